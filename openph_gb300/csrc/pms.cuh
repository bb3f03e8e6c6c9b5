// Shared between the pms driver (pms.cu) and the request server (server.cu).
#pragma once
#include "oph_host.h"

namespace oph {

// Device views of one pms reduction.  With `inst` set the columns belong to
// several independent instances (the server's active requests): each has its
// own pool region (ipool[2b] = bump pointer, ipool[2b+1] = end), its own
// repeated-low count per sweep (ireps[b]) and its own overflow flag.
struct PmsArgs {
    int64_t m;
    int32_t *low;
    int8_t *classes;
    uint8_t *clear;
    const int8_t *dim;
    int32_t *first;
    const int32_t *beta;
    int32_t *worklist;
    int32_t *widelist;
    int64_t *seg;
    PivRec *rec;
    int32_t *agg;
    int64_t ntiles;
    int *pool;
    DevStatus *st;
    int *inst;                    // per column: instance slot, or nullptr (one instance)
    unsigned long long *ipool;    // per instance: bump pointer, end
    int *ireps;                   // per instance: repeated lows seen by the last Phase I
    int *iover;                   // per instance: a pool allocation failed
    // compacted Phase I (single matrix): the unresolved columns in column
    // order, ping-ponged between two arrays; counts in ucur / unext
    int32_t *ulist;               // nullptr: Phase I visits every column
    int32_t *ulist_next;
    int *ucur, *unext;
    int32_t *kagg;                // per tile: columns kept, then their offsets
    // Phase II tier-0 queue (the compacted list, or the worklist)
    int32_t *t0_list;
    int *t0_count;
    // the scalar tier's hand-off list to tier 0 (nullptr: no scalar tier)
    int32_t *slist;
    // exact |P| + |T| + |T xor P| counters in the lazy tiers (profiling)
    int stats;
    // buckets in ascending order (with the compacted list): Phase II takes
    // columns of the lowest bucket that has unresolved ones and of those
    // below, so that the pivots of a bucket clear the next one's columns
    // before they are reduced (twist's order; for the anti-transpose)
    int ascending;
    // tier 3's bitmaps: bm_words 32-bit words per CTA of its grid (nullptr:
    // tier 3 merges)
    uint32_t *bm;
    int64_t bm_words;
    // tier 4: columns wider than a CTA's shared window go to the cluster
    // tier (a bitmap across a cluster's shared memory) instead of the
    // global bitmap (0: tier 3 keeps them)
    int cluster_tier;
    // the bitmap tiers' additions per column per sweep (0: no limit); a
    // column that reaches it is written back unresolved and goes on in the
    // next sweep, so no sweep waits on one long chain (the request server,
    // whose sweeps serve every active request)
    int chain_cap;
    // per-instance bucket order (the server, whose instances are reduced on
    // D or on their anti-transpose; nullptr: `ascending` above for all):
    // iasc[b] = 1 for an instance in ascending order, ibucket[b * MAXC + d]
    // its unresolved columns of bucket d seen by this sweep's Phase I, and
    // iopen[b] the highest bucket its Phase II takes (MAXC: every bucket)
    const int8_t *iasc;
    int *ibucket;
    int *iopen;
    int nslots;
};

// Launch geometry of the Phase II tiers (occupancy-derived, per device).
constexpr int T0_CANDIDATES = 7;
// Lanes per column and shared capacity of tier-0 candidate v (-1 if none).
int t0_candidate(int v, int *lanes, int *cap);

struct SweepGrids {
    int v0;                 // tier-0 candidate in use
    int m, t;               // grid of the per-column passes, Phase I tiles
    int g0, g1, g2, g3;     // Phase II tier grids
    int g4;                 //   the cluster tier's (a multiple of its cluster size; 0: none)
    int gs;                 //   and the scalar tier's
    size_t s0, s1, s2, ss;  // their dynamic shared memory
};

int sweep_grids(Context *ctx, int64_t m, int64_t ntiles, SweepGrids *g);
// One sweep (Phase I, Phase II tiers, sweep counter) on `stream`; with a
// compacted list, `parity` selects which of the two arrays is current; ev
// (optional, 6 events): before Phase I, after Phase I, after each tier.
void launch_sweep(const PmsArgs &a, const SweepGrids &g, cudaStream_t stream, int parity = 0,
                  cudaEvent_t *ev = nullptr);
// Phase 0 over columns [c0, c1).
void launch_phase0(const PmsArgs &a, int64_t c0, int64_t c1, int grid, cudaStream_t stream);

}  // namespace oph
