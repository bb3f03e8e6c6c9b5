#!/usr/bin/env python
"""Benchmark of the pms reduction on one GB300: a large complex, a batch of
complexes in one pass, and a served request stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload all|torus|batch|serve]

The default run (``--workload all``) prints ONE JSON line whose headline is
columns/s on one Rips complex of a noisy torus (400 points, 5,000,179
columns), with two more objects beside it:

* ``batch``: 4096 Rips complexes (n ~ U[20, 120], half cube, half noisy
  circle) reduced in one segmented pass, complexes/s against plain pms one
  complex at a time on the same GPU; every instance is checked against its
  one-at-a-time result and against the oracle's twist.
* ``serve``: a Poisson stream of requests (m log-uniform in [10^3, 2*10^6],
  the three generator families, fresh seeds) through the continuous-batching
  server, served complexes/s and p50/p99 latency at saturation, against plain
  sequential pms on the same GPU; every request is checked against plain pms
  and against the oracle's twist.
* ``configs``: the 50-point Rips cube (20,875 columns) and the 512x512
  lower-star image (1,568,771 columns), pms device and end-to-end time, low
  and ess checked against the oracle's twist.
* ``variants``: the reference's six other algorithms (standard, twist,
  ph_row and their parallel forms) and pms on one 128x128 lower-star image,
  device time of one reduction each, every low checked against the oracle.

For the headline, one step = one full reduction of the complex (set-up,
sweeps, outputs) by the library's own choice of matrix.  ``value`` is
columns/s with the boundary matrix already in HBM; ``e2e`` is the same metric
through the drop-in ``openph()`` C call with pinned host COO in and host
outputs, copies included.  The roofline is the Phase II kernel that takes the
most time, timed with CUDA events on the library's stream in a second pass of
the same steps.  ``cpu_baseline`` is one whole reduction of the same complex
by the fixed-slot port of the reference's CPU twist on one host core.

``--impl reference`` times that fixed-slot port of the reference's CPU twist
(the reference's own build needs its source tree) on the host cores: each
step is one whole reduction of the same complex, and the steps run side by
side in one process per core.  For N > 1 every rank reduces its own replica
of the torus (no collective on the data path); rank 0 prints.

CPU work (the oracle checks, the CPU baselines, request generation) runs in
a pool of worker processes started with ``spawn`` before any CUDA use, and
never beside a timed GPU region that it could slow down except for the two
single-core torus jobs, which overlap the torus timing on 2 of the cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {"name": "rips_torus", "points": 400, "target_m": 5_000_000, "seed": 2,
            "torus": {"R": 2.0, "r": 1.0, "sigma": 0.05}}
BATCH = {"count": 4096, "seed": 4, "lo": 20, "hi": 120}
VARIANTS = {"side": 128, "seed": 3}
CONFIGS = {"rips_cube_points": 50, "rips_cube_seed": 1, "lower_star_side": 512, "lower_star_seed": 3}
SERVE = {"requests": 160, "m_lo": 1_000, "m_hi": 2_000_000, "seed": 5, "budget_bytes": 150 * (1 << 30),
         "rates_x_plain": [0.5, 1, 2, 4, 8, 16, 32]}
L2_FLUSH_BYTES = 512 << 20
COL_WIDTH = 80  # slot width factor for the fixed-slot CPU port (p = 240 >= widest column)


def log(*a):
    print("[bench]", *a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(x: float, dist, device=None) -> float:
    """Max of a float over all ranks (identity without a process group)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        if device is not None:
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


def host_cpu() -> str:
    """The host CPU model and its core count, as lscpu reports them."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return f"{model or 'unknown CPU'} x {os.cpu_count()} cores"


def mem_available_bytes() -> int:
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 16 << 30


def make_workload():
    from openph_gb300 import complexes as cx
    w = WORKLOAD
    pts = cx.points_torus(w["points"], seed=w["seed"], **w["torus"])
    thr = cx.rips_threshold(pts, w["target_m"])
    t0 = time.perf_counter()
    bm = cx.rips(pts, thr)
    bm.meta.update(threshold=thr, points=pts, host_rips_s=time.perf_counter() - t0)
    return bm


# ------------------------------------------------------------ pool jobs
# Functions run in the spawned worker processes (they import what they use).

def _bm(colptr, rows):
    from openph_gb300.complexes import BoundaryMatrix
    return BoundaryMatrix(colptr, rows)


def _job_twist_full(job):
    """The oracle's twist on one matrix: lows, ess and its statistics."""
    import oracle
    colptr, rows = job
    t0 = time.perf_counter()
    low, ess, st = oracle.twist(_bm(colptr, rows))
    st["wall"] = time.perf_counter() - t0
    return low, ess, st


def _job_config_oracle(job):
    """The oracle's twist on config 0 or 2 (regenerated here)."""
    from openph_gb300 import complexes as cx
    import oracle
    kind, size, seed = job
    bm = cx.rips_cube(size, seed=seed) if kind == "rips_cube" else cx.lower_star_image(size, size, seed=seed)
    low, ess, _ = oracle.twist(bm)
    return kind, low, ess


def _job_variants_oracle(job):
    """The oracle's twist on the variants' image (regenerated here)."""
    from openph_gb300 import complexes as cx
    import oracle
    side, seed = job
    low, _, _ = oracle.twist(cx.lower_star_image(side, side, seed=seed))
    return low


def _job_fixed_full(job):
    """One whole reduction by the fixed-slot port of the reference's twist
    (slot width raised until the reduction fits, as the reference's users
    do); the low array's checksum is returned for a parity check."""
    import oracle
    colptr, rows, width = job
    bm = _bm(colptr, rows)
    while True:
        t0 = time.perf_counter()
        rc, low, _, st = oracle.twist_fixed_p(bm, width)
        wall = time.perf_counter() - t0
        if rc == 0:
            return {"seconds": st["seconds"], "wall": wall, "col_width": width, "columns": st["columns_done"],
                    "additions": st["additions"], "low_checksum": low_checksum(low)}
        width *= 2


def low_checksum(low) -> int:
    """A position-weighted checksum of a low array (parity of runs that do
    not hand their whole output back)."""
    w = np.arange(1, len(low) + 1, dtype=np.int64) % 1000003
    return int(np.sum((low.astype(np.int64) + 2) * w) % (1 << 61))


def _job_fixed_prefix(job):
    """A bounded prefix of the fixed-slot port (warm-up of the reference arm)."""
    import oracle
    colptr, rows, width, seconds = job
    oracle.twist_fixed_p(_bm(colptr, rows), width, max_columns=0, max_seconds=seconds)
    return os.getpid()


def _job_batch_oracle(items):
    """Batch instances regenerated from their (points, seed) and reduced by
    the oracle's twist: [(b, low, ess, seconds of the twist)]."""
    import oracle
    from openph_gb300 import complexes as cx
    out = []
    for b, n, seed in items:
        _, colptr, rows = cx.rips_mixed_instances([n], [seed], threads=1)
        t0 = time.perf_counter()
        low, ess, _ = oracle.twist(_bm(colptr, rows))
        out.append((b, low, ess, time.perf_counter() - t0))
    return out


def _serve_matrix(kind, m, seed):
    from openph_gb300 import complexes as cx
    if kind == "rips_cube":
        n = max(4, int(round((6 * m) ** (1 / 3))))
        return cx.rips_cube(n, seed=seed)
    if kind == "rips_torus":
        return cx.rips_torus(400, m, seed=seed)
    side = max(4, int(round((m / 6) ** 0.5)))
    return cx.lower_star_image(side, side, seed=seed)


def _job_serve_request(job):
    """One request of the serving stream: (kind, target m, seed) -> CSC."""
    kind, m, seed = job
    bm = _serve_matrix(kind, m, seed)
    return kind, bm.colptr, bm.rows


def _job_serve_oracle(job):
    """One request regenerated and reduced by the oracle's twist."""
    import oracle
    k, kind, m, seed = job
    bm = _serve_matrix(kind, m, seed)
    t0 = time.perf_counter()
    low, ess, _ = oracle.twist(bm)
    return k, low, ess, time.perf_counter() - t0


def _job_warm(_):
    import oracle  # noqa: F401  (the port's library loaded once per worker)
    from openph_gb300 import complexes  # noqa: F401
    return os.getpid()


def start_pool(processes=None):
    import multiprocessing as mp
    n = processes or os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(n)
    pool.map(_job_warm, range(2 * n))
    return pool, n


# ------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"oph_clocks_{os.getpid()}_{id(self)}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------- reference arm
def run_reference(args, ws, rank):
    """The fixed-slot port of the reference's CPU twist on the host cores:
    each step is one whole reduction of the torus, the steps side by side,
    one process per core (as many as the host's memory holds)."""
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    bm = make_workload()
    m, nnz = bm.m, bm.nnz
    width = COL_WIDTH
    per_proc = 2 * 4 * m * width * int(np.diff(bm.colptr).max()) + (1 << 30)
    procs = max(1, min(args.steps, os.cpu_count() or 1, int(0.75 * mem_available_bytes()) // per_proc))
    pool, _ = start_pool(procs)
    job = (bm.colptr, bm.rows)
    pool.map(_job_fixed_prefix, [job + (width, 1.0)] * max(args.warmup, procs))
    log(f"reference arm: {args.steps} whole reductions on {procs} processes")
    t0 = time.perf_counter()
    res = pool.map(_job_fixed_full, [job + (width,)] * args.steps, chunksize=1)
    wall = time.perf_counter() - t0
    pool.close()
    pool.join()
    value = args.steps * m / wall
    per_proc_rate = m / float(np.mean([r["seconds"] for r in res]))
    line = {
        "metric": "cols/s", "value": value, "unit": "cols/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "impl": "reference",
        "config": {"workload": f"rips_torus_{WORKLOAD['points']}pts_{m}cols", "m": m, "nnz": nnz,
                   "algorithm": "twist (reference CPU reduction, fixed-slot layout)",
                   "col_width": res[0]["col_width"], "seed": WORKLOAD["seed"]},
        "cpu_baseline": {"value": value, "unit": "cols/s", "cores": procs, "kind": "port",
                         "sample": f"{args.steps} whole reductions of the same matrix ({m} columns each), "
                                   f"{procs} at a time, one per process, on {host_cpu()}; one reduction takes "
                                   f"{np.mean([r['seconds'] for r in res]):.1f} s of twist "
                                   f"({per_proc_rate:.0f} cols/s per core); the reference's twist is "
                                   "single-threaded",
                         "per_core_value": per_proc_rate},
        "e2e": {"value": value, "unit": "cols/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- torus
# What bounds each Phase II kernel, from its ncu captures (profiles/).
ROOFLINE_NOTES = {
    "tier3": "latency-bound: chains of dependent additions on a few long columns of the anti-transpose "
             "(each addition waits on its low's pivot record, then the pivot's rows, from L2 or HBM); the "
             "merge-equivalent bytes are what a merge would move, far above the kernels' DRAM traffic",
    "narrow": "instruction-issue-bound (ncu: 60-89% issue active, DRAM 1-2%); T stays on chip per chain",
}


def load_traffic():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def algorithmic_bytes(bm, st) -> dict:
    """Bytes per reduction by the reference's layout: the CSC read once, low
    written, and for every twist addition |P| + |T| read and |T xor P| written
    (int32 slots)."""
    base = 4 * (bm.nnz + bm.m + 1) + 4 * bm.m
    adds = 4 * (st["slots_read"] + st["slots_written"])
    return {"total": base + adds, "additions": adds, "twist_additions": st["additions"]}


def device_generation(bm, ctx, device, reps=3) -> dict:
    """The same complex built on the GPU from the points (best of a few
    runs, wall time of the call, which returns with the matrix in HBM),
    beside the host generator's time, and whether the two are identical."""
    import torch

    from openph_gb300 import complexes as cx
    pts = torch.from_numpy(bm.meta["points"]).to(device)
    torch.cuda.synchronize()
    best, dm = None, None
    for _ in range(reps):
        t0 = time.perf_counter()
        dm = cx.rips_device(pts, bm.meta["threshold"], ctx=ctx, device=device)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    h = dm.to_host()
    same = bool(np.array_equal(h.colptr, bm.colptr) and np.array_equal(h.rows, bm.rows))
    return {"host_rips_s": bm.meta["host_rips_s"], "device_rips_ms": 1e3 * best, "device_equals_host": same,
            "api": "oph_rips_device (points in HBM -> sorted CSC in HBM)"}


def run_torus(args, ws, rank, local, bm, dist):
    """The headline: GPU timing of the torus (device-resident and end to
    end).  Returns the line without its oracle-dependent fields, and the
    device outputs to check."""
    import torch

    from openph_gb300 import api

    device = torch.device("cuda", local)
    m, nnz = bm.m, bm.nnz
    ctx = api.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    d_colptr = torch.from_numpy(bm.colptr).to(device)
    d_rows = torch.from_numpy(bm.rows).to(device)
    d_low = torch.empty(m, dtype=torch.int32, device=device)
    d_ess = torch.empty(m, dtype=torch.int32, device=device)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=device)
    torch.cuda.synchronize()

    def step():
        return ctx.reduce_device(m, d_colptr.data_ptr(), d_rows.data_ptr(), d_low.data_ptr(), d_ess.data_ptr(),
                                 None, "pms")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    infos = []
    barrier(dist, device)
    torch.cuda.synchronize()
    # the headline: the library's own schedule, no per-phase events
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(k)  # evict L2 between steps (512 MB write)
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            infos.append(step())
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    # the same steps again with CUDA events around every phase on the
    # library's stream (kernels launched one by one): the per-phase split,
    # the Phase II launch durations for the roofline and the launch count
    ctx.set_profile(True)
    narrow_ms, p1_ms, setup_ms, launches, p2_launches = 0.0, 0.0, 0.0, 0, 0
    tier_ms = [0.0, 0.0, 0.0]
    ev_prof = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k)
        torch.cuda.synchronize()
        ev_prof[k][0].record(stream)
        step()
        ev_prof[k][1].record(stream)
        prof = ctx.last_profile()
        narrow_ms += prof["phase2_narrow_ms"]
        tier_ms = [x + y for x, y in zip(tier_ms, prof["tier_ms"])]
        p1_ms += prof["phase1_ms"]
        setup_ms += prof["setup_ms"]
        launches += prof["kernel_launches"]
        p2_launches += prof["phase2_launches"]
    torch.cuda.synchronize()
    profiled_ms = sum(a.elapsed_time(b) for a, b in ev_prof) / args.steps
    # the exact |P| + |T| + |T xor P| of every addition per tier, from one
    # more (untimed) reduction of the same matrix with slot tracking on
    ctx.set_profile(True, slots=True)
    step()
    slot_prof = ctx.last_profile()
    ctx.set_profile(False)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = max_over_ranks(sum(step_ms) / 1e3, dist, device)
    barrier(dist, device)

    # end to end through the drop-in C call: pinned host COO in, host low/ess out
    r1, c1 = bm.to_coo1()
    h_r = torch.from_numpy(r1).pin_memory()
    h_c = torch.from_numpy(c1).pin_memory()
    h_low = torch.empty(m, dtype=torch.int32).pin_memory()
    h_ess = torch.empty(m, dtype=torch.int32).pin_memory()
    it = np.zeros(1, np.int32)
    L = api.lib()
    fn = L.oph_openph
    fn.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]

    def e2e_step():
        rc = fn(b"pms", h_r.data_ptr(), h_c.data_ptr(), m, 0, None, nnz, h_low.data_ptr(), h_ess.data_ptr(), None,
                None, None, None, None, it.ctypes.data, local)
        if rc != 0:
            raise api.OphError(rc, "openph")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sum(e2e_times), dist, device)

    generation = device_generation(bm, ctx, device) if rank == 0 else None
    low_gpu = d_low.cpu().numpy()
    ess_gpu = d_ess.cpu().numpy()
    low_e2e = h_low.numpy().copy()
    ess_e2e = h_ess.numpy().copy()

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    # the dominant Phase II kernel (one launch per sweep, CUDA events around
    # each tier on the library's stream): its algorithmic bytes are the
    # per-addition figure 4 (|P| + |T| + |T xor P|) summed over the additions
    # it performed (counted on the device), per launch, over its mean launch
    # time.  On the anti-transpose that is tier 3's bitmap kernel.
    comps = {"narrow": (narrow_ms, slot_prof["tier_slots"][0],
                        "k_p2_scalar + k_p2_tier<8,128,256> (scalar tier and tier 0, a pair per sweep)"),
             "tier1": (tier_ms[0], slot_prof["tier_slots"][1], "k_p2_tier1<32,512,256> (tier 1)"),
             "tier2": (tier_ms[1], slot_prof["tier_slots"][2], "k_p2_block<8192,256> (tier 2)"),
             "tier3": (tier_ms[2], slot_prof["tier_slots"][3],
                       "k_p2_bitmap<1024> + k_p2_cluster<8> (tier 3: bitmap columns in one CTA's shared window, "
                       "wider ones across a cluster's shared memory; one launch of each per sweep)")}
    dom = max(comps, key=lambda k: comps[k][0])
    dom_ms, dom_slots, dom_name = comps[dom]
    per_red_dom_s = dom_ms / 1e3 / args.steps
    launches_per_red = p2_launches / args.steps
    dom_bytes = 4 * dom_slots
    achieved = dom_bytes / per_red_dom_s / 1e9 if per_red_dom_s > 0 else None
    traffic = load_traffic()
    if traffic and traffic.get("component") != dom:
        traffic = None
    line = {
        "metric": "cols/s", "value": ws * m * args.steps / total_s, "unit": "cols/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator; replicas on every rank)",
        "config": {"workload": f"rips_torus_{WORKLOAD['points']}pts_{m}cols", "m": m, "nnz": nnz,
                   "algorithm": "pms", "seed": WORKLOAD["seed"], "threshold": bm.meta["threshold"],
                   "l2": "flushed between steps (512 MB write)", "parallelism": f"replicas x{ws}"},
        "complexes_per_s": ws * args.steps / total_s,
        "e2e": {"value": ws * m * args.steps / e2e_s, "unit": "cols/s", "h2d_bytes_per_step": 8 * nnz,
                "d2h_bytes_per_step": 8 * m, "ms_per_step": 1e3 * e2e_s / args.steps, "api": "openph() C ABI"},
        "roofline": {"bound": "hbm", "kernel": dom_name,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else "fallback",
                     "algorithmic_bytes_per_launch": dom_bytes / launches_per_red if launches_per_red else None,
                     "mean_launch_ms": dom_ms / max(1, p2_launches),
                     "launches_per_reduction": launches_per_red,
                     "traffic": (traffic or {}).get("bytes_per_launch"),
                     "traffic_source": (traffic or {}).get("source"),
                     "note": ROOFLINE_NOTES.get(dom)},
        "phases_ms_per_step": {"setup_and_transpose": setup_ms / args.steps, "phase1": p1_ms / args.steps,
                               "phase2_narrow": narrow_ms / args.steps, "tier1": tier_ms[0] / args.steps,
                               "tier2": tier_ms[1] / args.steps, "tier3": tier_ms[2] / args.steps,
                               "total_launched_one_by_one": profiled_ms,
                               "note": "a second pass of the same steps with events around every phase "
                                       "(no CUDA graph); the headline pass replays the captured sweeps"},
        "matrix_reduced": "anti-transpose D' (OPH_DUAL_AUTO)" if infos[-1]["dual"] else "D",
        "sweeps": infos[-1]["sweeps"], "device_additions": infos[-1]["additions"],
        "device_slots_per_tier": slot_prof["tier_slots"],
        "generation": generation,
        "clocks": clocks.summary(),
        "gpu_launches": launches,
        "gpu_launches_source": "kernel launches counted by the library over the profiled pass of the same steps",
    }
    ctx.close()
    del d_colptr, d_rows, d_low, d_ess, flush
    torch.cuda.empty_cache()
    return line, (low_gpu, ess_gpu, low_e2e, ess_e2e)


# --------------------------------------------------------------- batch
def run_batch(args, local, pool, cores, count, before_timing=None):
    """The batched workload: `count` Rips complexes in one segmented pass,
    against plain pms one complex at a time on the same GPU, every instance
    checked against its one-at-a-time result and the oracle's twist."""
    import torch

    from openph_gb300 import api
    from openph_gb300 import complexes as cx

    device = torch.device("cuda", local)
    t0 = time.perf_counter()
    col_off, colptr, rows, npts, seeds = cx.rips_mixed_batch(count, BATCH["seed"], lo=BATCH["lo"], hi=BATCH["hi"])
    gen_s = time.perf_counter() - t0
    total_m, total_nnz = int(col_off[-1]), int(colptr[-1])
    log(f"batch: {count} complexes, {total_m} columns, generated in {gen_s:.1f} s")
    if before_timing is not None:
        before_timing()  # no pool work beside the timed region
    ctx = api.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    d_off = torch.from_numpy(col_off).to(device)
    d_colptr = torch.from_numpy(colptr).to(device)
    d_rows = torch.from_numpy(rows).to(device)
    d_low = torch.empty(total_m, dtype=torch.int32, device=device)
    d_ess = torch.empty(total_m, dtype=torch.int32, device=device)
    torch.cuda.synchronize()

    def batched():
        return ctx.reduce_batch_device(count, d_off.data_ptr(), d_colptr.data_ptr(), d_rows.data_ptr(), total_m,
                                       total_nnz, d_low.data_ptr(), d_ess.data_ptr(), "pms")

    for _ in range(args.warmup):
        batched()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            info = batched()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    batch_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    # the kernel launches of one step, counted by the library in a profiled
    # (untimed) repeat of the same step
    ctx.set_profile(True)
    batched()
    launches = ctx.last_profile()["kernel_launches"] * args.steps
    ctx.set_profile(False)
    low_batch = d_low.cpu().numpy()
    ess_batch = d_ess.cpu().numpy()

    # plain pms, one complex at a time, device-resident inputs
    d_low1 = torch.empty(int(np.diff(col_off).max()), dtype=torch.int32, device=device)
    colptr_d = [torch.from_numpy(colptr[col_off[b]:col_off[b + 1] + 1] - colptr[col_off[b]]).to(device)
                for b in range(count)]
    rows_d = [d_rows[int(colptr[col_off[b]]):int(colptr[col_off[b + 1]])] for b in range(count)]
    for b in range(min(count, 8)):
        ctx.reduce_device(int(col_off[b + 1] - col_off[b]), colptr_d[b].data_ptr(), rows_d[b].data_ptr(),
                          d_low1.data_ptr(), None, None, "pms")
    torch.cuda.synchronize()
    mismatches = 0
    seq_ms = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for b in range(count):
        mb = int(col_off[b + 1] - col_off[b])
        e0.record(stream)
        ctx.reduce_device(mb, colptr_d[b].data_ptr(), rows_d[b].data_ptr(), d_low1.data_ptr(), None, None, "pms")
        e1.record(stream)
        e1.synchronize()
        seq_ms += e0.elapsed_time(e1)
        if not np.array_equal(d_low1[:mb].cpu().numpy(), low_batch[col_off[b]:col_off[b + 1]]):
            mismatches += 1
    seq_s = seq_ms / 1e3
    del colptr_d, rows_d, d_low1

    # end to end through the C ABI: pinned host CSC in, host lows out
    h_off = torch.from_numpy(col_off).pin_memory()
    h_colptr = torch.from_numpy(colptr).pin_memory()
    h_rows = torch.from_numpy(rows).pin_memory()
    h_low = torch.empty(total_m, dtype=torch.int32).pin_memory()
    L = api.lib()
    e2e_info = api.Info()

    def e2e_step():
        rc = L.oph_reduce_batch(ctx._h, api.algo_id("pms"), count, h_off.numpy(), h_colptr.numpy(),
                                C.c_void_p(h_rows.data_ptr()), h_low.numpy(), None, C.byref(e2e_info))
        if rc != 0:
            raise api.OphError(rc, "oph_reduce_batch")

    e2e_step()
    e2e_s = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_s += time.perf_counter() - t0
    e2e_equal = bool(np.array_equal(h_low.numpy(), low_batch))
    ctx.close()
    del d_off, d_colptr, d_rows, d_low, d_ess, h_off, h_colptr, h_rows, h_low
    torch.cuda.empty_cache()

    # every instance against the oracle's twist, regenerated in the workers
    # (all host cores; nothing on the GPU meanwhile)
    log("batch: oracle over every instance")
    order = np.argsort(-np.diff(col_off))  # largest first, for an even finish
    chunks = [[(int(b), int(npts[b]), int(seeds[b])) for b in order[i:i + 4]] for i in range(0, count, 4)]
    t0 = time.perf_counter()
    oracle_bad, twist_s = [], 0.0
    for res in pool.imap_unordered(_job_batch_oracle, chunks):
        for b, low, ess, secs in res:
            twist_s += secs
            c0, c1 = int(col_off[b]), int(col_off[b + 1])
            if not (np.array_equal(low, low_batch[c0:c1]) and np.array_equal(ess, ess_batch[c0:c1])):
                oracle_bad.append(b)
    oracle_wall = time.perf_counter() - t0
    return {
        "metric": "complexes/s", "value": count * args.steps / batch_s, "unit": "complexes/s",
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * batch_s / args.steps,
        "config": {"workload": f"rips_mixed_batch_{count}", "total_m": total_m, "total_nnz": total_nnz,
                   "points": [BATCH["lo"], BATCH["hi"]], "seed": BATCH["seed"], "algorithm": "pms",
                   "l2": "inputs (%.1f GB) larger than L2" % ((total_nnz * 4 + total_m * 8) / 1e9)},
        "plain_sequential": {"complexes_per_s": count / seq_s, "s_total": seq_s,
                             "api": "oph_reduce_device, one complex at a time, device-resident inputs"},
        "batched_over_plain": (count * args.steps / batch_s) / (count / seq_s),
        "e2e": {"value": count * args.steps / e2e_s, "unit": "complexes/s",
                "h2d_bytes_per_step": 8 * (count + 1) + 8 * (total_m + 1) + 4 * total_nnz,
                "d2h_bytes_per_step": 4 * total_m, "ms_per_step": 1e3 * e2e_s / args.steps,
                "api": "oph_reduce_batch C ABI", "equal_to_device_run": e2e_equal},
        "cpu_baseline": {"value": count / (twist_s / cores), "unit": "complexes/s", "cores": cores, "kind": "port",
                         "sample": f"all {count} instances through the oracle's twist (the reference's twist "
                                   f"restated on adaptive columns), one instance per process on {host_cpu()}: "
                                   f"{twist_s:.1f} core-seconds of twist, {oracle_wall:.1f} s wall"},
        "cols_per_s": total_m * args.steps / batch_s,
        "matrix_reduced": "anti-transpose D' (OPH_DUAL_AUTO)" if info["dual"] else "D",
        "sweeps": info["sweeps"], "device_additions": info["additions"], "regrows": info["regrows"],
        "pool_bytes": info["pool_bytes"],
        "parity": {"batched_equals_one_at_a_time": mismatches == 0, "mismatched_instances": mismatches,
                   "oracle_checked": count, "oracle_equal": not oracle_bad, "oracle_mismatches": oracle_bad[:20]},
        "generation_s": gen_s, "clocks": clocks.summary(), "gpu_launches": launches,
    }


# ------------------------------------------------------------- configs
def run_configs(local, pool):
    """The two single-complex configurations beside the headline: the
    50-point Rips cube (20,875 columns) and the 512x512 lower-star image
    (1,568,771 columns), pms through the library's own choice of matrix;
    device time (CUDA events) and wall time of the call with host CSC in and
    host low/ess out, the fastest of five after two warm-ups; low and ess
    checked against the oracle's twist (in the worker pool, waited for here,
    before the serve timing)."""
    from openph_gb300 import api
    from openph_gb300 import complexes as cx
    jobs = [("rips_cube", CONFIGS["rips_cube_points"], CONFIGS["rips_cube_seed"]),
            ("lower_star", CONFIGS["lower_star_side"], CONFIGS["lower_star_seed"])]
    want_async = pool.map_async(_job_config_oracle, jobs, chunksize=1)
    out = {}
    ctx = api.Context(local)
    for kind, size, seed in jobs:
        bm = cx.rips_cube(size, seed=seed) if kind == "rips_cube" else cx.lower_star_image(size, size, seed=seed)
        for _ in range(2):
            ctx.reduce(bm, "pms")
        dev, wall = [], []
        for _ in range(5):
            t0 = time.perf_counter()
            low, ess, info = ctx.reduce(bm, "pms")
            wall.append(time.perf_counter() - t0)
            dev.append(info["device_ms"])
        out[kind] = {"columns": bm.m, "device_ms": min(dev), "wall_ms": 1e3 * min(wall),
                     "cols_per_s": bm.m / (min(dev) / 1e3), "e2e_cols_per_s": bm.m / min(wall),
                     "matrix_reduced": {0: "D", 1: "D'", 2: "per block (D and D')"}[info["dual"]],
                     "sweeps": info["sweeps"], "low": low, "ess": ess}
    ctx.close()
    for kind, low, ess in want_async.get():
        v = out[kind]
        v["low_ess_equal_oracle"] = bool(np.array_equal(v.pop("low"), low) and np.array_equal(v.pop("ess"), ess))
    log("configs: " + ", ".join(f"{k} {v['device_ms']:.2f} ms" for k, v in out.items()))
    return out


# ------------------------------------------------------------ variants
def run_variants(local, pool):
    """The six other algorithms of the reference (standard, twist, ph_row and
    their parallel forms, each a single persistent GPU walker here) and pms
    on one lower-star image, one reduction each after a warm-up, device time
    of the call; every low checked against the oracle's twist."""
    from openph_gb300 import api
    from openph_gb300 import complexes as cx
    side, seed = VARIANTS["side"], VARIANTS["seed"]
    want_async = pool.apply_async(_job_variants_oracle, ((side, seed),))
    bm = cx.lower_star_image(side, side, seed=seed)
    out = {}
    ctx = api.Context(local)
    for algo in ("standard", "twist", "ph_row", "standard_parallel", "twist_parallel", "ph_row_parallel", "pms"):
        ctx.reduce(bm, algo)
        low, _, info = ctx.reduce(bm, algo)
        out[algo] = {"device_ms": info["device_ms"], "cols_per_s": bm.m / (info["device_ms"] / 1e3),
                     "low": low}
    ctx.close()
    want = want_async.get()
    for algo, v in out.items():
        v["low_equal_oracle"] = bool(np.array_equal(v.pop("low"), want))
    log("variants: " + ", ".join(f"{a} {v['device_ms']:.1f} ms" for a, v in out.items()))
    return {"matrix": f"lower-star image {side}x{side} (seed {seed}), {bm.m} columns", "algorithms": out,
            "api": "oph_reduce (host CSC in), device time of the reduction (CUDA events)"}


# --------------------------------------------------------------- serve
def serve_jobs(count, seed):
    """Request mix: sizes log-uniform in [m_lo, m_hi], kind uniform over the
    three generator families, fresh seeds."""
    rng = np.random.default_rng(seed)
    ms = np.exp(rng.uniform(np.log(SERVE["m_lo"]), np.log(SERVE["m_hi"]), size=count)).astype(np.int64)
    kinds = rng.choice(["rips_cube", "rips_torus", "lower_star"], size=count)
    seeds = rng.integers(1 << 30, size=count)
    return [(str(k), int(m), int(sd)) for k, m, sd in zip(kinds, ms, seeds)]


def run_serve(args, local, pool, cores, count, reqs_async):
    """Serving: a Poisson stream of reduction requests through the
    continuous-batching server (HBM budget 150 GB), rates swept to
    saturation; against plain pms one request at a time on the same GPU
    (host CSC in, host lows out, like the server); every request checked
    against plain pms and the oracle's twist."""
    import torch

    from openph_gb300 import api
    from openph_gb300.complexes import BoundaryMatrix
    jobs = serve_jobs(count, SERVE["seed"])
    reqs = [(k, BoundaryMatrix(cp, rw)) for k, cp, rw in reqs_async.get()]
    n = len(reqs)
    total_m = sum(bm.m for _, bm in reqs)
    log(f"serve: {n} requests, {total_m} columns")
    torch.cuda.set_device(local)
    # plain: one at a time, service time of each; two passes over the
    # stream, the faster one kept (the first also grows the context's
    # buffers to the largest request)
    ctx = api.Context(local)
    for _, bm in reqs[:3]:
        ctx.reduce(bm, "pms")
    passes, plain_low, plain_ess = [], [], []
    with ClockSampler(local) as clocks_plain:
        for p in range(2):
            service = []
            for _, bm in reqs:
                t0 = time.perf_counter()
                low, ess, _ = ctx.reduce(bm, "pms")
                service.append(time.perf_counter() - t0)
                if p == 0:
                    plain_low.append(low)
                    plain_ess.append(ess)
            passes.append(np.array(service))
    ctx.close()
    service = min(passes, key=lambda v: v.sum())
    plain_rate = n / service.sum()
    kinds = sorted({k for k, _ in reqs})
    log("serve: plain passes (ms) " + ", ".join(f"{1e3 * v.sum():.1f}" for v in passes) + " | by kind: " +
        ", ".join(f"{kd} {1e3 * sum(t for (k, _), t in zip(reqs, service) if k == kd):.1f}" for kd in kinds))

    srv = api.Server(local, budget_bytes=SERVE["budget_bytes"], max_active=4096)
    for _, bm in reqs[:3]:  # warm-up
        srv.wait(srv.submit(bm))
    rng = np.random.default_rng(SERVE["seed"] + 1)
    results, mism = [], 0
    with ClockSampler(local) as clocks:
        for x in SERVE["rates_x_plain"]:
            rate = x * plain_rate
            arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
            tickets = [None] * n
            t_start = time.perf_counter()

            def producer():
                for k, (_, bm) in enumerate(reqs):
                    delay = arrivals[k] - (time.perf_counter() - t_start)
                    if delay > 0:
                        time.sleep(delay)
                    tickets[k] = srv.submit(bm)

            th = threading.Thread(target=producer)
            th.start()
            lat, done_ms, sub_ms = [], [], []
            for k in range(n):
                while tickets[k] is None:
                    time.sleep(0.0002)
                low, ess, info = srv.wait(tickets[k])
                lat.append(info["latency_ms"])
                done_ms.append(info["done_ms"])
                sub_ms.append(info["submit_ms"])
                if not (np.array_equal(low, plain_low[k]) and np.array_equal(ess, plain_ess[k])):
                    mism += 1
            th.join()
            span_s = (max(done_ms) - min(sub_ms)) / 1e3
            # plain pms at the same arrivals: a FIFO single server with the
            # measured service times
            fin, plat = 0.0, []
            for k in range(n):
                fin = max(fin, arrivals[k]) + service[k]
                plat.append(1e3 * (fin - arrivals[k]))
            results.append({"offered_per_s": rate, "served_per_s": n / span_s,
                            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                            "plain_p50_ms": float(np.percentile(plat, 50)),
                            "plain_p99_ms": float(np.percentile(plat, 99)),
                            "plain_served_per_s": n / max(fin, arrivals[-1])})
    counters = srv.stats()
    srv.close()
    torch.cuda.empty_cache()

    # every request against the oracle's twist (regenerated in the workers)
    log("serve: oracle over every request")
    t0 = time.perf_counter()
    oracle_bad, twist_s = [], 0.0
    order = np.argsort([-bm.m for _, bm in reqs])
    for k, low, ess, secs in pool.imap_unordered(_job_serve_oracle, [(int(k),) + jobs[k] for k in order]):
        twist_s += secs
        if not (np.array_equal(low, plain_low[k]) and np.array_equal(ess, plain_ess[k])):
            oracle_bad.append(k)
    oracle_wall = time.perf_counter() - t0
    best = max(results, key=lambda r: r["served_per_s"])
    return {
        "metric": "complexes/s", "value": best["served_per_s"], "unit": "complexes/s",
        "rates": len(results),
        "config": {"workload": "serving_poisson_stream", "requests": n, "total_m": total_m,
                   "m_range": [SERVE["m_lo"], SERVE["m_hi"]], "budget_gb": SERVE["budget_bytes"] / (1 << 30),
                   "kinds": sorted({k for k, _ in reqs}), "seed": SERVE["seed"]},
        "plain_sequential": {"complexes_per_s": plain_rate, "mean_service_ms": 1e3 * service.mean(),
                             "passes_ms": [1e3 * float(v.sum()) for v in passes],
                             "api": "oph_reduce (host CSC in, host low/ess out), one request at a time; "
                                    "the faster of two passes over the stream",
                             "clocks": clocks_plain.summary()},
        "served_over_plain_at_saturation": best["served_per_s"] / plain_rate,
        "p50_ms_at_saturation": best["p50_ms"], "p99_ms_at_saturation": best["p99_ms"],
        "rate_sweep": results, "server": counters,
        "e2e": {"value": best["served_per_s"], "unit": "complexes/s",
                "h2d_bytes_per_step": int(np.mean([8 * (bm.m + 1) + 4 * bm.nnz for _, bm in reqs])),
                "d2h_bytes_per_step": int(np.mean([8 * bm.m for _, bm in reqs])),
                "api": "oph_server_submit / oph_server_wait (host CSC in, host lows and ess out; a step = one "
                       "request)"},
        "cpu_baseline": {"value": n / (twist_s / cores), "unit": "complexes/s", "cores": cores, "kind": "port",
                         "sample": f"all {n} requests through the oracle's twist, one request per process on "
                                   f"{host_cpu()}: {twist_s:.1f} core-seconds of twist, {oracle_wall:.1f} s wall"},
        "parity": {"served_equals_plain": mism == 0, "mismatches": mism, "oracle_checked": n,
                   "oracle_equal": not oracle_bad, "oracle_mismatches": oracle_bad[:20]},
        "clocks": clocks.summary(),
    }


# ---------------------------------------------------------------- main
def run_ours(args, ws, rank, local):
    # the worker pool first: spawned before this process touches CUDA
    pool, cores = (start_pool() if rank == 0 else (None, 0))
    bm = make_workload()
    m = bm.m
    torus_jobs = None
    if rank == 0 and args.workload in ("all", "torus"):
        # the oracle's twist (parity, algorithmic bytes) and one whole
        # reduction by the fixed-slot port (the CPU baseline), each on one
        # core, beside the torus timing
        torus_jobs = (pool.apply_async(_job_twist_full, ((bm.colptr, bm.rows),)),
                      pool.apply_async(_job_fixed_full, ((bm.colptr, bm.rows, COL_WIDTH),)))
    import torch

    from openph_gb300 import api
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    dist = init_dist(ws, "nccl")
    api.lib()

    line, outs = None, None
    if args.workload in ("all", "torus"):
        log("torus: GPU timing")
        line, outs = run_torus(args, ws, rank, local, bm, dist)
    if rank != 0:
        barrier(dist, device)
        return 0
    ok = True
    if line is None:
        # a batch-only or serve-only run: that object becomes the line
        line = {"n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators)"}
    serve_async = None
    if args.workload in ("all", "serve"):
        # request generation on the pool (CPU only), while the batch runs
        serve_async = pool.map_async(_job_serve_request, serve_jobs(args.count or SERVE["requests"], SERVE["seed"]),
                                     chunksize=1)
    if args.workload in ("all", "batch"):
        batch = run_batch(args, local, pool, cores, args.count or BATCH["count"],
                          serve_async.wait if serve_async is not None else None)
        ok &= batch["parity"]["batched_equals_one_at_a_time"] and batch["parity"]["oracle_equal"]
        if args.workload == "batch":
            line.update(batch)
        else:
            line["batch"] = batch
    if torus_jobs is not None:
        low_o, ess_o, st = torus_jobs[0].get()
        fixed = torus_jobs[1].get()
        low_gpu, ess_gpu, low_e2e, ess_e2e = outs
        parity = bool(np.array_equal(low_gpu, low_o) and np.array_equal(ess_gpu, ess_o))
        parity_e2e = bool(np.array_equal(low_e2e, low_o + 1) and np.array_equal(ess_e2e, ess_o))
        ok &= parity and parity_e2e
        ab = algorithmic_bytes(bm, st)
        step_s = line["ms_per_step"] / 1e3
        line["cpu_baseline"] = {
            "value": m / fixed["seconds"], "unit": "cols/s", "cores": 1, "kind": "port",
            "sample": f"one whole reduction of the same matrix ({fixed['columns']} columns reduced, "
                      f"{fixed['additions']} additions) by the fixed-slot port of the reference's twist "
                      f"(col_width {fixed['col_width']}), {fixed['seconds']:.1f} s on one core of {host_cpu()}",
            "adaptive_restatement_s": st["seconds"]}
        line["parity"] = {"low_ess_equal_oracle": parity, "e2e_low_ess_equal_oracle": parity_e2e,
                          "cpu_baseline_low_equal_oracle": fixed["low_checksum"] == low_checksum(low_o)}
        line["twist_additions_on_d"] = st["additions"]
        line["roofline"]["twist_on_d_algorithmic_bytes_per_reduction"] = ab["additions"]
        # the reduction-level figure of the algorithmic byte count: D's twist
        # work (the reference's) over the time this library takes for the
        # whole reduction; above 1 on the anti-transpose, which skips that work
        line["reduction_bytes"] = {
            "bytes_per_reduction": ab["total"], "per_s_gbs": ab["total"] / step_s / 1e9,
            "frac_of_peak": ab["total"] / step_s / 1e9 / line["roofline"]["peak"],
            "definition": "4 (nnz + m + 1) + 4 m + 4 (|P| + |T| + |T xor P|) over the CPU twist's additions on "
                          "D, per reduction; not a bandwidth achieved (the anti-transpose avoids that work)"}
    if args.workload == "all":
        configs = run_configs(local, pool)
        ok &= all(v["low_ess_equal_oracle"] for v in configs.values())
        line["configs"] = configs
        variants = run_variants(local, pool)
        ok &= all(v["low_equal_oracle"] for v in variants["algorithms"].values())
        line["variants"] = variants
    if serve_async is not None:
        serve = run_serve(args, local, pool, cores, args.count or SERVE["requests"], serve_async)
        ok &= serve["parity"]["served_equals_plain"] and serve["parity"]["oracle_equal"]
        if args.workload == "serve":
            line.update(serve)
        else:
            line["serve"] = serve
    pool.close()
    pool.join()
    print(json.dumps(line), flush=True)
    if dist is not None:
        barrier(dist, device)
    return 0 if ok else 3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["all", "torus", "batch", "serve"], default="all",
                    help="all: the torus headline with the batch and serve objects; torus: the ~5M-column "
                         "complex alone; batch: 4096 complexes in one pass; serve: a Poisson request stream "
                         "through the continuous-batching server")
    ap.add_argument("--count", type=int, default=0, help="batch/serve: number of complexes / requests")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if ws > 1 and args.workload == "all":
        args.workload = "torus"  # replicas of the headline; the batch and serve objects are 1-GPU runs
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
