#!/usr/bin/env python
"""Benchmark: pms on one Rips complex of a noisy torus (~5M columns).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one full pms reduction of the complex (set-up, sweeps, outputs),
by the library's own choice of matrix (the anti-transpose, for this complex).
``value`` is columns/s with the boundary matrix already resident in HBM;
``e2e`` is the same metric through the drop-in ``openph()`` C call with host
(pinned) COO input and host outputs, copies included.  The roofline is the
Phase II kernel that takes the most time, timed with CUDA events on the
library's stream in a second pass of the same steps.  ``cpu_baseline`` is the
fixed-slot port of the reference's CPU twist on a bounded prefix of the same
reduction.

``--impl reference`` times the reference's CPU twist (its port; the
reference's own build needs its source tree) on the host cores, on the same
matrix and metric.  For N > 1 every rank reduces its own replica (no
collective on the data path); rank 0 prints.
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
CPU_SAMPLE_SECONDS = 15.0
REF_STEP_SECONDS = 3.0
L2_FLUSH_BYTES = 512 << 20
COL_WIDTH = 80  # slot width factor for the fixed-slot CPU port (p = 240 >= widest column)


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


def make_workload():
    from openph_gb300 import complexes as cx
    w = WORKLOAD
    pts = cx.points_torus(w["points"], seed=w["seed"], **w["torus"])
    thr = cx.rips_threshold(pts, w["target_m"])
    t0 = time.perf_counter()
    bm = cx.rips(pts, thr)
    bm.meta.update(threshold=thr, points=pts, host_rips_s=time.perf_counter() - t0)
    return bm


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


def algorithmic_bytes(bm, st) -> dict:
    """Bytes per reduction by the reference's layout: the CSC read once, low
    written, and for every twist addition |P| + |T| read and |T xor P| written
    (int32 slots)."""
    base = 4 * (bm.nnz + bm.m + 1) + 4 * bm.m
    adds = 4 * (st["slots_read"] + st["slots_written"])
    return {"total": base + adds, "additions": adds, "twist_additions": st["additions"]}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"oph_clocks_{os.getpid()}.csv"

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


def cpu_port_sample(bm, seconds: float):
    """The fixed-slot twist port on a bounded prefix of the reduction order."""
    import oracle
    rc, _, _, st = oracle.twist_fixed_p(bm, COL_WIDTH, max_columns=0, max_seconds=seconds)
    if rc != 0:
        raise RuntimeError(f"CPU port failed with status {rc}")
    return st["columns_done"] / st["seconds"], st


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    bm = make_workload()
    for _ in range(args.warmup):
        cpu_port_sample(bm, 0.5)
    rates, cols, secs = [], 0, 0.0
    for _ in range(args.steps):
        r, st = cpu_port_sample(bm, REF_STEP_SECONDS)
        rates.append(r)
        cols += st["columns_done"]
        secs += st["seconds"]
    value = cols / secs
    line = {
        "metric": "cols/s", "value": value, "unit": "cols/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "impl": "reference",
        "config": {"workload": f"rips_torus_{WORKLOAD['points']}pts_{bm.m}cols", "m": bm.m, "nnz": bm.nnz,
                   "algorithm": "twist (reference CPU reduction, fixed-slot layout)", "col_width": COL_WIDTH,
                   "seed": WORKLOAD["seed"]},
        "cpu_baseline": {"value": value, "unit": "cols/s", "cores": 1, "kind": "port",
                         "sample": f"first columns of the twist order of the same matrix, {REF_STEP_SECONDS:.0f} s "
                                   f"per step ({cols} columns over {args.steps} steps); the reference's twist is "
                                   "single-threaded"},
        "e2e": {"value": value, "unit": "cols/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# What bounds each Phase II kernel, from its ncu captures (profiles/).
ROOFLINE_NOTES = {
    "tier3": "latency-bound: chains of dependent additions on a few long columns of the anti-transpose "
             "(ncu: 0.4% SM throughput, DRAM idle, the bitmaps in L2); the merge-equivalent bytes are "
             "what a merge would move, ~58x the kernel's DRAM traffic",
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


def run_ours(args, ws, rank, local):
    import torch

    from openph_gb300 import api

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    dist = init_dist(ws, "nccl")
    api.lib()
    bm = make_workload()
    m, nnz = bm.m, bm.nnz

    # the oracle: full CPU twist in the background (algorithmic bytes and a
    # bit-exact check of the GPU result at full size); rank 0 only
    oracle_out = {}

    def oracle_job():
        import oracle
        low, ess, st = oracle.twist(bm)
        oracle_out.update(low=low, ess=ess, st=st)

    th = None
    if rank == 0:
        import oracle
        oracle.build()
        th = threading.Thread(target=oracle_job, daemon=True)
        th.start()

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
    # the headline: the library's own schedule (sweeps replayed from its
    # captured CUDA graph), no per-phase events
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
    L.oph_openph.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_int]

    def e2e_step():
        rc = L.oph_openph(b"pms", h_r.data_ptr(), h_c.data_ptr(), m, 0, None, nnz, h_low.data_ptr(),
                          h_ess.data_ptr(), None, None, None, None, None, it.ctypes.data, local)
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

    if rank != 0:
        barrier(dist, device)
        return 0

    generation = device_generation(bm, ctx, device)
    th.join()
    st = oracle_out["st"]
    low_gpu = d_low.cpu().numpy()
    parity = bool(np.array_equal(low_gpu, oracle_out["low"]) and np.array_equal(d_ess.cpu().numpy(),
                                                                               oracle_out["ess"]))
    parity_e2e = bool(np.array_equal(h_low.numpy(), oracle_out["low"] + 1))
    cpu_rate, cpu_st = cpu_port_sample(bm, CPU_SAMPLE_SECONDS)

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    ab = algorithmic_bytes(bm, st)
    # the dominant Phase II kernel (one launch per sweep, CUDA events around
    # each tier on the library's stream): its algorithmic bytes are the
    # per-addition figure 4 (|P| + |T| + |T xor P|) summed over the additions
    # it performed (counted on the device), per launch, over its mean launch
    # time.  On the anti-transpose that is tier 3's bitmap kernel.
    comps = {"narrow": (narrow_ms, slot_prof["tier_slots"][0],
                        "k_p2_scalar + k_p2_tier<8,128,256> (scalar tier and tier 0, a pair per sweep)"),
             "tier1": (tier_ms[0], slot_prof["tier_slots"][1], "k_p2_tier1<32,512,256> (tier 1)"),
             "tier2": (tier_ms[1], slot_prof["tier_slots"][2], "k_p2_block<8192,256> (tier 2)"),
             "tier3": (tier_ms[2], slot_prof["tier_slots"][3], "k_p2_bitmap<1024> (tier 3, bitmap columns)")}
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
                     "twist_on_d_algorithmic_bytes_per_reduction": ab["additions"],
                     "traffic": (traffic or {}).get("bytes_per_launch"),
                     "traffic_source": (traffic or {}).get("source"),
                     "note": ROOFLINE_NOTES.get(dom)},
        # the reduction-level figure of the algorithmic byte count: D's twist
        # work (the reference's) over the time this library takes for the
        # whole reduction; above 1 on the anti-transpose, which skips that work
        "reduction_bytes": {"bytes_per_reduction": ab["total"],
                            "per_s_gbs": ab["total"] / (total_s / args.steps) / 1e9,
                            "frac_of_peak": ab["total"] / (total_s / args.steps) / 1e9 / peak,
                            "definition": "4 (nnz + m + 1) + 4 m + 4 (|P| + |T| + |T xor P|) over the CPU "
                                          "twist's additions on D, per reduction"},
        "phases_ms_per_step": {"setup_and_transpose": setup_ms / args.steps, "phase1": p1_ms / args.steps,
                               "phase2_narrow": narrow_ms / args.steps, "tier1": tier_ms[0] / args.steps,
                               "tier2": tier_ms[1] / args.steps, "tier3": tier_ms[2] / args.steps,
                               "total_launched_one_by_one": profiled_ms,
                               "note": "a second pass of the same steps with events around every phase "
                                       "(no CUDA graph); the headline pass replays the captured sweeps"},
        "matrix_reduced": "anti-transpose D' (OPH_DUAL_AUTO)" if infos[-1]["dual"] else "D",
        "sweeps": infos[-1]["sweeps"], "device_additions": infos[-1]["additions"],
        "device_slots_per_tier": slot_prof["tier_slots"],
        "twist_additions_on_d": st["additions"],
        "cpu_baseline": {"value": cpu_rate, "unit": "cols/s", "cores": 1, "kind": "port",
                         "sample": f"fixed-slot twist port, first {cpu_st['columns_done']} columns of the twist "
                                   f"order of the same matrix ({cpu_st['seconds']:.1f} s)"},
        "parity": {"low_ess_equal_oracle": parity, "e2e_low_equal_oracle": parity_e2e},
        "generation": generation,
        "clocks": clocks.summary(),
        "gpu_launches": launches,
        "gpu_launches_source": "kernel launches counted by the library over the profiled pass of the same steps",
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        barrier(dist, device)
    return 0 if (parity and parity_e2e) else 3


BATCH = {"count": 4096, "seed": 4, "lo": 20, "hi": 120}


def _batch_cpu_instance(job):
    """One batch instance through the reference-layout twist port (runs in a
    spawned worker; raises col_width until the instance fits, as the
    reference's users do)."""
    colptr, rows = job
    import oracle
    from openph_gb300.complexes import BoundaryMatrix
    bm = BoundaryMatrix(colptr, rows)
    width = COL_WIDTH
    while True:
        rc, _, _, st = oracle.twist_fixed_p(bm, width)
        if rc == 0:
            return st["seconds"]
        width *= 2


def cpu_batch_sample(col_off, colptr, rows, seconds: float) -> dict:
    """Complexes/s of the CPU twist port with one instance per process on
    every host core (spawned workers, the instances in order), over about
    `seconds` of wall time."""
    def jobs():
        for b in range(len(col_off) - 1):
            c0, c1 = int(col_off[b]), int(col_off[b + 1])
            yield colptr[c0:c1 + 1] - colptr[c0], rows[int(colptr[c0]):int(colptr[c1])]

    return cpu_pool_sample(jobs(), seconds, "instances of the batch")


def _pool_warm(_):
    import oracle  # noqa: F401  (loads the port's library once per worker)
    from openph_gb300 import complexes  # noqa: F401
    return os.getpid()


def cpu_pool_sample(jobs, seconds: float, what: str) -> dict:
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    done = 0
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_pool_warm, range(4 * cores))  # workers started and imported before the clock
        it = pool.imap(_batch_cpu_instance, jobs, chunksize=1)
        t0 = time.perf_counter()
        for _ in it:
            done += 1
            if time.perf_counter() - t0 >= seconds:
                break
        wall = time.perf_counter() - t0
        pool.terminate()
    return {"value": done / wall, "unit": "complexes/s", "cores": cores, "kind": "port",
            "sample": f"the first {done} {what}, one per process on {cores} host cores, "
                      f"reference-layout twist port ({wall:.1f} s wall)"}


def run_batch(args, ws, rank, local):
    """The batched workload: 4096 Rips complexes (n ~ U[20,120], half cube,
    half noisy circle) reduced in one segmented pass, against plain pms one
    complex at a time on the same GPU.  Bit-exactness: every instance of the
    batched result equals the one-at-a-time result, and a seeded sample of
    instances equals the oracle."""
    import torch

    import oracle
    from openph_gb300 import api
    from openph_gb300 import complexes as cx

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    dist = init_dist(ws, "nccl")
    t0 = time.perf_counter()
    col_off, colptr, rows, npts, seeds = cx.rips_mixed_batch(args.count or BATCH["count"], BATCH["seed"],
                                                             lo=BATCH["lo"], hi=BATCH["hi"])
    gen_s = time.perf_counter() - t0
    count = len(col_off) - 1
    total_m, total_nnz = int(col_off[-1]), int(colptr[-1])
    ctx = api.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=device)
    d_off = torch.from_numpy(col_off).to(device)
    d_colptr = torch.from_numpy(colptr).to(device)
    d_rows = torch.from_numpy(rows).to(device)
    d_low = torch.empty(total_m, dtype=torch.int32, device=device)
    torch.cuda.synchronize()

    def batched():
        return ctx.reduce_batch_device(count, d_off.data_ptr(), d_colptr.data_ptr(), d_rows.data_ptr(), total_m,
                                       total_nnz, d_low.data_ptr(), None, "pms")

    for _ in range(args.warmup):
        batched()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(dist, device)
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            info = batched()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    # the kernel launches of one step, counted by the library in a profiled
    # (untimed) repeat of the same step
    ctx.set_profile(True)
    batched()
    launches = ctx.last_profile()["kernel_launches"] * args.steps
    ctx.set_profile(False)
    batch_s = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / 1e3, dist, device)
    low_batch = d_low.cpu().numpy()

    # plain pms, one complex at a time, device-resident inputs
    d_low1 = torch.empty(int(np.diff(col_off).max()), dtype=torch.int32, device=device)
    colptr_d = [None] * count
    for b in range(count):
        c0, c1 = int(col_off[b]), int(col_off[b + 1])
        colptr_d[b] = torch.from_numpy(colptr[c0:c1 + 1] - colptr[c0]).to(device)
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
    seq_s = max_over_ranks(seq_ms / 1e3, dist, device)

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
    e2e_s = max_over_ranks(e2e_s, dist, device)
    e2e_equal = bool(np.array_equal(h_low.numpy(), low_batch))

    # oracle on a seeded sample of instances
    rng = np.random.default_rng(7)
    sample = sorted(rng.choice(count, size=min(count, 24), replace=False).tolist())
    oracle_ok = True
    for b in sample:
        bm = cx.batch_instance(col_off, colptr, rows, b)
        want, _, _ = oracle.twist(bm)
        oracle_ok &= bool(np.array_equal(want, low_batch[col_off[b]:col_off[b + 1]]))
    if rank == 0:
        line = {
            "metric": "complexes/s", "value": ws * count * args.steps / batch_s, "unit": "complexes/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * batch_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded generator)",
            "config": {"workload": f"rips_mixed_batch_{count}", "total_m": total_m, "total_nnz": total_nnz,
                       "points": [BATCH["lo"], BATCH["hi"]], "seed": BATCH["seed"], "algorithm": "pms",
                       "l2": "inputs (%.1f GB) larger than L2" % ((total_nnz * 4 + total_m * 8) / 1e9)},
            "plain_sequential": {"complexes_per_s": count / seq_s, "s_total": seq_s},
            "batched_over_plain": (count * args.steps / batch_s) / (count / seq_s),
            "e2e": {"value": ws * count * args.steps / e2e_s, "unit": "complexes/s",
                    "h2d_bytes_per_step": 8 * (count + 1) + 8 * (total_m + 1) + 4 * total_nnz,
                    "d2h_bytes_per_step": 4 * total_m, "ms_per_step": 1e3 * e2e_s / args.steps,
                    "api": "oph_reduce_batch C ABI", "equal_to_device_run": e2e_equal},
            "cpu_baseline": cpu_batch_sample(col_off, colptr, rows, CPU_SAMPLE_SECONDS),
            "cols_per_s": ws * total_m * args.steps / batch_s,
            "matrix_reduced": "anti-transpose D' (OPH_DUAL_AUTO)" if info["dual"] else "D",
            "sweeps": info["sweeps"], "device_additions": info["additions"], "regrows": info["regrows"],
            "pool_bytes": info["pool_bytes"],
            "parity": {"batched_equals_one_at_a_time": mismatches == 0, "mismatched_instances": mismatches,
                       "oracle_sample": len(sample), "oracle_sample_equal": oracle_ok},
            "generation_s": gen_s, "clocks": clocks.summary(), "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0 if (mismatches == 0 and oracle_ok) else 3


SERVE = {"requests": 160, "m_lo": 1_000, "m_hi": 2_000_000, "seed": 5, "budget_bytes": 150 * (1 << 30),
         "rates_x_plain": [0.5, 1, 2, 4, 8, 16, 32]}


def _serve_request(args):
    """One request of the serving stream: (kind, target m, seed) -> CSC."""
    kind, m, seed = args
    from openph_gb300 import complexes as cx
    if kind == "rips_cube":
        n = max(4, int(round((6 * m) ** (1 / 3))))
        bm = cx.rips_cube(n, seed=seed)
    elif kind == "rips_torus":
        bm = cx.rips_torus(400, m, seed=seed)
    else:
        side = max(4, int(round((m / 6) ** 0.5)))
        bm = cx.lower_star_image(side, side, seed=seed)
    return kind, bm.colptr, bm.rows


def serve_stream(count, seed):
    """Request mix: sizes log-uniform in [m_lo, m_hi], kind uniform over the
    three generator families, fresh seeds; generated on all host cores."""
    import concurrent.futures as cf
    import multiprocessing as mp
    rng = np.random.default_rng(seed)
    ms = np.exp(rng.uniform(np.log(SERVE["m_lo"]), np.log(SERVE["m_hi"]), size=count)).astype(np.int64)
    kinds = rng.choice(["rips_cube", "rips_torus", "lower_star"], size=count)
    seeds = rng.integers(1 << 30, size=count)
    jobs = [(str(k), int(m), int(sd)) for k, m, sd in zip(kinds, ms, seeds)]
    with cf.ProcessPoolExecutor(max_workers=os.cpu_count(), mp_context=mp.get_context("spawn")) as ex:
        out = list(ex.map(_serve_request, jobs, chunksize=1))
    from openph_gb300.complexes import BoundaryMatrix
    return [(k, BoundaryMatrix(cp, rw)) for k, cp, rw in out]


def run_serve(args, ws, rank, local):
    """Serving: a Poisson stream of reduction requests through the
    continuous-batching server (HBM budget 150 GB), rates swept to
    saturation; against plain pms one request at a time on the same GPU
    (host CSC in, host lows out, like the server)."""
    reqs = serve_stream(args.count or SERVE["requests"], SERVE["seed"])  # before any CUDA use
    import torch

    import oracle
    from openph_gb300 import api
    torch.cuda.set_device(local)
    n = len(reqs)
    total_m = sum(bm.m for _, bm in reqs)
    # plain: one at a time, service time of each
    ctx = api.Context(local)
    for _, bm in reqs[:3]:
        ctx.reduce(bm, "pms")
    service, plain_low = [], []
    for _, bm in reqs:
        t0 = time.perf_counter()
        low, _, _ = ctx.reduce(bm, "pms")
        service.append(time.perf_counter() - t0)
        plain_low.append(low)
    ctx.close()
    service = np.array(service)
    plain_rate = n / service.sum()

    srv = api.Server(local, budget_bytes=SERVE["budget_bytes"], max_active=4096)
    for _, bm in reqs[:3]:  # warm-up
        srv.wait(srv.submit(bm))
    rng = np.random.default_rng(SERVE["seed"] + 1)
    results, mism = [], 0
    for x in SERVE["rates_x_plain"]:
        rate = x * plain_rate
        gaps = rng.exponential(1.0 / rate, size=n)
        arrivals = np.cumsum(gaps)
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
            low, _, info = srv.wait(tickets[k])
            lat.append(info["latency_ms"])
            done_ms.append(info["done_ms"])
            sub_ms.append(info["submit_ms"])
            if not np.array_equal(low, plain_low[k]):
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
                        "plain_p50_ms": float(np.percentile(plat, 50)), "plain_p99_ms": float(np.percentile(plat, 99)),
                        "plain_served_per_s": n / max(fin, arrivals[-1])})
    counters = srv.stats()
    srv.close()
    # oracle on the smallest requests (the rest are checked against plain pms)
    order = np.argsort([bm.m for _, bm in reqs])[:16]
    oracle_ok = all(np.array_equal(oracle.twist(reqs[i][1])[0], plain_low[i]) for i in order)
    best = max(results, key=lambda r: r["served_per_s"])
    line = {
        "metric": "complexes/s", "value": best["served_per_s"], "unit": "complexes/s", "n_gpus": ws,
        "steps": len(results), "warmup": 3, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators, fresh seeds per request)",
        "config": {"workload": "serving_poisson_stream", "requests": n, "total_m": total_m,
                   "m_range": [SERVE["m_lo"], SERVE["m_hi"]], "budget_gb": SERVE["budget_bytes"] / (1 << 30),
                   "kinds": sorted({k for k, _ in reqs})},
        "plain_sequential": {"complexes_per_s": plain_rate, "mean_service_ms": 1e3 * service.mean()},
        "served_over_plain_at_saturation": best["served_per_s"] / plain_rate,
        "p50_ms_at_saturation": best["p50_ms"], "p99_ms_at_saturation": best["p99_ms"],
        "rate_sweep": results, "server": counters,
        "e2e": {"value": best["served_per_s"], "unit": "complexes/s",
                "h2d_bytes_per_step": int(np.mean([8 * (bm.m + 1) + 4 * bm.nnz for _, bm in reqs])),
                "d2h_bytes_per_step": int(np.mean([8 * bm.m for _, bm in reqs])),
                "api": "oph_server_submit / oph_server_wait (host CSC in, host lows and ess out; a step = one request)"},
        "cpu_baseline": cpu_pool_sample(((bm.colptr, bm.rows) for _, bm in reqs), CPU_SAMPLE_SECONDS,
                                        "requests of the stream"),
        "parity": {"served_equals_plain": mism == 0, "mismatches": mism, "oracle_checked_smallest": len(order),
                   "oracle_equal": bool(oracle_ok)},
    }
    print(json.dumps(line), flush=True)
    return 0 if (mism == 0 and oracle_ok) else 3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["torus", "batch", "serve"], default="torus",
                    help="torus: the ~5M-column complex (the headline); batch: 4096 complexes in one pass; "
                         "serve: a Poisson request stream through the continuous-batching server")
    ap.add_argument("--count", type=int, default=0, help="batch/serve: number of complexes / requests")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.workload == "batch":
        return run_batch(args, ws, rank, local)
    if args.workload == "serve":
        return run_serve(args, ws, rank, local)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
