"""Reduce one generated workload a few times on the GPU (for profiler runs).

    python -m openph_gb300.run_case [--workload rips_torus|lower_star|rips_cube|batch|rips_device|lower_star_device]
                                    [--target-m M] [--algo pms] [--steps K]
                                    [--tier0 LANES,CAP] [--profile] [--dual MODE]

Prints one JSON line with the device time per reduction and the library's
counters.  The matrix is device-resident before the first reduction.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def make(workload: str, target_m: int, seed: int):
    from . import complexes as cx
    if workload in ("rips_device", "lower_star_device"):
        return None  # built on the GPU in main()
    if workload == "rips_torus":
        return cx.rips_torus(400, target_m, seed=seed)
    if workload == "lower_star":
        side = int(round((target_m / 6) ** 0.5)) if target_m else 512
        return cx.lower_star_image(side, side, seed=seed)
    if workload == "rips_cube":
        return cx.rips_cube(50, seed=seed)
    if workload == "batch":
        return cx.rips_mixed_batch(target_m or 4096, seed)
    raise SystemExit(f"unknown workload {workload}")


def _prof(ctx, args) -> dict:
    if not args.profile:
        return {}
    p = ctx.last_profile()
    return {"profile": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in p.items()}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="rips_torus",
                    help="rips_torus, lower_star, rips_cube, batch, or rips_device / lower_star_device (built on "
                         "the GPU first)")
    ap.add_argument("--target-m", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--algo", default="pms")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--tier0", default="", help="tier-0 lanes,capacity (default: the library's choice)")
    ap.add_argument("--profile", action="store_true", help="print per-phase times of the last step")
    ap.add_argument("--dual", default="auto", help="pms on the anti-transpose: auto, never or always")
    args = ap.parse_args()

    import torch

    from . import api
    bm = make(args.workload, args.target_m, args.seed)
    dev = torch.device("cuda", 0)
    ctx = api.Context(0)
    if args.tier0:
        ctx.set_tier0(*map(int, args.tier0.split(",")))
    ctx.set_profile(args.profile)
    ctx.set_dual(args.dual)
    if args.workload in ("rips_device", "lower_star_device"):
        # the complex built on the GPU (the generator kernels), then reduced
        from . import complexes as cx
        out = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            if args.workload == "rips_device":
                pts = cx.points_torus(400, seed=args.seed)
                thr = cx.rips_threshold(pts, args.target_m)
                dm = cx.rips_device(torch.from_numpy(pts).to(dev), thr, ctx=ctx, device=dev)
            else:
                side = int(round((args.target_m / 6) ** 0.5))
                img = cx.image_smoothed(side, side, seed=args.seed)
                dm = cx.lower_star_device(torch.from_numpy(img).to(dev), ctx=ctx, device=dev)
            m = int(dm.colptr.shape[0]) - 1
            d_low = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
            out.append(ctx.reduce_device(m, dm.colptr.data_ptr(), dm.rows.data_ptr(), d_low.data_ptr(), None, None,
                                         args.algo))
        print(json.dumps({"workload": args.workload, "m": m, "device_ms": [o["device_ms"] for o in out],
                          "sweeps": out[-1]["sweeps"], "dual": out[-1]["dual"]}))
        ctx.close()
        return
    if args.workload == "batch":
        # --target-m is the number of complexes; one segmented pass each step
        col_off, colptr, rows = (torch.from_numpy(x).to(dev) for x in bm[:3])
        m, nnz = int(bm[0][-1]), int(bm[1][-1])
        d_low = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        out = [ctx.reduce_batch_device(len(bm[0]) - 1, col_off.data_ptr(), colptr.data_ptr(), rows.data_ptr(), m,
                                       nnz, d_low.data_ptr(), None, args.algo) for _ in range(args.steps)]
        print(json.dumps({"workload": "batch", "count": len(bm[0]) - 1, "m": m, "nnz": nnz,
                          "device_ms": [o["device_ms"] for o in out], "sweeps": out[-1]["sweeps"],
                          "additions": out[-1]["additions"], "dual": out[-1]["dual"], **_prof(ctx, args)}))
        ctx.close()
        return
    d_colptr = torch.from_numpy(bm.colptr).to(dev)
    d_rows = torch.from_numpy(bm.rows).to(dev)
    d_low = torch.empty(max(bm.m, 1), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    out = []
    for _ in range(args.steps):
        out.append(ctx.reduce_device(bm.m, d_colptr.data_ptr(), d_rows.data_ptr(), d_low.data_ptr(), None, None,
                                     args.algo))
    print(json.dumps({"workload": args.workload, "m": bm.m, "nnz": bm.nnz, "algo": args.algo,
                      "device_ms": [o["device_ms"] for o in out], "sweeps": out[-1]["sweeps"],
                      "additions": out[-1]["additions"], "dual": out[-1]["dual"], "pivots": int((d_low.cpu().numpy() >= 0).sum()),
                      **_prof(ctx, args)}))
    ctx.close()


if __name__ == "__main__":
    main()
