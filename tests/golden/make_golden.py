"""Generates the golden fixtures from the reference's own CPU reductions.

Runs the reference's standard, twist and ph_row (compiled from its sources by
oracle/Makefile into oracle/_ref/ref_ph; needs the reference checkout) on
small seeded complexes and stores, per case, the input CSC and each
algorithm's 0-based low and ess in golden_<case>.npz.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

import oracle  # noqa: E402
from openph_gb300 import complexes as cx  # noqa: E402
from cases import random_complex, triangle  # noqa: E402

CASES = {
    "triangle": lambda: triangle(),
    "rips_cube_12_s3": lambda: cx.rips_cube(12, seed=3),
    "rips_cube_50_s1": lambda: cx.rips_cube(50, seed=1),
    "rips_circle_30_s11": lambda: cx.rips_mixed(30, seed=11),
    "lower_star_32x32_s5": lambda: cx.lower_star_image(32, 32, seed=5, sigma=2.0),
    "random_flag_free_s100": lambda: random_complex(14, 0.5, 0.6, seed=100),
    "random_flag_free_s101": lambda: random_complex(14, 0.5, 0.6, seed=101),
}
COL_WIDTH = 40


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("the reference's CPU code is not built (needs the reference checkout)")
    for name, make in CASES.items():
        bm = make()
        out = {"colptr": bm.colptr, "rows": bm.rows}
        for alg in ("standard", "twist", "ph_row"):
            res = oracle.ref_run(bm, alg, COL_WIDTH)
            if res is None:
                raise SystemExit(f"{name}/{alg}: the reference overflowed col_width={COL_WIDTH}")
            low, ess, iters, _ = res
            out[f"{alg}_low"] = low
            out[f"{alg}_ess"] = ess
            out[f"{alg}_iters"] = np.array([iters], np.int32)
        np.savez_compressed(HERE / f"golden_{name}.npz", **out)
        print(name, bm.m, bm.nnz)


if __name__ == "__main__":
    main()
