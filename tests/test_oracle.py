"""The oracle, pinned: against the golden vectors made by the reference's own
CPU code, against a dense reduction, and (where the reference checkout
exists) against the reference's code run live."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from openph_gb300.complexes import BoundaryMatrix
from cases import random_complex, small_cases

GOLDEN = sorted((Path(__file__).parent / "golden").glob("golden_*.npz"))


def load_golden(path):
    z = np.load(path)
    return BoundaryMatrix(z["colptr"], z["rows"]), z


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_matches_golden(built, path):
    bm, z = load_golden(path)
    for alg, fn in (("twist", oracle.twist), ("standard", oracle.standard), ("ph_row", oracle.ph_row)):
        low, ess, st = fn(bm)
        np.testing.assert_array_equal(low, z[f"{alg}_low"], err_msg=alg)
        np.testing.assert_array_equal(ess, z[f"{alg}_ess"], err_msg=alg)
        assert st["iters"] == int(z[f"{alg}_iters"][0]), alg
    # pms (sequential interleaving) reaches the same reduced matrix
    low, ess, _ = oracle.pms(bm)
    np.testing.assert_array_equal(low, z["twist_low"])
    np.testing.assert_array_equal(ess, z["twist_ess"])


def test_golden_known_answer_triangle(built):
    bm, z = load_golden(Path(__file__).parent / "golden" / "golden_triangle.npz")
    np.testing.assert_array_equal(z["twist_low"] + 1, [0, 0, 0, 2, 3, 0, 6])


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_oracle_matches_dense(built, name):
    bm = small_cases()[name]
    want = oracle.dense_standard(bm)
    for fn in (oracle.twist, oracle.standard, oracle.ph_row, oracle.pms):
        np.testing.assert_array_equal(fn(bm)[0], want)


def test_fixed_slot_port_matches(built):
    bm = random_complex(16, 0.6, 0.7, seed=7)
    rc, low, ess, st = oracle.twist_fixed_p(bm, col_width=20)
    assert rc == 0
    np.testing.assert_array_equal(low, oracle.twist(bm)[0])
    np.testing.assert_array_equal(ess, oracle.twist(bm)[1])


def test_fixed_slot_port_overflow_is_reported(built):
    # col_width 1 leaves no room for fill-in: the port reports it instead of
    # exiting the process as the reference does (kernels_host.cu:21-24)
    from openph_gb300 import complexes as cx
    bm = cx.rips_cube(20, seed=2)
    rc, *_ = oracle.twist_fixed_p(bm, col_width=1)
    assert rc == 3


def test_planted_mistake_is_caught(built):
    # a wrong oracle must fail the comparison: flip one low
    bm, z = load_golden(Path(__file__).parent / "golden" / "golden_rips_cube_12_s3.npz")
    low, _, _ = oracle.twist(bm)
    bad = low.copy()
    k = int(np.nonzero(bad >= 0)[0][0])
    bad[k] = -1
    assert not np.array_equal(bad, z["twist_low"])


def test_transverse_restatement_matches_serial_walk(built):
    """The parallel Phase I rule (first occurrence + prefix max of repeated
    lows per bucket) marks exactly what the serial walk marks."""
    rng = np.random.default_rng(5)
    for trial in range(30):
        m = int(rng.integers(5, 200))
        cdim = 4
        dim = rng.integers(-1, 3, size=m).astype(np.int32)
        # graded: rows of bucket b live in a disjoint range
        low = np.full(m, -1, np.int32)
        for j in range(m):
            if dim[j] >= 1 and rng.random() < 0.8:
                low[j] = int(rng.integers(0, m // 4 + 1)) * 4 + (dim[j] + 1)
        low[low >= m] = -1
        classes = np.where(rng.random(m) < 0.2, -1, 0).astype(np.int32)
        arglow = np.full(m, -1, np.int32)
        ess = np.ones(m, np.int32)
        start = np.full(cdim, -1, np.int32)
        nxt = np.full(m, -1, np.int32)
        last = {}
        for j in range(m):
            b = dim[j] + 1
            if b in last:
                nxt[last[b]] = j
            else:
                start[b] = j
            last[b] = j
        _, _, cls_serial, clear_serial, _ = oracle.transverse(dim, start, nxt, low, arglow, classes, ess, cdim)
        # data-parallel restatement
        first = {}
        for j in range(m):
            if low[j] >= 0 and low[j] not in first:
                first[low[j]] = j
        ceil = {b: -1 for b in range(cdim)}
        piv = np.zeros(m, bool)
        for j in range(m):  # exclusive prefix max of repeated lows, per bucket
            if low[j] < 0:
                continue
            b = dim[j] + 1
            if first[low[j]] != j:
                ceil[b] = max(ceil[b], low[j])
            elif classes[j] == 0 and low[j] > ceil[b]:
                piv[j] = True
        np.testing.assert_array_equal(piv, (cls_serial == -1) & (classes == 0))
