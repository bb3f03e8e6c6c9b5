"""The duality the anti-transpose path rests on, checked on the oracle: the
low pairs of D and of its anti-transpose D' determine each other,
low_D(j) = i  <=>  low_D'(m-1-i) = m-1-j, and unpaired columns correspond.

D' is reduced by the oracle's standard algorithm (left to right, no
dimension buckets): the oracle's twist buckets columns by nnz - 1, which on
D' does not separate the columns that share rows."""
import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx

from cases import anti_transpose, random_complex, simplex_skeleton, small_cases


def mapped_back(low_d):
    m = len(low_d)
    low = np.full(m, -1, np.int32)
    c = np.nonzero(low_d >= 0)[0]
    low[m - 1 - low_d[c]] = m - 1 - c
    return low


CASES = small_cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_pairs_of_the_anti_transpose(built, name):
    bm = CASES[name]
    low, ess, _ = oracle.twist(bm)
    low_d, _, _ = oracle.standard(anti_transpose(bm))
    np.testing.assert_array_equal(mapped_back(low_d), low)
    np.testing.assert_array_equal(oracle.essential_from_low(low_d)[::-1], ess)


@pytest.mark.parametrize("seed", range(4))
def test_anti_transpose_larger_complexes(built, seed):
    for bm in (cx.rips_cube(14 + seed, seed=seed), cx.lower_star_image(10, 12, seed=seed, sigma=1.5),
               random_complex(18, 0.45, 0.5, seed=200 + seed), simplex_skeleton(6, seed=30 + seed)):
        low, _, _ = oracle.twist(bm)
        low_d, _, _ = oracle.standard(anti_transpose(bm))
        np.testing.assert_array_equal(mapped_back(low_d), low)


def test_anti_transpose_is_an_involution(built):
    bm = cx.rips_cube(9, seed=2)
    back = anti_transpose(anti_transpose(bm))
    np.testing.assert_array_equal(back.colptr, bm.colptr)
    np.testing.assert_array_equal(back.rows, bm.rows)


def test_rips_work_moves_to_the_vertices(built):
    """On a Rips complex even the standard algorithm (no clearing) on D'
    makes a small fraction of twist's additions on D."""
    bm = cx.rips_cube(30, seed=5)
    _, _, st = oracle.twist(bm)
    _, _, st_d = oracle.standard(anti_transpose(bm))
    assert st_d["additions"] * 5 < st["additions"]


def keep_columns(bm, mask):
    """bm with the columns outside mask emptied."""
    from openph_gb300.complexes import BoundaryMatrix
    return BoundaryMatrix.from_columns([list(bm.column(j)) if mask[j] else [] for j in range(bm.m)])


@pytest.mark.parametrize("case", ["lower_star", "volume", "random", "skeleton"])
def test_blocks_reduce_independently(built, case):
    """The per-block form the GPU path takes, on the oracle: the blocks of D
    (a bucket's columns with their rows) reduce on their own, some on D' and
    the others on D, the D part with the rows the D' part paired cleared
    (left as zero columns); the merged lows and the ess drawn from them
    equal twist on the whole of D."""
    from cases import lower_star_volume
    bm = {"lower_star": lambda: cx.lower_star_image(14, 11, seed=4, sigma=1.5),
          "volume": lambda: lower_star_volume(5, 6),
          "random": lambda: random_complex(16, 0.5, 0.6, seed=7),
          "skeleton": lambda: simplex_skeleton(7, seed=8, max_dim=3)}[case]()
    want, want_ess, _ = oracle.twist(bm)
    dims = np.diff(bm.colptr) - 1
    top = int(dims.max())
    for dual_dims in ({top}, {top, top - 1}, {1}):
        on_dual = np.isin(dims, list(dual_dims)) & (dims >= 1)
        low_d, _, _ = oracle.standard(anti_transpose(keep_columns(bm, on_dual)))
        mapped = mapped_back(low_d)
        # twist's clearing across blocks: a row the D' part paired is zero
        cleared = np.zeros(bm.m, bool)
        cleared[mapped[mapped >= 0]] = True
        low_p, _, _ = oracle.twist(keep_columns(bm, ~on_dual & ~cleared))
        low = np.where(on_dual, mapped, low_p)
        np.testing.assert_array_equal(low, want, err_msg=str(dual_dims))
        np.testing.assert_array_equal(oracle.essential_from_low(low), want_ess, err_msg=str(dual_dims))


@pytest.mark.parametrize("keep", [0.0, 0.3, 1.0])
def test_blocks_with_partial_clearing(built, keep):
    """The served form clears only the rows its D' part has paired by the
    time its D part starts: any subset of those clears (none, some, all)
    leaves the D part's lows exact."""
    bm = cx.lower_star_image(13, 12, seed=9, sigma=1.5)
    want, _, _ = oracle.twist(bm)
    dims = np.diff(bm.colptr) - 1
    on_dual = dims == 2
    mapped = mapped_back(oracle.standard(anti_transpose(keep_columns(bm, on_dual)))[0])
    paired = mapped[mapped >= 0]
    rng = np.random.default_rng(11)
    cleared = np.zeros(bm.m, bool)
    cleared[paired[rng.random(len(paired)) < keep]] = True
    low_p, _, _ = oracle.twist(keep_columns(bm, ~on_dual & ~cleared))
    np.testing.assert_array_equal(np.where(on_dual, mapped, low_p), want)
