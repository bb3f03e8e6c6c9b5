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
