"""Generators and the boundary-matrix formats (host only)."""
import numpy as np
import pytest

from openph_gb300 import complexes as cx
from openph_gb300.complexes import BoundaryMatrix


def boundary_squared_is_zero(bm):
    """d o d = 0 over Z/2 for every column (a valid boundary matrix)."""
    for j in range(bm.m):
        acc = {}
        for f in bm.column(j):
            for g in bm.column(int(f)):
                acc[int(g)] = acc.get(int(g), 0) ^ 1
        if any(acc.values()):
            return False
    return True


def test_rips_cube_50_shape(built):
    bm = cx.rips_cube(50, seed=1)
    assert bm.m == 20875 and bm.nnz == 61250
    assert np.bincount(bm.dims).tolist() == [50, 1225, 19600]


def test_rips_full_skeleton_counts(built):
    for n in (20, 35):
        bm = cx.rips_mixed(n, seed=n)
        assert bm.m == n + n * (n - 1) // 2 + n * (n - 1) * (n - 2) // 6


def test_lower_star_counts(built):
    bm = cx.lower_star_image(16, 16, seed=1, sigma=2.0)
    V, E, T = 256, 15 * 16 * 2 + 15 * 15, 2 * 15 * 15
    assert bm.m == V + E + T


@pytest.mark.parametrize("make", [lambda: cx.rips_cube(15, seed=2), lambda: cx.lower_star_image(9, 7, seed=3),
                                  lambda: cx.rips_mixed(14, seed=5)])
def test_valid_boundary_matrix(built, make):
    bm = make()
    assert boundary_squared_is_zero(bm)
    # filtration order: faces before cofaces, values non-decreasing
    for j in range(bm.m):
        col = bm.column(j)
        assert np.all(col < j) and np.all(np.diff(col) > 0)
    assert np.all(np.diff(bm.values) >= 0)


def test_generators_are_deterministic(built):
    a, b = cx.rips_cube(20, seed=4), cx.rips_cube(20, seed=4)
    np.testing.assert_array_equal(a.rows, b.rows)
    c = cx.rips_cube(20, seed=5)
    assert not np.array_equal(a.values, c.values)


def test_torus_threshold_hits_target(built):
    pts = cx.points_torus(60, seed=2)
    thr = cx.rips_threshold(pts, 8000)
    bm = cx.rips(pts, thr)
    # triangles sharing their longest edge tie at the threshold: within one edge star
    assert 8000 <= bm.m <= 8000 + 60


def test_coo_roundtrip_and_file(built, tmp_path):
    bm = cx.rips_cube(10, seed=1)
    r, c = bm.to_coo1()
    back = BoundaryMatrix.from_coo1(r, c, bm.m)
    np.testing.assert_array_equal(back.colptr, bm.colptr)
    np.testing.assert_array_equal(back.rows, bm.rows)
    p = tmp_path / "x.csc"
    bm.save(p)
    again = BoundaryMatrix.load(p)
    np.testing.assert_array_equal(again.rows, bm.rows)
