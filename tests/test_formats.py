"""PHAT ASCII round trip and persistence diagrams (host only)."""
import numpy as np

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.formats import persistence_diagram, persistence_pairs, read_phat_dat, write_phat_dat
from cases import triangle


def test_phat_round_trip(built, tmp_path):
    bm = cx.rips_cube(12, seed=3)
    p = tmp_path / "m.dat"
    write_phat_dat(bm, p, dims=bm.dims)
    back, dims = read_phat_dat(p)
    np.testing.assert_array_equal(back.colptr, bm.colptr)
    np.testing.assert_array_equal(back.rows, bm.rows)
    np.testing.assert_array_equal(dims, bm.dims)


def test_phat_comments_and_zero_cells(tmp_path):
    p = tmp_path / "t.dat"
    p.write_text("# triangle\n0\n0\n0\n\n1 0 1\n1 0 2\n1 1 2\n2 3 4 5\n")
    bm, dims = read_phat_dat(p)
    assert bm.m == 7 and bm.nnz == 9
    np.testing.assert_array_equal(oracle.twist(bm)[0] + 1, [0, 0, 0, 2, 3, 0, 6])


def test_pairs_and_diagram_triangle(built):
    bm = triangle()
    low, _, _ = oracle.twist(bm)
    pairs, ess = persistence_pairs(low)
    assert sorted(map(tuple, pairs.tolist())) == [(1, 3), (2, 4), (5, 6)]
    assert ess.tolist() == [0]
    values = np.array([0, 0, 0, 1, 1, 2, 3], float)
    dims = np.array([0, 0, 0, 1, 1, 1, 2])
    dgm = persistence_diagram(low, values, dims)
    assert dgm[0].tolist() == [[0, 1], [0, 1], [0, np.inf]]
    assert dgm[1].tolist() == [[2, 3]]


def test_diagram_counts_match_betti(built):
    # a noisy circle: H1 of the full 2-skeleton Rips complex dies, H0 has one essential
    bm = cx.rips_mixed(20, seed=1)
    low, ess, _ = oracle.twist(bm)
    dgm = persistence_diagram(low, bm.values, bm.dims)
    assert np.isinf(dgm[0][:, 1]).sum() == 1
    assert np.isinf(dgm[1][:, 1]).sum() == 0
    assert len(dgm[0]) == 20
