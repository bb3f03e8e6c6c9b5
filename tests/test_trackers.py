"""Per-iteration progress trackers of the sequential algorithms (the
reference's track_host after every column or row: standard.cu:44-49,
twist.cu:68-71, ph_row.cu:107-110; track on the device for the parallel
forms: standard_parallel.cu:40-43, twist_parallel.cu:75-78,
ph_row_parallel.cu:76-79; tracker.cu:92-172).  The oracle restates those loops
step by step (oracle.tracked); openph() keeps them from the GPU walk."""
import numpy as np
import pytest

import oracle
from cases import small_cases
from openph_gb300 import complexes as cx

ALGOS = ["standard", "twist", "standard_parallel", "twist_parallel", "ph_row", "ph_row_parallel"]
CASES = small_cases()


def _cases():
    out = dict(CASES)
    out["rips_cube_14"] = cx.rips_cube(14, seed=3)
    out["lower_star_10x12"] = cx.lower_star_image(10, 12, seed=4, sigma=1.5)
    return out


@pytest.mark.parametrize("name", sorted(_cases()))
def test_restated_reduction_matches_the_oracle(built, name):
    """The restatement's own column reduction ends at the oracle's lows."""
    bm = _cases()[name]
    want_s, _, _ = oracle.standard(bm)
    want_t, _, _ = oracle.twist(bm)
    want_r, _, _ = oracle.ph_row(bm)
    for algo, want in (("standard", want_s), ("twist", want_t), ("ph_row", want_r), ("ph_row_parallel", want_r)):
        *_, n, low = oracle.tracked(bm, algo, want_t)
        np.testing.assert_array_equal(low, want)
        assert n == (1 + int((np.diff(bm.colptr) - 1 >= 1).sum()) if algo == "twist" else bm.m + 1)


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("name", sorted(_cases()))
def test_trackers_every_iteration(cuda_lib, name, algo):
    """Every entry of err_linf, err_lone, err_redu and err_ess equals the
    restatement's (float32, within an ulp of the normalising divisions), the
    iteration count is the reference's, every iteration has a time, and
    nothing is written past num_iters."""
    from openph_gb300.api import ph
    bm = _cases()[name]
    want, _, _ = oracle.twist(bm)
    linf, lone, redu, eerr, n, _ = oracle.tracked(bm, algo, want)
    r, c = bm.to_coo1()
    low_true = (want + 1).astype(np.int32)
    low, ess, g_linf, g_lone, g_redu, g_eerr, tt, it = ph(algo, r, c, bm.m, 0, low_true)
    assert int(it[0]) == n
    for got, exp in ((g_linf, linf), (g_lone, lone), (g_redu, redu), (g_eerr, eerr)):
        np.testing.assert_allclose(got[:n], exp, rtol=2e-7, atol=0, equal_nan=True)
        assert np.all(got[n:] == -1)
    assert tt[0] == 0 and np.all(np.isfinite(tt[:n])) and np.all(tt[1:n] >= 0)
