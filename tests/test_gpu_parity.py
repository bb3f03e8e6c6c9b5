"""GPU parity: every algorithm, through the C ABI, against the oracle.

The lows of a reduced matrix are unique, so every algorithm must reproduce the
oracle's low bit for bit; ess must match the reference's per-algorithm
estimate (see the oracle's restatements)."""
import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import ALGORITHMS, OphError, ph

from cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()


def expected(bm, algo):
    low, ess, _ = oracle.twist(bm)
    if algo == "ph_row":
        _, ess, _ = oracle.ph_row(bm)
    elif algo == "ph_row_parallel":
        # the reference's GPU row variant never fills arglow, so its estimate
        # only clears rows that are some column's low (ph_row_parallel.cu:20-89)
        ess = np.ones(bm.m, np.int32)
        ess[low[low >= 0]] = 0
    return low, ess


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("algo", ALGORITHMS)
def test_small_cases_all_algorithms(cuda_lib, name, algo):
    bm = CASES[name]
    r, c = bm.to_coo1()
    low, ess, *_ = ph(algo, r, c, bm.m, 3, np.zeros(bm.m, np.int32))
    want_low, want_ess = expected(bm, algo)
    np.testing.assert_array_equal(low, want_low + 1)
    np.testing.assert_array_equal(ess, want_ess)


@pytest.mark.parametrize("algo", ALGORITHMS)
def test_rips_cube_50(cuda_lib, algo):
    bm = cx.rips_cube(50, seed=1)
    r, c = bm.to_coo1()
    low, ess, *_ = ph(algo, r, c, bm.m, 3, np.zeros(bm.m, np.int32))
    want_low, want_ess = expected(bm, algo)
    np.testing.assert_array_equal(low, want_low + 1)
    np.testing.assert_array_equal(ess, want_ess)


def test_context_reduce_arglow(ctx):
    bm = cx.rips_cube(30, seed=9)
    low, ess, arglow, info = ctx.reduce(bm, "pms", with_arglow=True)
    want, want_ess, _ = oracle.twist(bm)
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    want_arg = np.full(bm.m, -1, np.int32)
    j = np.nonzero(want >= 0)[0]
    want_arg[want[j]] = j
    np.testing.assert_array_equal(arglow, want_arg)
    assert info["sweeps"] >= 1


def test_lower_star_64(ctx):
    bm = cx.lower_star_image(64, 64, seed=11, sigma=4.0)
    want, want_ess, _ = oracle.twist(bm)
    for algo in ("pms", "twist", "standard", "ph_row"):
        low, ess, _ = ctx.reduce(bm, algo)
        np.testing.assert_array_equal(low, want, err_msg=algo)
    low, ess, _ = ctx.reduce(bm, "pms")
    np.testing.assert_array_equal(ess, want_ess)


def test_batch_mixed(ctx):
    mats = [cx.rips_mixed(n, seed=s) for s, n in enumerate([12, 20, 7, 25, 16, 9])]
    lows, esss, info = ctx.reduce_batch(mats, "pms")
    for bm, low, ess in zip(mats, lows, esss):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def test_batch_equals_alone(ctx):
    mats = [cx.rips_mixed(n, seed=40 + s) for s, n in enumerate([30, 22, 26])]
    lows, _, _ = ctx.reduce_batch(mats, "pms")
    for bm, low in zip(mats, lows):
        alone, _, _ = ctx.reduce(bm, "pms")
        np.testing.assert_array_equal(low, alone)


def test_regrow_from_tiny_pool(cuda_lib):
    from openph_gb300.api import Context
    bm = cx.lower_star_image(48, 48, seed=2, sigma=3.0)
    want, _, _ = oracle.twist(bm)
    with Context(0) as c:
        c.set_limits(initial_pool_bytes=1)  # the packed input only: any growth must regrow
        for algo in ("pms", "twist", "ph_row"):
            low, _, info = c.reduce(bm, algo)
            np.testing.assert_array_equal(low, want, err_msg=algo)
            assert info["regrows"] >= 1, algo


def test_sweep_cap_times_out(cuda_lib):
    from openph_gb300.api import Context, OPH_ERR_TIMEOUT
    bm = cx.rips_cube(40, seed=1)
    with Context(0) as c:
        c.set_dual("never")  # D itself needs several sweeps
        c.set_limits(max_sweeps=1)
        with pytest.raises(OphError) as e:
            c.reduce(bm, "pms")
        assert e.value.status == OPH_ERR_TIMEOUT
        c.set_limits(max_sweeps=0)
        low, _, _ = c.reduce(bm, "pms")  # the context stays usable
        np.testing.assert_array_equal(low, oracle.twist(bm)[0])


def test_budget_oom(cuda_lib):
    from openph_gb300.api import Context, OPH_ERR_OOM
    bm = cx.rips_cube(40, seed=1)
    with Context(0) as c:
        c.set_budget(4096)
        with pytest.raises(OphError) as e:
            c.reduce(bm, "pms")
        assert e.value.status == OPH_ERR_OOM


@pytest.mark.parametrize("bad", ["row_out_of_range", "unsorted_rows", "cols_decreasing"])
def test_malformed_input_rejected(cuda_lib, bad):
    from openph_gb300.api import OPH_ERR_BAD_INPUT
    bm = cases_triangle = CASES["triangle"]
    r, c = bm.to_coo1()
    r, c = r.copy(), c.copy()
    if bad == "row_out_of_range":
        r[-1] = bm.m + 1
    elif bad == "unsorted_rows":
        r[-1], r[-2] = r[-2], r[-1]
    else:
        c[0], c[-1] = c[-1], c[0]
    with pytest.raises(OphError) as e:
        ph("pms", r, c, bm.m, 3)
    assert e.value.status == OPH_ERR_BAD_INPUT


def test_unknown_algorithm(cuda_lib):
    r, c = CASES["triangle"].to_coo1()
    with pytest.raises(OphError):
        ph("spectral", r, c, 7, 3)


def test_zero_columns(cuda_lib):
    for algo in ALGORITHMS:
        low, ess, *_ = ph(algo, np.zeros(0, np.int32), np.zeros(0, np.int32), 4, 3)
        np.testing.assert_array_equal(low, np.zeros(4, np.int32))
        np.testing.assert_array_equal(ess, np.ones(4, np.int32))


@pytest.mark.parametrize("algo", ["pms", "twist"])
def test_lower_star_512_full_size(ctx, algo):
    """The 512 x 512 lower-star configuration (1,568,771 columns), bit-exact."""
    bm = cx.lower_star_image(512, 512, seed=3)
    want, want_ess, _ = oracle.twist(bm)
    low, ess, _ = ctx.reduce(bm, algo)
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


@pytest.fixture(scope="module")
def torus_1m():
    bm = cx.rips_torus(400, 1_000_000, seed=2)
    want, want_ess, _ = oracle.twist(bm)
    return bm, want, want_ess


@pytest.mark.parametrize("mode", ["never", "auto"])
def test_rips_torus_1m(cuda_lib, torus_1m, mode):
    """A 1M-column torus Rips complex (the 5M configuration's family), on D
    and on its anti-transpose."""
    from openph_gb300.api import Context
    bm, want, want_ess = torus_1m
    with Context(0) as c:
        c.set_dual(mode)
        low, ess, info = c.reduce(bm, "pms")
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    assert info["regrows"] == 0
    assert info["dual"] == (0 if mode == "never" else 1)


@pytest.mark.parametrize("lanes,cap", [(8, 128), (4, 128), (8, 64), (8, 256), (16, 128), (16, 256), (32, 128)])
def test_every_tier0_candidate_is_exact(cuda_lib, lanes, cap):
    from openph_gb300.api import Context
    bm = cx.lower_star_image(48, 48, seed=6, sigma=3.0)
    want, want_ess, _ = oracle.twist(bm)
    with Context(0) as c:
        c.set_tier0(lanes, cap)
        low, ess, _ = c.reduce(bm, "pms")
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


def test_autotune_picks_a_candidate(cuda_lib):
    from openph_gb300.api import Context
    bm = cx.rips_cube(30, seed=4)
    with Context(0) as c:
        choice = c.autotune(bm)
        assert (choice["lanes"], choice["cap"]) in {(8, 128), (4, 128), (8, 64), (8, 256), (16, 128), (16, 256), (32, 128)}
        low, _, _ = c.reduce(bm, "pms")
    np.testing.assert_array_equal(low, oracle.twist(bm)[0])
    with pytest.raises(OphError):
        Context(0).set_tier0(3, 100)


@pytest.fixture(scope="module")
def torus_200k():
    bm = cx.rips_torus(400, 200_000, seed=5)
    low, ess, st = oracle.twist(bm)
    return bm, low, ess, st


@pytest.mark.parametrize("lanes,cap", [(8, 128), (4, 128), (8, 64), (16, 256), (32, 128)])
def test_long_chains_every_tier0_candidate(cuda_lib, torus_200k, lanes, cap):
    """Top-dimension chains of up to ~200 rows: lazy columns with pending
    toggles of 4 to 16 lanes, flushes, wide pivots and tier hand-offs."""
    from openph_gb300.api import Context
    bm, want, want_ess, _ = torus_200k
    with Context(0) as c:
        c.set_dual("never")  # the chains of D's triangle columns
        c.set_tier0(lanes, cap)
        low, ess, _ = c.reduce(bm, "pms")
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


def test_slot_counters_match_twist(cuda_lib, torus_200k):
    """With slot tracking on, the device's |P| + |T| + |T xor P| total agrees
    with the twist oracle's to 0.5% (pms and twist add the same pivots, up to
    the few extra additions pms makes on columns twist clears), and the
    result is unchanged."""
    from openph_gb300.api import Context
    bm, want, want_ess, st = torus_200k
    with Context(0) as c:
        c.set_dual("never")  # the additions twist makes are those of D
        c.set_profile(True, slots=True)
        low, ess, info = c.reduce(bm, "pms")
        prof = c.last_profile()
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    slots = sum(prof["tier_slots"])
    want_slots = st["slots_read"] + st["slots_written"]
    assert sum(prof["tier_additions"]) == info["additions"]
    assert abs(info["additions"] - st["additions"]) <= 0.005 * st["additions"]
    assert abs(slots - want_slots) <= 0.005 * want_slots
    assert prof["tier_slots"][0] > 0


def test_pms_trackers_per_sweep(cuda_lib):
    """openph()'s progress outputs for pms: one entry per sweep as in the
    reference's track() calls (pms.cu:16,106, tracker.cu:92-134).  Entry 0
    (before Phase 0) is checked exactly against numpy, the last entry is the
    exact final state, and the entries between are finite progress values."""
    bm = cx.rips_torus(400, 200_000, seed=5)
    want, want_ess, _ = oracle.twist(bm)
    r, c = bm.to_coo1()
    low_true = (want + 1).astype(np.int32)
    low, ess, linf, lone, redu, eerr, tt, it = ph("pms", r, c, bm.m, 0, low_true)
    np.testing.assert_array_equal(low, low_true)
    n = int(it[0])
    assert n >= 3
    # entry 0: the initial lows (last row of every column, -1 when empty)
    lens = np.diff(bm.colptr)
    init = np.where(lens > 0, bm.rows[np.maximum(bm.colptr[1:] - 1, 0)], -1).astype(np.float64)
    d = np.abs(init - want)
    n1, ninf = np.abs(low_true).sum(dtype=np.float64), np.abs(low_true).max()
    assert lone[0] == pytest.approx(d.sum() / n1, rel=1e-6)
    assert linf[0] == pytest.approx(d.max() / ninf, rel=1e-6)
    assert redu[0] == pytest.approx(1.0)
    ess_true = np.ones(bm.m)
    ess_true[want >= 0] = 0
    ess_true[want[want >= 0]] = 0
    assert eerr[0] == pytest.approx(ess_true.sum() / bm.m, rel=1e-6)
    # the last entry: exact
    assert (lone[n - 1], linf[n - 1], redu[n - 1], eerr[n - 1]) == (0.0, 0.0, 0.0, 1.0)
    # between: progress values in range, positive sweep times, nothing past n
    for arr in (lone, linf, redu):
        assert np.all(np.isfinite(arr[:n])) and np.all(arr[:n] >= 0)
    assert np.all(redu[:n] <= 1.0) and np.all((eerr[:n] > 0) & (eerr[:n] <= 1.0))
    # what the schedule fixes although its interleaving does not: a column is
    # classified once for good (unclassified never grows) and the essential
    # estimate only loses rows (ess_true / ess_hat never falls)
    assert np.all(np.diff(redu[:n]) <= 0)
    assert np.all(np.diff(eerr[:n]) >= 0)
    assert np.all(tt[1:n] > 0) and tt[0] == 0
    assert np.all(lone[n:] == -1)


def test_columns_wider_than_pms_handles(cuda_lib):
    """The 7-simplex has a column of 8 rows: pms (whose Phase I keeps one
    running maximum per dimension -1..6) refuses it with an error; the other
    algorithms reduce it exactly."""
    from cases import simplex_skeleton
    bm = simplex_skeleton(8, seed=13)
    assert np.diff(bm.colptr).max() == 8
    r, c = bm.to_coo1()
    with pytest.raises(OphError):
        ph("pms", r, c, bm.m, 3, np.zeros(bm.m, np.int32))
    want, _, _ = oracle.twist(bm)
    for algo in ("standard", "twist", "standard_parallel", "twist_parallel", "ph_row", "ph_row_parallel"):
        low, *_ = ph(algo, r, c, bm.m, 3, np.zeros(bm.m, np.int32))
        np.testing.assert_array_equal(low, want + 1, err_msg=algo)


def test_batch_ragged_with_empty_instances(ctx):
    """Instances of 0, 1 and 5 columns, a triangle, a 6-simplex and a small
    Rips complex in one batch: each equals the oracle."""
    from cases import empty_columns, simplex_skeleton, triangle
    from openph_gb300.complexes import BoundaryMatrix
    mats = [BoundaryMatrix.from_columns([]), triangle(), BoundaryMatrix.from_columns([[]]), empty_columns(5),
            simplex_skeleton(7, seed=21), cx.rips_mixed(10, seed=3), BoundaryMatrix.from_columns([])]
    lows, esss, _ = ctx.reduce_batch(mats, "pms")
    for bm, low, ess in zip(mats, lows, esss):
        assert len(low) == bm.m
        if bm.m == 0:
            continue
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def test_void_openph_drop_in_symbol(cuda_lib):
    """The reference's own symbol, void openph(...) (src/cuda/openph.cu:29-35),
    called with the arguments the MEX gateway passes (src/matlab/ph/ph.cu:
    71-74): the outputs land in the caller's arrays; an unknown algorithm
    string prints and leaves low all zeros, as the drop-in contract says."""
    from cases import triangle
    for bm, algo in ((cx.rips_cube(24, seed=8), "pms"), (cx.rips_cube(24, seed=8), "twist"), (triangle(), "pms")):
        r, c = bm.to_coo1()
        m = bm.m
        low = np.full(m, -9, np.int32)
        ess = np.full(m, -9, np.int32)
        trk = [np.zeros(m + 1, np.float32) for _ in range(5)]
        it = np.zeros(1, np.int32)
        low_true = np.zeros(m, np.int32)
        cuda_lib.openph(algo.encode(), r, c, m, 4, low_true.ctypes.data, len(r), low, ess, *trk, it, 0)
        want_low, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want_low + 1, err_msg=algo)
        np.testing.assert_array_equal(ess, want_ess, err_msg=algo)
        assert it[0] >= 1
    bm = triangle()
    r, c = bm.to_coo1()
    low = np.full(bm.m, 5, np.int32)
    ess = np.zeros(bm.m, np.int32)
    trk = [np.zeros(bm.m + 1, np.float32) for _ in range(5)]
    cuda_lib.openph(b"not_an_algorithm", r, c, bm.m, 4, None, len(r), low, ess, *trk, np.zeros(1, np.int32), 0)
    np.testing.assert_array_equal(low, np.zeros(bm.m, np.int32))
