"""pms on the anti-transpose (OPH_DUAL_*): every output equal to the oracle's
twist on D, the automatic choice per matrix, the choice per dimension block
(some blocks on D', the others on D), the fall-back to D for inputs whose
buckets are not graded, batches, and the drop-in call."""
import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import Context

from cases import lower_star_volume, mixed_buckets, random_complex, simplex_skeleton, small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()


@pytest.fixture(scope="module")
def dctx(cuda_lib):
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("mode", ["always", "never", "auto", "blocks"])
def test_small_cases(dctx, name, mode):
    bm = CASES[name]
    dctx.set_dual(mode)
    low, ess, arglow, info = dctx.reduce(bm, "pms", with_arglow=True)
    dctx.set_dual("auto")
    want, want_ess, _ = oracle.twist(bm)
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    want_arg = np.full(bm.m, -1, np.int32)
    j = np.nonzero(want >= 0)[0]
    want_arg[want[j]] = j
    np.testing.assert_array_equal(arglow, want_arg)
    if mode in ("always", "never"):  # every small case is graded
        assert info["dual"] == (1 if mode == "always" else 0)


@pytest.mark.parametrize("seed", range(3))
def test_larger_complexes_both_ways(dctx, seed):
    mats = [cx.rips_cube(40 + 5 * seed, seed=seed), cx.rips_mixed(45, seed=seed),
            cx.lower_star_image(40, 56, seed=seed, sigma=2.0), random_complex(30, 0.4, 0.5, seed=300 + seed),
            simplex_skeleton(8, seed=40 + seed, max_dim=4)]
    for bm in mats:
        want, want_ess, _ = oracle.twist(bm)
        for mode in ("always", "never", "blocks"):
            dctx.set_dual(mode)
            low, ess, info = dctx.reduce(bm, "pms")
            np.testing.assert_array_equal(low, want, err_msg=f"{mode} m={bm.m}")
            np.testing.assert_array_equal(ess, want_ess, err_msg=f"{mode} m={bm.m}")
            if mode != "blocks":
                assert info["dual"] == (1 if mode == "always" else 0)
    dctx.set_dual("auto")


@pytest.mark.parametrize("shape", [(12, 12, 1.0), (40, 56, 2.0), (64, 33, 4.0), (97, 80, 3.0)])
def test_lower_star_split_by_block(dctx, shape):
    """A lower-star image's edges-on-vertices block on D, its
    triangles-on-edges block on D' (every edge has at most two triangles):
    the D' part first, then D with the edges it paired cleared; low and ess
    equal to the oracle's twist on D."""
    h, w, sigma = shape
    bm = cx.lower_star_image(h, w, seed=h + w, sigma=sigma)
    want, want_ess, _ = oracle.twist(bm)
    dctx.set_dual("blocks")
    low, ess, arglow, info = dctx.reduce(bm, "pms", with_arglow=True)
    dctx.set_dual("auto")
    assert info["dual"] == 2
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    want_arg = np.full(bm.m, -1, np.int32)
    j = np.nonzero(want >= 0)[0]
    want_arg[want[j]] = j
    np.testing.assert_array_equal(arglow, want_arg)


@pytest.mark.parametrize("n,seed", [(6, 1), (10, 2), (13, 3)])
def test_lower_star_volume_split(dctx, n, seed):
    """A 3-D lower-star volume: tetrahedra-on-triangles on D' (a triangle has
    at most two tetrahedra), triangles-on-edges and edges-on-vertices on D,
    with the triangles D' paired cleared; equal to the oracle's twist."""
    bm = lower_star_volume(n, seed)
    want, want_ess, _ = oracle.twist(bm)
    dctx.set_dual("blocks")
    low, ess, info = dctx.reduce(bm, "pms")
    dctx.set_dual("auto")
    assert info["dual"] == 2
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


def test_split_pool_regrow(dctx):
    """A split reduction whose D part (the triangles of a 3-D volume) grows
    its columns past a column store holding only the packed input."""
    bm = lower_star_volume(10, 5)
    want, want_ess, _ = oracle.twist(bm)
    with Context(0) as c:
        c.set_limits(initial_pool_bytes=1)
        c.set_dual("blocks")
        low, ess, info = c.reduce(bm, "pms")
    assert info["dual"] == 2 and info["regrows"] > 0
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


def test_auto_choice(dctx):
    """Rips complexes of 2^17 columns or more (top bucket >= 8x the bottom
    one) go to D'; a smaller one stays on D; a lower-star image of that size
    (triangles about twice the vertices, edges with at most two triangles)
    is split by block, a smaller one stays on D."""
    dctx.set_dual("auto")
    _, _, info = dctx.reduce(cx.rips_cube(100, seed=1), "pms")  # 166,750 columns
    assert info["dual"] == 1
    _, _, info = dctx.reduce(cx.rips_cube(30, seed=1), "pms")
    assert info["dual"] == 0
    bm = cx.lower_star_image(256, 256, seed=2)
    low, ess, info = dctx.reduce(bm, "pms")
    assert info["dual"] == 2
    dctx.set_dual("never")
    low_d, ess_d, info_d = dctx.reduce(bm, "pms")
    dctx.set_dual("auto")
    assert info_d["dual"] == 0
    np.testing.assert_array_equal(low, low_d)
    np.testing.assert_array_equal(ess, ess_d)
    _, _, info = dctx.reduce(cx.lower_star_image(64, 64, seed=2), "pms")
    assert info["dual"] == 0
    _, _, info = dctx.reduce(CASES["empty5"], "pms")
    assert info["dual"] == 0


def test_ungraded_input_stays_on_d(dctx):
    """Columns of three rows from two buckets: 'always' falls back to D and
    gives the same result as 'never'."""
    bm = mixed_buckets()
    dctx.set_dual("never")
    low_n, ess_n, info_n = dctx.reduce(bm, "pms")
    dctx.set_dual("always")
    low_a, ess_a, info_a = dctx.reduce(bm, "pms")
    dctx.set_dual("auto")
    assert info_a["dual"] == 0 and info_n["dual"] == 0
    np.testing.assert_array_equal(low_a, low_n)
    np.testing.assert_array_equal(ess_a, ess_n)


def test_dual_does_few_additions_on_rips(dctx):
    bm = cx.rips_torus(400, 200_000, seed=5)
    want, want_ess, st = oracle.twist(bm)
    dctx.set_dual("auto")
    low, ess, info = dctx.reduce(bm, "pms")
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
    assert info["dual"] == 1
    assert info["additions"] * 100 < st["additions"]


@pytest.mark.parametrize("mode", ["always", "auto", "never", "blocks"])
def test_batch(dctx, mode):
    from cases import empty_columns, triangle
    from openph_gb300.complexes import BoundaryMatrix
    mats = [cx.rips_mixed(n, seed=60 + n) for n in (9, 21, 14)] + [
        BoundaryMatrix.from_columns([]), triangle(), empty_columns(3), cx.lower_star_image(9, 7, seed=5),
        simplex_skeleton(6, seed=2)]
    dctx.set_dual(mode)
    lows, esss, info = dctx.reduce_batch(mats, "pms")
    dctx.set_dual("auto")
    for bm, low, ess in zip(mats, lows, esss):
        if bm.m == 0:
            continue
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def test_batch_of_images_split_by_block(dctx):
    """A batch of lower-star images reduced block by block (the batch's
    triangles on its anti-transpose, built per instance, its edges on D):
    every instance equal to the oracle's twist."""
    mats = [cx.lower_star_image(h, w, seed=h * w, sigma=2.0) for h, w in ((12, 9), (20, 20), (7, 31), (33, 25))]
    dctx.set_dual("blocks")
    lows, esss, info = dctx.reduce_batch(mats, "pms")
    dctx.set_dual("auto")
    assert info["dual"] == 2
    for bm, low, ess in zip(mats, lows, esss):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def star(n_leaves):
    """A vertex joined to n_leaves others: its column of D' holds n_leaves rows."""
    from openph_gb300.complexes import BoundaryMatrix
    return BoundaryMatrix.from_columns([[] for _ in range(n_leaves + 1)] + [[0, i] for i in range(1, n_leaves + 1)])


@pytest.mark.parametrize("odd", ["window", "wide_column", "none"])
def test_batch_transpose_fallback(dctx, odd):
    """A batch whose instances all fit the per-instance transpose (rows within
    16,384 of their first column, D' columns of at most 512 rows) takes it;
    one instance outside those bounds (a 90x90 lower-star image, 24K vertices
    and edges; a vertex of 600 edges) sends the whole batch to the general
    transpose.  Every instance equal to the oracle's twist either way."""
    mats = [cx.rips_mixed(30, seed=3), cx.rips_mixed(12, seed=5), star(40)]
    if odd == "window":
        mats.insert(1, cx.lower_star_image(90, 90, seed=4, sigma=3.0))
    elif odd == "wide_column":
        mats.insert(1, star(600))
    dctx.set_dual("always")
    lows, esss, info = dctx.reduce_batch(mats, "pms")
    dctx.set_dual("auto")
    assert info["dual"] == 1
    for bm, low, ess in zip(mats, lows, esss):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def test_batch_transpose_both_ways(dctx, monkeypatch):
    """64 instances of the batched mix through the per-instance transpose and
    through the general one (OPH_NO_INST_TRANSPOSE): both equal to the oracle,
    and the first launches fewer set-up kernels (it was taken, not fallen back
    from)."""
    col_off, colptr, rows, npts, _ = cx.rips_mixed_batch(64, seed=11)
    jobs = [(colptr[col_off[b]:col_off[b + 1] + 1] - colptr[col_off[b]],
             rows[colptr[col_off[b]]:colptr[col_off[b + 1]]]) for b in range(64)]
    want = oracle.twist_many(jobs)
    launches = []
    for inst in (True, False):
        if not inst:
            monkeypatch.setenv("OPH_NO_INST_TRANSPOSE", "1")
        dctx.set_profile(True)
        low, ess, info = dctx.reduce_batch_packed(col_off, colptr, rows, "pms")
        launches.append(dctx.last_profile()["kernel_launches"])
        dctx.set_profile(False)
        assert info["dual"] == 1
        for b in range(64):
            np.testing.assert_array_equal(low[col_off[b]:col_off[b + 1]], want[b][0])
            np.testing.assert_array_equal(ess[col_off[b]:col_off[b + 1]], want[b][1])
    assert launches[0] < launches[1], launches


def test_drop_in_call_without_trackers(cuda_lib):
    """openph() with no tracker outputs takes D' on a large Rips complex
    (1-based COO in, 1-based lows out); with trackers it reduces D."""
    from openph_gb300.api import ph
    bm = cx.rips_cube(100, seed=8)
    want, want_ess, _ = oracle.twist(bm)
    r, c = bm.to_coo1()
    low, ess, *_ = ph("pms", r, c, bm.m, 0)
    np.testing.assert_array_equal(low, want + 1)
    np.testing.assert_array_equal(ess, want_ess)
    low, ess, linf, *_ , it = ph("pms", r, c, bm.m, 0, (want + 1).astype(np.int32))
    np.testing.assert_array_equal(low, want + 1)
    assert linf[int(it[0]) - 1] == 0.0


def test_rips_torus_1m_device_input(dctx):
    """The torus family through oph_reduce_device, D' chosen automatically."""
    import torch
    bm = cx.rips_torus(400, 1_000_000, seed=2)
    want, want_ess, _ = oracle.twist(bm)
    cp = torch.as_tensor(bm.colptr, device="cuda")
    rw = torch.as_tensor(bm.rows, device="cuda")
    low = torch.empty(bm.m, dtype=torch.int32, device="cuda")
    ess = torch.empty(bm.m, dtype=torch.int32, device="cuda")
    info = dctx.reduce_device(bm.m, cp.data_ptr(), rw.data_ptr(), low.data_ptr(), ess.data_ptr())
    assert info["dual"] == 1
    np.testing.assert_array_equal(low.cpu().numpy(), want)
    np.testing.assert_array_equal(ess.cpu().numpy(), want_ess)


def fan(n_rim, seed):
    """A fan: vertex 0 joined to n_rim rim vertices, the rim a path, the
    triangles {0, k, k+1}; edges and triangles in a seeded filtration order
    (every face before its cofaces).  Vertex 0's column of the anti-transpose
    holds n_rim rows."""
    from openph_gb300.complexes import BoundaryMatrix
    rng = np.random.default_rng(seed)
    nv = n_rim + 1
    edges = [(0, k) for k in range(1, nv)] + [(k, k + 1) for k in range(1, nv - 1)]
    order = rng.permutation(len(edges))
    edges = [edges[i] for i in order]
    epos = {e: nv + i for i, e in enumerate(edges)}
    tris = [(0, k, k + 1) for k in range(1, nv - 1)]
    tris.sort(key=lambda t: max(epos[(0, t[1])], epos[(0, t[2])], epos[(t[1], t[2])]))
    cols = [[] for _ in range(nv)] + [[a, b] for a, b in edges]
    cols += [[epos[(0, k)], epos[(0, l)], epos[(k, l)]] for _, k, l in tris]
    return BoundaryMatrix.from_columns(cols)


@pytest.mark.parametrize("n_rim", [12, 40, 200, 700, 3000, 20000])
def test_transpose_long_columns(dctx, n_rim):
    """Columns of the anti-transpose of every length class: <= 8 rows (a
    thread), <= 32 and <= 128 (a warp's registers, 1 or 4 values a lane),
    <= 256 (8 values a lane) and beyond (a CTA's radix sort, several tiles
    of it at 20,000 rows)."""
    bm = fan(n_rim, seed=n_rim)
    dctx.set_dual("always")
    low, ess, info = dctx.reduce(bm, "pms")
    dctx.set_dual("auto")
    assert info["dual"] == 1
    want, want_ess, _ = oracle.twist(bm)
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)
