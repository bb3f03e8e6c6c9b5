"""The allocation-free pms entry point, oph_reduce_pms_noalloc, called
through the C ABI and checked against the oracle and against the allocating
entry point oph_reduce_device on the same device buffers.

Callers that cannot call cudaMalloc (a framework whose caching allocator owns
the GPU's memory, or a real-time pipeline that cannot afford cudaMalloc's
implicit synchronisation) use this entry point; its working arrays live in
one fixed scratch array inside the library that every call reuses.  Calls in
a row on different matrices must each equal the oracle and the allocating
path, so nothing of one call may leak into the next — also after a call that
failed; a matrix too large for the scratch must be refused, a column store
that would have to grow reports OPH_ERR_OVERFLOW, and a malformed CSC is
refused before anything is written.  This file is collected last on
purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import OPH_ERR_BAD_INPUT, OPH_ERR_OOM, OPH_ERR_OVERFLOW, OPH_OK, Context
from openph_gb300.complexes import BoundaryMatrix

pytestmark = pytest.mark.gpu


def _device(colptr, rows, torch):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(np.ascontiguousarray(colptr)).to(dev),
            torch.from_numpy(np.ascontiguousarray(rows) if len(rows) else np.zeros(1, np.int32)).to(dev))


def _noalloc(lib, bm, torch, stream, with_ess=True, colptr=None, rows=None):
    colptr, rows = _device(bm.colptr if colptr is None else colptr, bm.rows if rows is None else rows, torch)
    low = torch.full((max(bm.m, 1),), -7, dtype=torch.int32, device="cuda:0")
    ess = torch.full((max(bm.m, 1),), -7, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    rc = lib.oph_reduce_pms_noalloc(C.c_int64(bm.m), C.c_void_p(colptr.data_ptr()), C.c_void_p(rows.data_ptr()),
                                    C.c_void_p(low.data_ptr()), C.c_void_p(ess.data_ptr()) if with_ess else None,
                                    C.c_void_p(stream))
    return rc, low.cpu().numpy()[:bm.m], ess.cpu().numpy()[:bm.m]


def _allocating(ctx, bm, torch):
    colptr, rows = _device(bm.colptr, bm.rows, torch)
    low = torch.empty(max(bm.m, 1), dtype=torch.int32, device="cuda:0")
    ess = torch.empty(max(bm.m, 1), dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    ctx.reduce_device(bm.m, colptr.data_ptr(), rows.data_ptr(), low.data_ptr(), ess.data_ptr(), None, "pms")
    return low.cpu().numpy()[:bm.m], ess.cpu().numpy()[:bm.m]


def _check(lib, ctx, bm, torch, stream):
    """One call: equal to the oracle's twist and to the allocating path."""
    rc, low, ess = _noalloc(lib, bm, torch, stream)
    assert rc == OPH_OK
    want_low, want_ess, _ = oracle.twist(bm)
    np.testing.assert_array_equal(low, want_low)
    np.testing.assert_array_equal(ess, want_ess)
    a_low, a_ess = _allocating(ctx, bm, torch)
    np.testing.assert_array_equal(low, a_low)
    np.testing.assert_array_equal(ess, a_ess)


@pytest.fixture(scope="module")
def lib(cuda_lib):
    cuda_lib.oph_reduce_pms_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]
    cuda_lib.oph_reduce_pms_noalloc.restype = C.c_int
    return cuda_lib


def test_two_calls_in_a_row_match_the_oracle_and_the_allocating_path(lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    mats = [cx.lower_star_image(40, 40, seed=21, sigma=3.0), cx.rips_cube(30, seed=22),
            cx.rips_mixed(27, seed=23), cx.rips_cube(30, seed=22)]
    with Context(0) as ctx:
        for bm in mats:
            _check(lib, ctx, bm, torch, stream)


def test_default_stream_and_too_large_refused(lib):
    torch = pytest.importorskip("torch")
    small = cx.rips_cube(16, seed=5)
    with Context(0) as ctx:
        _check(lib, ctx, small, torch, None)
    big = cx.lower_star_image(400, 400, seed=2)  # ~960,000 columns: past the fixed scratch
    rc, _, _ = _noalloc(lib, big, torch, None)
    assert rc == OPH_ERR_OOM


def test_empty_inputs_and_no_ess(lib):
    """m == 0, columns without entries (nnz == 0), and d_ess == NULL."""
    torch = pytest.importorskip("torch")
    rc, low, _ = _noalloc(lib, BoundaryMatrix.from_columns([]), torch, None)
    assert rc == OPH_OK and low.size == 0
    verts = BoundaryMatrix.from_columns([[] for _ in range(6)])
    rc, low, ess = _noalloc(lib, verts, torch, None)
    assert rc == OPH_OK
    np.testing.assert_array_equal(low, np.full(6, -1, np.int32))
    np.testing.assert_array_equal(ess, np.ones(6, np.int32))
    bm = cx.rips_mixed(21, seed=8)
    rc, low, ess = _noalloc(lib, bm, torch, None, with_ess=False)
    assert rc == OPH_OK
    np.testing.assert_array_equal(low, oracle.twist(bm)[0])
    assert np.all(ess == -7)  # no ess requested: the buffer is untouched


def test_column_store_overflow_reported_then_next_call_exact(lib):
    """A full 2-skeleton Rips complex of 109 points (215,929 columns) fits
    the scratch with its packed input twice over, but reducing its triangle
    columns on the boundary matrix itself fills the column store past that
    (the allocating path uses ~2.3 times the packed size): the call returns
    OPH_ERR_OVERFLOW, and the calls after it are exact."""
    torch = pytest.importorskip("torch")
    bm = cx.rips_cube(109, seed=4)
    assert bm.m == 215_929
    rc, _, _ = _noalloc(lib, bm, torch, None)
    assert rc == OPH_ERR_OVERFLOW
    with Context(0) as ctx:
        _check(lib, ctx, cx.rips_cube(26, seed=31), torch, None)
        _check(lib, ctx, cx.lower_star_image(36, 36, seed=32, sigma=3.0), torch, None)


@pytest.mark.parametrize("how", ["colptr_decreasing", "colptr_past_nnz", "row_out_of_range", "rows_not_ascending"])
def test_malformed_csc_refused_before_anything_runs(lib, how):
    torch = pytest.importorskip("torch")
    bm = cx.rips_cube(14, seed=3)
    colptr, rows = bm.colptr.copy(), bm.rows.copy()
    if how == "colptr_decreasing":
        j = int(np.nonzero(np.diff(colptr) > 1)[0][0])
        colptr[j + 1] = colptr[j + 2] + 1
    elif how == "colptr_past_nnz":
        colptr[bm.m // 2] = colptr[-1] + 1000
    elif how == "row_out_of_range":
        rows[-1] = bm.m + 7
    else:
        a = int(colptr[-2])
        rows[a], rows[a + 1] = rows[a + 1], rows[a]
    rc, low, _ = _noalloc(lib, bm, torch, None, colptr=colptr, rows=rows)
    assert rc == OPH_ERR_BAD_INPUT
    assert np.all(low == -7)  # nothing written
    with Context(0) as ctx:
        _check(lib, ctx, bm, torch, None)
