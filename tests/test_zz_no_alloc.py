"""The allocation-free pms entry point, oph_reduce_pms_noalloc, called
through the C ABI and checked against the allocating entry point
oph_reduce_device on the same device buffers.

Callers that cannot call cudaMalloc (a framework whose caching allocator owns
the GPU's memory, a real-time pipeline, code inside a stream capture) use this
entry point; its working arrays live in one fixed scratch array inside the
library that every call reuses.  Two calls in a row on different matrices
must each equal the allocating path, so nothing of one call may leak into the
next; a matrix too large for the scratch must be refused.  This file is
collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from openph_gb300 import complexes as cx
from openph_gb300.api import OPH_ERR_OOM, OPH_OK, Context

pytestmark = pytest.mark.gpu


def _device(bm, torch):
    dev = torch.device("cuda", 0)
    colptr = torch.from_numpy(bm.colptr).to(dev)
    rows = torch.from_numpy(bm.rows if bm.nnz else np.zeros(1, np.int32)).to(dev)
    return colptr, rows


def _noalloc(lib, bm, torch, stream):
    colptr, rows = _device(bm, torch)
    low = torch.full((bm.m,), -7, dtype=torch.int32, device="cuda:0")
    ess = torch.full((bm.m,), -7, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    rc = lib.oph_reduce_pms_noalloc(C.c_int64(bm.m), C.c_void_p(colptr.data_ptr()), C.c_void_p(rows.data_ptr()),
                                    C.c_void_p(low.data_ptr()), C.c_void_p(ess.data_ptr()), C.c_void_p(stream))
    return rc, low.cpu().numpy(), ess.cpu().numpy()


def _allocating(ctx, bm, torch):
    colptr, rows = _device(bm, torch)
    low = torch.empty(bm.m, dtype=torch.int32, device="cuda:0")
    ess = torch.empty(bm.m, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    ctx.reduce_device(bm.m, colptr.data_ptr(), rows.data_ptr(), low.data_ptr(), ess.data_ptr(), None, "pms")
    return low.cpu().numpy(), ess.cpu().numpy()


@pytest.fixture(scope="module")
def lib(cuda_lib):
    cuda_lib.oph_reduce_pms_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]
    cuda_lib.oph_reduce_pms_noalloc.restype = C.c_int
    return cuda_lib


def test_two_calls_in_a_row_match_the_allocating_path(lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    mats = [cx.lower_star_image(40, 40, seed=21, sigma=3.0), cx.rips_cube(30, seed=22),
            cx.rips_mixed(27, seed=23), cx.rips_cube(30, seed=22)]
    with Context(0) as ctx:
        for bm in mats:
            rc, low, ess = _noalloc(lib, bm, torch, stream)
            assert rc == OPH_OK
            want_low, want_ess = _allocating(ctx, bm, torch)
            np.testing.assert_array_equal(low, want_low)
            np.testing.assert_array_equal(ess, want_ess)


def test_default_stream_and_too_large_refused(lib):
    torch = pytest.importorskip("torch")
    small = cx.rips_cube(16, seed=5)
    rc, low, _ = _noalloc(lib, small, torch, None)
    assert rc == OPH_OK
    with Context(0) as ctx:
        np.testing.assert_array_equal(low, _allocating(ctx, small, torch)[0])
    big = cx.lower_star_image(400, 400, seed=2)  # ~960,000 columns: past the fixed scratch
    rc, _, _ = _noalloc(lib, big, torch, None)
    assert rc == OPH_ERR_OOM
