"""Complexes built on the GPU equal the host generators' matrices bit for bit
(values, order, rows), and reduce to the oracle's lows."""
import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import Context, OphError

pytestmark = pytest.mark.gpu


def assert_same(dev, host):
    h = dev.to_host()
    np.testing.assert_array_equal(h.colptr, host.colptr)
    np.testing.assert_array_equal(h.rows, host.rows)
    np.testing.assert_array_equal(h.values.view(np.uint64), host.values.view(np.uint64))


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 3), (7, 2), (50, 1), (120, 8)])
def test_rips_full_equals_host(cuda_lib, n, seed):
    pts = cx.points_cube(n, seed)
    assert_same(cx.rips_device(pts), cx.rips(pts))


@pytest.mark.parametrize("target_m", [20_000, 200_000, 1_000_000])
def test_rips_torus_threshold_equals_host(cuda_lib, target_m):
    pts = cx.points_torus(400, 2)
    thr = cx.rips_threshold(pts, target_m)
    assert_same(cx.rips_device(pts, thr), cx.rips(pts, thr))


def test_rips_duplicate_points_and_zero_threshold(cuda_lib):
    pts = cx.points_circle(30, 5)
    pts = np.concatenate([pts, pts[:7]])  # zero-length edges tie with vertices on value
    assert_same(cx.rips_device(pts), cx.rips(pts))
    assert_same(cx.rips_device(pts, 0.0), cx.rips(pts, 0.0))


@pytest.mark.parametrize("h,w,seed", [(2, 2, 1), (3, 5, 2), (64, 64, 6), (512, 512, 3)])
def test_lower_star_equals_host(cuda_lib, h, w, seed):
    img = cx.image_smoothed(h, w, seed)
    assert_same(cx.lower_star_device(img), cx.lower_star(img))


def test_lower_star_ties(cuda_lib):
    img = np.round(cx.image_smoothed(40, 30, 4) * 4).astype(np.float32)  # many equal values
    assert_same(cx.lower_star_device(img), cx.lower_star(img))


def test_device_built_matrix_reduces_to_oracle(cuda_lib):
    import torch
    pts = cx.points_torus(400, 2)
    thr = cx.rips_threshold(pts, 300_000)
    with Context(0) as ctx:
        dm = cx.rips_device(pts, thr, ctx=ctx)
        low = torch.empty(dm.m, dtype=torch.int32, device="cuda")
        ctx.reduce_device(dm.m, dm.colptr.data_ptr(), dm.rows.data_ptr(), low.data_ptr())
    want, _, _ = oracle.twist(cx.rips(pts, thr))
    np.testing.assert_array_equal(low.cpu().numpy(), want)


def test_generator_input_errors(cuda_lib):
    import torch
    with Context(0) as ctx:
        with pytest.raises(OphError):
            ctx.rips_device(torch.zeros(1, 3, dtype=torch.float64, device="cuda").data_ptr(), 0, 3, 1.0,
                            lambda m, nnz: (0, 0, 0))
        with pytest.raises(OphError):
            ctx.lower_star_device(torch.zeros(4, dtype=torch.float32, device="cuda").data_ptr(), 1, 4,
                                  lambda m, nnz: (0, 0, 0))
        with pytest.raises(OphError):
            ctx.rips_device(torch.zeros(3, dtype=torch.float64, device="cuda").data_ptr(), 1, 3, float("nan"),
                            lambda m, nnz: (0, 0, 0))
