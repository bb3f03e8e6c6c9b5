"""Filtered simplicial complexes and their Z/2 boundary matrices.

A :class:`BoundaryMatrix` holds one complex in the canonical layout every
entry point here consumes: 0-based CSC with ``colptr`` (int64, m+1) and
``rows`` (int32, ascending inside each column), columns in filtration order
(value, dimension, lexicographic vertex tuple).  ``to_coo1()`` gives the
1-based (rows, cols) pair that the reference's ``ph``/``openph()`` call takes
(src/matlab/ph/ph.cu:29-40, src/cuda/openph.cu:29-35).

The generators stand in for the reference's Javaplex streams
(numerics/utils/example_factory.m:17-114 via stream2cmo.m:1-26): seeded
point clouds, Vietoris–Rips complexes of dimension <= 2 with FP64 distances,
and lower-star filtrations of smoothed FP32 images on the Freudenthal
triangulation.  They run natively (``gen/ophgen.c``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _build


class _Complex(C.Structure):
    _fields_ = [("m", C.c_int64), ("nnz", C.c_int64), ("colptr", C.POINTER(C.c_int64)),
                ("rows", C.POINTER(C.c_int32)), ("value", C.POINTER(C.c_double)),
                ("dim", C.POINTER(C.c_int8))]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        path = _build.GENLIB
        if not path.exists():
            _build.build_gen()
        lib = C.CDLL(str(path))
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        lib.oph_points_cube.argtypes = [C.c_int, C.c_int, C.c_uint64, dp]
        lib.oph_points_torus.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, dp]
        lib.oph_points_circle.argtypes = [C.c_int, C.c_double, C.c_uint64, dp]
        lib.oph_image_smoothed.argtypes = [C.c_int, C.c_int, C.c_double, C.c_uint64, fp]
        lib.oph_rips.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.POINTER(_Complex)]
        lib.oph_rips_threshold.argtypes = [dp, C.c_int, C.c_int, C.c_int64]
        lib.oph_rips_threshold.restype = C.c_double
        lib.oph_lower_star.argtypes = [fp, C.c_int, C.c_int, C.POINTER(_Complex)]
        lib.oph_complex_free.argtypes = [C.POINTER(_Complex)]
        lib.oph_rips_mixed_batch.argtypes = [C.c_int, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"),
                                             np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS"), C.c_int,
                                             np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS"),
                                             C.POINTER(_Complex)]
        _gen = lib
    return _gen


@dataclass
class BoundaryMatrix:
    """A Z/2 boundary matrix in 0-based CSC, columns in filtration order."""

    colptr: np.ndarray  # int64[m+1]
    rows: np.ndarray  # int32[nnz]
    values: np.ndarray | None = None  # float64[m] filtration values
    dims: np.ndarray | None = None  # int8[m] simplex dimensions
    meta: dict = field(default_factory=dict)

    def __post_init__(self):
        self.colptr = np.ascontiguousarray(self.colptr, dtype=np.int64)
        self.rows = np.ascontiguousarray(self.rows, dtype=np.int32)

    @property
    def m(self) -> int:
        return int(self.colptr.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.colptr[-1])

    def to_coo1(self):
        """1-based (rows, cols) int32 COO, column-major, as ``ph`` takes it."""
        counts = np.diff(self.colptr)
        cols = np.repeat(np.arange(1, self.m + 1, dtype=np.int32), counts)
        return (self.rows + 1).astype(np.int32), cols

    @staticmethod
    def from_coo1(r, c, m: int) -> "BoundaryMatrix":
        """From 1-based COO (columns non-decreasing, rows ascending per column)."""
        r = np.asarray(r, dtype=np.int64)
        c = np.asarray(c, dtype=np.int64)
        counts = np.bincount(c - 1, minlength=m) if c.size else np.zeros(m, np.int64)
        colptr = np.zeros(m + 1, np.int64)
        np.cumsum(counts, out=colptr[1:])
        return BoundaryMatrix(colptr, (r - 1).astype(np.int32))

    @staticmethod
    def from_columns(cols) -> "BoundaryMatrix":
        """From a list of row-index lists (0-based); each is sorted here."""
        colptr = np.zeros(len(cols) + 1, np.int64)
        for j, c in enumerate(cols):
            colptr[j + 1] = colptr[j] + len(c)
        rows = np.zeros(int(colptr[-1]), np.int32)
        for j, c in enumerate(cols):
            rows[colptr[j]:colptr[j + 1]] = sorted(c)
        return BoundaryMatrix(colptr, rows)

    def column(self, j: int) -> np.ndarray:
        return self.rows[self.colptr[j]:self.colptr[j + 1]]

    # canonical binary file: "OPHCSC01", int64 m, int64 nnz, colptr, rows
    def save(self, path) -> None:
        with open(path, "wb") as f:
            f.write(b"OPHCSC01")
            np.array([self.m, self.nnz], np.int64).tofile(f)
            self.colptr.tofile(f)
            self.rows.tofile(f)

    @staticmethod
    def load(path) -> "BoundaryMatrix":
        with open(path, "rb") as f:
            if f.read(8) != b"OPHCSC01":
                raise ValueError(f"{path}: not an OPHCSC01 file")
            m, nnz = np.fromfile(f, np.int64, 2)
            colptr = np.fromfile(f, np.int64, int(m) + 1)
            rows = np.fromfile(f, np.int32, int(nnz))
        return BoundaryMatrix(colptr, rows)


def _take(cx: _Complex, meta) -> BoundaryMatrix:
    m, nnz = cx.m, cx.nnz
    colptr = np.ctypeslib.as_array(cx.colptr, shape=(m + 1,)).copy()
    rows = np.ctypeslib.as_array(cx.rows, shape=(max(nnz, 1),))[:nnz].copy()
    values = np.ctypeslib.as_array(cx.value, shape=(m,)).copy()
    dims = np.ctypeslib.as_array(cx.dim, shape=(m,)).copy()
    _lib().oph_complex_free(C.byref(cx))
    return BoundaryMatrix(colptr, rows, values, dims, meta)


# ------------------------------------------------------------------ points
def points_cube(n: int, seed: int, d: int = 3) -> np.ndarray:
    out = np.empty(n * d, np.float64)
    _lib().oph_points_cube(n, d, seed, out)
    return out.reshape(n, d)


def points_torus(n: int, seed: int, R: float = 2.0, r: float = 1.0, sigma: float = 0.05) -> np.ndarray:
    out = np.empty(n * 3, np.float64)
    _lib().oph_points_torus(n, R, r, sigma, seed, out)
    return out.reshape(n, 3)


def points_circle(n: int, seed: int, sigma: float = 0.05) -> np.ndarray:
    out = np.empty(n * 3, np.float64)
    _lib().oph_points_circle(n, sigma, seed, out)
    return out.reshape(n, 3)


def image_smoothed(h: int, w: int, seed: int, sigma: float = 4.0) -> np.ndarray:
    out = np.empty(h * w, np.float32)
    if _lib().oph_image_smoothed(h, w, sigma, seed, out) != 0:
        raise MemoryError("image generation failed")
    return out.reshape(h, w)


# --------------------------------------------------------------- complexes
def rips(points: np.ndarray, threshold: float = float("inf")) -> BoundaryMatrix:
    """Vietoris–Rips complex of dimension <= 2 (edges of length <= threshold)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n, d = pts.shape
    cx = _Complex()
    if _lib().oph_rips(pts.reshape(-1), n, d, threshold, C.byref(cx)) != 0:
        raise MemoryError("rips generation failed")
    return _take(cx, {"kind": "rips", "n_points": n, "threshold": threshold})


def rips_threshold(points: np.ndarray, target_m: int) -> float:
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n, d = pts.shape
    return float(_lib().oph_rips_threshold(pts.reshape(-1), n, d, target_m))


def lower_star(image: np.ndarray) -> BoundaryMatrix:
    img = np.ascontiguousarray(image, dtype=np.float32)
    h, w = img.shape
    cx = _Complex()
    if _lib().oph_lower_star(img.reshape(-1), h, w, C.byref(cx)) != 0:
        raise MemoryError("lower-star generation failed")
    return _take(cx, {"kind": "lower_star", "shape": (h, w)})


# ------------------------------------------------------ on the device
@dataclass
class DeviceMatrix:
    """A boundary matrix built in device memory (torch tensors): 0-based
    CSC, columns in filtration order, and the FP64 filtration values."""

    colptr: object  # torch.int64[m + 1]
    rows: object  # torch.int32[nnz]
    values: object  # torch.float64[m]
    meta: dict = field(default_factory=dict)

    @property
    def m(self) -> int:
        return int(self.colptr.shape[0]) - 1

    @property
    def nnz(self) -> int:
        return int(self.rows.shape[0])

    def to_host(self) -> BoundaryMatrix:
        return BoundaryMatrix(self.colptr.cpu().numpy(), self.rows.cpu().numpy(), self.values.cpu().numpy(),
                              None, dict(self.meta))


def _device_build(ctx, device, build):
    import torch

    from . import api
    own = ctx is None
    if own:
        ctx = api.Context(device.index or 0)
    try:
        out = {}

        def alloc(m, nnz):
            out["colptr"] = torch.empty(m + 1, dtype=torch.int64, device=device)
            out["rows"] = torch.empty(max(nnz, 1), dtype=torch.int32, device=device)
            out["values"] = torch.empty(max(m, 1), dtype=torch.float64, device=device)
            return out["colptr"].data_ptr(), out["rows"].data_ptr(), out["values"].data_ptr()

        # inputs written on torch's stream must land before the context's
        # stream reads them
        torch.cuda.current_stream(device).synchronize()
        m, nnz = build(ctx, alloc)
        return out["colptr"], out["rows"][:nnz], out["values"][:m]
    finally:
        if own:
            ctx.close()


def rips_device(points, threshold: float = float("inf"), ctx=None, device=None) -> DeviceMatrix:
    """The Rips complex of ``rips`` built on the GPU from points (a numpy
    array or a CUDA tensor, n x d); identical output, device-resident."""
    import torch
    device = torch.device(device or "cuda")
    pts = torch.as_tensor(points, dtype=torch.float64).to(device).contiguous()
    n, d = pts.shape
    colptr, rows, values = _device_build(
        ctx, device, lambda c, alloc: c.rips_device(pts.data_ptr(), n, d, threshold, alloc))
    return DeviceMatrix(colptr, rows, values, {"kind": "rips", "n_points": n, "threshold": threshold})


def lower_star_device(image, ctx=None, device=None) -> DeviceMatrix:
    """The lower-star complex of ``lower_star`` built on the GPU from an
    h x w FP32 image (numpy or CUDA tensor)."""
    import torch
    device = torch.device(device or "cuda")
    img = torch.as_tensor(image, dtype=torch.float32).to(device).contiguous()
    h, w = img.shape
    colptr, rows, values = _device_build(ctx, device,
                                         lambda c, alloc: c.lower_star_device(img.data_ptr(), h, w, alloc))
    return DeviceMatrix(colptr, rows, values, {"kind": "lower_star", "shape": (h, w)})


# --------------------------------------------------- the benchmark shapes
def rips_cube(n_points: int = 50, seed: int = 1) -> BoundaryMatrix:
    """Full 2-skeleton Rips complex of n points uniform in [0,1]^3."""
    bm = rips(points_cube(n_points, seed))
    bm.meta.update(workload="rips_cube", seed=seed)
    return bm


def rips_torus(n_points: int = 400, target_m: int = 5_000_000, seed: int = 2) -> BoundaryMatrix:
    """Rips complex (dim <= 2) of a noisy torus (R=2, r=1, sigma=0.05) with
    the edge threshold chosen so the complex has about target_m simplices."""
    pts = points_torus(n_points, seed)
    thr = rips_threshold(pts, target_m)
    bm = rips(pts, thr)
    bm.meta.update(workload="rips_torus", seed=seed, target_m=target_m)
    return bm


def lower_star_image(h: int = 512, w: int = 512, seed: int = 3, sigma: float = 4.0) -> BoundaryMatrix:
    bm = lower_star(image_smoothed(h, w, seed, sigma))
    bm.meta.update(workload="lower_star", seed=seed)
    return bm


def rips_mixed(n_points: int, seed: int) -> BoundaryMatrix:
    """One instance of the batched mix: full 2-skeleton Rips of n points,
    uniform in [0,1]^3 (even seed) or on a noisy unit circle (odd seed)."""
    pts = points_cube(n_points, seed) if seed % 2 == 0 else points_circle(n_points, seed)
    bm = rips(pts)
    bm.meta.update(workload="rips_mixed", seed=seed)
    return bm


def mixed_batch_sizes(count: int, seed: int, lo: int = 20, hi: int = 120):
    """Point counts ~ U[lo, hi] and per-instance seeds of the batched mix."""
    rng = np.random.default_rng(seed)
    n = rng.integers(lo, hi + 1, size=count).astype(np.int32)
    seeds = (np.arange(count, dtype=np.uint64) * np.uint64(2654435761) + np.uint64(seed) * np.uint64(1000003))
    return n, seeds


def rips_mixed_batch(count: int = 4096, seed: int = 4, threads: int | None = None, lo: int = 20, hi: int = 120):
    """The batched workload: `count` full 2-skeleton Rips complexes, point
    counts uniform in [lo, hi], half uniform in the cube and half on a noisy
    circle (by instance seed parity).  Returns (col_off, colptr, rows_local,
    n_points, seeds) ready for Context.reduce_batch_packed."""
    n, seeds = mixed_batch_sizes(count, seed, lo, hi)
    col_off, colptr, rows = rips_mixed_instances(n, seeds, threads)
    return col_off, colptr, rows, n, seeds


def rips_mixed_instances(n_points, seeds, threads: int | None = None):
    """Instances of the batched mix for explicit point counts and instance
    seeds (instance b of rips_mixed_batch is rips_mixed_instances([n[b]],
    [seeds[b]])).  Returns (col_off, colptr, rows_local)."""
    import os
    n = np.ascontiguousarray(n_points, dtype=np.int32)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    count = int(n.shape[0])
    col_off = np.zeros(count + 1, np.int64)
    cx = _Complex()
    nt = threads or os.cpu_count() or 1
    if _lib().oph_rips_mixed_batch(count, n, seeds, nt, col_off, C.byref(cx)) != 0:
        raise MemoryError("batch generation failed")
    m, nnz = cx.m, cx.nnz
    colptr = np.ctypeslib.as_array(cx.colptr, shape=(m + 1,)).copy()
    rows = np.ctypeslib.as_array(cx.rows, shape=(max(nnz, 1),))[:nnz].copy()
    _lib().oph_complex_free(C.byref(cx))
    return col_off, colptr, rows


def batch_instance(col_off, colptr, rows, b: int) -> BoundaryMatrix:
    """Instance b of a packed batch as its own matrix (local rows)."""
    c0, c1 = int(col_off[b]), int(col_off[b + 1])
    cp = colptr[c0:c1 + 1] - colptr[c0]
    return BoundaryMatrix(cp, rows[colptr[c0]:colptr[c1]])
