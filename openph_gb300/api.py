"""Host-side mirror of the reference's MATLAB interface, over the C ABI.

``ph(algstr, r, c, m, col_width, low_true)`` returns the same eight outputs as
the reference's MEX call (src/matlab/ph/ph.cu:11-92) and
``openph(r, c, m, algo, col_width, low_true)`` the same record as its MATLAB
wrapper (src/matlab/ph/openph.m:3-20).  Both run the GPU reduction in
``libopenph_gb300.so``; there is no CPU path.  Missing library or device is an
error, never a silent fallback.

:class:`Context` wraps the context-based API for 0-based CSC input
(:meth:`Context.reduce`, :meth:`Context.reduce_batch`).
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import _build

ALGORITHMS = ("standard", "twist", "ph_row", "standard_parallel", "twist_parallel", "ph_row_parallel", "pms")

OPH_OK, OPH_ERR_BAD_INPUT, OPH_ERR_OOM, OPH_ERR_OVERFLOW, OPH_ERR_TIMEOUT, OPH_ERR_CUDA, OPH_ERR_ALGO = range(7)
OPH_DUAL_AUTO, OPH_DUAL_NEVER, OPH_DUAL_ALWAYS, OPH_DUAL_BLOCKS = range(4)


class OphError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {status_string(status)} (status {status})")


class Info(C.Structure):
    _fields_ = [("num_iters", C.c_int32), ("sweeps", C.c_int32), ("additions", C.c_int64),
                ("slots_moved", C.c_int64), ("pool_bytes", C.c_int64), ("regrows", C.c_int32),
                ("device_ms", C.c_float), ("dual", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RequestInfo(C.Structure):
    _fields_ = [("latency_ms", C.c_double), ("queue_ms", C.c_double), ("submit_ms", C.c_double),
                ("done_ms", C.c_double), ("sweeps", C.c_int32), ("status", C.c_int32), ("m", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerCounters(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("completed", "pending", "active", "sweeps", "regrows", "pool_bytes_in_use",
                                         "columns_in_use", "arena_bytes", "dual_admitted")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Profile(C.Structure):
    _fields_ = [("phase2_narrow_ms", C.c_float), ("phase2_wide_ms", C.c_float), ("phase1_ms", C.c_float),
                ("setup_ms", C.c_float), ("phase2_launches", C.c_int32), ("kernel_launches", C.c_int32),
                ("tier_additions", C.c_int64 * 4), ("tier_slots", C.c_int64 * 4), ("tier_ms", C.c_float * 3)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["tier_additions"] = list(self.tier_additions)
        d["tier_slots"] = list(self.tier_slots)
        d["tier_ms"] = list(self.tier_ms)
        return d


_lib = None


def library_path() -> Path:
    return _build.LIB


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise ImportError(f"{path} is missing: build it with openph_gb300._build.build_cuda() "
                              "(nvcc for sm_103a); openph_gb300 has no CPU fallback")
        L = C.CDLL(str(path))
        i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        i64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        vp = C.c_void_p
        L.oph_algo_from_string.argtypes = [C.c_char_p]
        L.oph_status_string.argtypes = [C.c_int]
        L.oph_status_string.restype = C.c_char_p
        L.oph_openph.argtypes = [C.c_char_p, i32, i32, C.c_int, C.c_int, vp, C.c_int, i32, i32, f32, f32, f32, f32,
                                 f32, i32, C.c_int]
        L.openph.argtypes = [C.c_char_p, i32, i32, C.c_int, C.c_int, vp, C.c_int, i32, i32, f32, f32, f32, f32, f32,
                             i32, C.c_int]
        L.openph.restype = None
        L.oph_context_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.oph_context_destroy.argtypes = [vp]
        L.oph_context_stream.argtypes = [vp]
        L.oph_context_stream.restype = vp
        L.oph_context_set_budget.argtypes = [vp, C.c_int64]
        L.oph_context_set_limits.argtypes = [vp, C.c_int32, C.c_int64]
        L.oph_reduce.argtypes = [vp, C.c_int, C.c_int64, i64, vp, i32, vp, vp, C.POINTER(Info)]
        L.oph_reduce_device.argtypes = [vp, C.c_int, C.c_int64, vp, vp, vp, vp, vp, C.POINTER(Info)]
        L.oph_rips_device.argtypes = [vp, vp, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64), vp, vp, vp]
        L.oph_lower_star_device.argtypes = [vp, vp, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                            vp, vp, vp]
        L.oph_reduce_batch.argtypes = [vp, C.c_int, C.c_int32, i64, i64, vp, i32, vp, C.POINTER(Info)]
        L.oph_reduce_batch_device.argtypes = [vp, C.c_int, C.c_int32, vp, vp, vp, C.c_int64, C.c_int64, vp, vp,
                                              C.POINTER(Info)]
        L.oph_server_create.argtypes = [C.c_int, C.c_int64, C.c_int32, C.POINTER(vp)]
        L.oph_server_submit.argtypes = [vp, C.c_int64, i64, vp, C.POINTER(C.c_int64)]
        L.oph_server_submit_device.argtypes = [vp, C.c_int64, vp, vp, C.POINTER(C.c_int64)]
        L.oph_server_wait.argtypes = [vp, C.c_int64, vp, vp, C.POINTER(RequestInfo), C.c_int64]
        L.oph_server_stats.argtypes = [vp, C.POINTER(ServerCounters)]
        L.oph_server_destroy.argtypes = [vp]
        L.oph_context_set_profile.argtypes = [vp, C.c_int]
        L.oph_context_autotune.argtypes = [vp, C.c_int64, i64, vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.POINTER(C.c_float)]
        L.oph_context_autotune_batch.argtypes = [vp, C.c_int32, i64, i64, vp, C.POINTER(C.c_int32),
                                                 C.POINTER(C.c_int32), C.POINTER(C.c_float)]
        L.oph_context_set_tier0.argtypes = [vp, C.c_int32, C.c_int32]
        L.oph_context_set_dual.argtypes = [vp, C.c_int32]
        L.oph_last_profile.argtypes = [vp, C.POINTER(Profile)]
        _lib = L
    return _lib


def status_string(status: int) -> str:
    return lib().oph_status_string(status).decode()


def algo_id(algstr: str) -> int:
    a = lib().oph_algo_from_string(algstr.encode())
    if a < 0:
        raise OphError(OPH_ERR_ALGO, f"algorithm {algstr!r}")
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def ph(algstr: str, r, c, m: int, col_width: int = 0, low_true=None, gpu_number: int = 0):
    """The reference's ``ph`` MEX call: 1-based int32 COO in, eight outputs out.

    Returns (low, ess, err_linf, err_lone, err_redu, err_ess, time_track,
    num_iters) with the reference's shapes: int32[m] x2, float32[m+1] x5,
    int32[1].  ``low`` is 1-based with 0 for a zero/cleared column.
    Raises OphError where the reference would print and carry on.
    """
    r = np.ascontiguousarray(r, dtype=np.int32).reshape(-1)
    c = np.ascontiguousarray(c, dtype=np.int32).reshape(-1)
    if r.shape != c.shape:
        raise OphError(OPH_ERR_BAD_INPUT, "ph: rows and cols differ in length")
    m = int(m)
    low = np.full(max(m, 1), -1, np.int32)
    ess = np.full(max(m, 1), -1, np.int32)
    errs = [np.full(m + 1, -1, np.float32) for _ in range(4)]
    tt = np.zeros(m + 1, np.float32)
    it = np.zeros(1, np.int32)
    lt = None
    if low_true is not None:
        lt = np.ascontiguousarray(low_true, dtype=np.int32).reshape(-1)
        if lt.shape[0] != m:
            raise OphError(OPH_ERR_BAD_INPUT, "ph: low_true must have m entries")
    rc = lib().oph_openph(algstr.encode(), r, c, m, int(col_width), _ptr(lt), int(r.shape[0]), low, ess, errs[0],
                          errs[1], errs[2], errs[3], tt, it, int(gpu_number))
    if rc != OPH_OK:
        raise OphError(rc, f"ph({algstr!r})")
    return low[:m], ess[:m], errs[0], errs[1], errs[2], errs[3], tt, it


def openph(r, c, m: int, algo: str, col_width: int = 0, low_true=None):
    """The reference's MATLAB wrapper: a record with low, ess, trackers,
    num_iters, time_inner (ms, device) and m; plus the wall time in seconds."""
    t0 = time.perf_counter()
    o = ph(algo, r, c, m, col_width, low_true if low_true is not None else np.zeros(m, np.int32))
    t = time.perf_counter() - t0
    n = int(o[7][0])
    out = {"low": o[0].astype(np.float64), "ess": o[1].astype(np.float64), "err_linf": o[2].astype(np.float64),
           "err_lone": o[3].astype(np.float64), "err_redu": o[4].astype(np.float64),
           "err_ess": o[5].astype(np.float64), "time_track": o[6].astype(np.float64), "num_iters": float(n),
           "time_inner": float(np.sum(o[6][:n])), "m": float(m)}
    return out, t


class Context:
    """A reduction context on one device (its own stream and cached buffers)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().oph_context_create(device, C.byref(self._h))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_create")
        self.device = device

    def close(self):
        if self._h:
            lib().oph_context_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(lib().oph_context_stream(self._h) or 0)

    def set_budget(self, nbytes: int):
        rc = lib().oph_context_set_budget(self._h, int(nbytes))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_set_budget")

    def set_limits(self, max_sweeps: int = 0, initial_pool_bytes: int = 0):
        rc = lib().oph_context_set_limits(self._h, int(max_sweeps), int(initial_pool_bytes))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_set_limits")

    def reduce(self, bm, algo: str = "pms", with_arglow: bool = False):
        """Reduce a 0-based CSC matrix; returns (low, ess[, arglow], info)."""
        m = bm.m
        low = np.empty(max(m, 1), np.int32)
        ess = np.empty(max(m, 1), np.int32)
        arg = np.empty(max(m, 1), np.int32) if with_arglow else None
        info = Info()
        rc = lib().oph_reduce(self._h, algo_id(algo), m, bm.colptr, _ptr(bm.rows if bm.nnz else None), low,
                              _ptr(ess), _ptr(arg), C.byref(info))
        if rc != OPH_OK:
            raise OphError(rc, f"oph_reduce({algo!r})")
        if with_arglow:
            return low[:m], ess[:m], arg[:m], info.as_dict()
        return low[:m], ess[:m], info.as_dict()

    def reduce_batch(self, mats, algo: str = "pms"):
        """Reduce several matrices in one pass; returns ([low_b], [ess_b], info)."""
        col_off = np.zeros(len(mats) + 1, np.int64)
        for b, bm in enumerate(mats):
            col_off[b + 1] = col_off[b] + bm.m
        nnz_off = np.zeros(len(mats) + 1, np.int64)
        for b, bm in enumerate(mats):
            nnz_off[b + 1] = nnz_off[b] + bm.nnz
        total_m = int(col_off[-1])
        colptr = np.zeros(total_m + 1, np.int64)
        for b, bm in enumerate(mats):
            colptr[col_off[b]:col_off[b + 1] + 1] = bm.colptr + nnz_off[b]
        rows = np.concatenate([bm.rows for bm in mats]) if nnz_off[-1] else np.zeros(1, np.int32)
        low, ess, info = self.reduce_batch_packed(col_off, colptr, rows, algo)
        lows = [low[col_off[b]:col_off[b + 1]] for b in range(len(mats))]
        esss = [ess[col_off[b]:col_off[b + 1]] for b in range(len(mats))]
        return lows, esss, info

    def reduce_batch_packed(self, col_off, colptr, rows, algo: str = "pms"):
        col_off = np.ascontiguousarray(col_off, np.int64)
        colptr = np.ascontiguousarray(colptr, np.int64)
        rows = np.ascontiguousarray(rows, np.int32)
        total_m = int(col_off[-1])
        low = np.empty(max(total_m, 1), np.int32)
        ess = np.empty(max(total_m, 1), np.int32)
        info = Info()
        rc = lib().oph_reduce_batch(self._h, algo_id(algo), len(col_off) - 1, col_off, colptr, _ptr(rows), low,
                                    _ptr(ess), C.byref(info))
        if rc != OPH_OK:
            raise OphError(rc, f"oph_reduce_batch({algo!r})")
        return low[:total_m], ess[:total_m], info.as_dict()

    def reduce_device(self, m: int, colptr_ptr: int, rows_ptr: int, low_ptr: int, ess_ptr: int | None = None,
                      arglow_ptr: int | None = None, algo: str = "pms"):
        """Reduce device-resident CSC (raw device pointers); returns info."""
        info = Info()
        rc = lib().oph_reduce_device(self._h, algo_id(algo), int(m), C.c_void_p(colptr_ptr), C.c_void_p(rows_ptr),
                                     C.c_void_p(low_ptr), C.c_void_p(ess_ptr) if ess_ptr else None,
                                     C.c_void_p(arglow_ptr) if arglow_ptr else None, C.byref(info))
        if rc != OPH_OK:
            raise OphError(rc, f"oph_reduce_device({algo!r})")
        return info.as_dict()

    def reduce_batch_device(self, count: int, col_off_ptr: int, colptr_ptr: int, rows_ptr: int, total_m: int,
                            total_nnz: int, low_ptr: int, ess_ptr: int | None = None, algo: str = "pms"):
        info = Info()
        rc = lib().oph_reduce_batch_device(self._h, algo_id(algo), int(count), C.c_void_p(col_off_ptr),
                                           C.c_void_p(colptr_ptr), C.c_void_p(rows_ptr), int(total_m),
                                           int(total_nnz), C.c_void_p(low_ptr),
                                           C.c_void_p(ess_ptr) if ess_ptr else None, C.byref(info))
        if rc != OPH_OK:
            raise OphError(rc, f"oph_reduce_batch_device({algo!r})")
        return info.as_dict()

    def rips_device(self, points_ptr: int, n: int, d: int, threshold: float, alloc):
        """Build the Rips complex of n x d FP64 points already on the device
        (raw pointer).  ``alloc(m, nnz)`` returns raw device pointers
        (colptr, rows, value) for the output (value may be None); returns
        (m, nnz)."""
        m, nnz = C.c_int64(), C.c_int64()
        rc = lib().oph_rips_device(self._h, C.c_void_p(points_ptr), int(n), int(d), float(threshold), C.byref(m),
                                   C.byref(nnz), None, None, None)
        if rc != OPH_OK:
            raise OphError(rc, "oph_rips_device")
        colptr, rows, value = alloc(m.value, nnz.value)
        rc = lib().oph_rips_device(self._h, C.c_void_p(points_ptr), int(n), int(d), float(threshold), C.byref(m),
                                   C.byref(nnz), C.c_void_p(colptr), C.c_void_p(rows),
                                   C.c_void_p(value) if value else None)
        if rc != OPH_OK:
            raise OphError(rc, "oph_rips_device")
        return m.value, nnz.value

    def lower_star_device(self, image_ptr: int, h: int, w: int, alloc):
        """Build the lower-star complex of an h x w FP32 image on the device;
        ``alloc`` as for rips_device; returns (m, nnz)."""
        m, nnz = C.c_int64(), C.c_int64()
        rc = lib().oph_lower_star_device(self._h, C.c_void_p(image_ptr), int(h), int(w), C.byref(m), C.byref(nnz),
                                         None, None, None)
        if rc != OPH_OK:
            raise OphError(rc, "oph_lower_star_device")
        colptr, rows, value = alloc(m.value, nnz.value)
        rc = lib().oph_lower_star_device(self._h, C.c_void_p(image_ptr), int(h), int(w), C.byref(m), C.byref(nnz),
                                         C.c_void_p(colptr), C.c_void_p(rows), C.c_void_p(value) if value else None)
        if rc != OPH_OK:
            raise OphError(rc, "oph_lower_star_device")
        return m.value, nnz.value

    def autotune(self, bm):
        """Pick the narrow-tier lanes/capacity on a representative matrix."""
        lanes, cap, ms = C.c_int32(), C.c_int32(), C.c_float()
        rc = lib().oph_context_autotune(self._h, bm.m, bm.colptr, _ptr(bm.rows if bm.nnz else None),
                                        C.byref(lanes), C.byref(cap), C.byref(ms))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_autotune")
        return {"lanes": lanes.value, "cap": cap.value, "ms": ms.value}

    def autotune_batch(self, col_off, colptr, rows):
        lanes, cap, ms = C.c_int32(), C.c_int32(), C.c_float()
        rows = np.ascontiguousarray(rows, np.int32)
        rc = lib().oph_context_autotune_batch(self._h, len(col_off) - 1, np.ascontiguousarray(col_off, np.int64),
                                              np.ascontiguousarray(colptr, np.int64), _ptr(rows), C.byref(lanes),
                                              C.byref(cap), C.byref(ms))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_autotune_batch")
        return {"lanes": lanes.value, "cap": cap.value, "ms": ms.value}

    def set_tier0(self, lanes: int, cap: int):
        rc = lib().oph_context_set_tier0(self._h, int(lanes), int(cap))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_set_tier0")

    def set_dual(self, mode):
        """Which matrix pms reduces: "auto" (the anti-transpose for graded
        inputs of >= 2^17 columns whose top dimension bucket holds >= 8x the
        columns of the bottom one, else at that size a choice per dimension
        block), "never", "always" (the anti-transpose when graded) or
        "blocks" (the per-block choice at any size: D' for a block whose row
        simplices have at most two cofaces on average, D for the others)."""
        code = {"auto": OPH_DUAL_AUTO, "never": OPH_DUAL_NEVER, "always": OPH_DUAL_ALWAYS,
                "blocks": OPH_DUAL_BLOCKS}.get(mode, mode)
        rc = lib().oph_context_set_dual(self._h, int(code))
        if rc != OPH_OK:
            raise OphError(rc, "oph_context_set_dual")

    def set_profile(self, on: bool = True, slots: bool = False):
        """Per-phase event timing (``on``); ``slots`` also tracks the exact
        |P| + |T| + |T xor P| of every addition in the lazy tiers (slower)."""
        lib().oph_context_set_profile(self._h, (1 if on else 0) | (2 if slots else 0))

    def last_profile(self):
        p = Profile()
        lib().oph_last_profile(self._h, C.byref(p))
        return p.as_dict()


class Server:
    """Continuous-batching reduction server (one worker thread per server).

    ``submit(bm)`` queues a matrix and returns a ticket; ``wait(ticket)``
    returns (low, ess, info).  Requests are admitted between pms sweeps while
    they fit in the device arena of ``budget_bytes``."""

    def __init__(self, device: int = 0, budget_bytes: int = 8 << 30, max_active: int = 4096):
        self._h = C.c_void_p()
        rc = lib().oph_server_create(device, int(budget_bytes), int(max_active), C.byref(self._h))
        if rc != OPH_OK:
            raise OphError(rc, "oph_server_create")
        self._m = {}

    def submit(self, bm) -> int:
        t = C.c_int64()
        rc = lib().oph_server_submit(self._h, bm.m, bm.colptr, _ptr(bm.rows if bm.nnz else None), C.byref(t))
        if rc != OPH_OK:
            raise OphError(rc, "oph_server_submit")
        self._m[t.value] = bm.m
        return t.value

    def submit_device(self, dm) -> int:
        """Queue a matrix already in device memory (a complexes.DeviceMatrix,
        or anything with torch ``colptr``/``rows`` on this server's device);
        the server copies it on the device before returning."""
        import torch
        torch.cuda.current_stream(dm.colptr.device).synchronize()
        t = C.c_int64()
        m = int(dm.colptr.shape[0]) - 1
        rc = lib().oph_server_submit_device(self._h, m, C.c_void_p(dm.colptr.data_ptr()),
                                            C.c_void_p(dm.rows.data_ptr()), C.byref(t))
        if rc != OPH_OK:
            raise OphError(rc, "oph_server_submit_device")
        self._m[t.value] = m
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        m = self._m.pop(ticket)
        low = np.empty(max(m, 1), np.int32)
        ess = np.empty(max(m, 1), np.int32)
        info = RequestInfo()
        rc = lib().oph_server_wait(self._h, ticket, _ptr(low), _ptr(ess), C.byref(info), int(timeout_ms))
        if rc != OPH_OK:
            raise OphError(rc, "oph_server_wait")
        return low[:m], ess[:m], info.as_dict()

    def stats(self):
        c = ServerCounters()
        lib().oph_server_stats(self._h, C.byref(c))
        return c.as_dict()

    def close(self):
        if self._h:
            lib().oph_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
