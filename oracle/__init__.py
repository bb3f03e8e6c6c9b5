"""ORACLE — test infrastructure only.

The checker for the GPU reduction: a C restatement of the reference's CPU
algorithms (``oracle.c``), a dense NumPy reduction restating the reference's
own test oracle (src/test/std_test.m:10-31), and a driver for the reference's
own CPU code compiled from its sources (``_ref/ref_ph``, built where the
reference checkout exists).  Only tests, the smoke check and the bench's CPU
baseline leg may import this package; the product path never does.

All functions take a 0-based CSC boundary matrix (``colptr`` int64[m+1],
``rows`` int32) and return 0-based ``low`` (-1 = zero or cleared column) and
``ess`` (1 = estimated essential), both int32[m].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboph_oracle.so"
REF_BIN = HERE / "_ref" / "ref_ph"


class Stats(C.Structure):
    _fields_ = [("additions", C.c_int64), ("slots_read", C.c_int64), ("slots_written", C.c_int64),
                ("max_len", C.c_int64), ("iters", C.c_int64), ("columns_done", C.c_int64),
                ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build(force: bool = False) -> None:
    """Compile the restatement, and the reference's CPU code where it exists."""
    src = HERE / "oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "liboph_oracle.so"], check=True)
    # the reference's own CPU code, where its checkout exists (the recipe
    # takes the checkout from OPENPH_REFERENCE)
    subprocess.run(["make", "-s", "-C", str(HERE), "ref-if-present"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        for name in ("oracle_twist", "oracle_standard", "oracle_ph_row", "oracle_pms"):
            f = getattr(L, name)
            f.argtypes = [C.c_int64, i64p, i32p, i32p, i32p, C.POINTER(Stats)]
            f.restype = C.c_int
        L.oracle_twist_fixed_p.argtypes = [C.c_int64, i64p, i32p, C.c_int, C.c_int64, C.c_double, i32p, i32p,
                                           C.POINTER(Stats)]
        L.oracle_twist_fixed_p.restype = C.c_int
        L.oracle_transverse.argtypes = [C.c_int64, C.c_int32] + [i32p] * 10
        L.oracle_setup.argtypes = [C.c_int64, i64p, i32p, i32p, i32p, i32p, i32p, C.POINTER(C.c_int32)]
        _lib = L
    return _lib


def _run(name, bm):
    m = bm.m
    low = np.empty(max(m, 1), np.int32)
    ess = np.empty(max(m, 1), np.int32)
    st = Stats()
    rc = getattr(lib(), name)(m, bm.colptr, bm.rows, low, ess, C.byref(st))
    if rc != 0:
        raise RuntimeError(f"{name} failed with status {rc}")
    return low[:m], ess[:m], st.as_dict()


def twist(bm):
    """CPU twist (src/cuda/algorithms/twist/twist.cu:10-87)."""
    return _run("oracle_twist", bm)


class _Csc:
    """The fields of a boundary matrix that the oracle reads."""

    def __init__(self, colptr, rows):
        self.colptr = np.ascontiguousarray(colptr, dtype=np.int64)
        self.rows = np.ascontiguousarray(rows, dtype=np.int32)
        self.m = int(self.colptr.shape[0] - 1)


def _twist_job(job):
    low, ess, _ = twist(_Csc(*job))
    return low, ess


def twist_many(jobs, processes: int | None = None):
    """The CPU twist over many matrices, each a (colptr, rows) pair, in
    worker processes started with ``spawn`` (safe in a parent that has
    already initialised CUDA).  Returns [(low, ess), ...] in job order."""
    import multiprocessing as mp
    jobs = list(jobs)
    if not jobs:
        return []
    n = max(1, min(processes or os.cpu_count() or 1, len(jobs)))
    with mp.get_context("spawn").Pool(n) as pool:
        return pool.map(_twist_job, jobs, chunksize=max(1, len(jobs) // (8 * n)))


def standard(bm):
    """CPU standard (src/cuda/algorithms/standard/standard.cu:1-57)."""
    return _run("oracle_standard", bm)


def ph_row(bm):
    """CPU row algorithm (src/cuda/algorithms/ph_row/ph_row.cu:2-121)."""
    return _run("oracle_ph_row", bm)


def pms(bm):
    """pms sweeps, one thread at a time (src/cuda/algorithms/pms/pms.cu:1-118)."""
    return _run("oracle_pms", bm)


def twist_fixed_p(bm, col_width: int, max_columns: int = 0, max_seconds: float = 0.0):
    """Twist on the reference's m x p slot layout: the timed CPU baseline."""
    m = bm.m
    low = np.empty(max(m, 1), np.int32)
    ess = np.empty(max(m, 1), np.int32)
    st = Stats()
    rc = lib().oracle_twist_fixed_p(m, bm.colptr, bm.rows, col_width, max_columns, max_seconds, low, ess,
                                    C.byref(st))
    return rc, low[:m], ess[:m], st.as_dict()


def setup(bm):
    """low, beta, left, dim, complex_dim as the reference's set-up computes them."""
    m = bm.m
    arrs = [np.empty(max(m, 1), np.int32) for _ in range(4)]
    cd = C.c_int32()
    lib().oracle_setup(m, bm.colptr, bm.rows, *arrs, C.byref(cd))
    low, beta, left, dim = (a[:m] for a in arrs)
    return low, beta, left, dim, int(cd.value)


def transverse(dim, start, next_, low, arglow, classes, ess, cdim):
    """One serial Phase I walk (pms_functions.cu:55-85) on copies of the state."""
    m = len(low)
    low, arglow, classes, ess = (np.array(a, np.int32) for a in (low, arglow, classes, ess))
    clear = np.zeros(max(m, 1), np.int32)
    visited = np.zeros(max(m, 1), np.int32)
    ceil = np.full(cdim + 1, -1, np.int32)
    lib().oracle_transverse(m, cdim, np.ascontiguousarray(dim, np.int32), np.ascontiguousarray(start, np.int32),
                            np.ascontiguousarray(next_, np.int32), low, arglow, classes, clear, visited, ess, ceil)
    return low, arglow, classes, clear[:m], ess


def dense_standard(bm):
    """Dense Z/2 standard reduction (src/test/std_test.m:10-31), for m <= ~3000.

    Returns 0-based low; zero columns get -1."""
    m = bm.m
    R = np.zeros((m, m), np.uint8)
    for j in range(m):
        R[bm.column(j), j] = 1
    low = np.full(m, -1, np.int64)
    nz = R.any(axis=0)
    low[nz] = m - 1 - np.argmax(R[::-1, nz], axis=0)
    for j in range(m):
        while low[j] >= 0:
            prev = np.nonzero(low[:j] == low[j])[0]
            if prev.size == 0:
                break
            R[:, j] ^= R[:, prev[0]]
            col = np.nonzero(R[:, j])[0]
            low[j] = col[-1] if col.size else -1
    return low.astype(np.int32)


def essential_from_low(low):
    """ess implied by a reduced low array: unpaired columns are essential."""
    low = np.asarray(low)
    ess = np.ones(len(low), np.int32)
    neg = low >= 0
    ess[neg] = 0
    ess[low[neg]] = 0
    return ess


def ref_available() -> bool:
    return REF_BIN.exists() and os.access(REF_BIN, os.X_OK)


def ref_run(bm, alg: str = "twist", col_width: int = 10, timeout: float = 600.0):
    """Run the reference's own CPU code on bm; None when it overflowed its slots."""
    with tempfile.TemporaryDirectory() as td:
        inp, out = Path(td) / "in.csc", Path(td) / "out.bin"
        bm.save(inp)
        r = subprocess.run([str(REF_BIN), alg, str(col_width), str(inp), str(out)], capture_output=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_ph exited {r.returncode}: {r.stderr.decode()}")
        if not out.exists():
            return None  # the reference hit its fixed slot limit and exited
        m = bm.m
        raw = out.read_bytes()
        low = np.frombuffer(raw, np.int32, m, 0).copy()
        ess = np.frombuffer(raw, np.int32, m, 4 * m).copy()
        iters = int(np.frombuffer(raw, np.int32, 1, 8 * m)[0])
        secs = float(np.frombuffer(raw, np.float64, 1, 8 * m + 4)[0])
        return low, ess, iters, secs


def tracked(bm, algo: str, low_true):
    """The reference's per-iteration progress trackers of standard, twist,
    the row algorithm and their parallel forms, restated step by step in
    Python for small matrices (O(m) work per iteration, as the reference's
    own tracker).  The row forms follow _tracked_rows.

    The reduction follows reduce_col_host (algorithms/kernels_host.cu:62-75;
    the device reduce_col, algorithms/kernels.cu:62-77, is the same without
    the essential-estimate step) column by column in the algorithm's order
    (standard.cu:17-53; twist.cu:36-86 with twist_step_host, twist.cu:1-8,
    dimensions by nnz - 1 from the top, columns in order within one);
    classes and ess are updated as the CPU forms do after each column
    (standard.cu:26-37, twist.cu:50-64) or, for the parallel forms, by
    update_classes and ess_hat over every column (kernels.cu:93-124).  After
    each column the four sums of track_host (tracker.cu:136-172) are taken
    with float32 accumulation, and normalised as openph.cu:184-193.

    ``low_true`` is 0-based (-1 = none).  Returns (err_linf, err_lone,
    err_redu, err_ess) as float32 arrays of num_iters entries, num_iters, and
    the final 0-based low.
    """
    par = algo.endswith("_parallel")
    twist = algo.startswith("twist")
    m = bm.m
    cols = [set(bm.rows[bm.colptr[j]:bm.colptr[j + 1]].tolist()) for j in range(m)]
    low = [max(c) if c else -1 for c in cols]
    arglow = [-1] * m
    classes = [0] * m
    ess = [1] * m
    lt = np.asarray(low_true, np.int64)
    ess_true = np.ones(m, np.int64)
    for j in range(m):
        if lt[j] > -1:
            ess_true[j] = 0
            ess_true[lt[j]] = 0
    f32 = np.float32
    norm1 = f32(0)
    norminf = f32(0)
    for v in (lt + 1):  # the 1-based low_true's norms (openph.cu:106-110)
        norm1 = f32(norm1 + f32(abs(v)))
        norminf = max(norminf, f32(abs(v)))
    num_ess_true = f32(0)
    for v in ess_true:
        num_ess_true = f32(num_ess_true + f32(v))
    out = []

    def track():
        s, mx, red, eh = f32(0), f32(0), f32(0), f32(0)
        for i in range(m):
            d = f32(abs(low[i] - int(lt[i])))
            s = f32(s + d)
            mx = max(mx, d)
            red = f32(red + f32(1 if classes[i] == 0 else 0))
            eh = f32(eh + f32(ess[i]))
        out.append((mx, s, f32(red / f32(m)), f32(1) if eh == num_ess_true else f32(num_ess_true / eh)))

    track()
    order = []
    if algo in ("ph_row", "ph_row_parallel"):
        _tracked_rows(cols, low, classes, ess, par, track)
    elif twist:
        dims = [len(c) - 1 for c in cols]
        order = [j for d in range(max(dims, default=-1), 0, -1) for j in range(m) if dims[j] == d]
    else:
        order = list(range(m))
    for j in (order if algo not in ("ph_row", "ph_row_parallel") else []):
        lj = low[j]
        while lj > -1 and arglow[lj] != -1:
            if not par:
                ess[lj] = 0
            cols[j] ^= cols[arglow[lj]]
            low[j] = max(cols[j]) if cols[j] else -1
            lj = low[j]
        if lj > -1:
            arglow[lj] = j
        if twist and low[j] > -1:
            low[low[j]] = -1
        if not par:
            if low[j] > -1:
                classes[j] = -1
                classes[low[j]] = 1
                ess[j] = 0
                ess[low[j]] = 0
            else:
                classes[j] = 1
        else:
            for t in range(m):
                if arglow[t] > -1:
                    classes[arglow[t]] = -1
                    classes[t] = 1
            for t in range(m):
                if low[t] > -1:
                    ess[low[t]] = 0
                if arglow[t] > -1:
                    ess[arglow[t]] = 0
                    ess[t] = 0
        track()
    n = len(out)
    with np.errstate(divide="ignore", invalid="ignore"):  # an empty low_true has norm 0, as in the reference
        linf = np.array([f32(o[0] / norminf) for o in out], np.float32)
        lone = np.array([f32(o[1] / norm1) for o in out], np.float32)
    redu = np.array([o[2] for o in out], np.float32)
    eerr = np.array([o[3] for o in out], np.float32)
    return linf, lone, redu, eerr, n, np.array(low, np.int32)


def _tracked_rows(cols, low, classes, ess, par, track):
    """The row algorithm's loop for oracle.tracked, one tracker entry per row
    i = m-1 .. 0.  CPU form (ph_row.cu:38-121): the pivot of row i is the
    first column ever to hold low i; every later column of its dimension
    list with that low takes the pivot once (left_to_right_neighbours_host,
    ph_row.cu:2-31: ess cleared at the row and the pivot pair before the
    addition, a column that is then the first ever to hold its new low
    marked as a pair; the reference reads pivots[-1] for a new low of -1,
    taken here as no mark), and after row 0 every pair is marked and the
    remaining essentials classified 2 (ph_row.cu:91-103).  Parallel form
    (ph_row_parallel.cu:20-89): the pivot is the least column with low i
    (mark_neighbours), every other takes it, arglow stays empty, so
    update_classes marks nothing and ess_hat clears every current low."""
    m = len(cols)
    dims = [len(c) - 1 for c in cols]
    pivots = [-1] * m
    for j in range(m):
        if low[j] != -1 and (pivots[low[j]] == -1 or j < pivots[low[j]]):
            pivots[low[j]] = j
    for i in range(m - 1, -1, -1):
        if not par:
            piv = pivots[i]
            if piv != -1:
                nbs = [c for c in range(piv + 1, m) if dims[c] == dims[piv] and low[c] == low[piv]]
                for j in nbs:
                    if low[j] > -1:
                        ess[low[j]] = 0
                    ess[piv] = 0
                    ess[low[piv]] = 0
                    cols[j] ^= cols[piv]
                    low[j] = max(cols[j]) if cols[j] else -1
                    if low[j] != -1 and (pivots[low[j]] == -1 or j < pivots[low[j]]):
                        pivots[low[j]] = j
                    if low[j] != -1 and pivots[low[j]] == j:
                        classes[j] = -1
                        classes[low[j]] = 1
                        ess[j] = 0
                        ess[low[j]] = 0
            if i == 0:
                for c in range(m):
                    if low[c] > -1:
                        ess[c] = 0
                        ess[low[c]] = 0
                        classes[c] = -1
                        classes[low[c]] = 1
                for c in range(m):
                    if ess[c] == 1 and classes[c] == 0:
                        classes[c] = 2
        else:
            nbs = [c for c in range(m) if low[c] == i]
            if nbs:
                piv = min(nbs)
                for j in nbs:
                    if j > piv:
                        cols[j] ^= cols[piv]
                        low[j] = max(cols[j]) if cols[j] else -1
            for c in range(m):
                if low[c] > -1:
                    ess[low[c]] = 0
        track()
