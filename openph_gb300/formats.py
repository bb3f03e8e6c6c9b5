"""File formats and persistence diagrams around the reduction.

* PHAT ASCII boundary matrices (one column per line: ``dim r1 r2 ...`` with
  0-based rows; ``#`` comments and blank lines skipped), the format the
  reference converts with numerics/utils/dat2cmo.m:2-48 and
  numerics/utils/cmo2dat.m:2-38.  A column whose line is ``0`` is a
  zero-dimensional cell with no boundary.  Reading gives the canonical 0-based
  CSC; ``BoundaryMatrix.to_coo1()`` then gives the reference's 1-based COO.
  Unlike dat2cmo.m (which keeps an ``r = -1`` marker row for 0-cells that
  callers filter out, numerics/benchmark_datasets.m:53) empty columns simply
  have no entries.
* Persistence pairs from a reduced ``low`` array: (birth, death) simplex
  indices for every nonzero low, and the unpaired (essential) simplices; with
  filtration values, the diagram per dimension.
"""
from __future__ import annotations

import numpy as np

from .complexes import BoundaryMatrix


def read_phat_dat(path) -> tuple[BoundaryMatrix, np.ndarray]:
    """Read a PHAT ASCII file; returns (matrix, dims) with dims[j] the
    declared dimension of column j."""
    cols, dims = [], []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            parts = s.split()
            d = int(parts[0])
            rows = sorted(int(x) for x in parts[1:])
            if d == 0 and rows:
                raise ValueError(f"{path}: a 0-dimensional cell with boundary entries")
            dims.append(d)
            cols.append(rows)
    bm = BoundaryMatrix.from_columns(cols)
    if bm.nnz and (bm.rows.max() >= bm.m or bm.rows.min() < 0):
        raise ValueError(f"{path}: row index out of range")
    bm.dims = np.asarray(dims, np.int8)
    return bm, bm.dims


def write_phat_dat(bm: BoundaryMatrix, path, dims=None) -> None:
    """Write a PHAT ASCII file; dims defaults to nnz(col) - 1 (0 for an
    empty column)."""
    if dims is None:
        nz = np.diff(bm.colptr)
        dims = np.where(nz > 0, nz - 1, 0)
    with open(path, "w") as f:
        f.write("# boundary matrix: one column per line, dimension then 0-based rows\n")
        for j in range(bm.m):
            col = bm.column(j)
            f.write(" ".join([str(int(dims[j]))] + [str(int(r)) for r in col]) + "\n")


def persistence_pairs(low) -> tuple[np.ndarray, np.ndarray]:
    """(pairs, essential): pairs[k] = (birth simplex, death simplex) for every
    column j with low[j] = i >= 0 (i is born, j kills it); essential = the
    simplices in no pair.  low is 0-based with -1 for zero columns."""
    low = np.asarray(low)
    j = np.nonzero(low >= 0)[0]
    pairs = np.stack([low[j], j], axis=1).astype(np.int64)
    paired = np.zeros(len(low), bool)
    paired[j] = True
    paired[low[j]] = True
    return pairs, np.nonzero(~paired)[0].astype(np.int64)


def persistence_diagram(low, values, dims) -> dict:
    """Per homology dimension d: an (n, 2) array of (birth, death) filtration
    values, death = inf for essential classes.  Pairs of zero persistence are
    kept (they are part of the pairing)."""
    pairs, ess = persistence_pairs(low)
    values = np.asarray(values, np.float64)
    dims = np.asarray(dims)
    out = {}
    for d in np.unique(dims):
        pb = pairs[dims[pairs[:, 0]] == d] if len(pairs) else np.zeros((0, 2), np.int64)
        e = ess[dims[ess] == d]
        dgm = np.concatenate([np.stack([values[pb[:, 0]], values[pb[:, 1]]], axis=1),
                              np.stack([values[e], np.full(len(e), np.inf)], axis=1)])
        out[int(d)] = dgm
    return out
