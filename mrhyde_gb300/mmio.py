"""MatrixMarket interchange of the assembled system (J, r, u).

The reference dumps the Jacobian, residual and solution with Tpetra's MatrixMarket writer when
"dump jacobian/residual/solution" is set (src/interfaces/linear_algebra/linearAlgebraInterface_util.hpp:316-335,
writeToFile; readStateVectorFromFile for restarts).  This module writes the same formats from device
or host arrays: "coordinate real general" with 1-based indices for the CSR matrix, "array real general"
for vectors, so files can be diffed against a reference dump or loaded by scipy.io.mmread.
"""
from __future__ import annotations

import numpy as np


def _np(a):
    try:
        import torch

        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


def write_csr(path, row_ptr, col_idx, vals, n_cols=None):
    rp, ci, v = _np(row_ptr).astype(np.int64), _np(col_idx).astype(np.int64), _np(vals).astype(np.float64)
    n = len(rp) - 1
    m = int(n_cols) if n_cols is not None else n
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate real general\n")
        fh.write(f"{n} {m} {len(v)}\n")
        data = np.column_stack([rows + 1, ci + 1, v])
        np.savetxt(fh, data, fmt=["%d", "%d", "%.17g"])


def write_vector(path, x):
    x = _np(x).astype(np.float64).ravel()
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix array real general\n")
        fh.write(f"{len(x)} 1\n")
        np.savetxt(fh, x, fmt="%.17g")


def read_csr(path):
    """Returns (row_ptr, col_idx, vals) with 0-based, row-sorted entries."""
    with open(path) as fh:
        header = fh.readline()
        if "coordinate" not in header:
            raise ValueError("not a MatrixMarket coordinate file")
        line = fh.readline()
        while line.startswith("%"):
            line = fh.readline()
        n, m, nnz = (int(t) for t in line.split())
        data = np.loadtxt(fh, ndmin=2) if nnz else np.zeros((0, 3))
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2]
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp), c.astype(np.int32), v


def read_vector(path):
    with open(path) as fh:
        header = fh.readline()
        if "array" not in header:
            raise ValueError("not a MatrixMarket array file")
        line = fh.readline()
        while line.startswith("%"):
            line = fh.readline()
        n = int(line.split()[0])
        x = np.loadtxt(fh, ndmin=1)
    return x[:n]
