"""Seeded synthetic inputs with the shapes the local kernels are measured on.

All matrices are returned as column-major CSC triples (colptr int64[n+1],
rowidx int64[nnz] sorted within each column, values) -- the same layout the
reference's ``SpCCols``/``Csc`` holds (``csc.h:70-74``) and, with empty
columns dropped, its ``SpDCCols``/``Dcsc`` (``dcsc.h:125-131``).

* ``rmat``: Kronecker (R-MAT) edges with initiator (a, b, c, d), duplicates
  merged, self-loops removed, symmetrized -- the input family of the
  reference's Graph500 generator (``graph500-1.2/generator``), restated with
  numpy; vertex ids are not scrambled.
* ``mcl_planted``: column-stochastic matrix with planted clusters, the
  expansion input of ``Applications/MCL.cpp``.
* ``poisson27`` / ``aggregation``: 27-point Poisson stencil and the 2x2x2
  aggregation restriction used for Galerkin products (as
  ``ReleaseTests/GalerkinNew.cpp`` multiplies them).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSC:
    """Column-compressed sparse matrix on the host (int64 indices)."""

    nrow: int
    ncol: int
    colptr: np.ndarray  # int64[ncol+1]
    rowidx: np.ndarray  # int64[nnz]
    values: np.ndarray | None  # [nnz] or None for a pattern matrix

    @property
    def nnz(self) -> int:
        return int(self.colptr[-1])

    def with_values(self, values: np.ndarray | None) -> "CSC":
        return CSC(self.nrow, self.ncol, self.colptr, self.rowidx, values)

    def astype(self, dtype) -> "CSC":
        v = None if self.values is None else self.values.astype(dtype)
        return self.with_values(v)

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.nrow, self.ncol), dtype=self.values.dtype if self.values is not None else np.int8)
        cols = np.repeat(np.arange(self.ncol), np.diff(self.colptr))
        d[self.rowidx, cols] = 1 if self.values is None else self.values
        return d

    def col_ids(self) -> np.ndarray:
        return np.repeat(np.arange(self.ncol, dtype=np.int64), np.diff(self.colptr))


def csc_from_coo(nrow: int, ncol: int, rows: np.ndarray, cols: np.ndarray, values=None, dedupe=True) -> CSC:
    """Sort (col, row) and build CSC.  Duplicates are merged by keeping the
    first occurrence when ``dedupe`` (pattern generators) -- callers that need
    summed duplicates build their own values afterwards."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    key = cols * np.int64(nrow) + rows
    order = np.argsort(key, kind="stable")
    key = key[order]
    if dedupe and key.size:
        keep = np.empty(key.size, dtype=bool)
        keep[0] = True
        np.not_equal(key[1:], key[:-1], out=keep[1:])
        order = order[keep]
        key = key[keep]
    r = key % nrow
    c = key // nrow
    colptr = np.zeros(ncol + 1, dtype=np.int64)
    colptr[1:] = np.cumsum(np.bincount(c, minlength=ncol), dtype=np.int64)
    vals = None if values is None else np.asarray(values)[order]
    return CSC(nrow, ncol, colptr, r.astype(np.int64), vals)


def rmat_edges(scale: int, edge_factor: int, seed: int, a=0.57, b=0.19, c=0.19, d=0.05):
    """Raw Kronecker edge list (may hold duplicates and self-loops)."""
    rng = np.random.default_rng(seed)
    ne = edge_factor << scale
    u = np.zeros(ne, dtype=np.int64)
    v = np.zeros(ne, dtype=np.int64)
    ab = a + b
    abc = a + b + c
    chunk = 1 << 22
    for s0 in range(0, ne, chunk):
        s1 = min(ne, s0 + chunk)
        uu = np.zeros(s1 - s0, dtype=np.int64)
        vv = np.zeros(s1 - s0, dtype=np.int64)
        for lvl in range(scale):
            r = rng.random(s1 - s0, dtype=np.float32)
            rbit = r >= ab  # quadrants c, d: lower half of rows
            cbit = ((r >= a) & (r < ab)) | (r >= abc)  # quadrants b, d: right half of cols
            uu |= rbit.astype(np.int64) << lvl
            vv |= cbit.astype(np.int64) << lvl
        u[s0:s1] = uu
        v[s0:s1] = vv
    return u, v


def rmat(scale: int, edge_factor: int, seed: int = 1, values: str | None = "uniform", dtype=np.float64,
         a=0.57, b=0.19, c=0.19, d=0.05) -> CSC:
    """Symmetric R-MAT pattern of 2**scale vertices without self-loops.

    ``values``: None for a pattern matrix, "uniform" for U(0,1] drawn per
    stored entry (column-major order) from ``seed + 1``, "ones" for all ones.
    """
    n = 1 << scale
    u, v = rmat_edges(scale, edge_factor, seed, a, b, c, d)
    keep = u != v
    u, v = u[keep], v[keep]
    rows = np.concatenate([u, v])
    cols = np.concatenate([v, u])
    del u, v
    M = csc_from_coo(n, n, rows, cols)
    if values == "uniform":
        rng = np.random.default_rng(seed + 1)
        # (0, 1]: 1 - U[0,1)
        M.values = (1.0 - rng.random(M.nnz)).astype(dtype)
    elif values == "ones":
        M.values = np.ones(M.nnz, dtype=dtype)
    return M


def mcl_planted(n: int = 1 << 20, cluster: int = 1024, intra_nnz: float = 24.0, inter_nnz: float = 6.0,
                seed: int = 3) -> CSC:
    """Column-stochastic fp32 matrix with ``n // cluster`` planted clusters.

    Each column j draws ~``intra_nnz`` rows uniformly inside its own cluster
    and ~``inter_nnz`` rows uniformly over all vertices; a self-loop is added;
    duplicates merged; values U(0,1] then each column normalised to sum 1.
    """
    rng = np.random.default_rng(seed)
    k_in = rng.poisson(intra_nnz, n).astype(np.int64)
    k_out = rng.poisson(inter_nnz, n).astype(np.int64)
    cols_in = np.repeat(np.arange(n, dtype=np.int64), k_in)
    base = (cols_in // cluster) * cluster
    rows_in = base + rng.integers(0, cluster, cols_in.size)
    cols_out = np.repeat(np.arange(n, dtype=np.int64), k_out)
    rows_out = rng.integers(0, n, cols_out.size)
    diag = np.arange(n, dtype=np.int64)
    rows = np.concatenate([rows_in, rows_out, diag])
    cols = np.concatenate([cols_in, cols_out, diag])
    M = csc_from_coo(n, n, rows, cols)
    vals = (1.0 - rng.random(M.nnz)).astype(np.float32)
    colsum = np.add.reduceat(vals, M.colptr[:-1]) if M.nnz else np.zeros(n, np.float32)
    vals = (vals / np.repeat(colsum, np.diff(M.colptr))).astype(np.float32)
    M.values = vals
    return M


def poisson27(side: int, dtype=np.float64) -> CSC:
    """27-point stencil on a side^3 grid: diagonal 26, each neighbour -1.
    Built directly in column order: neighbour offsets taken in (dz, dy, dx)
    lexicographic order are ascending row ids."""
    n = side ** 3
    idx = np.arange(n, dtype=np.int64)
    x = idx % side
    y = (idx // side) % side
    z = idx // (side * side)
    rows = np.empty((n, 27), dtype=np.int64)
    valid = np.empty((n, 27), dtype=bool)
    vals = np.empty(27, dtype=np.float64)
    k = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                xx, yy, zz = x + dx, y + dy, z + dz
                valid[:, k] = (xx >= 0) & (xx < side) & (yy >= 0) & (yy < side) & (zz >= 0) & (zz < side)
                rows[:, k] = (zz * side + yy) * side + xx
                vals[k] = 26.0 if (dx, dy, dz) == (0, 0, 0) else -1.0
                k += 1
    cnt = valid.sum(1)
    colptr = np.zeros(n + 1, dtype=np.int64)
    colptr[1:] = np.cumsum(cnt)
    return CSC(n, n, colptr, rows[valid], np.broadcast_to(vals, (n, 27))[valid].astype(dtype))


def aggregation(side: int, dtype=np.float64) -> CSC:
    """Restriction R (n/8 x n) that sums each 2x2x2 block of a side^3 grid
    (side even); entries are ones.  Column c (a fine point) holds one row."""
    assert side % 2 == 0
    n = side ** 3
    h = side // 2
    idx = np.arange(n, dtype=np.int64)
    x = idx % side
    y = (idx // side) % side
    z = idx // (side * side)
    agg = ((z // 2) * h + (y // 2)) * h + (x // 2)
    return CSC(h ** 3, n, np.arange(n + 1, dtype=np.int64), agg, np.ones(n, dtype=dtype))


def transpose(M: CSC) -> CSC:
    cols = M.col_ids()
    return csc_from_coo(M.ncol, M.nrow, cols, M.rowidx, M.values, dedupe=False)


def batch_c4(nprob: int = 256, seed: int = 4, rmat_scales=(10, 18), sides=(16, 64)):
    """The uneven batch: half R-MAT products A*A (n log-uniform over
    2^rmat_scales, edge factor uniform 4..16), half Galerkin triple products
    R*A*R^T with A a 27-point Poisson stencil on a cube (side uniform over
    the even values in `sides`) and R its 2x2x2 aggregation.  Returns
    (rmat_list, galerkin_list) with rmat entries A and galerkin entries
    (A, R, R^T)."""
    rng = np.random.default_rng(seed)
    rm, gk = [], []
    for q in range(nprob // 2):
        scale = int(rng.integers(rmat_scales[0], rmat_scales[1] + 1))
        ef = int(rng.integers(4, 17))
        rm.append(rmat(scale, ef, seed=seed * 1000 + q))
    evens = np.arange(sides[0], sides[1] + 1, 2)
    for q in range(nprob - nprob // 2):
        side = int(rng.choice(evens))
        A = poisson27(side)
        R = aggregation(side)
        gk.append((A, R, transpose(R)))
    return rm, gk


def random_sparse(m: int, n: int, density: float, seed: int, dtype=np.float64, empty_cols: float = 0.0) -> CSC:
    """Uniform random sparse matrix with optional fraction of forced-empty
    columns (exercises the DCSC path where nzc < n)."""
    rng = np.random.default_rng(seed)
    nnz = int(m * n * density)
    rows = rng.integers(0, m, nnz)
    cols = rng.integers(0, n, nnz)
    if empty_cols > 0:
        dead = rng.random(n) < empty_cols
        keep = ~dead[cols]
        rows, cols = rows[keep], cols[keep]
    M = csc_from_coo(m, n, rows, cols)
    if np.issubdtype(np.dtype(dtype), np.floating):
        M.values = (1.0 - rng.random(M.nnz)).astype(dtype)
    elif np.dtype(dtype) == np.bool_:
        M.values = np.ones(M.nnz, dtype=np.bool_)
    else:
        M.values = rng.integers(1, 10, M.nnz).astype(dtype)
    return M
