"""Seeded synthetic inputs for the five workloads (numpy PCG64).

The reference is measured on SuiteSparse matrices that are not available
here; these generators stand in with the shapes and value distributions of
the workloads the benchmark names:

  laplacian_2d(256, 256)        5-point Laplacian (4 on the diagonal, -1 off
                                it), the poisson5pt gallery matrix of
                                bhsparse/main.cu:41-45
  rmat(18, 8) / rmat(21, 16)    R-MAT power-law graphs, (a,b,c,d) =
                                (.57,.19,.19,.05), deduplicated, columns sorted,
                                values 1 - U[0,1) in (0, 1]
  batched_pairs(512)            uneven independent pairs: n log-uniform in
                                [1024, 65536], uniform-random rows with
                                Poisson(12) entries or a band |i-j| <= 32
                                (65 diagonals), values U[-1, 1]
  uniform_rows(100000, 16)      exactly k entries per row at uniform columns,
                                values N(0, 1)

All return CSR with int32 indices, sorted unique columns and float64 values.
"""
import numpy as np

from .csr import CSR


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def _from_coo(n_rows, n_cols, rows, cols, vals):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    ptr = np.zeros(n_rows + 1, np.int64)
    np.add.at(ptr, rows + 1, 1)
    ptr = np.cumsum(ptr)
    return CSR(n_rows, n_cols, ptr.astype(np.int32), cols.astype(np.int32), vals.astype(np.float64))


def laplacian_2d(nx, ny=None):
    """5-point Laplacian of an nx-by-ny grid: n = nx*ny rows."""
    ny = nx if ny is None else ny
    n = nx * ny
    i = np.arange(n, dtype=np.int64)
    x, y = i % nx, i // nx
    rows = [i]
    cols = [i]
    vals = [np.full(n, 4.0)]
    for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny)
        rows.append(i[ok])
        cols.append(i[ok] + dx + dy * nx)
        vals.append(np.full(int(ok.sum()), -1.0))
    return _from_coo(n, n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def rmat(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=0, int_values=False):
    """Seeded R-MAT: one uniform draw per level and edge picks the quadrant
    (row bit = u >= a+b; column bit = a <= u < a+b or u >= a+b+c); edges are
    deduplicated and each row's columns sorted.  Values 1 - U[0,1) (or
    integers 1..9 with int_values, a value set on which the reference's
    value-based structure test cannot fire)."""
    n = 1 << scale
    m = n * edge_factor
    rng = _rng(seed)
    r = np.zeros(m, np.int64)
    cc = np.zeros(m, np.int64)
    for _ in range(scale):
        u = rng.random(m)
        rb = u >= a + b
        cb = ((u >= a) & (u < a + b)) | (u >= a + b + c)
        r = (r << 1) | rb
        cc = (cc << 1) | cb
    # Sorted distinct keys (np.unique's result, by a plain sort and a mask:
    # np.unique takes ~35 s on the 33.5M keys of scale 21, this ~1 s).
    key = np.sort(r * n + cc)
    keep = np.ones(key.size, bool)
    keep[1:] = key[1:] != key[:-1]
    key = key[keep]
    rows = key // n
    cols = key % n
    if int_values:
        vals = rng.integers(1, 10, key.size).astype(np.float64)
    else:
        vals = 1.0 - rng.random(key.size)
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(np.bincount(rows, minlength=n))
    return CSR(n, n, ptr.astype(np.int32), cols.astype(np.int32), vals)


def _distinct_cols(rng, counts, n):
    """Per-row distinct uniform columns in [0, n), counts[i] of them, sorted."""
    rows = np.repeat(np.arange(counts.size, dtype=np.int64), counts)
    cols = rng.integers(0, n, rows.size)
    while True:
        key = rows * n + cols
        order = np.argsort(key, kind="stable")
        ks = key[order]
        dup = np.zeros(ks.size, bool)
        dup[1:] = ks[1:] == ks[:-1]
        if not dup.any():
            break
        bad = order[dup]
        cols[bad] = rng.integers(0, n, bad.size)
    return rows, cols


def uniform_rows(n, k, seed=0, n_cols=None, dist="normal"):
    """n rows with exactly k distinct uniform columns each."""
    n_cols = n if n_cols is None else n_cols
    rng = _rng(seed)
    rows, cols = _distinct_cols(rng, np.full(n, k, np.int64), n_cols)
    vals = rng.standard_normal(rows.size) if dist == "normal" else rng.uniform(-1.0, 1.0, rows.size)
    return _from_coo(n, n_cols, rows, cols, vals)


def poisson_rows(n, lam, seed=0):
    """n x n, Poisson(lam) distinct uniform columns per row, values U[-1, 1].

    Columns are drawn per row, sorted by (row, column) key, and duplicates
    redrawn until every row's columns are distinct; the values are drawn in
    CSR order."""
    rng = _rng(seed)
    counts = np.minimum(rng.poisson(lam, n), n).astype(np.int64)
    ptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=ptr[1:])
    rows = np.repeat(np.arange(n, dtype=np.int64), counts)
    key = np.sort(rows * n + rng.integers(0, n, rows.size))
    while True:
        dup = np.flatnonzero(key[1:] == key[:-1]) + 1
        if dup.size == 0:
            break
        key[dup] = (key[dup] // n) * n + rng.integers(0, n, dup.size)
        key.sort()
    cols = key - rows * n
    return CSR(n, n, ptr.astype(np.int32), cols.astype(np.int32), rng.uniform(-1.0, 1.0, key.size))


def banded(n, half_bandwidth=32, seed=0):
    """n x n with a_ij != 0 iff |i - j| <= half_bandwidth, values U[-1, 1].

    Built row by row in CSR order directly (the entries are generated sorted)."""
    rng = _rng(seed)
    r = np.arange(n, dtype=np.int64)
    first = np.maximum(r - half_bandwidth, 0)
    counts = np.minimum(r + half_bandwidth, n - 1) - first + 1
    ptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=ptr[1:])
    nnz = int(ptr[-1])
    cols = np.arange(nnz, dtype=np.int64) - np.repeat(ptr[:-1] - first, counts)
    return CSR(n, n, ptr.astype(np.int32), cols.astype(np.int32), rng.uniform(-1.0, 1.0, nnz))


def batched_pairs(count=512, seed=0, n_min=1024, n_max=65536):
    """`count` independent (A_i, B_i) pairs of one kind each (50/50 by seed)."""
    rng = _rng(seed)
    ns = np.rint(np.exp(rng.uniform(np.log(n_min), np.log(n_max), count))).astype(np.int64)
    kinds = rng.integers(0, 2, count)
    pairs = []
    for q in range(count):
        s = int(rng.integers(0, 2**62))
        n = int(ns[q])
        if kinds[q] == 0:
            pairs.append((poisson_rows(n, 12, s), poisson_rows(n, 12, s + 1), "uniform"))
        else:
            pairs.append((banded(n, 32, s), banded(n, 32, s + 1), "banded"))
    return pairs


WORKLOADS = {
    "laplacian256": dict(desc="A*A, A = 5-point Laplacian 256x256 (n=65,536), blocksize 4096",
                         rows_per_block=4096),
    "rmat18": dict(desc="A*A, A = R-MAT scale 18, edge factor 8, seed 0, blocksize 4096",
                   rows_per_block=4096),
    "rmat21": dict(desc="out-of-core A*A, A = R-MAT scale 21, edge factor 16, seed 0, blocksize 512",
                   rows_per_block=512),
}


def workload(name, seed=0):
    if name == "laplacian256":
        return laplacian_2d(256)
    if name == "rmat18":
        return rmat(18, 8, seed=seed)
    if name == "rmat21":
        return rmat(21, 16, seed=seed)
    raise KeyError(name)
