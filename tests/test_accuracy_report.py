"""Max and mean error against the sequential FP64 oracle, per workload.

Each case asserts the parity bar (bit-exact structure, |c - o| <= 1e-12 *
sum|a*b| per entry) and prints one line with the maximum and mean relative
error |c - o| / |o| and the maximum scaled error |c - o| / sum|a*b|
(`pytest -s` shows them).  The out-of-core R-MAT 2^21 workload is checked on
its first 32 rows (the power-law hubs) and a seeded sample of the others:
those rows of A times A, through the same kernels (a row's kernel depends on
the row alone).
"""
import json

import numpy as np
import pytest

from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR

pytestmark = pytest.mark.gpu


def errors(C, A, B, orc):
    Cp, Ci, Cv, Ca = orc.spgemm(A, B, with_abs=True)
    assert np.array_equal(C.row_ptr, Cp) and np.array_equal(C.col_idx, Ci)
    err = np.abs(C.val - Cv)
    assert np.all(err <= 1e-12 * Ca)
    nz = np.abs(Cv) > 0
    rel = err[nz] / np.abs(Cv[nz])
    scaled = err / np.maximum(Ca, 1e-300)
    return {"nnz_c": int(Cv.size), "max_rel": float(rel.max(initial=0.0)), "mean_rel": float(rel.mean()) if rel.size else 0.0,
            "max_scaled": float(scaled.max(initial=0.0))}


def rows_of(A, rows):
    rows = np.sort(rows)
    lens = np.diff(A.row_ptr)[rows]
    ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    take = np.concatenate([np.arange(A.row_ptr[r], A.row_ptr[r + 1]) for r in rows])
    return CSR(rows.size, A.n_cols, ptr, A.col_idx[take], A.val[take])


def report(name, e):
    print(json.dumps({"workload": name, **e}))


def test_laplacian256(ctx, orc):
    L = gen.laplacian_2d(256)
    report("laplacian256", errors(ctx.spgemm(L, scope="kernel").C, L, L, orc))


def test_rmat18(ctx, orc):
    A = gen.rmat(18, 8, seed=0)
    report("rmat18", errors(ctx.spgemm(A, scope="kernel").C, A, A, orc))


def test_batched_pairs(ctx, orc):
    pairs = gen.batched_pairs(24, seed=0)
    As, Bs = [a for a, _, _ in pairs], [b for _, b, _ in pairs]
    res = ctx.spgemm_batched(As, Bs, scope="kernel")
    agg = {"nnz_c": 0, "max_rel": 0.0, "mean_rel": 0.0, "max_scaled": 0.0}
    n = 0
    for q in range(len(As)):
        e = errors(res.C[q], As[q], Bs[q], orc)
        agg["max_rel"] = max(agg["max_rel"], e["max_rel"])
        agg["max_scaled"] = max(agg["max_scaled"], e["max_scaled"])
        agg["mean_rel"] += e["mean_rel"] * e["nnz_c"]
        n += e["nnz_c"]
    agg["nnz_c"] = n
    agg["mean_rel"] /= max(n, 1)
    report("batched (first 24 of the 512 pairs)", agg)


def test_forward_100k(ctx, orc):
    A = gen.uniform_rows(100_000, 16, seed=31)
    B = gen.uniform_rows(100_000, 16, seed=32)
    report("adjoint100k forward", errors(ctx.spgemm(A, B, scope="kernel").C, A, B, orc))


def test_rmat21_sampled_rows(ctx, orc):
    A = gen.rmat(21, 16, seed=0)
    rng = np.random.default_rng(0)
    rows = np.union1d(np.arange(32), rng.choice(A.n_rows, 2000, replace=False))  # the hub rows and a sample
    S = rows_of(A, rows)
    res = ctx.spgemm(S, A, scope="kernel")
    assert res.stats["rows_per_bin"][8] > 0  # the dense bin
    report(f"rmat21 ({rows.size} rows: the first 32 and a seeded sample)", errors(res.C, S, A, orc))
