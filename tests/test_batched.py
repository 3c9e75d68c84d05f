"""Batched products (dbd_spgemm_batched) against the oracle, pair by pair.

Every pair's C_q must match the oracle's product of that pair alone: the same
bit-exact structure and FP64 tolerance as the single-product parity tests,
with pair-local column indices.
"""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR
from test_gpu_parity import check, mixed_rows

pytestmark = pytest.mark.gpu


def empty(m, n):
    return CSR(m, n, np.zeros(m + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))


def mixed_batch(seed=0):
    """Uneven pairs: uniform Poisson rows, bands, rectangular pairs, empty
    pairs and operands, and pairs whose rows reach every numeric bin."""
    rng = np.random.default_rng(seed)
    As, Bs = [], []
    for q in range(12):
        n = int(rng.integers(50, 3000))
        s = int(rng.integers(0, 2**31))
        if q % 2:
            As.append(gen.poisson_rows(n, 12, s))
            Bs.append(gen.poisson_rows(n, 12, s + 1))
        else:
            As.append(gen.banded(n, 32, s))
            Bs.append(gen.banded(n, 32, s + 1))
    A, B = mixed_rows(rng, 600, 3000, 600000)   # hash CTA rows and dense windows
    As.append(A), Bs.append(B)
    A, B = mixed_rows(rng, 600, 3000, 20000)    # CTA rank rows
    As.append(A), Bs.append(B)
    As.append(empty(0, 7)), Bs.append(empty(7, 5))                                       # no rows
    As.append(empty(9, 4)), Bs.append(gen.poisson_rows(4, 2, 3))                          # A without entries
    As.append(gen.uniform_rows(40, 3, seed=5, n_cols=30)), Bs.append(empty(30, 11))       # B without entries
    As.append(gen.uniform_rows(70, 5, seed=6, n_cols=33, dist="uniform"))                 # rectangular
    Bs.append(gen.uniform_rows(33, 4, seed=7, n_cols=91, dist="uniform"))
    As.append(CSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.5])))
    Bs.append(CSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([-4.0])))
    perm = rng.permutation(len(As))
    return [As[i] for i in perm], [Bs[i] for i in perm]


def test_batched_pairs_match_oracle(ctx, orc):
    As, Bs = mixed_batch(0)
    res = ctx.spgemm_batched(As, Bs, scope="kernel")
    assert len(res.C) == len(As)
    for q, (A, B) in enumerate(zip(As, Bs)):
        check(res.C[q], A, B, orc)
    assert res.row_off[-1] == sum(A.n_rows for A in As)
    assert res.nnz_off[-1] == res.stats["nnz_c"]
    used = {i for i, v in enumerate(res.stats["rows_per_bin"]) if v}
    assert used >= set(range(1, 9)), used  # the column shift is applied in every numeric kernel


def test_batched_offsets_match_single_products(ctx, orc):
    As, Bs = mixed_batch(1)
    res = ctx.spgemm_batched(As, Bs, scope="kernel")
    for q, (A, B) in enumerate(zip(As, Bs)):
        one = ctx.spgemm(A, B, scope="kernel")
        assert res.nnz_off[q + 1] - res.nnz_off[q] == one.stats["nnz_c"]
        assert np.array_equal(res.C[q].row_ptr, one.C.row_ptr)
        assert np.array_equal(res.C[q].col_idx, one.C.col_idx)


def test_batched_squares_and_d2h(ctx, orc):
    As = [gen.banded(int(n), 32, seed=int(n)) for n in (100, 257, 1024)] + [gen.rmat(10, 8, seed=2)]
    res = ctx.spgemm_batched(As, None, scope="d2h")
    for q, A in enumerate(As):
        check(res.C[q], A, A, orc)


def test_batched_device_and_host_views(ctx, orc):
    torch = pytest.importorskip("torch")
    As, Bs = mixed_batch(2)
    keep = []

    def dev(M):
        p, i, v = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (M.row_ptr, M.col_idx, M.val))
        keep.append((p, i, v))
        return CSR.from_device(M.n_rows, M.n_cols, M.nnz, p.data_ptr(), i.data_ptr(), v.data_ptr())

    dA = [dev(A) if q % 2 == 0 else A for q, A in enumerate(As)]
    dB = [dev(B) if q % 3 == 0 else B for q, B in enumerate(Bs)]
    torch.cuda.synchronize()
    res = ctx.spgemm_batched(dA, dB, scope="kernel")
    for q, (A, B) in enumerate(zip(As, Bs)):
        check(res.C[q], A, B, orc)


def test_batched_invalid_pairs_rejected(ctx, orc):
    good = gen.poisson_rows(50, 4, 1)
    bad_col = CSR(2, 2, np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32), np.array([1.0, 1.0]))
    bad_ptr = CSR(2, 2, np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    bad_end = CSR(2, 2, np.array([0, 1, 1], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    rect = CSR(2, 3, np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    for As, Bs in [([good, bad_col], [good, bad_col]), ([good, bad_ptr], None), ([bad_end, good], None),
                   ([good, rect], [good, rect])]:
        with pytest.raises(dbd.DBDError) as ei:
            ctx.spgemm_batched(As, Bs, scope="kernel")
        assert ei.value.code == -1
    with pytest.raises(dbd.DBDError):
        ctx.spgemm_batched(As=[good], Bs=[good], scope="io")
    res = ctx.spgemm_batched([good, good], None, scope="kernel")  # the context stays usable
    for C_ in res.C:
        check(C_, good, good, orc)


def test_single_products_after_a_batch(ctx, orc):
    """A plain multiply after a batched one writes global columns again."""
    As, Bs = mixed_batch(3)
    ctx.spgemm_batched(As, Bs, scope="kernel")
    A = gen.rmat(11, 8, seed=3)
    res = ctx.spgemm(A, scope="kernel")
    check(res.C, A, A, orc)
