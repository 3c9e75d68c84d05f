"""dbd_update_values: new values on the last multiply's patterns, replayed
from the captured CUDA graph of the numeric kernels, against the oracle."""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR
from test_batched import mixed_batch
from test_gpu_parity import check, mixed_rows

pytestmark = pytest.mark.gpu


def revalue(M, seed):
    rng = np.random.default_rng(seed)
    return CSR(M.n_rows, M.n_cols, M.row_ptr, M.col_idx, rng.uniform(-2.0, 2.0, M.nnz))


def test_single_product_host_values(ctx, orc):
    rng = np.random.default_rng(1)
    A, B = mixed_rows(rng, 600, 3000, 20000)
    ctx.spgemm(A, B, scope="kernel", fetch=False)
    for seed in (2, 3, 4):  # the first call captures, the others replay
        A2, B2 = revalue(A, seed), revalue(B, seed + 100)
        ctx.update_values(A2.val, B2.val)
        check(ctx.result(), A2, B2, orc)


def test_every_numeric_bin_replayed(ctx, orc):
    """Rows in all numeric bins (dense windows and CTA hash tables included)."""
    rng = np.random.default_rng(7)
    A, B = mixed_rows(rng, 600, 3000, 600000)
    res = ctx.spgemm(A, B, scope="kernel", fetch=False)
    A2, B2 = revalue(A, 5), revalue(B, 6)
    ctx.update_values(A2.val, B2.val)
    check(ctx.result(), A2, B2, orc)
    assert {i for i, v in enumerate(res.stats["rows_per_bin"]) if v} >= {6, 7, 8}


def test_square_device_values(ctx, orc):
    torch = pytest.importorskip("torch")
    A = gen.rmat(12, 8, seed=4)
    t = [torch.from_numpy(x).cuda() for x in (A.row_ptr, A.col_idx, A.val)]
    D = CSR.from_device(A.n_rows, A.n_cols, A.nnz, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())
    ctx.spgemm(D, scope="kernel", fetch=False)
    A2 = revalue(A, 9)
    v2 = torch.from_numpy(A2.val).cuda()
    torch.cuda.synchronize()
    ctx.update_values(v2)
    check(ctx.result(), A2, A2, orc)


def test_batched_values(ctx, orc):
    As, Bs = mixed_batch(4)
    ctx.spgemm_batched(As, Bs, scope="kernel", fetch=False)
    for seed in (10, 11):
        A2 = [revalue(A, seed + q) for q, A in enumerate(As)]
        B2 = [revalue(B, seed + 1000 + q) for q, B in enumerate(Bs)]
        ctx.update_values([a.val for a in A2], [b.val for b in B2])
        whole = ctx.result()
        rows = np.concatenate([[0], np.cumsum([A.n_rows for A in As])])
        ents = whole.row_ptr[rows]
        for q in range(len(As)):
            Cq = whole.slice_pair(rows[q], rows[q + 1], ents[q], ents[q + 1], Bs[q].n_cols)
            check(Cq, A2[q], B2[q], orc)


def test_update_needs_a_resident_kernel_scope_product(orc):
    A = gen.rmat(10, 8, seed=1)
    with dbd.Context(cpu_gib=8, gpu_gib=8) as c:
        with pytest.raises(dbd.DBDError):
            c.update_values(A.val)  # nothing multiplied yet
        c.spgemm(A, scope="d2h", fetch=False)
        with pytest.raises(dbd.DBDError):
            c.update_values(A.val)  # C was not left on the device
        c.spgemm(A, scope="kernel", fetch=False)
        with pytest.raises(dbd.DBDError):
            c.update_values([A.val, A.val])  # count differs
        A2 = revalue(A, 3)
        c.update_values(A2.val)
        check(c.result(), A2, A2, orc)
        B = gen.rmat(11, 8, seed=2)  # a new multiply replaces the plan and its graph
        c.spgemm(B, scope="kernel", fetch=False)
        B2 = revalue(B, 4)
        c.update_values(B2.val)
        check(c.result(), B2, B2, orc)


def test_update_with_kernel_timing(orc):
    """A context that times its kernels captures the serial launch order."""
    rng = np.random.default_rng(3)
    A, B = mixed_rows(rng, 300, 2000, 20000)
    with dbd.Context(cpu_gib=8, gpu_gib=8, time_kernels=True) as c:
        c.spgemm(A, B, scope="kernel", fetch=False)
        A2, B2 = revalue(A, 1), revalue(B, 2)
        c.update_values(A2.val, B2.val)
        check(c.result(), A2, B2, orc)
