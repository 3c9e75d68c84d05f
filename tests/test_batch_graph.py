"""The device-driven batched multiply (dbd_batch_plan / _enqueue / _result):
run eagerly, captured into a CUDA graph and replayed after the pairs'
contents -- values and sparsity pattern -- changed in place, against the
host-synchronous batched multiply (itself checked against the oracle) and
the oracle; capacity overflow and a malformed pair reported after a replay."""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def to_dev(M, keep):
    t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (M.row_ptr, M.col_idx, M.val)]
    keep.append(t)
    return CSR.from_device(M.n_rows, M.n_cols, M.nnz, *[x.data_ptr() for x in t]), t


def reference(As, Bs):
    with dbd.Context(cpu_gib=8, gpu_gib=8) as c:
        return c.spgemm_batched(As, Bs, scope="kernel").C


def assert_same(got, ref):
    assert len(got) == len(ref)
    for q, (g, r) in enumerate(zip(got, ref)):
        assert np.array_equal(g.row_ptr, r.row_ptr), q
        assert np.array_equal(g.col_idx, r.col_idx), q
        # Sums in another order (N(0,1) values cancel): absolute error at the
        # scale of the pair's largest entry.
        scale = float(np.abs(r.val).max()) if r.nnz else 1.0
        assert np.allclose(g.val, r.val, rtol=1e-12, atol=1e-12 * scale), q


def new_contents(M, rng):
    """Same shape and entry count, other columns and values (rows ascending)."""
    cols = np.empty_like(M.col_idx)
    for r in range(M.n_rows):
        a, b = int(M.row_ptr[r]), int(M.row_ptr[r + 1])
        if b > a:
            cols[a:b] = np.sort(rng.choice(M.n_cols, b - a, replace=False))
    return CSR(M.n_rows, M.n_cols, M.row_ptr.copy(), cols.astype(np.int32), rng.standard_normal(M.nnz))


def test_eager_and_graph_replays_follow_the_pairs(orc):
    pairs = gen.batched_pairs(24, seed=3, n_min=64, n_max=1500)
    As = [p[0] for p in pairs]
    Bs = [p[1] for p in pairs]
    keep = []
    dA = [to_dev(A, keep) for A in As]
    dB = [to_dev(B, keep) for B in Bs]
    ref = reference(As, Bs)
    rng = np.random.default_rng(5)
    As2 = [new_contents(A, rng) for A in As]
    Bs2 = [new_contents(B, rng) for B in Bs]
    ref2 = reference(As2, Bs2)
    cap = max(sum(C.nnz for C in ref), sum(C.nnz for C in ref2))
    s = torch.cuda.Stream()
    with dbd.Context(cpu_gib=8, gpu_gib=8) as c:
        c.batch_plan([d for d, _ in dA], [d for d, _ in dB], capacity=cap)
        c.batch_enqueue(s.cuda_stream)
        s.synchronize()
        assert_same(c.batch_result().C, ref)

        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            c.batch_enqueue(s.cuda_stream)
        g.replay()
        torch.cuda.synchronize()
        assert_same(c.batch_result().C, ref)

        # New values and a new pattern in the same arrays, then a replay.
        for (_, t), M in zip(dA + dB, As2 + Bs2):
            t[1].copy_(torch.from_numpy(M.col_idx))
            t[2].copy_(torch.from_numpy(M.val))
        g.replay()
        torch.cuda.synchronize()
        got = c.batch_result().C
        assert_same(got, ref2)
        # Two pairs against the oracle directly.
        for q in (0, 17):
            Cp, Ci, Cv = orc.spgemm(As2[q], Bs2[q])
            assert np.array_equal(got[q].row_ptr, Cp)
            assert np.array_equal(got[q].col_idx, Ci)
            assert np.allclose(got[q].val, Cv, rtol=1e-12, atol=1e-12 * float(np.abs(Cv).max()))


def test_capacity_and_bad_pair_reported_after_replay():
    pairs = gen.batched_pairs(8, seed=4, n_min=64, n_max=400)
    As = [p[0] for p in pairs]
    keep = []
    dA = [to_dev(A, keep) for A in As]
    ref = reference(As, None)
    need = sum(C.nnz for C in ref)
    s = torch.cuda.Stream()
    with dbd.Context(cpu_gib=4, gpu_gib=4) as c:
        c.batch_plan([d for d, _ in dA], None, capacity=need - 1)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            c.batch_enqueue(s.cuda_stream)
        g.replay()
        torch.cuda.synchronize()
        with pytest.raises(dbd.DBDError) as e:
            c.batch_result()
        assert e.value.code == -4  # DBD_ERR_BUDGET
    with dbd.Context(cpu_gib=4, gpu_gib=4) as c:
        c.batch_plan([d for d, _ in dA], None, capacity=need)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            c.batch_enqueue(s.cuda_stream)
        t = dA[3][1]
        saved = t[1][0].item()
        t[1][0] = As[3].n_cols + 5  # a column out of range
        g.replay()
        torch.cuda.synchronize()
        with pytest.raises(dbd.DBDError) as e:
            c.batch_result()
        assert e.value.code == -1  # DBD_ERR_INVALID
        t[1][0] = saved
        g.replay()
        torch.cuda.synchronize()
        assert_same(c.batch_result().C, ref)
