"""Adjoint of C = A*B over fixed patterns, through the torch.autograd harness.

dA = mask_A(G B^T), dB = mask_B(A^T G) for G = dL/dC; with L = sum(W * C) the
loss is bilinear, so central differences are exact up to rounding.  Checked
against the sequential FP64 oracle (|d - oracle| <= 1e-12 * scale), a dense
reference, and central differences (h = 1e-6) on sampled entries.
"""
import numpy as np
import pytest

from dbd_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def to_dev(torch, M):
    return (torch.from_numpy(np.ascontiguousarray(M.row_ptr, np.int32)).cuda(),
            torch.from_numpy(np.ascontiguousarray(M.col_idx, np.int32)).cuda(),
            torch.from_numpy(np.ascontiguousarray(M.val, np.float64)).cuda())


def setup(torch, A, B):
    from dbd_gb300.autograd import Pattern
    ap, ai, av = to_dev(torch, A)
    bp, bi, bv = to_dev(torch, B)
    pat = Pattern(ap, ai, (A.n_rows, A.n_cols), bp, bi, (B.n_rows, B.n_cols))
    return pat, av.requires_grad_(True), bv.requires_grad_(True)


def dense(M):
    D = np.zeros((M.n_rows, M.n_cols))
    for r in range(M.n_rows):
        s, e = M.row_ptr[r], M.row_ptr[r + 1]
        np.add.at(D[r], M.col_idx[s:e], M.val[s:e])
    return D


@pytest.mark.parametrize("keep", [True, False])
def test_adjoint_matches_oracle_and_dense(orc, keep):
    torch = pytest.importorskip("torch")
    from dbd_gb300.autograd import spgemm, engine
    A = gen.uniform_rows(300, 7, seed=11, n_cols=200)
    B = gen.uniform_rows(200, 9, seed=12, n_cols=250)
    pat, av, bv = setup(torch, A, B)
    with engine() as eng:
        c = spgemm(av, bv, pat, eng, keep_pattern=keep)
        rng = np.random.default_rng(5)
        w = torch.from_numpy(rng.standard_normal(c.numel())).cuda()
        (w * c).sum().backward()
        Cp, Ci = pat.c_ptr.cpu().numpy(), pat.c_idx.cpu().numpy()
        dA_o, dB_o = orc.adjoint(A, B, Cp, Ci, w.cpu().numpy())
        dA, dB = av.grad.cpu().numpy(), bv.grad.cpu().numpy()
        assert np.allclose(dA, dA_o, rtol=1e-12, atol=1e-12)
        assert np.allclose(dB, dB_o, rtol=1e-12, atol=1e-12)
        G = np.zeros((300, 250))
        for r in range(300):
            G[r, Ci[Cp[r]:Cp[r + 1]]] = w.cpu().numpy()[Cp[r]:Cp[r + 1]]
        dAd, dBd = G @ dense(B).T, dense(A).T @ G
        assert np.allclose(dA, dAd[np.repeat(np.arange(300), np.diff(A.row_ptr)), A.col_idx], rtol=1e-10, atol=1e-12)
        assert np.allclose(dB, dBd[np.repeat(np.arange(200), np.diff(B.row_ptr)), B.col_idx], rtol=1e-10, atol=1e-12)


def test_deterministic_db_matches_and_repeats(orc):
    """DBD_ADJ_DETERMINISTIC: dB from its own pass over B's pattern equals the
    oracle and the default reductions within tolerance, and two runs give the
    same bits; dA is the same in both modes.  Power-law operands, so that
    columns of A hold from one to hundreds of rows."""
    torch = pytest.importorskip("torch")
    from dbd_gb300.autograd import spgemm, engine
    A = gen.rmat(11, 8, seed=21)
    B = gen.rmat(11, 8, seed=22)
    grads = []
    with engine() as eng:
        for det in (False, True, True):
            pat, av, bv = setup(torch, A, B)
            c = spgemm(av, bv, pat, eng, deterministic=det)
            w = torch.from_numpy(np.random.default_rng(6).standard_normal(c.numel())).cuda()
            (w * c).sum().backward()
            grads.append((av.grad.cpu().numpy(), bv.grad.cpu().numpy()))
        Cp, Ci = pat.c_ptr.cpu().numpy(), pat.c_idx.cpu().numpy()
        dA_o, dB_o = orc.adjoint(A, B, Cp, Ci, w.cpu().numpy())
    (dA0, dB0), (dA1, dB1), (dA2, dB2) = grads
    scale = float(np.abs(dB_o).max())
    assert np.allclose(dB1, dB_o, rtol=1e-12, atol=1e-12 * scale)
    assert np.allclose(dB0, dB1, rtol=1e-12, atol=1e-12 * scale)
    assert np.array_equal(dB1.view(np.uint64), dB2.view(np.uint64))
    assert np.array_equal(dA0.view(np.uint64), dA1.view(np.uint64))
    assert np.allclose(dA1, dA_o, rtol=1e-12, atol=1e-12 * float(np.abs(dA_o).max()))


def loss_at(torch, eng, pat, av, bv, w):
    from dbd_gb300.autograd import spgemm
    with torch.no_grad():
        return float((w * spgemm(av, bv, pat, eng)).sum())


def test_adjoint_2048_dense_reference_and_central_differences():
    """The fwd+adjoint workload at its 2,048 x 2,048 sub-size: A, B with 16
    entries per row, N(0,1) values, W ~ N(0,1) on C's pattern."""
    torch = pytest.importorskip("torch")
    from dbd_gb300.autograd import spgemm, engine
    n = 2048
    A = gen.uniform_rows(n, 16, seed=21)
    B = gen.uniform_rows(n, 16, seed=22)
    pat, av, bv = setup(torch, A, B)
    with engine() as eng:
        c = spgemm(av, bv, pat, eng)
        rng = np.random.default_rng(7)
        w = torch.from_numpy(rng.standard_normal(c.numel())).cuda()
        (w * c).sum().backward()
        Cp, Ci = pat.c_ptr.cpu().numpy(), pat.c_idx.cpu().numpy()
        G = np.zeros((n, n))
        wv = w.cpu().numpy()
        for r in range(n):
            G[r, Ci[Cp[r]:Cp[r + 1]]] = wv[Cp[r]:Cp[r + 1]]
        Ad, Bd = dense(A), dense(B)
        assert np.allclose(dense_vals(G @ Bd.T, A), av.grad.cpu().numpy(), rtol=1e-10, atol=1e-12)
        assert np.allclose(dense_vals(Ad.T @ G, B), bv.grad.cpu().numpy(), rtol=1e-10, atol=1e-12)
        h = 1e-6
        for which, vals, grad in (("A", av, av.grad), ("B", bv, bv.grad)):
            idx = rng.choice(vals.numel(), 25, replace=False)
            for i in idx:
                base = vals.detach().clone()
                up, dn = base.clone(), base.clone()
                up[i] += h
                dn[i] -= h
                if which == "A":
                    fd = (loss_at(torch, eng, pat, up, bv.detach(), w) - loss_at(torch, eng, pat, dn, bv.detach(), w)) / (2 * h)
                else:
                    fd = (loss_at(torch, eng, pat, av.detach(), up, w) - loss_at(torch, eng, pat, av.detach(), dn, w)) / (2 * h)
                g = float(grad[i])
                assert abs(fd - g) <= 1e-6 * max(1.0, abs(g)), (which, i, fd, g)


def dense_vals(D, M):
    rows = np.repeat(np.arange(M.n_rows), np.diff(M.row_ptr))
    return D[rows, M.col_idx]


def test_adjoint_full_size_central_differences():
    """The fwd+adjoint workload at full size (100,000 x 100,000, 16 per row):
    central differences on 1,000 sampled entries (500 of A, 500 of B)."""
    torch = pytest.importorskip("torch")
    from dbd_gb300.autograd import spgemm, engine
    n = 100_000
    A = gen.uniform_rows(n, 16, seed=31)
    B = gen.uniform_rows(n, 16, seed=32)
    pat, av, bv = setup(torch, A, B)
    with engine() as eng:
        c = spgemm(av, bv, pat, eng)
        assert c.numel() > 25_000_000
        rng = np.random.default_rng(9)
        w = torch.from_numpy(rng.standard_normal(c.numel())).cuda()
        (w * c).sum().backward()
        h = 1e-6
        worst = 0.0
        for which, vals, grad in (("A", av, av.grad), ("B", bv, bv.grad)):
            for i in rng.choice(vals.numel(), 500, replace=False):
                up, dn = vals.detach().clone(), vals.detach().clone()
                up[i] += h
                dn[i] -= h
                if which == "A":
                    fd = (loss_at(torch, eng, pat, up, bv.detach(), w) - loss_at(torch, eng, pat, dn, bv.detach(), w)) / (2 * h)
                else:
                    fd = (loss_at(torch, eng, pat, av.detach(), up, w) - loss_at(torch, eng, pat, av.detach(), dn, w)) / (2 * h)
                g = float(grad[i])
                worst = max(worst, abs(fd - g) / max(1.0, abs(g)))
        # |loss| ~ sqrt(nnz(C)) ~ 5e3: rounding of the loss / (2h) is ~ 1e-9
        assert worst <= 1e-5, worst


def test_adjoint_refuses_mismatched_inner_dimensions():
    """A kept-pattern call whose A has more columns than B has rows is refused
    before anything is launched, and the context stays usable."""
    import ctypes as C_
    import dbd_gb300 as dbd
    A = gen.uniform_rows(300, 7, seed=11, n_cols=200)
    B = gen.uniform_rows(200, 9, seed=12, n_cols=250)
    with dbd.Context(cpu_gib=1, gpu_gib=1) as ctx:
        nnz = ctx.spgemm(A, B, scope="kernel").C.nnz
        va, _ka = A.view()
        vb, _kb = B.view()
        g = np.ones(nnz)
        da, db = np.empty(A.nnz), np.empty(B.nnz)
        va.n_cols = 201
        rc = ctx._lib.dbd_spgemm_adjoint(ctx.handle, C_.byref(va), C_.byref(vb), g.ctypes.data, da.ctypes.data,
                                         db.ctypes.data, 0, 0)
        assert rc == -1  # DBD_ERR_INVALID
        assert b"inner dimensions" in ctx._lib.dbd_last_error(ctx.handle)
        va.n_cols = 200
        dbd._check(ctx._lib.dbd_spgemm_adjoint(ctx.handle, C_.byref(va), C_.byref(vb), g.ctypes.data,
                                               da.ctypes.data, db.ctypes.data, 0, 2), ctx.handle)
        # L = sum(C): dA(i,k) is B's row sum k, dB(k,j) is A's column sum k.
        assert np.allclose(da, np.add.reduceat(B.val, B.row_ptr[:-1])[A.col_idx], rtol=1e-12)
        colsum = np.bincount(A.col_idx, weights=A.val, minlength=200)
        assert np.allclose(db, np.repeat(colsum, np.diff(B.row_ptr)), rtol=1e-12)
