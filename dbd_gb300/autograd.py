"""torch.autograd harness over libdbd's multiply and adjoint (test harness).

    pat = Pattern(a_ptr, a_idx, a_shape, b_ptr, b_idx, b_shape)   # int32 CUDA tensors
    c_val = spgemm(a_val, b_val, pat, engine)                      # FP64 values on C's pattern
    loss = (w * c_val).sum(); loss.backward()                      # a_val.grad, b_val.grad

Forward runs dbd_spgemm in the kernel scope on device-resident operands;
backward runs dbd_spgemm_adjoint, which computes dA = mask_A(G B^T) and
dB = mask_B(A^T G) for G = dL/dC on C's pattern.  With keep_pattern=False the
backward recomputes C's pattern instead of relying on the one the engine kept
from the forward (for engines that run other multiplies in between).
"""
import ctypes as C

import torch

from . import Context, _check
from . import _ffi


class Pattern:
    """Fixed sparsity patterns of A (m x k) and B (k x n), int32 CUDA tensors."""

    def __init__(self, a_ptr, a_idx, a_shape, b_ptr, b_idx, b_shape):
        self.a_ptr, self.a_idx, self.a_shape = a_ptr.contiguous(), a_idx.contiguous(), tuple(a_shape)
        self.b_ptr, self.b_idx, self.b_shape = b_ptr.contiguous(), b_idx.contiguous(), tuple(b_shape)
        self.c_ptr = None
        self.c_idx = None

    def views(self, a_val, b_val):
        va = _ffi.CsrView()
        va.n_rows, va.n_cols, va.nnz = self.a_shape[0], self.a_shape[1], self.a_idx.numel()
        va.row_ptr, va.col_idx, va.val = self.a_ptr.data_ptr(), self.a_idx.data_ptr(), a_val.data_ptr()
        va.val_fp32, va.on_device = 0, 1
        vb = _ffi.CsrView()
        vb.n_rows, vb.n_cols, vb.nnz = self.b_shape[0], self.b_shape[1], self.b_idx.numel()
        vb.row_ptr, vb.col_idx, vb.val = self.b_ptr.data_ptr(), self.b_idx.data_ptr(), b_val.data_ptr()
        vb.val_fp32, vb.on_device = 0, 1
        return va, vb


class _SpGEMM(torch.autograd.Function):
    @staticmethod
    def forward(fctx, a_val, b_val, pat, engine, keep_pattern, deterministic):
        a_val = a_val.detach().contiguous()
        b_val = b_val.detach().contiguous()
        lib = engine._lib
        va, vb = pat.views(a_val, b_val)
        engine.set_stream(torch.cuda.current_stream().cuda_stream)
        _check(lib.dbd_spgemm(engine.handle, C.byref(va), C.byref(vb), 0, b".", None, None), engine.handle)
        o = _ffi.CsrOut()
        _check(lib.dbd_result(engine.handle, C.byref(o)), engine.handle)
        c_val = torch.empty(o.nnz, dtype=torch.float64, device=a_val.device)
        c_ptr = torch.empty(o.n_rows + 1, dtype=torch.int64, device=a_val.device)
        c_idx = torch.empty(o.nnz, dtype=torch.int32, device=a_val.device)
        _check(lib.dbd_result_copy(engine.handle, c_ptr.data_ptr(), c_idx.data_ptr(), c_val.data_ptr()),
               engine.handle)
        pat.c_ptr, pat.c_idx = c_ptr, c_idx
        fctx.save_for_backward(a_val, b_val)
        fctx.pat = pat
        fctx.engine = engine
        fctx.keep = keep_pattern
        fctx.det = deterministic
        return c_val

    @staticmethod
    def backward(fctx, grad_c):
        a_val, b_val = fctx.saved_tensors
        engine, pat = fctx.engine, fctx.pat
        g = grad_c.detach().to(torch.float64).contiguous()
        da = torch.empty_like(a_val)
        db = torch.empty_like(b_val)
        va, vb = pat.views(a_val, b_val)
        engine.set_stream(torch.cuda.current_stream().cuda_stream)
        _check(engine._lib.dbd_spgemm_adjoint(engine.handle, C.byref(va), C.byref(vb), g.data_ptr(), da.data_ptr(),
                                              db.data_ptr(), 1, (0 if fctx.keep else 1) | (2 if fctx.det else 0)),
               engine.handle)
        return da, db, None, None, None, None


def spgemm(a_val, b_val, pat, engine, keep_pattern=True, deterministic=False):
    """C's values (FP64, on C's pattern, which is left in pat.c_ptr / pat.c_idx).
    deterministic=True computes dB by its own pass over B's pattern (run-to-run
    identical gradients) instead of reductions from A's rows."""
    return _SpGEMM.apply(a_val, b_val, pat, engine, keep_pattern, deterministic)


def engine(device=0, gpu_gib=64.0):
    return Context(cpu_gib=16, gpu_gib=gpu_gib, device=device)
