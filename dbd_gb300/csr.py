"""CSR container used by the host API (numpy arrays, or device arrays by pointer)."""
import ctypes as C

import numpy as np

from . import _ffi


class CSR:
    """CSR matrix: int32 row_ptr (int64 for products), int32 col_idx, float64 (or float32) val.

    On the host the arrays are numpy arrays.  A device-resident operand is
    made with CSR.from_device(n_rows, n_cols, nnz, ptr_addr, idx_addr,
    val_addr) from raw device addresses (e.g. torch tensors' data_ptr()).
    """

    def __init__(self, n_rows, n_cols, row_ptr, col_idx, val):
        self.n_rows = int(n_rows)
        self.n_cols = int(n_cols)
        self.row_ptr = row_ptr
        self.col_idx = col_idx
        self.val = val
        self._dev = None

    @property
    def nnz(self):
        if self._dev is not None:
            return self._dev[0]
        return int(self.col_idx.shape[0])

    @classmethod
    def from_device(cls, n_rows, n_cols, nnz, ptr_addr, idx_addr, val_addr, val_fp32=False):
        m = cls(n_rows, n_cols, None, None, None)
        m._dev = (int(nnz), int(ptr_addr), int(idx_addr), int(val_addr), bool(val_fp32))
        return m

    @classmethod
    def from_scipy(cls, s):
        s = s.tocsr()
        return cls(s.shape[0], s.shape[1], s.indptr.astype(np.int32), s.indices.astype(np.int32),
                   s.data.astype(np.float64))

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col_idx, self.row_ptr), shape=(self.n_rows, self.n_cols))

    def view(self):
        """(dbd_csr_view, keep-alive tuple) for the C ABI."""
        v = _ffi.CsrView()
        v.n_rows = self.n_rows
        v.n_cols = self.n_cols
        if self._dev is not None:
            nnz, p, i, x, f32 = self._dev
            v.nnz = nnz
            v.row_ptr, v.col_idx, v.val = p, i, x
            v.val_fp32 = int(f32)
            v.on_device = 1
            return v, None
        ptr = np.ascontiguousarray(self.row_ptr, dtype=np.int32)
        idx = np.ascontiguousarray(self.col_idx, dtype=np.int32)
        if self.val.dtype == np.float32:
            val = np.ascontiguousarray(self.val)
            v.val_fp32 = 1
        else:
            val = np.ascontiguousarray(self.val, dtype=np.float64)
            v.val_fp32 = 0
        v.nnz = idx.shape[0]
        v.row_ptr = ptr.ctypes.data
        v.col_idx = idx.ctypes.data if idx.size else ptr.ctypes.data
        v.val = val.ctypes.data if val.size else ptr.ctypes.data
        v.on_device = 0
        return v, (ptr, idx, val)

    def slice_pair(self, r0, r1, e0, e1, n_cols):
        """Rows [r0, r1) with entries [e0, e1) as their own matrix (row_ptr rebased to 0)."""
        r0, r1, e0, e1 = int(r0), int(r1), int(e0), int(e1)
        return CSR(r1 - r0, n_cols, self.row_ptr[r0:r1 + 1] - e0, self.col_idx[e0:e1], self.val[e0:e1])

    def __repr__(self):
        return f"CSR({self.n_rows}x{self.n_cols}, nnz={self.nnz})"
