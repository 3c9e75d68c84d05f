"""dbd_gb300 -- GB300-native out-of-core SpGEMM (C = A*B, CSR) behind DBD's interface.

Host-side mirror of the reference's stage functions (ZIP:dbd/src/SSpMM.hpp:126-149)
over the C ABI of libdbd (include/dbd.h):

    read_CSR(path)                      -> readInput.cpp:18  read_CSR
    ctx = Context(cpu_gib, gpu_gib)     -> main.cpp:152      initialize (+ preProc.cu:23 initialize_GPU)
    ctx.initialize_A(A), initialize_B   -> preProc.cu:28-46
    ctx.divide_Blocks()                 -> main.cpp:259      divide_Blocks (+ get_UpperBound)
    ctx.distribute_Workload(scope, dir) -> distributeWorkload.cpp:25 distribute_Workload
    ctx.spgemm(A, B, scope)             -> one call of all of the above

Errors: the reference prints to stderr and returns -1 / exits; here every
failure raises DBDError carrying the library's error code and message.
"""
import ctypes as C
import os

import numpy as np

from . import _ffi
from .csr import CSR

__all__ = ["CSR", "Context", "DBDError", "Writer", "read_CSR", "write_CSR", "lib_path", "SCOPES"]

SCOPES = dict(_ffi.SCOPES)


def lib_path():
    return _ffi.LIB_PATH


class DBDError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        name = _ffi.ERR_NAMES.get(code, str(code))
        super().__init__(f"{name}: {msg}" if msg else name)


def _check(rc, ctx=None):
    if rc != _ffi.DBD_OK:
        msg = ""
        if ctx is not None:
            m = _ffi.load().dbd_last_error(ctx)
            msg = m.decode() if m else ""
        raise DBDError(rc, msg)


def _scope(scope):
    if isinstance(scope, str):
        return SCOPES[scope]
    return int(scope)


def read_CSR(path, gpu=None):
    """Reads <path>.dcsr, <path>.csr (reference layout) or converts <path>
    (.mtx/.dat): on the host, or on CUDA device `gpu` when given."""
    lib = _ffi.load()
    h = _ffi.CsrHost()
    if gpu is None:
        _check(lib.dbd_read_csr(os.fsencode(path), C.byref(h)))
    else:
        _check(lib.dbd_read_csr_gpu(os.fsencode(path), int(gpu), C.byref(h)))
    try:
        n, nnz = h.n_rows, h.nnz
        ptr = np.ctypeslib.as_array(C.cast(h.row_ptr, C.POINTER(C.c_int32)), shape=(n + 1,)).copy()
        if nnz:
            idx = np.ctypeslib.as_array(C.cast(h.col_idx, C.POINTER(C.c_int32)), shape=(nnz,)).copy()
            val = np.ctypeslib.as_array(C.cast(h.val, C.POINTER(C.c_double)), shape=(nnz,)).copy()
        else:
            idx = np.zeros(0, np.int32)
            val = np.zeros(0, np.float64)
        return CSR(h.n_rows, h.n_cols, ptr, idx, val)
    finally:
        lib.dbd_csr_host_free(C.byref(h))


def write_CSR(path, m, fp64=True):
    """Writes m as .dcsr (fp64=True) or in the reference .csr layout (float32 values)."""
    lib = _ffi.load()
    v, _keep = m.view()
    _check(lib.dbd_write_csr(os.fsencode(path), C.byref(v), 1 if fp64 else 0))


class Writer:
    """The +I/O output writer on the caller's chunks (dbd_writer_*): Idx.output
    and Val.output appended in row order with aligned O_DIRECT writes (or
    through the page cache), Ptr.output at finish().  With resume=True a
    progress manifest makes every append durable; reopening the same product
    (n_rows, nnz, fingerprint, layout) continues at .resume_row."""

    def __init__(self, out_dir, n_rows, nnz, fingerprint=0, buffered=False, val_fp32=False, ptr32=False,
                 resume=False, rotate_gib=0.0):
        self._lib = _ffi.load()
        flags = ((_ffi.WRITER_BUFFERED if buffered else 0) | (_ffi.WRITER_VAL_FP32 if val_fp32 else 0) |
                 (_ffi.WRITER_PTR32 if ptr32 else 0) | (_ffi.WRITER_RESUME if resume else 0))
        h = C.c_void_p()
        row = C.c_int64()
        _check(self._lib.dbd_writer_open(os.fsencode(out_dir), int(n_rows), int(nnz), int(fingerprint), flags,
                                         float(rotate_gib), C.byref(h), C.byref(row)))
        self._h = h
        self.resume_row = row.value
        self.direct = bool(self._lib.dbd_writer_is_direct(h))

    def _check(self, rc):
        if rc != _ffi.DBD_OK:
            m = self._lib.dbd_writer_error(self._h)
            raise DBDError(rc, m.decode() if m else "")

    def append(self, row_end, col_idx, val):
        ci = np.ascontiguousarray(col_idx, np.int32)
        cv = np.ascontiguousarray(val, np.float64)
        if ci.size != cv.size:
            raise ValueError("col_idx and val differ in length")
        self._check(self._lib.dbd_writer_append(self._h, int(row_end), ci.ctypes.data, cv.ctypes.data, ci.size))

    def finish(self, row_ptr):
        rp = np.ascontiguousarray(row_ptr, np.int64)
        t = C.c_double()
        self._check(self._lib.dbd_writer_finish(self._h, rp.ctypes.data, C.byref(t)))
        return t.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.dbd_writer_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Result:
    """Product of one multiply: C (host CSR with int64 row_ptr) and the stats."""

    def __init__(self, C_, stats):
        self.C = C_
        self.stats = stats

    @property
    def gflops(self):
        t = self.stats["t_total"]
        return 2.0 * self.stats["products"] / t / 1e9 if t > 0 else float("nan")


class BatchResult:
    """Product of one batched multiply: per-pair offsets into the concatenated
    C (row_off, nnz_off: count + 1 each), the stats and, when fetched, the
    per-pair host products C[q]."""

    def __init__(self, row_off, nnz_off, stats):
        self.row_off = row_off
        self.nnz_off = nnz_off
        self.stats = stats
        self.C = None

    @property
    def gflops(self):
        t = self.stats["t_total"]
        return 2.0 * self.stats["products"] / t / 1e9 if t > 0 else float("nan")


class Context:
    """A libdbd context: device, budgets, streams, buffers (one per host thread)."""

    def __init__(self, cpu_gib=28.0, gpu_gib=22.0, rows_per_block=4096, device=0, out_val_fp32=False,
                 out_ptr32=False, verbose=False, io_rotate_gib=0.0, time_kernels=False, io_buffered=False,
                 io_resume=False):
        self._lib = _ffi.load()
        cfg = _ffi.Config()
        self._lib.dbd_config_default(C.byref(cfg))
        cfg.host_gib = float(cpu_gib)
        cfg.gpu_gib = float(gpu_gib)
        cfg.rows_per_block = int(rows_per_block)
        cfg.device = int(device)
        cfg.out_val_fp32 = int(bool(out_val_fp32))
        cfg.out_ptr32 = int(out_ptr32)
        cfg.verbose = int(bool(verbose))
        cfg.time_kernels = int(bool(time_kernels))
        cfg.io_rotate_gib = float(io_rotate_gib)
        cfg.io_buffered = int(bool(io_buffered))
        cfg.io_resume = int(bool(io_resume))
        h = C.c_void_p()
        _check(self._lib.dbd_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.dbd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle):
        """Runs the device pipeline on this cudaStream_t (an int), or the context's own (None)."""
        _check(self._lib.dbd_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None), self._h)

    # ---- the reference's stage functions ----
    def initialize_A(self, A):
        v, keep = A.view()
        self._keep = [keep]
        _check(self._lib.dbd_load_a(self._h, C.byref(v)), self._h)

    def initialize_B(self, B):
        v, keep = B.view()
        self._keep.append(keep)
        _check(self._lib.dbd_load_b(self._h, C.byref(v)), self._h)

    def divide_Blocks(self):
        nb = C.c_int64()
        _check(self._lib.dbd_divide_blocks(self._h, C.byref(nb)), self._h)
        return nb.value

    def block_info(self, num_blocks):
        p = np.zeros(num_blocks, np.int64)
        cat = np.zeros(num_blocks, np.int32)
        _check(self._lib.dbd_block_info(self._h, p.ctypes.data, cat.ctypes.data), self._h)
        return p, cat

    def distribute_Workload(self, scope="kernel", out_dir="."):
        _check(self._lib.dbd_distribute_workload(self._h, _scope(scope), os.fsencode(out_dir)), self._h)
        return self.stats()

    def stats(self):
        st = _ffi.Stats()
        _check(self._lib.dbd_get_stats(self._h, C.byref(st)), self._h)
        return st.as_dict()

    def result(self):
        """Copies the last product to host numpy arrays."""
        o = _ffi.CsrOut()
        _check(self._lib.dbd_result(self._h, C.byref(o)), self._h)
        ptr = np.empty(o.n_rows + 1, np.int64)
        idx = np.empty(o.nnz, np.int32)
        if o.val_fp32:
            # float32 values (out_val_fp32 in a copying scope), in host memory
            val = np.empty(o.nnz, np.float32)
            if o.nnz:
                C.memmove(val.ctypes.data, o.val, 4 * o.nnz)
            _check(self._lib.dbd_result_copy(self._h, ptr.ctypes.data, idx.ctypes.data, None), self._h)
        else:
            val = np.empty(o.nnz, np.float64)
            _check(self._lib.dbd_result_copy(self._h, ptr.ctypes.data, idx.ctypes.data, val.ctypes.data), self._h)
        return CSR(o.n_rows, o.n_cols, ptr, idx, val)

    # ---- one-shot ----
    def spgemm(self, A, B=None, scope="kernel", out_dir=".", fetch=True):
        """C = A*B (B=None: A*A).  fetch=False leaves C where the scope put it."""
        va, ka = A.view()
        if B is None or B is A:
            pb = None
            kb = None
        else:
            vb, kb = B.view()
            pb = C.byref(vb)
        st = _ffi.Stats()
        _check(self._lib.dbd_spgemm(self._h, C.byref(va), pb, _scope(scope), os.fsencode(out_dir), None,
                                    C.byref(st)), self._h)
        del ka, kb
        stats = st.as_dict()
        if not fetch or _scope(scope) == SCOPES["io"]:
            return Result(None, stats)
        return Result(self.result(), stats)

    def spgemm_batched(self, As, Bs=None, scope="kernel", fetch=True):
        """C_q = A_q * B_q for every pair (Bs=None: A_q * A_q) in one multiply.

        Returns a BatchResult: the pairs' row and entry offsets in the
        concatenated product, the stats and, with fetch=True, the list of
        per-pair host CSR products (local columns, row_ptr from 0)."""
        count = len(As)
        if Bs is not None and len(Bs) != count:
            raise ValueError("As and Bs differ in length")
        va = (_ffi.CsrView * count)()
        keep = []
        for q, A in enumerate(As):
            v, k = A.view()
            va[q] = v
            keep.append(k)
        pb = None
        if Bs is not None:
            vb = (_ffi.CsrView * count)()
            for q, B in enumerate(Bs):
                v, k = B.view()
                vb[q] = v
                keep.append(k)
            pb = vb
        row_off = np.zeros(count + 1, np.int64)
        nnz_off = np.zeros(count + 1, np.int64)
        st = _ffi.Stats()
        _check(self._lib.dbd_spgemm_batched(self._h, count, va, pb, _scope(scope), row_off.ctypes.data,
                                            nnz_off.ctypes.data, None, C.byref(st)), self._h)
        del keep
        res = BatchResult(row_off, nnz_off, st.as_dict())
        if fetch:
            whole = self.result()
            ncols = [(Bs[q] if Bs is not None else As[q]).n_cols for q in range(count)]
            res.C = [whole.slice_pair(row_off[q], row_off[q + 1], nnz_off[q], nnz_off[q + 1], ncols[q])
                     for q in range(count)]
        return res

    # ---- the capturable batched multiply ----
    def batch_plan(self, As, Bs=None, capacity=0):
        """Plans the device-driven batched multiply (dbd_batch_plan): device
        pairs (CSR.from_device views) whose arrays stay in place, C with room
        for `capacity` entries."""
        count = len(As)
        va = (_ffi.CsrView * count)()
        keep = []
        for q, A in enumerate(As):
            v, k = A.view()
            va[q] = v
            keep.append(k)
        pb = None
        if Bs is not None:
            vb = (_ffi.CsrView * count)()
            for q, B in enumerate(Bs):
                v, k = B.view()
                vb[q] = v
                keep.append(k)
            pb = C.cast(vb, C.c_void_p)
        _check(self._lib.dbd_batch_plan(self._h, count, C.cast(va, C.c_void_p), pb, int(capacity)), self._h)
        ncols = [(Bs[q] if Bs is not None else As[q]).n_cols for q in range(count)]
        self._batch = (count, keep, ncols)

    def batch_enqueue(self, stream=None):
        """Enqueues the planned multiply on `stream` (a cudaStream_t as an
        int; None: the context's) without synchronising: capturable."""
        _check(self._lib.dbd_batch_enqueue(self._h, C.c_void_p(stream) if stream else None), self._h)

    def batch_result(self, fetch=True):
        """Status and product of the last enqueued run (after it completed)."""
        count, _, ncols = self._batch
        row_off = np.zeros(count + 1, np.int64)
        nnz_off = np.zeros(count + 1, np.int64)
        o = _ffi.CsrOut()
        _check(self._lib.dbd_batch_result(self._h, row_off.ctypes.data, nnz_off.ctypes.data, C.byref(o)), self._h)
        res = BatchResult(row_off, nnz_off, None)
        if fetch:
            whole = self.result()
            res.C = [whole.slice_pair(row_off[q], row_off[q + 1], nnz_off[q], nnz_off[q + 1], ncols[q])
                     for q in range(count)]
        return res

    # ---- tuning ----
    @property
    def tuning(self):
        """The bin thresholds in use (dict of dbd_tuning's fields)."""
        t = _ffi.Tuning()
        _check(self._lib.dbd_get_tuning(self._h, C.byref(t)), self._h)
        return t.as_dict()

    def set_tuning(self, **kw):
        """Changes some bin thresholds (names as in dbd_tuning)."""
        t = _ffi.Tuning()
        _check(self._lib.dbd_get_tuning(self._h, C.byref(t)), self._h)
        for k, v in kw.items():
            if not hasattr(t, k):
                raise KeyError(k)
            setattr(t, k, int(v))
        _check(self._lib.dbd_set_tuning(self._h, C.byref(t)), self._h)

    def autotune(self, repeats=2):
        """Tunes the bin thresholds on the operands loaded now; returns (tuning, ms)."""
        t = _ffi.Tuning()
        ms = C.c_double()
        _check(self._lib.dbd_autotune(self._h, int(repeats), C.byref(t), C.byref(ms)), self._h)
        return t.as_dict(), ms.value

    def update_values(self, a_vals, b_vals=None):
        """New values of A (and B) on the last kernel-scope multiply's patterns:
        only the numeric kernels run, replayed from a captured CUDA graph.

        a_vals / b_vals: one array per pair (a single array after spgemm),
        all numpy float64 (host) or all CUDA tensors (device)."""
        if not isinstance(a_vals, (list, tuple)):
            a_vals = [a_vals]
            b_vals = None if b_vals is None else [b_vals]

        def table(vals):
            on_dev = hasattr(vals[0], "data_ptr")
            keep = [v if on_dev else np.ascontiguousarray(v, np.float64) for v in vals]
            t = (C.c_void_p * len(keep))(*[(v.data_ptr() if on_dev else v.ctypes.data) for v in keep])
            return t, keep, on_dev

        ta, ka, on_dev = table(a_vals)
        tb, kb = None, None
        if b_vals is not None:
            tb, kb, on_dev_b = table(b_vals)
            if on_dev_b != on_dev:
                raise ValueError("A and B values must both be host or both be device arrays")
        _check(self._lib.dbd_update_values(self._h, len(a_vals), ta, tb, 1 if on_dev else 0), self._h)
        del ka, kb

    # ---- output digest ----
    def set_digest(self, device=True, host=False):
        """Per-row digest of C on every later multiply: on the device after each
        chunk's kernels (device) and from each chunk's pinned host copy in the
        d2h / io scopes (host)."""
        flags = (_ffi.DIGEST_DEVICE if device else 0) | (_ffi.DIGEST_HOST if host else 0)
        _check(self._lib.dbd_set_digest(self._h, flags), self._h)

    def digest(self, n_rows, which="device"):
        """The last multiply's digest (C has n_rows rows): dict of per-row
        numpy arrays count, col_hash, val_hash (uint64), sum, wsum and the
        count of bad rows."""
        m = int(n_rows)
        out = {"count": np.empty(m, np.int64), "col_hash": np.empty(m, np.uint64),
               "val_hash": np.empty(m, np.uint64), "sum": np.empty(m), "wsum": np.empty(m)}
        bad = C.c_int64()
        w = _ffi.DIGEST_DEVICE if which == "device" else _ffi.DIGEST_HOST
        _check(self._lib.dbd_digest_copy(self._h, w, out["count"].ctypes.data, out["col_hash"].ctypes.data,
                                         out["val_hash"].ctypes.data, out["sum"].ctypes.data,
                                         out["wsum"].ctypes.data, C.byref(bad)), self._h)
        out["bad_rows"] = int(bad.value)
        return out

    def spgemm_files(self, path_a, path_b=None, scope="io", out_dir="."):
        st = _ffi.Stats()
        _check(self._lib.dbd_spgemm_files(self._h, os.fsencode(path_a),
                                          os.fsencode(path_b) if path_b else None, _scope(scope),
                                          os.fsencode(out_dir), C.byref(st)), self._h)
        return st.as_dict()
