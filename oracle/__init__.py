"""Oracle: CPU restatement of DBD's SpGEMM path (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs as the checker / the timed CPU restatement of the
reference's algorithm.  The product (dbd_gb300, libdbd) never imports it.

    spgemm(A, B)            FP64 Gustavson, sorted, index-determined structure
                            (the oracle of record); also returns sum|a*b| per
                            entry for the tolerance
    ref_cpu(A, B, threads)  FP32 restatement of the reference's CPU worker
                            compute_CPU (value-based structure, first-touch order)
    row_products / divide_blocks / criteria / analyze_block / threads_per_row
                            the reference's work estimate, segmenter and categoriser
    adjoint(A, B, C, G)     dA = mask_A(G B^T), dB = mask_B(A^T G)
    reference()             the reference's own CPU code built by build_ref.py
                            (None when the reference tree was not available)
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libdbdref.so")

_orc = None
_ref = None

P = C.c_void_p
I64 = C.c_int64


def build():
    """Compiles liborc.so (make) and, when the reference tree is present, oracle/_ref."""
    subprocess.check_call(["make", "-s", "-C", HERE])
    from . import build_ref
    build_ref.build()


def lib():
    global _orc
    if _orc is None:
        if not os.path.exists(LIB):
            subprocess.check_call(["make", "-s", "-C", HERE])
        L = C.CDLL(LIB)
        L.orc_row_products.restype = I64
        L.orc_row_products.argtypes = [I64, P, P, P, P]
        L.orc_exclusive_scan_i64.argtypes = [I64, P, P]
        L.orc_divide_blocks.restype = I64
        L.orc_divide_blocks.argtypes = [I64, P, I64, P, P, P]
        L.orc_criteria.restype = C.c_int32
        L.orc_criteria.argtypes = [I64, P, I64, I64]
        L.orc_analyze_block.restype = C.c_int32
        L.orc_analyze_block.argtypes = [C.c_int32, I64]
        L.orc_threads_per_row.restype = C.c_int32
        L.orc_threads_per_row.argtypes = [I64]
        L.orc_spgemm_symbolic.restype = I64
        L.orc_spgemm_symbolic.argtypes = [I64, I64, P, P, P, P, P]
        L.orc_spgemm_numeric.argtypes = [I64, I64, P, P, P, P, P, P, P, P, P, P]
        L.orc_ref_cpu_rows.argtypes = [I64, I64, I64, P, P, P, P, P, P, P, P, P, P, C.c_int]
        L.orc_adjoint.argtypes = [I64, P, P, P, P, P, P, I64, P, P, P, P, P]
        L.orc_row_col_digest.argtypes = [I64, I64, I64, P, P, P, P, P, P]
        L.orc_row_sums.argtypes = [I64, P, P, P, I64, P, P, P, C.c_int, P, P]
        L.orc_col_weight.restype = C.c_double
        L.orc_col_weight.argtypes = [C.c_int32]
        _orc = L
    return _orc


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


def _csr(M, vdt=np.float64):
    return _a(M.row_ptr, np.int32), _a(M.col_idx, np.int32), _a(M.val, vdt)


def row_products(A, B):
    Ap, Ai, _ = _csr(A)
    Bp, _, _ = _csr(B)
    out = np.zeros(A.n_rows, np.int64)
    tot = lib().orc_row_products(A.n_rows, Ap.ctypes.data, Ai.ctypes.data, Bp.ctypes.data, out.ctypes.data)
    return out, tot


def exclusive_scan(x):
    x = _a(x, np.int64)
    out = np.zeros(x.size + 1, np.int64)
    lib().orc_exclusive_scan_i64(x.size, x.ctypes.data, out.ctypes.data)
    return out


def divide_blocks(m, upp, rows_per_block):
    upp = _a(upp, np.int64)
    nb = (m - 1) // rows_per_block + 1 if m > 0 else 0
    bptr = np.zeros(nb + 1, np.int64)
    binfo = np.zeros(max(nb, 1), np.int64)
    mx = C.c_int64()
    n = lib().orc_divide_blocks(m, upp.ctypes.data, rows_per_block, bptr.ctypes.data, binfo.ctypes.data,
                                C.byref(mx))
    return bptr, binfo[:n], mx.value


def criteria(block_info, rows_per_block, neC):
    b = _a(block_info, np.int64)
    return lib().orc_criteria(b.size, b.ctypes.data, rows_per_block, neC)


def analyze_block(crit, avg):
    return lib().orc_analyze_block(crit, avg)


def threads_per_row(block_products):
    return lib().orc_threads_per_row(block_products)


def spgemm(A, B=None, with_abs=False):
    """FP64 oracle of record: returns (Cp int64, Ci int32, Cv f64[, Cabs f64])."""
    B = A if B is None else B
    Ap, Ai, Av = _csr(A)
    Bp, Bi, Bv = _csr(B)
    m, n = A.n_rows, B.n_cols
    Cp = np.zeros(m + 1, np.int64)
    nnz = lib().orc_spgemm_symbolic(m, n, Ap.ctypes.data, Ai.ctypes.data, Bp.ctypes.data, Bi.ctypes.data,
                                    Cp.ctypes.data)
    Ci = np.zeros(max(nnz, 1), np.int32)
    Cv = np.zeros(max(nnz, 1), np.float64)
    Ca = np.zeros(max(nnz, 1), np.float64) if with_abs else None
    lib().orc_spgemm_numeric(m, n, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, Bp.ctypes.data,
                             Bi.ctypes.data, Bv.ctypes.data, Cp.ctypes.data, Ci.ctypes.data, Cv.ctypes.data,
                             Ca.ctypes.data if with_abs else None)
    if with_abs:
        return Cp, Ci[:nnz], Cv[:nnz], Ca[:nnz]
    return Cp, Ci[:nnz], Cv[:nnz]


def ref_cpu(A, B=None, threads=0, row0=0, row1=None):
    """FP32 restatement of compute_CPU.  Returns (slot_off, rowcnt, idx_slots, val_slots):
    row r's entries (first-touch order, duplicates possible) are
    idx_slots[slot_off[r] - slot_off[row0] : ... + rowcnt[r]]."""
    B = A if B is None else B
    Ap, Ai, Av = _csr(A, np.float32)
    Bp, Bi, Bv = _csr(B, np.float32)
    m = A.n_rows
    row1 = m if row1 is None else row1
    rp, _ = row_products(A, B)
    off = exclusive_scan(rp)
    total = int(off[row1] - off[row0])
    cnt = np.zeros(m, np.int32)
    idx = np.zeros(max(total, 1), np.int32)
    val = np.zeros(max(total, 1), np.float32)
    lib().orc_ref_cpu_rows(row0, row1, B.n_cols, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, Bp.ctypes.data,
                           Bi.ctypes.data, Bv.ctypes.data, off.ctypes.data, cnt.ctypes.data, idx.ctypes.data,
                           val.ctypes.data, int(threads))
    return off, cnt, idx, val


def slots_to_rows(off, cnt, idx, val, row0=0, row1=None):
    """Per-row (cols, vals) lists from the slot layout of ref_cpu / reference()."""
    row1 = cnt.size if row1 is None else row1
    out = []
    for r in range(row0, row1):
        s = off[r] - off[row0]
        out.append((idx[s:s + cnt[r]], val[s:s + cnt[r]]))
    return out


def canonicalise(off, cnt, idx, val):
    """Reference output -> (Cp, Ci, Cv, n_duplicates): rows sorted by column;
    duplicate columns (the reference's value-based structure) are summed and
    counted."""
    m = cnt.size
    Cp = np.zeros(m + 1, np.int64)
    cols, vals = [], []
    dups = 0
    for r in range(m):
        s = off[r]
        c = idx[s:s + cnt[r]].astype(np.int64)
        v = val[s:s + cnt[r]].astype(np.float64)
        u, inv = np.unique(c, return_inverse=True)
        dups += c.size - u.size
        acc = np.zeros(u.size)
        np.add.at(acc, inv, v)
        cols.append(u.astype(np.int32))
        vals.append(acc)
        Cp[r + 1] = Cp[r] + u.size
    Ci = np.concatenate(cols) if cols else np.zeros(0, np.int32)
    Cv = np.concatenate(vals) if vals else np.zeros(0)
    return Cp, Ci, Cv, dups


def adjoint(A, B, Cp, Ci, G):
    Ap, Ai, Av = _csr(A)
    Bp, Bi, Bv = _csr(B)
    Cp = _a(Cp, np.int64)
    Ci = _a(Ci, np.int32)
    G = _a(G, np.float64)
    dA = np.zeros(max(Ai.size, 1))
    dB = np.zeros(max(Bi.size, 1))
    lib().orc_adjoint(A.n_rows, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, Bp.ctypes.data, Bi.ctypes.data,
                      Bv.ctypes.data, Bi.size, Cp.ctypes.data, Ci.ctypes.data, G.ctypes.data, dA.ctypes.data,
                      dB.ctypes.data)
    return dA[:Ai.size], dB[:Bi.size]


def col_weights(cols):
    """w(c) = 0.5 + (mix64(c) >> 11) * 2^-53 of the library's digest, vectorised."""
    z = np.asarray(cols).astype(np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return 0.5 + (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def mix64(x):
    """SplitMix64's output function on uint64 arrays (the digest's column hash)."""
    z = np.asarray(x).astype(np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def row_col_digest(A, B=None, r0=0, r1=None):
    """(count, col_hash) of rows [r0, r1) of A*B: distinct columns per row and
    the sum of mix64(col) over them, without forming C (O(products))."""
    B = A if B is None else B
    r1 = A.n_rows if r1 is None else r1
    Ap, Ai, _ = _csr(A)
    Bp, Bi, _ = _csr(B)
    cnt = np.zeros(max(r1 - r0, 1), np.int64)
    h = np.zeros(max(r1 - r0, 1), np.uint64)
    lib().orc_row_col_digest(r0, r1, B.n_cols, Ap.ctypes.data, Ai.ctypes.data, Bp.ctypes.data, Bi.ctypes.data,
                             cnt.ctypes.data, h.ctypes.data)
    return cnt[:r1 - r0], h[:r1 - r0]


def row_sums(A, B=None, weighted=False):
    """(A*(B*w), |A|*(|B|*w)) per row by compensated sums; w = 1 or the
    digest's column weights."""
    B = A if B is None else B
    Ap, Ai, Av = _csr(A)
    Bp, Bi, Bv = _csr(B)
    out = np.zeros(max(A.n_rows, 1))
    out_abs = np.zeros(max(A.n_rows, 1))
    lib().orc_row_sums(A.n_rows, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, B.n_rows, Bp.ctypes.data,
                       Bi.ctypes.data, Bv.ctypes.data, 1 if weighted else 0, out.ctypes.data, out_abs.ctypes.data)
    return out[:A.n_rows], out_abs[:A.n_rows]


# ---- the reference's own CPU code (built only where the reference tree exists) ----

def reference():
    """ctypes handle on oracle/_ref/libdbdref.so, or None when it was not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            return None
        L = C.CDLL(REF_LIB)
        L.ref_read_csr.argtypes = [C.c_char_p, P, P, P, P, P, P]
        L.ref_cpu_spgemm.argtypes = [C.c_int, C.c_int, P, P, P, C.c_int, C.c_int, P, P, P, P, P, P, P]
        L.ref_free.argtypes = [P]
        L.ref_rows_in_block.restype = C.c_int
        L.ref_divide.restype = C.c_int
        L.ref_divide.argtypes = [C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P]
        L.ref_criteria.restype = C.c_int
        L.ref_criteria.argtypes = [C.c_int, P, C.c_longlong]
        L.ref_cpu_blocks.restype = C.c_int
        L.ref_cpu_blocks.argtypes = [C.c_int, C.c_int, P, P, P, C.c_int, C.c_int, P, P, P, C.c_int, REF_BLOCK_CB,
                                     P]
        _ref = L
    return _ref


# Callback of ref_cpu_blocks: (r0, r1, cnt, hash, idx, n_idx, dups, user).
REF_BLOCK_CB = C.CFUNCTYPE(None, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_uint64),
                           C.POINTER(C.c_int32), C.c_longlong, C.c_longlong, C.c_void_p)


def ref_cpu_blocks(A, B=None, rows_per_block=512, on_block=None):
    """Runs the reference's compute_CPU over A*B block by block of
    rows_per_block rows and hands each block's canonical output to
    on_block(r0, r1, cnt, hash, idx, dups): cnt the entries of each row,
    hash the sum of mix64(col) over each row's entries, idx the rows' columns
    (each row sorted, duplicates kept), dups the number of repeated columns in
    the block (0 on quirk-inert inputs).  The arrays are
    valid only during the call.  Memory: the largest block's products, not
    the whole product."""
    L = reference()
    B = A if B is None else B
    Ap, Ai, Av = _csr(A, np.float32)
    Bp, Bi, Bv = _csr(B, np.float32)

    def cb(r0, r1, cnt, hsh, idx, n, dups, user):
        c = np.ctypeslib.as_array(cnt, shape=(r1 - r0,)) if r1 > r0 else np.zeros(0, np.int32)
        h = np.ctypeslib.as_array(hsh, shape=(r1 - r0,)) if r1 > r0 else np.zeros(0, np.uint64)
        i = np.ctypeslib.as_array(idx, shape=(n,)) if n else np.zeros(0, np.int32)
        on_block(r0, r1, c, h, i, dups)
    fn = REF_BLOCK_CB(cb)
    rc = L.ref_cpu_blocks(A.n_rows, A.n_cols, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, B.n_rows, B.n_cols,
                          Bp.ctypes.data, Bi.ctypes.data, Bv.ctypes.data, int(rows_per_block), fn, None)
    if rc:
        raise RuntimeError(f"ref_cpu_blocks failed ({rc})")


def ref_divide(A, B=None):
    """divide_Blocks of the reference on A*B (its ROWS_IN_BLOCK = 4096):
    (block_info int32, block_ptr int32, neC)."""
    L = reference()
    B = A if B is None else B
    Ap, Ai, _ = _csr(A)
    Bp, _, _ = _csr(B)
    nb = (A.n_rows - 1) // L.ref_rows_in_block() + 1
    info = np.zeros(nb, np.int32)
    bptr = np.zeros(nb + 1, np.int32)
    tot = C.c_longlong()
    got = L.ref_divide(A.n_rows, A.n_cols, Ap.ctypes.data, Ai.ctypes.data, B.n_rows, B.n_cols, Bp.ctypes.data,
                       info.ctypes.data, bptr.ctypes.data, C.byref(tot))
    return info[:max(got, 0)], bptr[:max(got, 0) + 1], tot.value


def ref_criteria(block_info, neC):
    L = reference()
    b = _a(block_info, np.int32)
    return L.ref_criteria(b.size, b.ctypes.data, int(neC))


def ref_read_csr(path):
    """read_CSR of the reference (converts .mtx and writes <path>.csr if needed)."""
    L = reference()
    nr, nc, ne = C.c_int(), C.c_int(), C.c_int()
    p, i, v = C.c_void_p(), C.c_void_p(), C.c_void_p()
    L.ref_read_csr(os.fsencode(path), C.byref(nr), C.byref(nc), C.byref(ne), C.byref(p), C.byref(i), C.byref(v))
    ptr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int32)), shape=(nr.value + 1,)).copy()
    idx = np.ctypeslib.as_array(C.cast(i, C.POINTER(C.c_int32)), shape=(ne.value,)).copy() if ne.value else np.zeros(0, np.int32)
    val = np.ctypeslib.as_array(C.cast(v, C.POINTER(C.c_float)), shape=(ne.value,)).copy() if ne.value else np.zeros(0, np.float32)
    for q in (p, i, v):
        L.ref_free(q)
    return nr.value, nc.value, ptr, idx, val


def ref_cpu_spgemm(A, B=None):
    """The reference's compute_CPU over all blocks: (slot_off, rowcnt, idx_slots, val_slots)."""
    L = reference()
    B = A if B is None else B
    Ap, Ai, Av = _csr(A, np.float32)
    Bp, Bi, Bv = _csr(B, np.float32)
    m = A.n_rows
    off = np.zeros(m + 1, np.int64)
    rp, total = row_products(A, B)
    cnt = np.zeros(m, np.int32)
    idx = np.zeros(max(total, 1), np.int32)
    val = np.zeros(max(total, 1), np.float32)
    L.ref_cpu_spgemm(m, A.n_cols, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, B.n_rows, B.n_cols,
                     Bp.ctypes.data, Bi.ctypes.data, Bv.ctypes.data, off.ctypes.data, cnt.ctypes.data,
                     idx.ctypes.data, val.ctypes.data)
    return off, cnt, idx, val
