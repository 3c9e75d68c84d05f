"""Generates the golden fixtures of tests/golden from the reference's own code.

Run in a checkout that has the reference tree (it needs oracle/_ref, built by
oracle/build_ref.py from the reference's computeCPU.cpp and readInput.cpp):

    python tests/golden/make_golden.py

Fixtures written (all small):
  kat_bhsparse.npz    the 4x6 * 6x4 known-answer operands of bhsparse/main.cu:194-234
                      and their product as computed by the reference's compute_CPU
  cage4.csr           the reference's read_CSR conversion of bhsparse/cage4.mtx
                      (byte-exact .csr cache), plus cage4_ref.npz: cage4*cage4
                      through compute_CPU (raw slot layout)
  *.mtx / edges.dat   synthetic Matrix Market / edge-list inputs written for
                      these tests, and <name>.ref.csr: the reference's
                      conversion of each
  lap16_ref.npz       16x16-grid Laplacian squared through compute_CPU
  rmat9_ref.npz       R-MAT scale 9, edge factor 4, integer values 1..9, squared
  quirk_ref.npz       a row whose running sum returns to zero: the reference's
                      value-based structure test emits a duplicate column
  lap256_ref.json     checksums of the reference's output for the 256x256-grid
                      Laplacian squared (the benchmark's CPU-runnable workload)
  rmat18_int_ref.json the reference's output structure for R-MAT scale 18,
                      edge factor 8, seed 0 with integer values 1..9 (the
                      quirk-inert form of that workload): sha256 of the
                      canonical row_ptr (int64) and col_idx (int32)
  rmat21_int_ref.json the same for R-MAT scale 21, edge factor 16, seed 0 in
                      blocks of 512 rows (2.65e10 entries, never held whole):
                      sha256 of the per-row entry counts (int64) and column
                      hashes (uint64, sum of SplitMix64's mix64 of each column)

    python tests/golden/make_golden.py [--only small|rmat18|rmat21]

The R-MAT records take the reference's compute_CPU about 20 s (scale 18) and
25 min (scale 21) on 8 cores; each is also checked against the oracle's own
structure before it is written.
"""
import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from dbd_gb300 import generators as gen  # noqa: E402
from dbd_gb300.csr import CSR  # noqa: E402

from oracle.build_ref import reference_root  # noqa: E402

CAGE4 = os.path.join(reference_root() or ".", "bhsparse", "cage4.mtx")
MTX_FIXTURES = ["mtx_general.mtx", "mtx_symmetric.mtx", "mtx_pattern.mtx", "edges.dat"]


def kat_operands():
    # bhsparse/main.cu:188-234 (test_small_spgemm)
    A = CSR(4, 6, np.array([0, 1, 4, 5, 6], np.int32), np.array([0, 1, 2, 3, 3, 1], np.int32),
            np.array([(i + 1) * 10 for i in range(6)], np.float64))
    B = CSR(6, 4, np.array([0, 1, 3, 5, 5, 5, 7], np.int32), np.array([0, 1, 3, 0, 1, 1, 3], np.int32),
            np.array([i + 1 for i in range(7)], np.float64))
    return A, B


def quirk_operands():
    A = CSR(1, 3, np.array([0, 3], np.int32), np.array([0, 1, 2], np.int32), np.array([1.0, -1.0, 1.0]))
    B = CSR(3, 2, np.array([0, 1, 2, 3], np.int32), np.array([0, 0, 0], np.int32), np.array([1.0, 1.0, 1.0]))
    return A, B


def save_ref(name, A, B):
    off, cnt, idx, val = oracle.ref_cpu_spgemm(A, B)
    np.savez_compressed(os.path.join(HERE, name), a_ptr=A.row_ptr, a_idx=A.col_idx, a_val=A.val,
                        a_shape=np.array([A.n_rows, A.n_cols]), b_ptr=B.row_ptr, b_idx=B.col_idx, b_val=B.val,
                        b_shape=np.array([B.n_rows, B.n_cols]), off=off, cnt=cnt,
                        idx=idx[:int(off[-1])] if off[-1] else idx[:0], val=val[:int(off[-1])] if off[-1] else val[:0])


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def rmat_structure(scale, edge_factor, rows_per_block, name):
    """Streams the reference's compute_CPU output of A*A, A = rmat(scale,
    edge_factor, seed 0, integer values), block by block and records hashes of
    its canonical structure; asserts it equals the oracle's."""
    import time
    A = gen.rmat(scale, edge_factor, seed=0, int_values=True)
    m = A.n_rows
    cnt = np.zeros(m, np.int64)
    chash = np.zeros(m, np.uint64)
    h_idx = hashlib.sha256()
    state = {"dups": 0}

    def on_block(r0, r1, c, hh, idx, dups):
        cnt[r0:r1] = c
        chash[r0:r1] = hh
        state["dups"] += int(dups)
        h_idx.update(np.ascontiguousarray(idx, np.int32).tobytes())

    t0 = time.time()
    oracle.ref_cpu_blocks(A, rows_per_block=rows_per_block, on_block=on_block)
    t_ref = time.time() - t0
    ocnt, ohash = oracle.row_col_digest(A)
    assert np.array_equal(ocnt, cnt), "reference row counts differ from the oracle's"
    assert np.array_equal(ohash, chash), "reference column hashes differ from the oracle's"
    row_ptr = np.zeros(m + 1, np.int64)
    np.cumsum(cnt, out=row_ptr[1:])
    rec = {"workload": f"rmat({scale}, {edge_factor}, seed=0, int_values=True) squared through the reference's "
                       f"compute_CPU in blocks of {rows_per_block} rows, each row's columns sorted",
           "n_rows": int(m), "nnz_a": int(A.nnz), "products": int(oracle.row_products(A, A)[1]),
           "nnz_c": int(row_ptr[-1]), "duplicates": state["dups"],
           "sha256_row_ptr_i64": digest(row_ptr),
           "sha256_col_idx_i32": h_idx.hexdigest(),
           "sha256_row_count_i64": digest(cnt),
           "sha256_row_col_hash_u64": digest(chash),
           "first_rows": {"count": cnt[:8].tolist(), "col_hash": [str(x) for x in chash[:8]]},
           "reference_seconds": round(t_ref, 1)}
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec, indent=1))


def main():
    if oracle.reference() is None:
        oracle.build()
    if oracle.reference() is None:
        sys.exit("the reference's CPU code is not built (reference tree absent)")
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "rmat18":
        return rmat_structure(18, 8, 4096, "rmat18_int_ref.json")
    if only == "rmat21":
        return rmat_structure(21, 16, 512, "rmat21_int_ref.json")
    A, B = kat_operands()
    save_ref("kat_bhsparse.npz", A, B)
    A, B = quirk_operands()
    save_ref("quirk_ref.npz", A, B)

    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "cage4.mtx")
        shutil.copy(CAGE4, p)
        nr, nc, ptr, idx, val = oracle.ref_read_csr(p)
        shutil.copy(p + ".csr", os.path.join(HERE, "cage4.csr"))
        # The reference's conversion of the synthetic Matrix Market fixtures.
        for name in MTX_FIXTURES:
            q = os.path.join(tmp, name)
            shutil.copy(os.path.join(HERE, name), q)
            oracle.ref_read_csr(q)
            shutil.copy(q + ".csr", os.path.join(HERE, name + ".ref.csr"))
    M = CSR(nr, nc, ptr, idx, val.astype(np.float64))
    save_ref("cage4_ref.npz", M, M)

    L = gen.laplacian_2d(16)
    save_ref("lap16_ref.npz", L, L)
    R = gen.rmat(9, 4, seed=1, int_values=True)
    save_ref("rmat9_ref.npz", R, R)

    L = gen.laplacian_2d(256)
    off, cnt, idx, val = oracle.ref_cpu_spgemm(L, L)
    Cp, Ci, Cv, dups = oracle.canonicalise(off, cnt, idx, val)
    rec = {"workload": "laplacian_2d(256) squared through the reference's compute_CPU",
           "n_rows": int(L.n_rows), "products": int(off[-1]), "nnz_c": int(Cp[-1]), "duplicates": int(dups),
           "sha256_row_ptr_col_idx": digest(Cp.astype(np.int64), Ci.astype(np.int32)),
           "sha256_values_f32": digest(Cv.astype(np.float32)),
           "value_sum": float(Cv.sum())}
    with open(os.path.join(HERE, "lap256_ref.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec, indent=1))


if __name__ == "__main__":
    main()
