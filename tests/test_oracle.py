"""The oracle pinned against the reference's own code and known answers (CPU only)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR

GOLDEN_REF = ["kat_bhsparse.npz", "quirk_ref.npz", "cage4_ref.npz", "lap16_ref.npz", "rmat9_ref.npz"]
QUIRK_INERT = ["kat_bhsparse.npz", "cage4_ref.npz", "lap16_ref.npz", "rmat9_ref.npz"]


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name))
    A = CSR(*d["a_shape"], d["a_ptr"], d["a_idx"], d["a_val"])
    B = CSR(*d["b_shape"], d["b_ptr"], d["b_idx"], d["b_val"])
    return A, B, d


def test_kat_bhsparse_known_answer(orc):
    # bhsparse/main.cu:182-279: 4x6 * 6x4, values (i+1)*10 and i+1.
    A, B, _ = load_golden("kat_bhsparse.npz")
    Cp, Ci, Cv = orc.spgemm(A, B)
    assert Cp.tolist() == [0, 1, 4, 4, 6]
    assert Ci.tolist() == [0, 0, 1, 3, 1, 3]
    assert Cv.tolist() == [10.0, 120.0, 190.0, 60.0, 120.0, 180.0]


@pytest.mark.parametrize("name", GOLDEN_REF)
def test_ref_restatement_bit_exact_vs_reference_output(orc, name):
    """orc_ref_cpu_rows reproduces the reference's compute_CPU bit for bit
    (counts, first-touch column order, FP32 values, duplicates)."""
    A, B, d = load_golden(name)
    off, cnt, idx, val = orc.ref_cpu(A, B, threads=3)
    assert np.array_equal(off, d["off"])
    assert np.array_equal(cnt, d["cnt"])
    m = A.n_rows
    for r in range(m):
        s = off[r]
        assert np.array_equal(idx[s:s + cnt[r]], d["idx"][s:s + cnt[r]]), r
        assert np.array_equal(val[s:s + cnt[r]].view(np.uint32), d["val"][s:s + cnt[r]].view(np.uint32)), r


@pytest.mark.parametrize("name", QUIRK_INERT)
def test_oracle_structure_equals_canonical_reference(orc, name):
    """On inputs where the reference's value-based structure test cannot fire,
    its canonicalised output (rows sorted) has exactly the oracle's structure,
    and its FP32 values agree to FP32 rounding."""
    A, B, d = load_golden(name)
    rp, cp, ci, cv, dups = d["off"], None, None, None, None
    Cp_r, Ci_r, Cv_r, dups = orc.canonicalise(d["off"], d["cnt"], d["idx"], d["val"])
    assert dups == 0
    Cp, Ci, Cv = orc.spgemm(A, B)
    assert np.array_equal(Cp, Cp_r)
    assert np.array_equal(Ci, Ci_r)
    assert np.allclose(Cv, Cv_r, rtol=2e-6, atol=0)


def test_quirk_duplicate_is_a_documented_deviation(orc):
    """Row sum 1 - 1 + 1 on one column: the reference re-lists the column when
    its running sum returns inside (-1e-4, 1e-4) (computeCPU.cpp:48), giving
    (col 0: 1, col 0: 0); the index-determined oracle gives one entry, 1."""
    A, B, d = load_golden("quirk_ref.npz")
    assert d["cnt"].tolist() == [2]
    assert d["idx"][:2].tolist() == [0, 0] and d["val"][:2].tolist() == [1.0, 0.0]
    Cp, Ci, Cv = orc.spgemm(A, B)
    assert Cp.tolist() == [0, 1] and Ci.tolist() == [0] and Cv.tolist() == [1.0]


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_laplacian256_matches_reference_checksums(orc):
    """The CPU-runnable workload (256x256-grid Laplacian squared): structure
    and FP32-rounded values equal the reference's output, by checksum."""
    with open(os.path.join(GOLDEN, "lap256_ref.json")) as f:
        ref = json.load(f)
    L = gen.laplacian_2d(256)
    Cp, Ci, Cv = orc.spgemm(L)
    assert Cp[-1] == ref["nnz_c"] == 846852
    assert ref["products"] == 1629192
    assert _digest(Cp.astype(np.int64), Ci.astype(np.int32)) == ref["sha256_row_ptr_col_idx"]
    assert _digest(Cv.astype(np.float32)) == ref["sha256_values_f32"]


def test_oracle_vs_scipy_random(orc):
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(7)
    for m, k, n, dens in [(50, 40, 60, 0.1), (1, 1, 1, 1.0), (200, 30, 5, 0.2), (64, 64, 64, 0.02)]:
        A = sp.random(m, k, dens, format="csr", random_state=rng, data_rvs=lambda s: rng.uniform(0.5, 2, s))
        B = sp.random(k, n, dens, format="csr", random_state=rng, data_rvs=lambda s: rng.uniform(0.5, 2, s))
        Cs = (A @ B).tocsr()
        Cs.sort_indices()
        Cp, Ci, Cv = orc.spgemm(CSR.from_scipy(A), CSR.from_scipy(B))
        assert np.array_equal(Cp, Cs.indptr)
        assert np.array_equal(Ci, Cs.indices)
        assert np.allclose(Cv, Cs.data, rtol=1e-14)


def test_oracle_keeps_structural_zeros(orc):
    # 1*1 + 1*(-1) = 0 stays an entry (structure by index only).
    A = CSR(1, 2, np.array([0, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    B = CSR(2, 1, np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32), np.array([1.0, -1.0]))
    Cp, Ci, Cv = orc.spgemm(A, B)
    assert Cp.tolist() == [0, 1] and Ci.tolist() == [0] and Cv.tolist() == [0.0]


def test_segmenter_and_categoriser_match_reference(orc):
    """divide_Blocks (main.cpp:259-310) and calculate_Criteria
    (distributeWorkload.cpp:249-264) of the reference against the oracle."""
    if orc.reference() is None:
        pytest.skip("reference tree absent")
    rpb = orc.reference().ref_rows_in_block()
    for A in (gen.laplacian_2d(64), gen.rmat(14, 8, seed=2), gen.laplacian_2d(256)):
        info_r, bptr_r, tot_r = orc.ref_divide(A)
        rp, tot = orc.row_products(A, A)
        upp = orc.exclusive_scan(rp)
        bptr, info, mx = orc.divide_blocks(A.n_rows, upp, rpb)
        assert tot == tot_r
        assert np.array_equal(info, info_r.astype(np.int64))
        assert np.array_equal(bptr, bptr_r.astype(np.int64))
        assert mx == info_r.max()
        assert orc.criteria(info, rpb, tot) == orc.ref_criteria(info_r, tot_r)


def test_threads_per_row_rule(orc):
    # computeGPU.cu:9-13
    assert [orc.threads_per_row(p) for p in (0, 128, 129, 512, 513, 10**9)] == [64, 64, 256, 256, 1024, 1024]
    # distributeWorkload.cpp:266-270
    assert orc.analyze_block(100, 101) == 0
    assert orc.analyze_block(100, 64) == 1
    assert orc.analyze_block(100, 65) == 2


def test_adjoint_oracle_matches_dense(orc):
    rng = np.random.default_rng(3)
    A = gen.uniform_rows(30, 4, seed=1, n_cols=20)
    B = gen.uniform_rows(20, 5, seed=2, n_cols=25)
    Cp, Ci, _ = orc.spgemm(A, B)
    G = rng.standard_normal(Ci.size)
    dA, dB = orc.adjoint(A, B, Cp, Ci, G)
    Gd = np.zeros((30, 25))
    for r in range(30):
        Gd[r, Ci[Cp[r]:Cp[r + 1]]] = G[Cp[r]:Cp[r + 1]]
    Ad, Bd = A.to_scipy().toarray(), B.to_scipy().toarray()
    dAd, dBd = Gd @ Bd.T, Ad.T @ Gd
    for r in range(30):
        for e in range(A.row_ptr[r], A.row_ptr[r + 1]):
            assert np.isclose(dA[e], dAd[r, A.col_idx[e]], rtol=1e-12, atol=1e-13)
    for j in range(20):
        for f in range(B.row_ptr[j], B.row_ptr[j + 1]):
            assert np.isclose(dB[f], dBd[j, B.col_idx[f]], rtol=1e-12, atol=1e-13)


def test_rmat_generator_matches_published_statistics():
    """The R-MAT generator reproduces the statistics quoted for the scale-18
    workload: 2,016,992 entries, 139,756 empty rows, longest row 9,628."""
    A = gen.rmat(18, 8, seed=0)
    lens = np.diff(A.row_ptr)
    assert A.nnz == 2016992
    assert int((lens == 0).sum()) == 139756
    assert int(lens.max()) == 9628
    assert all(np.all(np.diff(A.col_idx[A.row_ptr[r]:A.row_ptr[r + 1]]) > 0) for r in range(0, A.n_rows, 997))


def test_oracle_structure_equals_reference_output_rmat18(orc):
    """The oracle's index-determined structure of the full R-MAT 2^18 product
    equals the reference's own compute_CPU output (hashed by
    tests/golden/make_golden.py on the integer-valued form of the workload)."""
    with open(os.path.join(GOLDEN, "rmat18_int_ref.json")) as f:
        ref = json.load(f)
    A = gen.rmat(18, 8, seed=0)
    cnt, h = orc.row_col_digest(A)
    assert int(cnt.sum()) == ref["nnz_c"]
    assert hashlib.sha256(cnt.astype(np.int64).tobytes()).hexdigest() == ref["sha256_row_count_i64"]
    assert hashlib.sha256(h.tobytes()).hexdigest() == ref["sha256_row_col_hash_u64"]
    row_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    assert hashlib.sha256(row_ptr.tobytes()).hexdigest() == ref["sha256_row_ptr_i64"]


def test_digest_oracle_against_full_product(orc):
    """row_col_digest and row_sums (the checks of out-of-core products) agree
    with the full oracle product they summarise."""
    B = gen.rmat(12, 6, seed=2)
    A = gen.uniform_rows(3000, 9, seed=4, n_cols=B.n_rows)
    Cp, Ci, Cv = orc.spgemm(A, B)
    rows = np.repeat(np.arange(A.n_rows), np.diff(Cp))
    cnt, h = orc.row_col_digest(A, B)
    hh = np.zeros(A.n_rows, np.uint64)
    np.add.at(hh, rows, orc.mix64(Ci))
    assert np.array_equal(cnt, np.diff(Cp)) and np.array_equal(h, hh)
    for weighted in (False, True):
        s, sa = orc.row_sums(A, B, weighted=weighted)
        w = orc.col_weights(Ci) if weighted else 1.0
        ref = np.zeros(A.n_rows)
        np.add.at(ref, rows, Cv * w)
        assert np.all(np.abs(s - ref) <= 1e-13 * sa + 1e-300)
    assert orc.lib().orc_col_weight(77) == orc.col_weights(np.array([77]))[0]


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libdbdref.so")), reason="reference CPU code not built")
def test_reference_block_stream_matches_oracle(orc):
    """ref_cpu_blocks (the reference's compute_CPU, block by block) gives the
    oracle's per-row counts and column hashes on a quirk-inert R-MAT."""
    A = gen.rmat(12, 8, seed=3, int_values=True)
    cnt, h = orc.row_col_digest(A)
    got_c = np.zeros(A.n_rows, np.int64)
    got_h = np.zeros(A.n_rows, np.uint64)
    dups = []

    def on_block(r0, r1, c, hh, idx, d):
        got_c[r0:r1] = c
        got_h[r0:r1] = hh
        dups.append(d)
        assert idx.size == int(c.sum())
    orc.ref_cpu_blocks(A, rows_per_block=512, on_block=on_block)
    assert np.array_equal(got_c, cnt) and np.array_equal(got_h, h) and sum(dups) == 0
