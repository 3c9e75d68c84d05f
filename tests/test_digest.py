"""The per-row digest of C (dbd_set_digest / dbd_digest_copy) on small cases.

The digest is what checks out-of-core products at full size, so it is checked
itself here against the whole product: every row's count, column hash, value
hash and sums recomputed with numpy from C, in every scope, with the output
forced through several device chunks and a recycled host ring.
"""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen

pytestmark = pytest.mark.gpu
GOLD = 0x9E3779B97F4A7C15


def numpy_digest(orc, Cp, Ci, Cv):
    m = Cp.size - 1
    rows = np.repeat(np.arange(m), np.diff(Cp))
    col = np.zeros(m, np.uint64)
    np.add.at(col, rows, orc.mix64(Ci.astype(np.uint32)))
    with np.errstate(over="ignore"):
        key = Cv.view(np.uint64) + np.uint64(GOLD) * (Ci.astype(np.uint64) + np.uint64(1))
    val = np.zeros(m, np.uint64)
    np.add.at(val, rows, orc.mix64(key))
    s = np.zeros(m)
    np.add.at(s, rows, Cv)
    ws = np.zeros(m)
    np.add.at(ws, rows, Cv * orc.col_weights(Ci))
    sabs = np.zeros(m)
    np.add.at(sabs, rows, np.abs(Cv))
    return {"count": np.diff(Cp), "col_hash": col, "val_hash": val, "sum": s, "wsum": ws, "abs": sabs}


def assert_digest_of(d, ref):
    assert d["bad_rows"] == 0
    assert np.array_equal(d["count"], ref["count"])
    assert np.array_equal(d["col_hash"], ref["col_hash"])
    assert np.array_equal(d["val_hash"], ref["val_hash"])
    # numpy's sequential sums err by up to (entries) units of the last place
    # of sum|c|; the digest's compensated sums by about one.
    tol = (ref["count"] + 4) * 2.3e-16 * ref["abs"] + 1e-300
    assert np.all(np.abs(d["sum"] - ref["sum"]) <= tol)
    assert np.all(np.abs(d["wsum"] - ref["wsum"]) <= 2 * tol)


def test_digest_matches_product_in_every_scope(orc, tmp_path):
    A = gen.rmat(14, 8, seed=5)
    gib = 1024 ** 3
    with dbd.Context(cpu_gib=8, gpu_gib=8, rows_per_block=512) as c:
        c.set_digest(device=True, host=True)
        res = c.spgemm(A, scope="kernel")
        C = res.C
        ref = numpy_digest(orc, C.row_ptr, C.col_idx, C.val)
        assert_digest_of(c.digest(A.n_rows, "device"), ref)
        with pytest.raises(dbd.DBDError):
            c.digest(A.n_rows, "host")  # the kernel scope copies nothing to the host
    out_bytes = 12 * C.nnz
    # Budgets that force several chunks, two device slots and a host ring.
    with dbd.Context(cpu_gib=0.6 * out_bytes / gib, gpu_gib=(8 << 20) / gib + 0.3 * out_bytes / gib,
                     rows_per_block=512) as c:
        c.set_digest(device=True, host=True)
        for scope in ("kernel", "d2h", "io"):
            st = c.spgemm(A, scope=scope, out_dir=str(tmp_path), fetch=False).stats
            assert st["n_chunks"] >= 3, st["n_chunks"]
            dev = c.digest(A.n_rows, "device")
            assert np.array_equal(dev["count"], ref["count"]) and np.array_equal(dev["col_hash"], ref["col_hash"])
            assert dev["bad_rows"] == 0
            if scope != "kernel":
                host = c.digest(A.n_rows, "host")
                for k in ("count", "col_hash", "val_hash"):
                    assert np.array_equal(host[k], dev[k]), k
                assert host["bad_rows"] == 0
        # The io scope's files hold what the digests summarise.
        ptr = np.fromfile(tmp_path / "Ptr.output", np.int64)
        idx = np.fromfile(tmp_path / "Idx.output", np.int32)
        val = np.fromfile(tmp_path / "Val.output", np.float64)
        assert np.array_equal(numpy_digest(orc, ptr, idx, val)["val_hash"], host["val_hash"])


def test_digest_sums_against_oracle_row_sums(orc):
    A = gen.uniform_rows(1 << 13, 12, seed=9)  # N(0,1) values: rows with cancellation
    B = gen.uniform_rows(1 << 13, 12, seed=10)
    with dbd.Context(cpu_gib=4, gpu_gib=4) as c:
        c.set_digest(device=True)
        c.spgemm(A, B, scope="kernel", fetch=False)
        d = c.digest(A.n_rows)
    cnt, h = orc.row_col_digest(A, B)
    assert np.array_equal(d["count"], cnt) and np.array_equal(d["col_hash"], h)
    s, sa = orc.row_sums(A, B)
    w, wa = orc.row_sums(A, B, weighted=True)
    assert np.all(np.abs(d["sum"] - s) <= 2e-12 * sa)
    assert np.all(np.abs(d["wsum"] - w) <= 2e-12 * wa)


def test_digest_off_by_default_and_flags_checked():
    A = gen.laplacian_2d(16)
    with dbd.Context(cpu_gib=1, gpu_gib=1) as c:
        c.spgemm(A, scope="kernel", fetch=False)
        with pytest.raises(dbd.DBDError):
            c.digest(A.n_rows)
        assert c._lib.dbd_set_digest(c.handle, 4) == -1  # DBD_ERR_INVALID: unknown flag
