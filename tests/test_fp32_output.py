"""C's values in the reference's float32 layout (out_val_fp32) in the copying
scopes: rounded once on the device after the FP64 accumulation, 8 bytes per
entry over the link, float32 in host memory and in Val.output, and a digest
(device and host) of the values as they left the device."""
import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from test_digest import assert_digest_of, numpy_digest

pytestmark = pytest.mark.gpu
GIB = 1024 ** 3


def fp64_product(A):
    with dbd.Context(cpu_gib=8, gpu_gib=8, rows_per_block=512) as c:
        return c.spgemm(A, scope="kernel").C


def assert_rounded(v32, v64):
    """v32 is v64 rounded to float32 (the FP64 sums themselves may differ in
    their last bits between runs: reductions in place add in any order)."""
    assert v32.dtype == np.float32
    half_ulp = np.spacing(np.abs(v64).astype(np.float32)).astype(np.float64) / 2
    assert np.all(np.abs(v32.astype(np.float64) - v64) <= half_ulp + 1e-12 * np.abs(v64))


def test_d2h_float32_values_chunked():
    A = gen.rmat(14, 8, seed=5)
    C64 = fp64_product(A)
    nnz, m = C64.nnz, A.n_rows
    # Budgets that force several chunks through two device slots; C lands whole in host memory.
    with dbd.Context(cpu_gib=8, gpu_gib=(8 << 20) / GIB + 0.3 * 16 * nnz / GIB, rows_per_block=512,
                     out_val_fp32=True) as c:
        res = c.spgemm(A, scope="d2h")
    st = res.stats
    assert st["n_chunks"] >= 3, st["n_chunks"]
    assert st["bytes_d2h"] == 8 * nnz + 8 * (m + 1)
    C = res.C
    assert np.array_equal(C.row_ptr, C64.row_ptr) and np.array_equal(C.col_idx, C64.col_idx)
    assert_rounded(C.val, C64.val)


def test_float32_digests_and_files(orc, tmp_path):
    A = gen.rmat(14, 8, seed=6)
    C64 = fp64_product(A)
    nnz = C64.nnz
    # A host ring smaller than C: the consumer thread takes the host digest and the files.
    with dbd.Context(cpu_gib=0.6 * 8 * nnz / GIB, gpu_gib=(8 << 20) / GIB + 0.3 * 16 * nnz / GIB,
                     rows_per_block=512, out_val_fp32=True, out_ptr32=0) as c:
        c.set_digest(device=True, host=True)
        st = c.spgemm(A, scope="io", out_dir=str(tmp_path), fetch=False).stats
        assert st["n_chunks"] >= 3
        dev = c.digest(A.n_rows, "device")
        host = c.digest(A.n_rows, "host")
    idx = np.fromfile(tmp_path / "Idx.output", np.int32)
    val = np.fromfile(tmp_path / "Val.output", np.float32)
    ptr = np.fromfile(tmp_path / "Ptr.output", np.int64)
    assert np.array_equal(ptr, C64.row_ptr) and np.array_equal(idx, C64.col_idx)
    assert_rounded(val, C64.val)
    # Both digests describe the float32 values that left the device, and agree bit for bit.
    ref = numpy_digest(orc, ptr, idx, val.astype(np.float64))
    assert_digest_of(dev, ref)
    for k in ("count", "col_hash", "val_hash", "sum", "wsum"):
        assert np.array_equal(host[k], dev[k]), k
    assert host["bad_rows"] == 0


def test_kernel_scope_stays_fp64():
    A = gen.laplacian_2d(64)
    with dbd.Context(cpu_gib=1, gpu_gib=1, out_val_fp32=True) as c:
        C = c.spgemm(A, scope="kernel").C
    assert C.val.dtype == np.float64
