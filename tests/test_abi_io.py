"""C ABI surface and CSR file formats (CPU only: no compute call needs a GPU here)."""
import ctypes as C
import os
import re
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
import dbd_gb300 as dbd
from dbd_gb300 import _ffi
from dbd_gb300.csr import CSR

HEADER = os.path.join(ROOT, "include", "dbd.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dbd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _ffi.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes mirror covers the whole header
    assert set(names) == set(_ffi.SIGNATURES)


def test_error_strings():
    lib = _ffi.load()
    for code, name in _ffi.ERR_NAMES.items():
        assert lib.dbd_error_string(code)
    assert lib.dbd_error_string(0) == b"ok"


def test_create_without_device_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(dbd.DBDError) as ei:
        dbd.Context()
    assert ei.value.code == -10


def test_invalid_config_rejected():
    lib = _ffi.load()
    cfg = _ffi.Config()
    lib.dbd_config_default(C.byref(cfg))
    assert cfg.host_gib == 28.0 and cfg.gpu_gib == 22.0 and cfg.rows_per_block == 4096
    cfg.rows_per_block = 1000  # not a multiple of the 256-row tile
    h = C.c_void_p()
    assert lib.dbd_create(C.byref(cfg), C.byref(h)) == -1


@pytest.mark.parametrize("name", ["mtx_general.mtx", "mtx_symmetric.mtx", "mtx_pattern.mtx", "edges.dat"])
def test_mtx_conversion_byte_identical_to_reference(tmp_path, name):
    """dbd_read_csr converts .mtx/.dat exactly like the reference's make_CSR
    (readInput.cpp:48-176) and caches a byte-identical <path>.csr."""
    p = tmp_path / name
    shutil.copy(os.path.join(GOLDEN, name), p)
    M = dbd.read_CSR(str(p))
    got = open(str(p) + ".csr", "rb").read()
    want = open(os.path.join(GOLDEN, name + ".ref.csr"), "rb").read()
    assert got == want
    # the second read takes the cache
    M2 = dbd.read_CSR(str(p))
    assert np.array_equal(M.row_ptr, M2.row_ptr) and np.array_equal(M.val, M2.val)


def test_mtx_quirks(tmp_path):
    p = tmp_path / "mtx_general.mtx"
    shutil.copy(os.path.join(GOLDEN, "mtx_general.mtx"), p)
    M = dbd.read_CSR(str(p))
    # 1-based indices kept: header 5 x 6 -> 6 x 7, row 0 empty
    assert (M.n_rows, M.n_cols) == (6, 7)
    assert M.row_ptr[1] == 0
    p = tmp_path / "mtx_pattern.mtx"
    shutil.copy(os.path.join(GOLDEN, "mtx_pattern.mtx"), p)
    assert np.all(dbd.read_CSR(str(p)).val == 1.0)


def test_trailing_empty_rows_are_filled(tmp_path):
    """Rows after the last non-empty one get ptr = nnz (the reference leaves
    those ptr entries uninitialised, readInput.cpp:133-152)."""
    p = tmp_path / "t.dat"
    p.write_text("5 5 2\n0 1 1.0\n1 2 2.0\n")
    M = dbd.read_CSR(str(p))
    assert M.row_ptr.tolist() == [0, 1, 2, 2, 2, 2, 2]


def test_reference_csr_roundtrip(tmp_path):
    M = dbd.read_CSR(os.path.join(GOLDEN, "cage4"))
    assert (M.n_rows, M.n_cols, M.nnz) == (10, 10, 49)
    out = tmp_path / "copy.csr"
    dbd.write_CSR(str(out), M, fp64=False)
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, "cage4.csr"), "rb").read()


def test_dcsr_roundtrip_fp64(tmp_path):
    rng = np.random.default_rng(0)
    M = CSR(3, 4, np.array([0, 2, 2, 5], np.int32), np.array([0, 3, 1, 2, 3], np.int32), rng.standard_normal(5))
    dbd.write_CSR(str(tmp_path / "m.dcsr"), M, fp64=True)
    R = dbd.read_CSR(str(tmp_path / "m"))
    assert np.array_equal(R.row_ptr, M.row_ptr) and np.array_equal(R.col_idx, M.col_idx)
    assert np.array_equal(R.val, M.val)


def test_missing_file_raises(tmp_path):
    with pytest.raises(dbd.DBDError) as ei:
        dbd.read_CSR(str(tmp_path / "nope"))
    assert ei.value.code == -5


def test_cli_binaries_built():
    for name in ("SSpMM", "compute", "d2h", "debug"):
        assert os.access(os.path.join(ROOT, "dbd_gb300", "bin", name), os.X_OK), name
