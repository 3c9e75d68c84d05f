"""ctypes mirror of include/dbd.h and the loader of libdbd.so.

The library is built in-tree (dbd_gb300/_lib/libdbd.so, see dbd_gb300/build.py);
loading fails loudly when it is missing -- there is no fallback path.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdbd.so")

DBD_OK = 0
ERR_NAMES = {
    -1: "DBD_ERR_INVALID", -2: "DBD_ERR_OOM_DEVICE", -3: "DBD_ERR_OOM_HOST", -4: "DBD_ERR_BUDGET",
    -5: "DBD_ERR_IO", -6: "DBD_ERR_CUDA", -7: "DBD_ERR_TIMEOUT", -8: "DBD_ERR_OVERFLOW",
    -9: "DBD_ERR_DEVICE_CHECK", -10: "DBD_ERR_NO_DEVICE",
}
SCOPES = {"kernel": 0, "d2h": 1, "io": 2}
NUM_BINS = 12


class CsrView(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("val", C.c_void_p),
                ("val_fp32", C.c_int32), ("on_device", C.c_int32)]


class CsrOut(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("val", C.c_void_p),
                ("on_device", C.c_int32), ("owner", C.c_int32), ("val_fp32", C.c_int32)]


class CsrHost(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("val", C.c_void_p),
                ("src_fp32", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("host_gib", C.c_double), ("gpu_gib", C.c_double), ("rows_per_block", C.c_int64),
                ("device", C.c_int32), ("out_val_fp32", C.c_int32), ("out_ptr32", C.c_int32),
                ("verbose", C.c_int32), ("time_kernels", C.c_int32), ("io_rotate_gib", C.c_double),
                ("io_buffered", C.c_int32), ("io_resume", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("warp_span_words", C.c_int32), ("warp_max_nnz", C.c_int32), ("sym_warp_max_products", C.c_int32),
                ("rank_words_max", C.c_int32), ("rank_shared_max_nnz", C.c_int32),
                ("sym_hash_span_words", C.c_int32), ("dense_warp_span_words", C.c_int32),
                ("mid_span_words", C.c_int32), ("dense_method", C.c_int32)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("t_preprocess", C.c_double), ("t_compute_gpu", C.c_double), ("t_write_file", C.c_double),
                ("t_kernel_exec", C.c_double), ("t_total", C.c_double), ("t_d2h", C.c_double),
                ("t_fsync", C.c_double), ("t_device_ms", C.c_double), ("t_numeric_ms", C.c_double),
                ("products", C.c_int64), ("nnz_c", C.c_int64), ("n_blocks", C.c_int64),
                ("max_block_products", C.c_int64), ("criteria", C.c_int32), ("n_chunks", C.c_int32),
                ("blocks_per_category", C.c_int64 * 3), ("rows_per_bin", C.c_int64 * NUM_BINS),
                ("sym_rows_per_bin", C.c_int64 * NUM_BINS), ("bytes_d2h", C.c_int64),
                ("bytes_written", C.c_int64), ("gpu_launches", C.c_int64), ("t_analysis_ms", C.c_double),
                ("t_sym_bin_ms", C.c_double * NUM_BINS), ("t_scan_ms", C.c_double),
                ("t_num_bin_ms", C.c_double * NUM_BINS), ("io_direct", C.c_int64), ("resumed_from_row", C.c_int64),
                ("heavy_rows", C.c_int64), ("t_chunks_ms", C.c_double), ("t_copy_ms", C.c_double)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


# Every function the header declares: name -> (restype, argtypes).
SIGNATURES = {
    "dbd_config_default": (None, [C.POINTER(Config)]),
    "dbd_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "dbd_destroy": (None, [C.c_void_p]),
    "dbd_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dbd_error_string": (C.c_char_p, [C.c_int]),
    "dbd_last_error": (C.c_char_p, [C.c_void_p]),
    "dbd_read_csr": (C.c_int, [C.c_char_p, C.POINTER(CsrHost)]),
    "dbd_read_csr_gpu": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(CsrHost)]),
    "dbd_csr_host_free": (None, [C.POINTER(CsrHost)]),
    "dbd_write_csr": (C.c_int, [C.c_char_p, C.POINTER(CsrView), C.c_int]),
    "dbd_load_a": (C.c_int, [C.c_void_p, C.POINTER(CsrView)]),
    "dbd_load_b": (C.c_int, [C.c_void_p, C.POINTER(CsrView)]),
    "dbd_divide_blocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "dbd_block_info": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "dbd_distribute_workload": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "dbd_result": (C.c_int, [C.c_void_p, C.POINTER(CsrOut)]),
    "dbd_result_copy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "dbd_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "dbd_spgemm": (C.c_int, [C.c_void_p, C.POINTER(CsrView), C.POINTER(CsrView), C.c_int, C.c_char_p,
                             C.POINTER(CsrOut), C.POINTER(Stats)]),
    "dbd_spgemm_files": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.c_char_p,
                                   C.POINTER(Stats)]),
    "dbd_csr_free": (None, [C.POINTER(CsrOut)]),
    "dbd_spgemm_noalloc": (C.c_int, [C.POINTER(CsrView), C.POINTER(CsrView), C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_int64, C.POINTER(C.c_int64), C.c_void_p]),
    "dbd_spgemm_adjoint": (C.c_int, [C.c_void_p, C.POINTER(CsrView), C.POINTER(CsrView), C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_int]),
    "dbd_batch_plan": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64]),
    "dbd_batch_enqueue": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dbd_batch_result": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(CsrOut)]),
    "dbd_spgemm_batched": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(CsrView), C.POINTER(CsrView), C.c_int,
                                     C.c_void_p, C.c_void_p, C.POINTER(CsrOut), C.POINTER(Stats)]),
    "dbd_update_values": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int]),
    "dbd_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "dbd_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "dbd_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_double)]),
    "dbd_set_digest": (C.c_int, [C.c_void_p, C.c_int]),
    "dbd_writer_open": (C.c_int, [C.c_char_p, C.c_int64, C.c_int64, C.c_uint64, C.c_int, C.c_double,
                                  C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "dbd_writer_append": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64]),
    "dbd_writer_finish": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "dbd_writer_is_direct": (C.c_int, [C.c_void_p]),
    "dbd_writer_error": (C.c_char_p, [C.c_void_p]),
    "dbd_writer_close": (None, [C.c_void_p]),
    "dbd_digest_copy": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.POINTER(C.c_int64)]),
}

DIGEST_DEVICE = 1
DIGEST_HOST = 2
WRITER_BUFFERED = 1
WRITER_VAL_FP32 = 2
WRITER_PTR32 = 4
WRITER_RESUME = 8

_lib = None


def load():
    """Loads libdbd.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"libdbd.so not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
