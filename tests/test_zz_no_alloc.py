"""dbd_spgemm_noalloc: the multiply for callers that cannot allocate device memory.

Callers inside a caching allocator's hooks, frameworks that forbid allocation
outside their own pool, or loops that cannot afford cudaMalloc's implicit
synchronisation pass device-resident inputs and outputs; the entry point keeps
every temporary array in one file-scope device array of fixed size.  This file
checks, through the C ABI, that two calls in a row (different matrices, so the
second call starts from the first call's leftovers in that array) give the
same product as the regular entry point dbd_spgemm, within the tolerance of
the other parity tests, that an input too large for the array is refused, and
that after its first call on the device (the set-up) further calls whose rows
land in different kernel bins leave the device's free memory unchanged, and
that a call on a stream being captured is refused before it enqueues work.
It is collected last so that a failure here stops a -x run only after every
other test ran; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import dbd_gb300 as dbd
from dbd_gb300 import _ffi
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR

pytestmark = pytest.mark.gpu
TOL = 1e-12


def device_view(torch, A):
    t = (torch.from_numpy(np.ascontiguousarray(A.row_ptr, np.int32)).cuda(),
         torch.from_numpy(np.ascontiguousarray(A.col_idx, np.int32)).cuda(),
         torch.from_numpy(np.ascontiguousarray(A.val, np.float64)).cuda())
    v = _ffi.CsrView()
    v.n_rows, v.n_cols, v.nnz = A.n_rows, A.n_cols, A.nnz
    v.row_ptr, v.col_idx, v.val = t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr()
    v.val_fp32, v.on_device = 0, 1
    return v, t


def noalloc_multiply(torch, lib, A, capacity):
    va, keep = device_view(torch, A)
    cp = torch.empty(A.n_rows + 1, dtype=torch.int64, device="cuda")
    ci = torch.empty(max(capacity, 1), dtype=torch.int32, device="cuda")
    cv = torch.empty(max(capacity, 1), dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.dbd_spgemm_noalloc(C.byref(va), None, C.c_void_p(cp.data_ptr()), C.c_void_p(ci.data_ptr()),
                                C.c_void_p(cv.data_ptr()), capacity, C.byref(nnz), C.c_void_p(stream))
    torch.cuda.synchronize()
    n = nnz.value
    return rc, n, cp.cpu().numpy(), ci[:max(n, 0)].cpu().numpy(), cv[:max(n, 0)].cpu().numpy()


def wide_rows(n=300_000, heavy=40, k=3000, seed=3):
    """n x n with `heavy` rows of k columns spread over all n columns (their
    rows of A*A land in the dense-window bin) and two columns in every other
    row."""
    rng = np.random.default_rng(seed)
    rows = [np.repeat(np.arange(heavy), k), np.repeat(np.arange(heavy, n), 2)]
    cols = [np.concatenate([rng.choice(n, k, replace=False) for _ in range(heavy)]),
            rng.integers(0, n, 2 * (n - heavy))]
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    return gen._from_coo(n, n, rows, cols, rng.uniform(-1, 1, rows.size))


def test_noalloc_matches_regular_entry_point_twice(orc):
    torch = pytest.importorskip("torch")
    lib = _ffi.load()
    mats = [gen.rmat(14, 8, seed=5), gen.laplacian_2d(128), wide_rows()]
    with dbd.Context(cpu_gib=8, gpu_gib=8) as ctx:
        for A in mats:
            ref = ctx.spgemm(A, scope="kernel").C
            _, _, _, Ca = orc.spgemm(A, with_abs=True)
            rc, n, cp, ci, cv = noalloc_multiply(torch, lib, A, capacity=ref.nnz + 16)
            assert rc == 0, _ffi.ERR_NAMES.get(rc, rc)
            assert n == ref.nnz
            assert np.array_equal(cp, ref.row_ptr)
            assert np.array_equal(ci, ref.col_idx)
            assert np.all(np.abs(cv - ref.val) <= 2 * TOL * Ca)


def test_noalloc_reports_short_capacity_and_size_limit():
    torch = pytest.importorskip("torch")
    lib = _ffi.load()
    A = gen.laplacian_2d(32)
    rc, n, cp, _, _ = noalloc_multiply(torch, lib, A, capacity=10)
    assert rc == -4 and n > 10 and cp[-1] == n
    # ~1.6M empty rows need more scratch than the fixed array holds.
    m = 1_600_000
    big = CSR(m, m, np.zeros(m + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    vb, keep = device_view(torch, big)
    cp = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    nnz = C.c_int64(0)
    rc = lib.dbd_spgemm_noalloc(C.byref(vb), None, C.c_void_p(cp.data_ptr()), None, None, 0, C.byref(nnz),
                                None)
    assert rc == -4


def test_noalloc_allocates_nothing_after_setup():
    """After the first call (which sets the device up), calls on inputs that
    reach different kernels leave cudaMemGetInfo's free memory unchanged."""
    torch = pytest.importorskip("torch")
    lib = _ffi.load()
    mats = [gen.laplacian_2d(128), gen.rmat(13, 8, seed=9), wide_rows(n=200_000, heavy=20)]
    prepared = []
    for A in mats:
        va, keep = device_view(torch, A)
        cap = int(np.diff(A.row_ptr).astype(np.int64)[A.col_idx].sum()) + 16  # products bound nnz(C)
        out = (torch.empty(A.n_rows + 1, dtype=torch.int64, device="cuda"),
               torch.empty(cap, dtype=torch.int32, device="cuda"),
               torch.empty(cap, dtype=torch.float64, device="cuda"))
        prepared.append((va, keep, out, cap))
    stream = torch.cuda.current_stream().cuda_stream
    nnz = C.c_int64(0)

    def call(i):
        va, _, (cp, ci, cv), cap = prepared[i]
        rc = lib.dbd_spgemm_noalloc(C.byref(va), None, C.c_void_p(cp.data_ptr()), C.c_void_p(ci.data_ptr()),
                                    C.c_void_p(cv.data_ptr()), cap, C.byref(nnz), C.c_void_p(stream))
        torch.cuda.synchronize()
        return rc

    assert call(0) == 0  # set-up (and the first call)
    free0 = torch.cuda.mem_get_info()[0]
    for i in (1, 2, 0, 2):
        assert call(i) == 0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_refuses_a_capturing_stream():
    """The call reads sizes back to the host, so on a stream being captured it
    returns DBD_ERR_INVALID before enqueueing anything; the capture itself
    stays valid and the stream works afterwards."""
    torch = pytest.importorskip("torch")
    lib = _ffi.load()
    A = gen.laplacian_2d(32)
    rc, n, _, _, _ = noalloc_multiply(torch, lib, A, capacity=1 << 16)  # device set up
    assert rc == 0
    va, keep = device_view(torch, A)
    cp = torch.empty(A.n_rows + 1, dtype=torch.int64, device="cuda")
    ci = torch.empty(n, dtype=torch.int32, device="cuda")
    cv = torch.empty(n, dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = lib.dbd_spgemm_noalloc(C.byref(va), None, C.c_void_p(cp.data_ptr()), C.c_void_p(ci.data_ptr()),
                                    C.c_void_p(cv.data_ptr()), n, C.byref(nnz), C.c_void_p(s.cuda_stream))
        cp.zero_()  # the capture holds something
    assert rc == -1  # DBD_ERR_INVALID
    g.replay()
    torch.cuda.synchronize()
    rc2, n2, _, _, _ = noalloc_multiply(torch, lib, A, capacity=1 << 16)
    assert rc2 == 0 and n2 == n
