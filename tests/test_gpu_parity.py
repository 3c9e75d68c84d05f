"""GPU parity: libdbd through its C ABI against the oracle.

Structure (row_ptr, col_idx) must be bit-exact.  Values are FP64 and must
satisfy |c - oracle| <= 1e-12 * sum|a_ik * b_kj| per entry (the oracle computes
that scale; it equals 1e-12 relative wherever no cancellation occurs).  Rows
on the register path (<= 32 products) are summed in the oracle's order and
must match bit for bit.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
import dbd_gb300 as dbd
from dbd_gb300 import generators as gen
from dbd_gb300.csr import CSR

pytestmark = pytest.mark.gpu
TOL = 1e-12


def check(C, A, B, orc, exact=False):
    Cp, Ci, Cv, Ca = orc.spgemm(A, B, with_abs=True)
    assert C.n_rows == A.n_rows and C.n_cols == B.n_cols
    assert np.array_equal(C.row_ptr, Cp), "row_ptr"
    assert np.array_equal(C.col_idx, Ci), "col_idx"
    err = np.abs(C.val - Cv)
    if exact:
        assert np.array_equal(C.val.view(np.uint64), Cv.view(np.uint64))
    assert np.all(err <= TOL * Ca), f"max err {err.max()} scale {Ca[np.argmax(err)]}"
    rel = err / np.maximum(np.abs(Cv), 1e-300)
    return float(rel.max(initial=0.0)), float(rel.mean()) if rel.size else 0.0


def bins_used(st):
    return [i for i, v in enumerate(st["rows_per_bin"]) if v]


def test_laplacian256_kernel_scope_bit_exact(ctx, orc):
    L = gen.laplacian_2d(256)
    res = ctx.spgemm(L, scope="kernel")
    check(res.C, L, L, orc, exact=True)
    st = res.stats
    assert st["products"] == 1629192 and st["nnz_c"] == 846852
    assert st["n_blocks"] == 16
    assert st["gpu_launches"] > 0


@pytest.mark.parametrize("scope", ["d2h", "io"])
def test_laplacian256_other_scopes(ctx, orc, scope, tmp_path):
    L = gen.laplacian_2d(256)
    res = ctx.spgemm(L, scope=scope, out_dir=str(tmp_path))
    if scope == "d2h":
        check(res.C, L, L, orc, exact=True)
    else:
        Cp, Ci, Cv = orc.spgemm(L)
        ptr = np.fromfile(tmp_path / "Ptr.output", np.int64)
        idx = np.fromfile(tmp_path / "Idx.output", np.int32)
        val = np.fromfile(tmp_path / "Val.output", np.float64)
        assert np.array_equal(ptr, Cp) and np.array_equal(idx, Ci) and np.array_equal(val, Cv)
        assert res.stats["bytes_written"] == 8 * (L.n_rows + 1) + 12 * Cv.size


def test_io_reference_layout(orc, tmp_path):
    """DBD_OUT_FP32 / ptr32: the reference's int32 Ptr, int32 Idx, float32 Val."""
    L = gen.laplacian_2d(64)
    with dbd.Context(cpu_gib=4, gpu_gib=4, out_val_fp32=True, out_ptr32=True) as c:
        c.spgemm(L, scope="io", out_dir=str(tmp_path))
    Cp, Ci, Cv = orc.spgemm(L)
    assert np.array_equal(np.fromfile(tmp_path / "Ptr.output", np.int32), Cp.astype(np.int32))
    assert np.array_equal(np.fromfile(tmp_path / "Idx.output", np.int32), Ci)
    assert np.array_equal(np.fromfile(tmp_path / "Val.output", np.float32), Cv.astype(np.float32))


@pytest.mark.parametrize("name", ["kat_bhsparse.npz", "cage4_ref.npz", "lap16_ref.npz", "rmat9_ref.npz",
                                  "quirk_ref.npz"])
def test_golden_operands(ctx, orc, name):
    d = np.load(os.path.join(GOLDEN, name))
    A = CSR(*d["a_shape"], d["a_ptr"], d["a_idx"], d["a_val"])
    B = CSR(*d["b_shape"], d["b_ptr"], d["b_idx"], d["b_val"])
    res = ctx.spgemm(A, B, scope="kernel")
    check(res.C, A, B, orc)
    if name != "quirk_ref.npz":
        Cp_r, Ci_r, Cv_r, dups = orc.canonicalise(d["off"], d["cnt"], d["idx"], d["val"])
        assert dups == 0
        assert np.array_equal(res.C.row_ptr, Cp_r) and np.array_equal(res.C.col_idx, Ci_r)
        assert np.allclose(res.C.val, Cv_r, rtol=2e-6, atol=0)


def test_cage4_from_reference_csr_file(ctx, orc):
    M = dbd.read_CSR(os.path.join(GOLDEN, "cage4"))
    res = ctx.spgemm(M, scope="kernel")
    check(res.C, M, M, orc)


@pytest.mark.parametrize("scale,ef,seed", [(10, 8, 1), (12, 8, 2), (14, 8, 3), (13, 16, 4)])
def test_rmat_small(ctx, orc, scale, ef, seed):
    A = gen.rmat(scale, ef, seed=seed)
    res = ctx.spgemm(A, scope="kernel")
    check(res.C, A, A, orc)


def mixed_rows(rng, m, k, n):
    """m x k A with row lengths from 1 to 2500, k x n B with Poisson(6) rows."""
    rows, cols = [], []
    lens = np.concatenate([rng.integers(1, 3, 200), rng.integers(5, 20, 150), rng.integers(40, 80, 100),
                           rng.integers(150, 300, 100), rng.integers(1500, 2500, 50)])[:m]
    rng.shuffle(lens)
    for r in range(m):
        c = rng.choice(k, size=int(lens[r]), replace=False)
        rows.append(np.full(c.size, r))
        cols.append(c)
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    A = gen._from_coo(m, k, rows, cols, rng.uniform(-1, 1, rows.size))
    br, bc = gen._distinct_cols(rng, rng.poisson(6, k).astype(np.int64), n)
    B = gen._from_coo(k, n, br, bc, rng.uniform(-1, 1, br.size))
    return A, B


def random_band(rng, n, k, half):
    """n x n, k distinct columns per row drawn from [i - half, i + half]."""
    rows, cols = [], []
    for i in range(n):
        lo, hi = max(0, i - half), min(n - 1, i + half)
        c = rng.choice(hi - lo + 1, size=min(k, hi - lo + 1), replace=False) + lo
        rows.append(np.full(c.size, i))
        cols.append(c)
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    return gen._from_coo(n, n, rows, cols, rng.uniform(-1, 1, rows.size))


def test_every_numeric_bin_exercised(ctx, orc):
    """Rows in every numeric bin: narrow rows (bands: warp dense windows and
    warp rank), rows within 2^18 columns (CTA rank, shared and in place), and
    rows spanning more than 2^18 columns (CTA hash of both sizes, dense
    windows)."""
    rng = np.random.default_rng(11)
    used = set()
    sym_used = set()
    cases = [mixed_rows(rng, 600, 3000, 20000), mixed_rows(rng, 600, 3000, 600000),
             (gen.banded(3000, 8, seed=3), gen.banded(3000, 8, seed=4)),
             (random_band(rng, 2000, 8, 400), random_band(rng, 2000, 8, 400))]
    for A, B in cases:
        res = ctx.spgemm(A, B, scope="kernel")
        check(res.C, A, B, orc)
        used |= set(bins_used(res.stats))
        sym_used |= {i for i, v in enumerate(res.stats["sym_rows_per_bin"]) if v}
    assert used >= set(range(1, 10)), used
    assert sym_used >= set(range(1, 6)), sym_used
    # The warp rank-window bin (off by default) on the rows it would take.
    with dbd.Context(cpu_gib=8, gpu_gib=8) as c:
        c.set_tuning(mid_span_words=2048)
        A, B = cases[0]
        res = c.spgemm(A, B, scope="kernel")
        check(res.C, A, B, orc)
        assert res.stats["rows_per_bin"][10] > 0


def shuffled_rows(rng, M):
    """M with every row's entries in random order (B rows not ascending)."""
    idx, val = M.col_idx.copy(), M.val.copy()
    for r in range(M.n_rows):
        s, e = M.row_ptr[r], M.row_ptr[r + 1]
        p = rng.permutation(e - s)
        idx[s:e], val[s:e] = idx[s:e][p], val[s:e][p]
    return CSR(M.n_rows, M.n_cols, M.row_ptr, idx, val)


def test_narrow_rows_every_enumeration(ctx, orc):
    """Narrow rows (warp flag and dense-window kernels) through each path:
    contiguous B rows (banded: flagged a word at a time), long B rows with
    gaps (row-wise, a column at a time), short B rows (flattened), and B rows
    out of column order (row-wise with atomics)."""
    rng = np.random.default_rng(21)
    band = gen.banded(1500, 24, seed=5)
    gappy = random_band(rng, 1500, 20, 40)
    short = random_band(rng, 1500, 3, 40)
    for A, B in ((band, band), (gappy, gappy), (gappy, short), (band, shuffled_rows(rng, band)),
                 (gappy, shuffled_rows(rng, gappy))):
        res = ctx.spgemm(A, B, scope="kernel")
        check(res.C, A, B, orc)
        assert res.stats["sym_rows_per_bin"][2] > 0 and res.stats["rows_per_bin"][9] > 0


def run_rows(rng, n, step, lmin, lmax, permute=False, gap_every=0):
    """n x (step n + lmax): row k is one contiguous run of lmin..lmax columns
    starting at step * k (starts ascending with k; overlapping, nested or
    disjoint runs by the step).  permute: rows shuffled within blocks of 8
    (starts no longer ascending); gap_every: every such row loses an interior
    column."""
    lens = rng.integers(lmin, lmax + 1, n)
    rows = np.repeat(np.arange(n), lens)
    cols = np.concatenate([step * k + np.arange(L) for k, L in enumerate(lens)])
    keep = np.ones(cols.size, bool)
    if gap_every:
        starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
        keep[starts[::gap_every] + 1] = False
    M = gen._from_coo(n, step * n + lmax, rows[keep], cols[keep], rng.uniform(-1, 1, int(keep.sum())))
    if permute:  # rows shuffled within blocks of 8, so that the window stays narrow
        p = np.concatenate([b0 + rng.permutation(min(8, n - b0)) for b0 in range(0, n, 8)])
        lens2 = np.diff(M.row_ptr)[p]
        ptr = np.concatenate([[0], np.cumsum(lens2)]).astype(np.int32)
        take = np.concatenate([np.arange(M.row_ptr[r], M.row_ptr[r + 1]) for r in p])
        M = CSR(n, M.n_cols, ptr, M.col_idx[take], M.val[take])
    return M


def test_narrow_rows_runs_of_columns(ctx, orc):
    """Narrow rows whose B rows are single runs of columns (the symbolic
    count is the length of the runs' union): overlapping and nested runs,
    disjoint runs, runs whose starts do not ascend with the entry, and some
    B rows with a gap (the warp-flag path takes over)."""
    rng = np.random.default_rng(33)
    A = gen.banded(1500, 24, seed=7)
    for B in (run_rows(rng, 1500, 2, 16, 40), run_rows(rng, 1500, 1, 16, 64), run_rows(rng, 1500, 30, 16, 25),
              run_rows(rng, 1500, 2, 16, 40, permute=True), run_rows(rng, 1500, 2, 16, 40, gap_every=97)):
        res = ctx.spgemm(A, B, scope="kernel")
        check(res.C, A, B, orc)
        assert res.stats["sym_rows_per_bin"][2] > 0


def test_dense_rows_long_and_thin_b_rows(ctx, orc):
    """Dense-window rows both ways: B rows of 2,000 consecutive columns (many
    products per entry and window: one warp per entry) and B rows of a few
    scattered columns over 600,000 (one thread per entry)."""
    rng = np.random.default_rng(8)
    n = 600_000
    k = 400
    starts = (np.arange(k) * 1487) % (n - 2000)
    rows = np.repeat(np.arange(k), 2000)
    cols = (starts[:, None] + np.arange(2000)[None, :]).ravel()
    B_long = gen._from_coo(k, n, rows, cols, rng.uniform(-1, 1, rows.size))
    A_long = gen.uniform_rows(48, 60, seed=4, n_cols=k, dist="uniform")
    B_thin = gen.uniform_rows(4000, 5, seed=3, n_cols=n, dist="uniform")
    A_thin = gen.uniform_rows(48, 1000, seed=5, n_cols=4000, dist="uniform")
    # Every method of the dense bin: rank windows, global slots, FP64 windows,
    # one pass into scratch rows.
    for method in (0, 1, 2, 3):
        with dbd.Context(cpu_gib=8, gpu_gib=16) as c:
            c.set_tuning(dense_method=method)
            for A, B in ((A_long, B_long), (A_thin, B_thin)):
                res = c.spgemm(A, B, scope="kernel")
                check(res.C, A, B, orc)
                assert res.stats["rows_per_bin"][8] > 0  # the dense bin
    # Global slots or scratch rows without room for them (a small budget):
    # FP64 windows.
    for method in (1, 3):
        with dbd.Context(cpu_gib=4, gpu_gib=0.5) as small:
            small.set_tuning(dense_method=method)
            for A, B in ((A_long, B_long), (A_thin, B_thin)):
                res = small.spgemm(A, B, scope="kernel")
                check(res.C, A, B, orc)


def test_dense_rows_over_several_windows(ctx, orc):
    """Rows over 2.5M columns (five 2^19-column windows, symbolic and
    numeric): B rows scattered over the whole range (each window takes its
    part of them), B rows inside one 2^20-column range, B rows ending
    exactly at a window edge; then the same B with its rows out of column
    order."""
    rng = np.random.default_rng(12)
    n = 2_500_000
    rows, cols = [], []
    for r in range(3000):
        kind = r % 3
        if kind == 0:
            c = rng.choice(n, 40, replace=False)
        elif kind == 1:
            w0 = (r % 3) * (1 << 20)
            c = w0 + rng.choice(min(1 << 20, n - w0), 40, replace=False)
        else:
            edge = (1 + r % 4) << 19
            c = np.concatenate([np.arange(edge - 20, edge), rng.choice(n, 20, replace=False)])
            c = np.unique(c)
        rows.append(np.full(c.size, r))
        cols.append(c)
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    B = gen._from_coo(3000, n, rows, cols, rng.uniform(-1, 1, rows.size))
    A = gen.uniform_rows(24, 600, seed=9, n_cols=3000, dist="uniform")
    Bu = shuffled_rows(rng, B)
    for method in (0, 3):  # rank windows, one pass into scratch rows
        with dbd.Context(cpu_gib=8, gpu_gib=32) as c:
            c.set_tuning(dense_method=method)
            res = c.spgemm(A, B, scope="kernel")
            check(res.C, A, B, orc)
            assert res.stats["rows_per_bin"][8] > 0 and res.stats["sym_rows_per_bin"][5] > 0
            res = c.spgemm(A, Bu, scope="kernel")
            check(res.C, A, B, orc)


def test_dense_rows_cut_into_pieces(ctx, orc):
    """Dense-bin rows of more than 2^16 entries over 2.5M columns: the
    symbolic pass keeps their per-slab counts and the numeric pass cuts them
    into column pieces of about 2^16 entries, each its own work item; B rows
    mix scattered columns with runs that cross slab and window edges."""
    rng = np.random.default_rng(44)
    n = 2_500_000
    rows, cols = [], []
    for r in range(3000):
        c = rng.choice(n, 50, replace=False)
        if r % 5 == 0:  # a run across a slab edge (2^16) or a window edge (2^20)
            edge = ((1 + r % 7) << 16) if r % 2 else ((1 + r % 2) << 20)
            c = np.unique(np.concatenate([c, np.arange(edge - 30, edge + 30)]))
        rows.append(np.full(c.size, r))
        cols.append(c)
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    B = gen._from_coo(3000, n, rows, cols, rng.uniform(-1, 1, rows.size))
    A = gen.uniform_rows(12, 2600, seed=13, n_cols=3000, dist="uniform")
    res = ctx.spgemm(A, B, scope="kernel")
    check(res.C, A, B, orc)
    assert res.stats["rows_per_bin"][8] == A.n_rows and res.stats["heavy_rows"] == A.n_rows
    assert np.diff(res.C.row_ptr).min() > 65536  # every row is cut into pieces
    # B's rows out of column order: no pieces (each row one item).
    res = ctx.spgemm(A, shuffled_rows(rng, B), scope="kernel")
    check(res.C, A, B, orc)
    assert res.stats["heavy_rows"] == 0


def test_dense_rows_unsorted_b(ctx, orc):
    """Dense-window rows with B rows out of column order take the rescanning path."""
    rng = np.random.default_rng(5)
    A = gen.uniform_rows(64, 1500, seed=1, n_cols=4000, dist="uniform")
    B = gen.uniform_rows(4000, 12, seed=2, n_cols=600000, dist="uniform")
    perm_idx = B.col_idx.copy()
    for r in range(B.n_rows):
        s, e = B.row_ptr[r], B.row_ptr[r + 1]
        p = rng.permutation(e - s)
        perm_idx[s:e] = B.col_idx[s:e][p]
        B.val[s:e] = B.val[s:e][p]
    B = CSR(B.n_rows, B.n_cols, B.row_ptr, perm_idx, B.val)
    for method in (0, 3):
        with dbd.Context(cpu_gib=8, gpu_gib=16) as c:
            c.set_tuning(dense_method=method)
            res = c.spgemm(A, B, scope="kernel")
            check(res.C, A, B, orc)
            assert res.stats["rows_per_bin"][8] > 0  # dense windows


def test_edge_cases(ctx, orc):
    z = np.zeros(0)
    cases = [
        (CSR(0, 5, np.zeros(1, np.int32), np.zeros(0, np.int32), z), CSR(5, 3, np.zeros(6, np.int32), np.zeros(0, np.int32), z)),
        (CSR(4, 4, np.zeros(5, np.int32), np.zeros(0, np.int32), z), None),
        (CSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0])), None),
        (CSR(3, 2, np.array([0, 2, 2, 4], np.int32), np.array([1, 0, 0, 1], np.int32), np.array([1., 2., 3., 4.])),
         CSR(2, 7, np.array([0, 3, 3], np.int32), np.array([6, 0, 2], np.int32), np.array([1., -1., .5]))),
        # duplicate columns inside a row of A and of B
        (CSR(2, 3, np.array([0, 3, 4], np.int32), np.array([1, 1, 2, 0], np.int32), np.array([1., 2., 3., 4.])),
         CSR(3, 3, np.array([0, 1, 3, 4], np.int32), np.array([2, 1, 1, 0], np.int32), np.array([1., 1., 1., 1.]))),
    ]
    for A, B in cases:
        Bx = A if B is None else B
        res = ctx.spgemm(A, B, scope="kernel")
        check(res.C, A, Bx, orc)


def test_fp32_operands_promoted(ctx, orc):
    A = gen.rmat(11, 8, seed=9)
    A32 = CSR(A.n_rows, A.n_cols, A.row_ptr, A.col_idx, A.val.astype(np.float32))
    res = ctx.spgemm(A32, scope="kernel")
    A64 = CSR(A.n_rows, A.n_cols, A.row_ptr, A.col_idx, A.val.astype(np.float32).astype(np.float64))
    check(res.C, A64, A64, orc)


def test_device_resident_operands(ctx, orc):
    torch = pytest.importorskip("torch")
    A = gen.rmat(12, 8, seed=4)
    p = torch.from_numpy(A.row_ptr).cuda()
    i = torch.from_numpy(A.col_idx).cuda()
    v = torch.from_numpy(A.val).cuda()
    D = CSR.from_device(A.n_rows, A.n_cols, A.nnz, p.data_ptr(), i.data_ptr(), v.data_ptr())
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        res = ctx.spgemm(D, scope="kernel")
    finally:
        ctx.set_stream(None)
    check(res.C, A, A, orc)


def test_invalid_operands_rejected(ctx):
    bad = CSR(2, 2, np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32), np.array([1.0, 1.0]))
    with pytest.raises(dbd.DBDError) as ei:
        ctx.spgemm(bad)
    assert ei.value.code == -1
    A = CSR(2, 3, np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    with pytest.raises(dbd.DBDError):
        ctx.spgemm(A, A)  # 2x3 * 2x3
    torch = pytest.importorskip("torch")
    p = torch.tensor([0, 2, 1], dtype=torch.int32, device="cuda")  # decreasing row_ptr
    i = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    v = torch.ones(2, dtype=torch.float64, device="cuda")
    D = CSR.from_device(2, 2, 2, p.data_ptr(), i.data_ptr(), v.data_ptr())
    with pytest.raises(dbd.DBDError) as ei:
        ctx.spgemm(D)
    assert ei.value.code == -1


def test_out_of_core_chunks_and_ring(orc, tmp_path):
    """Small budgets force several device output chunks, a host ring and the
    writer's ordered appends; files must still hold the exact product."""
    A = gen.uniform_rows(1 << 14, 10, seed=6, dist="uniform")
    Cp, Ci, Cv, Ca = orc.spgemm(A, with_abs=True)
    out_bytes = 12 * Cv.size
    gib = 1024 ** 3
    work = 4 << 20  # operands and work arrays of this size, generously
    with dbd.Context(cpu_gib=1, gpu_gib=(work + 0.5 * out_bytes) / gib, rows_per_block=512) as c:
        res = c.spgemm(A, scope="io", out_dir=str(tmp_path))
        assert res.stats["n_chunks"] >= 3
        ptr = np.fromfile(tmp_path / "Ptr.output", np.int64)
        idx = np.fromfile(tmp_path / "Idx.output", np.int32)
        val = np.fromfile(tmp_path / "Val.output", np.float64)
        assert np.array_equal(ptr, Cp) and np.array_equal(idx, Ci)
        assert np.all(np.abs(val - Cv) <= TOL * Ca)
        res = c.spgemm(A, scope="d2h")
        assert res.stats["n_chunks"] >= 3
        check(res.C, A, A, orc)


def test_io_rotation_bounds_file_size(tmp_path):
    A = gen.rmat(13, 8, seed=7)
    with dbd.Context(cpu_gib=1, gpu_gib=0.06, rows_per_block=512, io_rotate_gib=0.001) as c:
        res = c.spgemm(A, scope="io", out_dir=str(tmp_path))
    assert os.path.getsize(tmp_path / "Idx.output") <= 0.001 * 1024 ** 3
    assert res.stats["bytes_written"] >= 12 * res.stats["nnz_c"]


def test_stage_functions_mirror_reference(orc):
    """initialize_A/B -> divide_Blocks -> distribute_Workload, as main.cpp drives them."""
    A = gen.rmat(13, 8, seed=8)
    with dbd.Context(cpu_gib=4, gpu_gib=4, rows_per_block=4096) as c:
        c.initialize_A(A)
        c.initialize_B(A)
        nb = c.divide_Blocks()
        assert nb == 2
        prods, cats = c.block_info(nb)
        rp, tot = orc.row_products(A, A)
        upp = orc.exclusive_scan(rp)
        _, info, _ = orc.divide_blocks(A.n_rows, upp, 4096)
        assert np.array_equal(prods, info)
        crit = orc.criteria(info, 4096, tot)
        assert [orc.analyze_block(crit, int(p // 4096)) for p in prods] == cats.tolist()
        st = c.distribute_Workload("kernel")
        assert st["criteria"] == crit
        check(c.result(), A, A, orc)


def test_cli_binaries(tmp_path, orc):
    L = gen.laplacian_2d(32)
    dbd.write_CSR(str(tmp_path / "lap.dcsr"), L, fp64=True)
    for name in ("compute", "d2h", "SSpMM", "debug"):
        out = subprocess.run([os.path.join(ROOT, "dbd_gb300", "bin", name), "4", "4", "lap"], cwd=tmp_path,
                             capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
        for line in ("Preprocessing\t\t", "Compute GPU\t\t", "Kernel Execution\t", "Total Execution\t\t"):
            assert line in out.stdout
    Cp, Ci, Cv = orc.spgemm(L)
    assert np.array_equal(np.fromfile(tmp_path / "Idx.output", np.int32), Ci)
    out = subprocess.run([os.path.join(ROOT, "dbd_gb300", "bin", "SSpMM")], cwd=tmp_path, capture_output=True,
                         text=True, timeout=60)
    assert out.returncode != 0 and "Invalid Arguments." in out.stdout


def test_rmat18_full_size_properties(ctx, orc):
    """The scale-18 workload at full size: structure equal to the oracle's,
    values within the tolerance, per-row sums (a size-independent checksum)
    equal to A*(A*1)."""
    A = gen.rmat(18, 8, seed=0)
    res = ctx.spgemm(A, scope="kernel")
    C = res.C
    assert res.stats["products"] == 867505158
    relmax, relmean = check(C, A, A, orc)
    S = A.to_scipy()
    ones = np.ones(A.n_cols)
    rows = np.add.reduceat(np.concatenate([C.val, [0.0]]), np.minimum(C.row_ptr[:-1], C.val.size))
    rows[np.diff(C.row_ptr) == 0] = 0.0
    assert np.allclose(rows, S @ (S @ ones), rtol=1e-10)
    print(f"rmat18: nnz(C)={C.nnz} max rel err {relmax:.3e} mean {relmean:.3e}")
