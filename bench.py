#!/usr/bin/env python3
"""SpGEMM GFLOPS (2 x intermediate products / s) of C = A*A on one GB300.

Workload (default): A = R-MAT scale 18, edge factor 8, (a,b,c,d) =
(.57,.19,.19,.05), seed 0 (n = 262,144, nnz = 2,016,992, P = 867,505,158
products), FP64 values 1 - U[0,1), row blocks of 4096.  One step = one full
multiply in the kernel scope (work estimate + segmentation + categorisation +
symbolic + numeric, device-synchronised, C left in HBM), inputs resident in
HBM, L2 flushed between steps by a 512 MiB device write outside the timed
events.

Also reported: e2e = the same multiply through the C ABI (dbd_spgemm) with
host buffers, H2D of A and D2H of the whole C inside the timed region (the
+D2H scope); the +I/O scope (Ptr/Idx/Val.output written and fsynced); the
roofline of the dominant kernel from CUDA events recorded around it inside
the library; and the reference's CPU algorithm (a restatement of its
compute_CPU worker, FP32) timed on this host's cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dbd|reference]
"""
import argparse
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpGEMM GFLOPS (2×products/s) kernel/+D2H/+I/O; batched & adjoint vs plain"
WORKLOADS = {
    "rmat18": ("A*A, A = R-MAT scale 18 (n=262,144), edge factor 8, (a,b,c,d)=(.57,.19,.19,.05), seed 0, "
               "FP64 values 1-U[0,1), blocksize 4096", 4096),
    "laplacian256": ("A*A, A = 5-point Laplacian on a 256x256 grid (n=65,536), FP64 values 4/-1, blocksize 4096",
                     4096),
}


def make_workload(name):
    from dbd_gb300 import generators as gen
    if name == "rmat18":
        return gen.rmat(18, 8, seed=0)
    if name == "laplacian256":
        return gen.laplacian_2d(256)
    if name.startswith("rmat"):
        return gen.rmat(int(name[4:]), 8, seed=0)
    raise SystemExit(f"unknown workload {name}")


def row_products(A):
    lens = np.diff(A.row_ptr).astype(np.int64)
    per_entry = lens[A.col_idx]
    cs = np.concatenate([[0], np.cumsum(per_entry)])
    return cs[A.row_ptr[1:]] - cs[A.row_ptr[:-1]]


def thresholds():
    """Bin thresholds of the library (dbd_internal.h), for per-kernel byte counts."""
    text = open(os.path.join(ROOT, "dbd_gb300", "csrc", "dbd_internal.h")).read()
    names = ["kTinyMax", "kSymWarpMax", "kSymCtaMax", "kNumWarpMax", "kNumCtaSMax", "kNumCtaLMax",
             "kWarpSpanWords", "kRankWordsMax", "kWideHashSpanWords"]
    return {n: int(re.search(rf"\b{n}\s*=\s*(\d+)", text).group(1)) for n in names}


def span_words(A, B=None, col_off=0):
    """Words of 32 columns spanned by each row of A*B (0 for empty rows); B's
    rows have ascending columns, which sit at col_off in C."""
    B = A if B is None else B
    lens = np.diff(B.row_ptr)
    imax = np.iinfo(np.int64).max
    first = np.where(lens > 0, B.col_idx[np.minimum(B.row_ptr[:-1], max(B.nnz - 1, 0))].astype(np.int64), imax)
    last = np.where(lens > 0, B.col_idx[np.maximum(B.row_ptr[1:] - 1, 0)].astype(np.int64), -1)
    nA = np.diff(A.row_ptr)
    lo = np.full(A.n_rows, imax, np.int64)
    hi = np.full(A.n_rows, -1, np.int64)
    nz = nA > 0
    if A.nnz:
        starts = A.row_ptr[:-1][nz]
        lo[nz] = np.minimum.reduceat(first[A.col_idx], starts)
        hi[nz] = np.maximum.reduceat(last[A.col_idx], starts)
    ok = hi >= lo
    return np.where(ok, ((hi + col_off) >> 5) - ((np.where(ok, lo, 0) + col_off) >> 5) + 1, 0)


def bins(A, rowP, nnz_r, sw):
    """Symbolic and numeric bin of every row (the rules of dbd_internal.h)."""
    t = thresholds()
    nA = np.diff(A.row_ptr)
    tiny = (rowP <= t["kTinyMax"]) & (nA <= 32)
    sym = np.select([rowP == 0, tiny, sw <= t["kWarpSpanWords"], rowP <= t["kSymWarpMax"],
                     (rowP <= t["kSymCtaMax"]) & (sw > t["kWideHashSpanWords"])], [0, 1, 2, 3, 4], 5)
    num = np.select([nnz_r == 0, tiny, (sw <= t["kWarpSpanWords"]) & (nnz_r <= t["kNumWarpMax"]),
                     nnz_r <= t["kNumWarpMax"], (sw <= t["kRankWordsMax"]) & (nnz_r <= t["kNumCtaLMax"]),
                     sw <= t["kRankWordsMax"], nnz_r <= t["kNumCtaSMax"], nnz_r <= t["kNumCtaLMax"]],
                    [0, 1, 2, 3, 4, 5, 6, 7], 8)
    return sym, num


SYM_NAMES = {1: "k_sym_tiny", 2: "k_sym_bitw<8>", 3: "k_sym_hash_warp<8,1024>", 4: "k_sym_hash_cta<256,8192>",
             5: "k_sym_wide<512>"}
NUM_NAMES = {1: "k_num_tiny", 2: "k_num_rankw<8>", 3: "k_num_hash_warp<4,512>", 4: "k_num_rank<256,shared>",
             5: "k_num_rank<512,in-place>", 6: "k_num_hash_cta<256,2048>", 7: "k_num_hash_cta<512,8192>",
             8: "k_num_dense<512,8192>"}


def kernel_bytes(A, rowP, nnz_r, sym, num):
    """Algorithmic bytes per launch of each kernel family: every A entry of its
    rows (int32 index + FP64 value), the B (int32 column, FP64 value) of
    every product, and C's output (int32 + FP64 per entry) and row pointer."""
    nA = np.diff(A.row_ptr).astype(np.int64)
    out = {}
    for b, name in SYM_NAMES.items():
        m = sym == b
        out[("sym", b)] = (name, int(4 * nA[m].sum() + 4 * rowP[m].sum() + 4 * m.sum()))
    for b, name in NUM_NAMES.items():
        m = num == b
        out[("num", b)] = (name, int(12 * nA[m].sum() + 12 * rowP[m].sum() + 12 * nnz_r[m].sum() + 8 * m.sum()))
    return out


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            f = line.split()
            if len(f) >= 3 and not line.startswith("#"):
                out[(f[0], f[1])] = float(f[2])
    return out


def cpu_reference_port(A, threads, repeats=1):
    """The reference's CPU worker (compute_CPU, FP32) restated in oracle/,
    block by block of 4096 rows like the reference, one reused slot buffer of
    the largest block (h_IdxC / h_ValC)."""
    import ctypes as C
    import oracle
    L = oracle.lib()
    Ap = np.ascontiguousarray(A.row_ptr, np.int32)
    Ai = np.ascontiguousarray(A.col_idx, np.int32)
    Av = np.ascontiguousarray(A.val, np.float32)
    rowP = row_products(A)
    off = np.concatenate([[0], np.cumsum(rowP)]).astype(np.int64)
    rpb = 4096
    nb = (A.n_rows + rpb - 1) // rpb
    edges = [min(b * rpb, A.n_rows) for b in range(nb + 1)]
    maxblk = max(int(off[edges[b + 1]] - off[edges[b]]) for b in range(nb))
    cnt = np.zeros(A.n_rows, np.int32)
    idx = np.zeros(max(maxblk, 1), np.int32)
    val = np.zeros(max(maxblk, 1), np.float32)
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        for b in range(nb):
            L.orc_ref_cpu_rows(edges[b], edges[b + 1], A.n_cols, Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data,
                               Ap.ctypes.data, Ai.ctypes.data, Av.ctypes.data, off.ctypes.data, cnt.ctypes.data,
                               idx.ctypes.data, val.ctypes.data, C.c_int(threads))
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return int(off[-1]), best


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    desc, _ = WORKLOADS.get(args.workload, (args.workload, 4096))
    A = make_workload(args.workload)
    threads = os.cpu_count() or 1
    P, _ = cpu_reference_port(A, threads, 1)
    for _ in range(args.warmup):
        cpu_reference_port(A, threads, 1)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_reference_port(A, threads, 1)
        times.append(dt)
    t = float(np.mean(times))
    v = 2.0 * P / t / 1e9
    sample = f"the whole workload ({P} products), row blocks of 4096, one step = one full pass"
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GFLOPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "products": P, "path": "reference CPU worker compute_CPU "
                       "(ZIP:dbd/src/computeCPU.cpp:10-98) restated in oracle/oracle.c, OpenMP over rows"},
            "cpu_baseline": {"value": round(v, 4), "unit": "GFLOPS", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "GFLOPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def pinned_copy(torch, M):
    """M with its arrays in pinned host memory (numpy views of pinned tensors)."""
    from dbd_gb300.csr import CSR
    out = []
    for x in (M.row_ptr, M.col_idx, M.val):
        t = torch.empty(x.shape[0], dtype=getattr(torch, x.dtype.name), pin_memory=True)
        t.numpy()[:] = x
        out.append(t)
    C_ = CSR(M.n_rows, M.n_cols, out[0].numpy(), out[1].numpy(), out[2].numpy())
    C_._pinned = out
    return C_


def run_batched(args, local):
    """512 independent A_q*B_q products: one dbd_spgemm_batched call per step
    against 512 plain dbd_spgemm calls on the same device-resident pairs."""
    import torch
    import dbd_gb300 as dbd
    from dbd_gb300 import generators as gen
    from dbd_gb300.csr import CSR
    count = 512
    pairs = gen.batched_pairs(count, seed=0)
    As = [a for a, _, _ in pairs]
    Bs = [b for _, b, _ in pairs]
    kinds = [k for _, _, k in pairs]
    dev = torch.device("cuda", local)
    torch.cuda.set_device(local)
    keep = []

    def on_dev(M):
        t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (M.row_ptr, M.col_idx, M.val)]
        keep.append(t)
        return CSR.from_device(M.n_rows, M.n_cols, M.nnz, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())

    dA = [on_dev(A) for A in As]
    dB = [on_dev(B) for B in Bs]
    rowP, nA_all, sw_all = [], [], []
    col_off = 0
    for A, B in zip(As, Bs):
        lens = np.diff(B.row_ptr).astype(np.int64)
        cs = np.concatenate([[0], np.cumsum(lens[A.col_idx])])
        rowP.append(cs[A.row_ptr[1:]] - cs[A.row_ptr[:-1]])
        nA_all.append(np.diff(A.row_ptr))
        sw_all.append(span_words(A, B, col_off))
        col_off += B.n_cols
    rowP = np.concatenate(rowP)
    P = int(rowP.sum())
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    ctx = dbd.Context(cpu_gib=96, gpu_gib=200, rows_per_block=4096, device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
            flush.zero_()
        torch.cuda.synchronize()
        ms, out = [], None
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            flush.zero_()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.mean(ms)) / 1e3, out

    with Clocks(local) as clk:
        t_batch, res = timed(lambda: ctx.spgemm_batched(dA, dB, scope="kernel", fetch=False), args.steps,
                             args.warmup)
    launches = int(res.stats["gpu_launches"])
    nnzC = int(res.stats["nnz_c"])
    # Roofline of the dominant kernel family of the batched multiply.
    Cp = np.empty(int(res.row_off[-1]) + 1, np.int64)
    ctx._lib.dbd_result_copy(ctx.handle, Cp.ctypes.data, None, None)
    nnz_r = np.diff(Cp)
    Acat = CSR(len(rowP), col_off, np.concatenate([[0], np.cumsum(np.concatenate(nA_all))]), None, None)
    Acat.col_idx = np.zeros(0, np.int32)
    sym, num = bins(Acat, rowP, nnz_r, np.concatenate(sw_all))
    kb = kernel_bytes(Acat, rowP, nnz_r, sym, num)
    # Per-kernel times: the same batched multiply on a context that times
    # every kernel family, the bins one after another.
    pctx = dbd.Context(cpu_gib=96, gpu_gib=200, rows_per_block=4096, device=local, time_kernels=True)
    pctx.set_stream(stream.cuda_stream)
    pctx.spgemm_batched(dA, dB, scope="kernel", fetch=False)
    flush.zero_()
    st = pctx.spgemm_batched(dA, dB, scope="kernel", fetch=False).stats
    torch.cuda.synchronize()
    pctx.close()
    ktime = {("num", b): st["t_num_bin_ms"][b] for b in NUM_NAMES}
    ktime.update({("sym", b): st["t_sym_bin_ms"][b] for b in SYM_NAMES})
    dom = max(ktime, key=ktime.get)
    dom_ms = ktime[dom]
    dom_name, dom_bytes = kb[dom]
    peak, peak_kind = peaks()
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0

    def sequential():
        for q in range(count):
            ctx.spgemm(dA[q], dB[q], scope="kernel", fetch=False)
    t_seq, _ = timed(sequential, max(1, min(args.steps, 3)), 1)

    # e2e: host pairs in pinned memory, C back to (pinned) host memory.
    hA = [pinned_copy(torch, A) for A in As]
    hB = [pinned_copy(torch, B) for B in Bs]
    ctx.set_stream(None)
    ctx.spgemm_batched(hA, hB, scope="d2h", fetch=False)
    te = []
    for _ in range(max(1, args.e2e_steps)):
        t0 = time.perf_counter()
        ctx.spgemm_batched(hA, hB, scope="d2h", fetch=False)
        te.append(time.perf_counter() - t0)
    te = float(np.mean(te))
    t0 = time.perf_counter()
    for q in range(count):
        ctx.spgemm(hA[q], hB[q], scope="d2h", fetch=False)
    te_seq = time.perf_counter() - t0
    nnz_in = sum(A.nnz + B.nnz for A, B in zip(As, Bs))
    rows_in = sum(A.n_rows + B.n_rows + 2 for A, B in zip(As, Bs))
    h2d = 12 * nnz_in + 4 * rows_in
    d2h = 12 * nnzC + 8 * (len(rowP) + 1)
    ctx.close()
    g = lambda t: round(2.0 * P / t / 1e9, 4)
    line = {"metric": METRIC, "value": g(t_batch), "unit": "GFLOPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_batch * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded pairs, numpy PCG64)",
            "config": {"workload": "batched: 512 independent A_q*B_q, n_q log-uniform in [1024, 65536], "
                       "uniform Poisson(12) rows or band |i-j|<=32 (50/50 by seed), values U[-1,1], seed 0",
                       "pairs": count, "banded_pairs": int(sum(k == "banded" for k in kinds)),
                       "rows": int(len(rowP)), "nnz_a": int(sum(A.nnz for A in As)),
                       "nnz_b": int(sum(B.nnz for B in Bs)), "products": P, "nnz_c": nnzC,
                       "scope": "kernel (pairs resident in HBM, C left in HBM)",
                       "l2": "flushed between steps (512 MiB device write outside the timed events)"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                         "peak_kind": f"of {peak_kind}", "algorithmic_bytes_per_launch": dom_bytes,
                         "launch_ms": round(dom_ms, 4),
                         "kernel_ms_per_step": {kb[k][0]: round(v, 4) for k, v in
                                                sorted(ktime.items(), key=lambda x: -x[1]) if v}},
            "sequential": {"gflops": g(t_seq), "ms": round(t_seq * 1e3, 3),
                           "what": "512 plain dbd_spgemm calls (kernel scope) on the same device-resident pairs"},
            "batched_vs_sequential": round(t_seq / t_batch, 3),
            "e2e": {"value": g(te), "unit": "GFLOPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": round(te * 1e3, 3),
                    "scope": "+D2H through dbd_spgemm_batched with pinned host pairs and pinned host C",
                    "sequential_gflops": g(te_seq), "sequential_ms": round(te_seq * 1e3, 3)},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="dbd", choices=["dbd", "reference"])
    ap.add_argument("--workload", default="rmat18")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-io", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.workload == "batched512":
        if rank != 0:
            return 0
        return run_batched(args, local)

    import torch
    import dbd_gb300 as dbd
    from dbd_gb300.csr import CSR

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    desc, rpb = WORKLOADS.get(args.workload, (args.workload, 4096))
    A = make_workload(args.workload)
    rowP = row_products(A)
    P = int(rowP.sum())
    dev = torch.device("cuda", local)
    tp = torch.from_numpy(A.row_ptr).to(dev)
    ti = torch.from_numpy(A.col_idx).to(dev)
    tv = torch.from_numpy(A.val).to(dev)
    D = CSR.from_device(A.n_rows, A.n_cols, A.nnz, tp.data_ptr(), ti.data_ptr(), tv.data_ptr())
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    ctx = dbd.Context(cpu_gib=96, gpu_gib=200, rows_per_block=rpb, device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.initialize_A(D)
    ctx.initialize_B(D)

    def step(c=ctx):
        c.divide_Blocks()
        return c.distribute_Workload("kernel")

    for _ in range(args.warmup):
        step()
        flush.zero_()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    with Clocks(local) as clk:
        t_wall0 = time.perf_counter()
        for i in range(args.steps):
            evs[i][0].record(stream)
            stats.append(step())
            evs[i][1].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    t_step = float(np.mean(ms)) / 1e3
    if dist:
        tt = torch.tensor([t_step], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    value = world * 2.0 * P / t_step / 1e9
    nnzC = int(stats[-1]["nnz_c"])
    launches = int(sum(s["gpu_launches"] for s in stats))

    # Roofline of the dominant kernel family: a second context runs the same
    # multiply with CUDA events around every kernel family, the bins one
    # after another on its stream (outside the timed steps above).
    Cp = np.empty(A.n_rows + 1, np.int64)
    ctx._lib.dbd_result_copy(ctx.handle, Cp.ctypes.data, None, None)
    nnz_r = np.diff(Cp)
    sym, num = bins(A, rowP, nnz_r, span_words(A))
    kb = kernel_bytes(A, rowP, nnz_r, sym, num)
    pctx = dbd.Context(cpu_gib=96, gpu_gib=200, rows_per_block=rpb, device=local, time_kernels=True)
    pctx.set_stream(stream.cuda_stream)
    pctx.initialize_A(D)
    pctx.initialize_B(D)
    pstats = []
    for i in range(args.warmup + 3):
        st_i = step(pctx)
        flush.zero_()
        if i >= args.warmup:
            pstats.append(st_i)
    torch.cuda.synchronize()
    pctx.close()
    ktime = {}
    for s in pstats:
        for b in NUM_NAMES:
            ktime[("num", b)] = ktime.get(("num", b), 0.0) + s["t_num_bin_ms"][b]
        for b in SYM_NAMES:
            ktime[("sym", b)] = ktime.get(("sym", b), 0.0) + s["t_sym_bin_ms"][b]
    dom = max(ktime, key=ktime.get)
    dom_ms = ktime[dom] / len(pstats)
    dom_name, dom_bytes = kb[dom]
    peak, peak_kind = peaks()
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    traffic = profiled_traffic().get((args.workload, dom_name))
    bytes_alg = 12 * P + 12 * A.nnz + 4 * (A.n_rows + 1) + 12 * nnzC + 8 * (A.n_rows + 1)
    shares = {f"{kb[k][0]}": round(v / len(pstats), 4) for k, v in sorted(ktime.items(), key=lambda x: -x[1]) if v}

    line = {"metric": METRIC, "value": round(value, 4), "unit": "GFLOPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded R-MAT, numpy PCG64)",
            "config": {"workload": desc, "n": A.n_rows, "nnz": A.nnz, "products": P, "nnz_c": nnzC,
                       "rows_per_block": rpb, "scope": "kernel (inputs resident in HBM, C left in HBM)",
                       "l2": "flushed between steps (512 MiB device write outside the timed events)",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_kind": f"of {peak_kind}", "algorithmic_bytes_per_launch": dom_bytes,
                         "launch_ms": round(dom_ms, 4),
                         "pipeline": {"bytes_alg": bytes_alg, "achieved": round(bytes_alg / t_step / 1e9, 2),
                                      "frac": round(bytes_alg / t_step / 1e9 / peak, 4)},
                         "kernel_ms_per_step": shares},
            "wall_s": round(t_wall, 3)}
    line["clocks"] = clk.summary()

    if rank == 0 or world == 1:
        # e2e: the public API with host buffers (H2D of A, D2H of all of C).
        ctx.set_stream(None)
        res = ctx.spgemm(A, scope="d2h", fetch=False)
        e2e_t = []
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            res = ctx.spgemm(A, scope="d2h", fetch=False)
            e2e_t.append(time.perf_counter() - t0)
        te = float(np.mean(e2e_t))
        h2d = 4 * (A.n_rows + 1) + 12 * A.nnz
        d2h = 12 * nnzC + 8 * (A.n_rows + 1)
        line["e2e"] = {"value": round(world * 2.0 * P / te / 1e9, 4), "unit": "GFLOPS", "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": d2h, "ms_per_step": round(te * 1e3, 3),
                       "scope": "+D2H through dbd_spgemm with host (pageable) A and pinned host C"}
        scopes = {"kernel_gflops": round(2.0 * P / t_step / 1e9, 4), "d2h_gflops": round(2.0 * P / te / 1e9, 4)}
        if not args.no_io:
            tmp = tempfile.mkdtemp(prefix="dbd_io_", dir=ROOT)
            try:
                ctx.spgemm(A, scope="io", out_dir=tmp, fetch=False)
                t0 = time.perf_counter()
                r = ctx.spgemm(A, scope="io", out_dir=tmp, fetch=False)
                tio = time.perf_counter() - t0
                scopes["io_gflops"] = round(2.0 * P / tio / 1e9, 4)
                scopes["io_s"] = round(tio, 3)
                scopes["io_fsync_s"] = round(r.stats["t_fsync"], 3)
                scopes["io_bytes"] = int(r.stats["bytes_written"])
            finally:
                shutil.rmtree(tmp, ignore_errors=True)
        line["scopes"] = scopes
        if world == 1 and not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            Pc, tc = cpu_reference_port(A, threads, 1)
            line["cpu_baseline"] = {"value": round(2.0 * Pc / tc / 1e9, 4), "unit": "GFLOPS", "cores": threads,
                                    "kind": "port",
                                    "sample": "the whole workload, FP32 restatement of the reference's "
                                              "compute_CPU, row blocks of 4096, one pass"}
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
