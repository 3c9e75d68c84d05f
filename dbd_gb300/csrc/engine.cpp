// engine.cpp -- host side of libdbd: context, budgets, the row-block
// pipeline and the dynamic block distributor, and the C ABI of include/dbd.h.
//
// Reference structure (ZIP:dbd/src): main.cpp drives initialize ->
// read_CSR -> initialize_A/B -> divide_Blocks -> distribute_Workload; the
// distributor (distributeWorkload.cpp:25-223) hands row blocks to a CPU and a
// GPU pthread through plain bool flags polled every 2 us, the GPU thread
// (computeGPU.cu:15-98) runs its kernels and blocking cudaMemcpys per block on
// the default stream, and a writer pthread (writeFile.cpp) fwrites finished
// blocks in order.
//
// GB300 design: the whole matrix is categorised and symbolically sized on the
// device first; then consecutive row blocks are grouped into output chunks
// sized by the device budget.  Each chunk's numeric kernels run on the
// compute stream, its device->host copy on a copy stream (event-chained, so
// chunk i+1 computes while chunk i copies), and in the +I/O scope a writer
// thread appends finished chunks to Idx.output / Val.output in block order
// while the next chunks compute.  There is no CPU compute path.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <errno.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "../../include/dbd.h"
#include "dbd_internal.h"
#include "dbd_io.h"
#include "writer.h"

using namespace dbd;

namespace {

using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

constexpr double kGiB = 1024.0 * 1024.0 * 1024.0;

// Device allocation that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Pinned host allocation that only grows.
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

struct Operand {
    CsrDev dev;
    DevBuf ptr, idx, val, tmp;
    DevBuf bmin, bmax;  // first and last column of every row (as the right operand)
    bool loaded = false;
    int sorted = 0;
};

// A chunk: rows [r0, r1) (multiples of the tile size or m) and their output.
struct Chunk {
    int64_t r0, r1;
    int64_t c0, c1;  // Cp[r0], Cp[r1]
};

struct WriteJob {
    int64_t chunk;
    int slot;
    int64_t n;
    cudaEvent_t ready;
    int64_t r0, r1, c0;  // the chunk's rows and its first entry
    int64_t lead_i, lead_v;  // its indices / values start this many bytes into their slots
};

}  // namespace

struct dbd_ctx {
    dbd_config cfg;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr, copy_stream = nullptr, stream = nullptr;
    std::string last_error;

    Operand A, B;
    bool b_is_a = false;

    // work arrays
    DevBuf rowP, symBin, numBin, rowNnz, symList, numList, hist, symTileOff, numTileOff, symStart,
        numStart, part, Cp, cursor, err, blockP, flags;
    DevBuf Ci, Cv;           // resident product or device output ring
    DevBuf Cf;               // float32 values of each device slot (out_val_fp32 in the copying scopes)
    DevBuf ctrs;             // row counters of the persistent kernels
    DevBuf gdense;           // global dense slots of the dense bin
    int gSlots = 0;
    int64_t gStride = 0;
    DevBuf heavySlot, slabCnt;  // slab counts of heavy rows (symbolic -> dense-bin pieces)
    DevBuf items;               // dense-bin work items
    int heavyCap = 0, itemCap = 0;
    bool pieces = false;        // the dense bin cuts heavy rows into pieces in this multiply
    DevBuf dscr;             // FP64 scratch rows of the one-pass dense kernel
    int scrSlots = 0;
    int64_t scrStride = 0;
    DevBuf wideBits, wideSlot;  // column bitmaps of wide rows kept for the numeric pass
    bool wideKept = false;      // the symbolic pass of this multiply kept them
    DevBuf rowLo, rowHi;        // column window of every row of C
    // C's pattern left on the device by the last multiply (for the adjoint).
    bool patternOk = false;
    int64_t patA = -1, patB = -1;
    DevBuf adjG, adjA, adjB;    // device copies for host-side adjoint arguments
    DevBuf adjT;                // A grouped by column for the deterministic dB pass
    // Batched products: the pairs' placement (device copy of the pair
    // descriptors and offsets, staged through pinned memory), the per-row
    // column shift of the concatenated A, and the pair count of the last
    // batched multiply (0: the last multiply was a single product).
    DevBuf batchDev, rowShift;
    HostBuf batchHost;
    int64_t batchCount = 0;
    // Device-driven batched multiply (dbd_batch_plan / _enqueue / _result):
    // the planned pairs' shapes and the output's capacity.
    bool bpOk = false, bpSquare = false;
    int64_t bpCount = 0, bpCap = 0, bpColsC = 0, bpNnzB = 0, bpRowsB = 0;
    std::vector<int64_t> bpRowOff;
    std::vector<int64_t> batchNnzA, batchNnzB;  // per-pair entry offsets of the last batch (count + 1)
    // The numeric launches of the last multiply captured as a CUDA graph,
    // replayed by dbd_update_values (dropped by the next multiply).
    cudaGraph_t numGraph = nullptr;
    cudaGraphExec_t numExec = nullptr;
    bool capturing = false;
    bool replayOk = false;  // the last multiply left its plan and C on the device (kernel scope)
    Tuning tune;            // bin thresholds (dbd_set_tuning / dbd_autotune)
    int64_t m = 0, ncols = 0, nnzC = 0, products = 0;
    int64_t nblocks = 0, ntiles = 0;
    bool divided = false;
    std::vector<int64_t> blockP_h;
    std::vector<int32_t> blockCat_h;
    int32_t symStart_h[kMaxBins + 1] = {0};
    int32_t numStart_h[kMaxBins + 1] = {0};
    std::vector<int32_t> numTileOff_h;

    // Per-row digest of C (dbd_set_digest): the device digest is taken
    // after every chunk's numeric kernels, the host digest from every
    // chunk's pinned copy.  *Ok: the last multiply filled them.
    int digest = 0;
    DevBuf dgCount, dgCol, dgVal, dgSum, dgWsum, dgBad;
    DevBuf hashOut;  // operand hash of a resumable +I/O run
    bool dgDevOk = false, dgHostOk = false;
    std::vector<int64_t> hdCount;
    std::vector<uint64_t> hdCol, hdVal;
    std::vector<double> hdSum, hdWsum;
    std::atomic<int64_t> hdBad{0};

    // host result / ring
    HostBuf hCp, hCi, hCv;
    bool host_full = false;  // hCp/hCi/hCv hold the complete product
    bool host_f32 = false;   // hCv holds float32 values (out_val_fp32 in the copying scopes)
    bool dev_resident = false;
    dbd_scope last_scope = DBD_SCOPE_KERNEL;

    cudaEvent_t evStart = nullptr, evPre = nullptr, evSym = nullptr, evEnd = nullptr;
    cudaEvent_t evNumA = nullptr, evNumB = nullptr;
    dbd_stats stats;
    int launches = 0;

    // One stream per bin so that the kernels of different bins overlap.
    cudaStream_t bin_streams[kMaxBins] = {};
    // Event pools, reset at the start of every multiply (all earlier work is
    // complete by then): timing events (time_kernels) and fork/join events.
    std::vector<cudaEvent_t> tpool, spool;
    size_t tused = 0, sused = 0;
    struct Timed {
        int kind;  // 0 symbolic bin, 1 numeric bin, 2 scan + numeric binning
        int bin;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;

    cudaEvent_t time_ev(cudaStream_t s) {
        if (!cfg.time_kernels || capturing) return nullptr;
        if (tused == tpool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            tpool.push_back(e);
        }
        cudaEvent_t e = tpool[tused++];
        cudaEventRecord(e, s);
        return e;
    }
    cudaEvent_t sync_ev() {
        if (sused == spool.size()) {
            cudaEvent_t e;
            cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            spool.push_back(e);
        }
        return spool[sused++];
    }
};

namespace {

// Fork the context's stream into per-bin streams and join them back.
struct Fork {
    dbd_ctx *c;
    cudaStream_t origin;
    cudaEvent_t start;
    bool used[kMaxBins] = {};
    explicit Fork(dbd_ctx *ctx, cudaStream_t from = nullptr) : c(ctx), origin(from ? from : ctx->stream) {
        start = c->sync_ev();
        cudaEventRecord(start, origin);
    }
    cudaStream_t stream(int b) {
        if (c->cfg.time_kernels) return origin;  // serial: per-kernel events time that kernel alone
        if (!used[b]) cudaStreamWaitEvent(c->bin_streams[b], start, 0);
        used[b] = true;
        return c->bin_streams[b];
    }
    void join() {
        for (int b = 0; b < kMaxBins; ++b) {
            if (!used[b]) continue;
            cudaEvent_t e = c->sync_ev();
            cudaEventRecord(e, c->bin_streams[b]);
            cudaStreamWaitEvent(origin, e, 0);
        }
    }
};

RowInfo row_info(dbd_ctx *c) {
    RowInfo ri;
    ri.rowP = c->rowP.as<int64_t>();
    ri.lo = c->rowLo.as<int32_t>();
    ri.hi = c->rowHi.as<int32_t>();
    return ri;
}

void drop_graph(dbd_ctx *c) {
    if (c->numExec) cudaGraphExecDestroy(c->numExec);
    if (c->numGraph) cudaGraphDestroy(c->numGraph);
    c->numExec = nullptr;
    c->numGraph = nullptr;
}

int set_err(dbd_ctx *c, int code, const std::string &msg) {
    if (c) c->last_error = msg;
    return code;
}

int cuda_fail(dbd_ctx *c, cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? DBD_ERR_OOM_DEVICE : DBD_ERR_CUDA;
    return set_err(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(ctx, call)                                               \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return cuda_fail((ctx), _e, #call);  \
    } while (0)

int check_device_err(dbd_ctx *c, const char *stage) {
    int h = 0;
    CK(c, cudaMemcpyAsync(&h, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (h != DEV_OK) {
        const char *what = h == DEV_TABLE_FULL       ? "hash table full"
                           : h == DEV_COUNT_MISMATCH ? "numeric/symbolic count mismatch"
                           : h == DEV_ROW_TOO_LONG   ? "a row has more than 2^31 products"
                           : h == DEV_OUT_OF_WINDOW  ? "a column lies outside its row's window (B changed after loading?)"
                                                     : "unknown";
        return set_err(c, DBD_ERR_DEVICE_CHECK, std::string(stage) + ": device check failed: " + what);
    }
    return DBD_OK;
}

// Host-side validation of a host CSR operand (O(n + nnz)).
int validate_host(dbd_ctx *c, const dbd_csr_view *v, const char *name) {
    if (v->n_rows < 0 || v->n_cols < 0 || v->nnz < 0 || v->n_rows >= INT32_MAX || v->n_cols > INT32_MAX ||
        v->nnz > INT32_MAX)
        return set_err(c, DBD_ERR_INVALID, std::string(name) + ": size out of range");
    if (!v->row_ptr || (v->nnz > 0 && (!v->col_idx || !v->val)))
        return set_err(c, DBD_ERR_INVALID, std::string(name) + ": null array");
    if (v->on_device) return DBD_OK;
    if (v->row_ptr[0] != 0 || v->row_ptr[v->n_rows] != v->nnz)
        return set_err(c, DBD_ERR_INVALID, std::string(name) + ": row_ptr does not span [0, nnz]");
    for (int64_t r = 0; r < v->n_rows; ++r)
        if (v->row_ptr[r + 1] < v->row_ptr[r])
            return set_err(c, DBD_ERR_INVALID, std::string(name) + ": row_ptr decreases");
    for (int64_t i = 0; i < v->nnz; ++i)
        if (v->col_idx[i] < 0 || v->col_idx[i] >= v->n_cols)
            return set_err(c, DBD_ERR_INVALID, std::string(name) + ": column index out of range");
    return DBD_OK;
}

int finish_operand(dbd_ctx *c, Operand &op, const CsrDev &d);

int load_operand(dbd_ctx *c, Operand &op, const dbd_csr_view *v, const char *name) {
    int rc = validate_host(c, v, name);
    if (rc) return rc;
    op.loaded = false;
    c->batchCount = 0;
    c->replayOk = false;  // operand buffers may move: the captured numeric graph is stale
    drop_graph(c);
    CsrDev d;
    d.m = v->n_rows;
    d.n = v->n_cols;
    d.nnz = v->nnz;
    const size_t ne = (size_t)v->nnz;
    if (v->on_device) {
        // Validate on the device: row_ptr first, then indices (only once the
        // row_ptr is known to span [0, nnz]).
        CK(c, c->flags.ensure(4 * sizeof(int)));
        CK(c, cudaMemsetAsync(c->flags.p, 0, 4 * sizeof(int), c->stream));
        launch_validate_ptr(v->row_ptr, v->n_rows, v->nnz, c->flags.as<int>(), c->stream);
        int hf[4];
        CK(c, cudaMemcpyAsync(hf, c->flags.p, sizeof(hf), cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        if (hf[0]) return set_err(c, DBD_ERR_INVALID, std::string(name) + ": malformed row_ptr");
        launch_validate_idx(v->col_idx, v->nnz, v->n_cols, c->flags.as<int>() + 1, c->stream);
        CK(c, cudaMemcpyAsync(hf, c->flags.p, sizeof(hf), cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        if (hf[1]) return set_err(c, DBD_ERR_INVALID, std::string(name) + ": column index out of range");
        d.ptr = v->row_ptr;
        d.idx = v->col_idx;
        if (v->val_fp32) {
            CK(c, op.val.ensure(sizeof(double) * ne));
            launch_f32_to_f64((const float *)v->val, op.val.as<double>(), v->nnz, c->stream);
            d.val = op.val.as<double>();
        } else {
            d.val = (const double *)v->val;
        }
    } else {
        CK(c, op.ptr.ensure(sizeof(int32_t) * (size_t)(v->n_rows + 1)));
        CK(c, op.idx.ensure(sizeof(int32_t) * ne));
        CK(c, op.val.ensure(sizeof(double) * ne));
        CK(c, cudaMemcpyAsync(op.ptr.p, v->row_ptr, sizeof(int32_t) * (size_t)(v->n_rows + 1),
                              cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaMemcpyAsync(op.idx.p, v->col_idx, sizeof(int32_t) * ne, cudaMemcpyHostToDevice, c->stream));
        if (v->val_fp32) {
            CK(c, op.tmp.ensure(sizeof(float) * ne));
            CK(c, cudaMemcpyAsync(op.tmp.p, v->val, sizeof(float) * ne, cudaMemcpyHostToDevice, c->stream));
            launch_f32_to_f64(op.tmp.as<float>(), op.val.as<double>(), v->nnz, c->stream);
        } else {
            CK(c, cudaMemcpyAsync(op.val.p, v->val, sizeof(double) * ne, cudaMemcpyHostToDevice, c->stream));
        }
        d.ptr = op.ptr.as<int32_t>();
        d.idx = op.idx.as<int32_t>();
        d.val = op.val.as<double>();
    }
    return finish_operand(c, op, d);
}

// Sortedness and row column ranges of an operand now on the device.
int finish_operand(dbd_ctx *c, Operand &op, const CsrDev &d) {
    op.dev = d;
    // Row column ranges (the column windows of the products' rows) and
    // whether every row ascends strictly (cursors, plain accumulation, runs).
    CK(c, c->flags.ensure(4 * sizeof(int)));
    CK(c, cudaMemsetAsync(c->flags.as<int>() + 2, 0, sizeof(int), c->stream));
    CK(c, op.bmin.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(d.m, 1)));
    CK(c, op.bmax.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(d.m, 1)));
    launch_row_minmax(d, op.bmin.as<int32_t>(), op.bmax.as<int32_t>(), c->flags.as<int>() + 2, c->stream,
                      c->num_sms);
    int unsorted = 0;
    CK(c, cudaMemcpyAsync(&unsorted, c->flags.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    op.sorted = unsorted ? 0 : 1;
    op.loaded = true;
    c->divided = false;
    return DBD_OK;
}

const CsrDev &opB(dbd_ctx *c) { return c->b_is_a ? c->A.dev : c->B.dev; }
int opB_sorted(dbd_ctx *c) { return c->b_is_a ? c->A.sorted : c->B.sorted; }

// ---- stage 1: work estimate, segmentation, categorisation ----------------

int divide_blocks(dbd_ctx *c) {
    if (!c->A.loaded || (!c->b_is_a && !c->B.loaded))
        return set_err(c, DBD_ERR_INVALID, "load A and B before dividing blocks");
    const CsrDev &A = c->A.dev;
    const CsrDev &B = opB(c);
    if (A.n != B.m) return set_err(c, DBD_ERR_INVALID, "inner dimensions differ (A.n_cols != B.n_rows)");
    const auto t0 = Clock::now();
    drop_graph(c);  // the plan it replays is replaced
    c->launches = 0;
    c->tused = c->sused = 0;
    c->timed.clear();
    c->m = A.m;
    c->ncols = B.n;
    const int64_t m = A.m;
    const int64_t rpb = c->cfg.rows_per_block;
    c->nblocks = m > 0 ? ceil_div(m, rpb) : 0;
    c->ntiles = ceil_div(m, kTileRows);
    const size_t mm = (size_t)std::max<int64_t>(m, 1);
    const size_t nt = (size_t)c->ntiles;
    CK(c, c->rowP.ensure(sizeof(int64_t) * mm));
    CK(c, c->rowLo.ensure(sizeof(int32_t) * mm));
    CK(c, c->rowHi.ensure(sizeof(int32_t) * mm));
    CK(c, c->symBin.ensure(mm));
    CK(c, c->numBin.ensure(mm));
    CK(c, c->rowNnz.ensure(sizeof(int32_t) * mm));
    CK(c, c->symList.ensure(sizeof(int32_t) * mm));
    CK(c, c->numList.ensure(sizeof(int32_t) * mm));
    CK(c, c->hist.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->symTileOff.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->numTileOff.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->symStart.ensure(sizeof(int32_t) * (kMaxBins + 1)));
    CK(c, c->numStart.ensure(sizeof(int32_t) * (kMaxBins + 1)));
    CK(c, c->part.ensure(sizeof(int64_t) * (size_t)(ceil_div(m, kScanTile) + 1)));
    CK(c, c->Cp.ensure(sizeof(int64_t) * (mm + 1)));
    CK(c, c->cursor.ensure(2 * sizeof(int32_t) * (size_t)std::max<int64_t>(A.nnz, 1)));
    CK(c, c->err.ensure(sizeof(int)));
    CK(c, c->blockP.ensure(sizeof(int64_t) * (size_t)std::max<int64_t>(c->nblocks, 1)));

    CK(c, cudaEventRecord(c->evStart, c->stream));
    CK(c, cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
    const Operand &opb = c->b_is_a ? c->A : c->B;
    launch_row_products(A, B.ptr, opb.bmin.as<int32_t>(), opb.bmax.as<int32_t>(), row_info(c),
                        c->symBin.as<uint8_t>(), c->err.as<int>(), c->tune, c->stream, c->num_sms);
    launch_block_products(m, c->rowP.as<int64_t>(), rpb, c->blockP.as<int64_t>(), c->stream);
    Binning sb{c->symBin.as<uint8_t>(), c->symList.as<int32_t>(), c->hist.as<int32_t>(),
               c->symTileOff.as<int32_t>(), c->symStart.as<int32_t>()};
    launch_bin_lists(m, sb, SB_COUNT, c->stream);
    c->launches += 5;
    CK(c, cudaGetLastError());
    c->blockP_h.assign((size_t)c->nblocks, 0);
    if (c->nblocks)
        CK(c, cudaMemcpyAsync(c->blockP_h.data(), c->blockP.p, sizeof(int64_t) * (size_t)c->nblocks,
                              cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaMemcpyAsync(c->symStart_h, c->symStart.p, sizeof(c->symStart_h), cudaMemcpyDeviceToHost,
                          c->stream));
    CK(c, cudaEventRecord(c->evPre, c->stream));
    int rc = check_device_err(c, "work estimate");
    if (rc) return rc;

    // Segmenter + categoriser on the per-block products (host, O(blocks)).
    int64_t total = 0, mx = 0;
    for (int64_t b = 0; b < c->nblocks; ++b) {
        total += c->blockP_h[(size_t)b];
        mx = std::max(mx, c->blockP_h[(size_t)b]);
    }
    c->products = total;
    int32_t crit = 0;
    if (c->nblocks > 0) {
        const int64_t avg = (total / c->nblocks) / rpb;
        float var = 0.0f;
        for (int64_t b = 0; b < c->nblocks; ++b) {
            const int64_t d = avg - c->blockP_h[(size_t)b] / rpb;
            var += (float)(d * d);
        }
        var /= (float)c->nblocks;
        crit = (int32_t)(1.28f * std::sqrt(var)) + (int32_t)avg;
    }
    c->blockCat_h.assign((size_t)c->nblocks, 0);
    memset(&c->stats, 0, sizeof(c->stats));
    for (int64_t b = 0; b < c->nblocks; ++b) {
        const int64_t avgb = c->blockP_h[(size_t)b] / rpb;
        const int cat = avgb > crit ? 0 : (avgb <= 64 ? 1 : 2);
        c->blockCat_h[(size_t)b] = cat;
        c->stats.blocks_per_category[cat]++;
    }
    c->stats.products = total;
    c->stats.n_blocks = c->nblocks;
    c->stats.max_block_products = mx;
    c->stats.criteria = crit;
    for (int q = 0; q < SB_COUNT; ++q) c->stats.sym_rows_per_bin[q] = c->symStart_h[q + 1] - c->symStart_h[q];
    c->stats.t_preprocess = seconds_since(t0);
    c->divided = true;
    if (c->cfg.verbose)
        printf("Divide Matrix A into %lld Blocks (Block Size: %lld)\n\n", (long long)c->nblocks, (long long)rpb);
    return DBD_OK;
}

// ---- stage 2: symbolic over all rows, row_ptr, numeric bins --------------

int symbolic(dbd_ctx *c) {
    const int64_t m = c->m;
    CK(c, cudaMemsetAsync(c->rowNnz.p, 0, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1), c->stream));
    SymArgs sa;
    sa.A = c->A.dev;
    sa.B = opB(c);
    sa.list = c->symList.as<int32_t>();
    sa.binStart = c->symStart.as<int32_t>();
    sa.rowNnz = c->rowNnz.as<int32_t>();
    CK(c, c->ctrs.ensure(sizeof(uint32_t) * CTR_COUNT));
    CK(c, cudaMemsetAsync(c->ctrs.p, 0, sizeof(uint32_t) * CTR_COUNT, c->stream));
    sa.ctr = c->ctrs.as<uint32_t>();
    sa.numSms = c->num_sms;
    sa.bSorted = opB_sorted(c);
    sa.err = c->err.as<int>();
    sa.rowLo = c->rowLo.as<int32_t>();
    sa.rowP = c->rowP.as<int64_t>();
    sa.rowHi = c->rowHi.as<int32_t>();
    sa.tune = c->tune;
    // Slab counts of heavy rows for the dense bin's pieces (rank windows,
    // B's rows ascending): at most one slot per kHeavyP products.
    c->heavyCap = 0;
    c->pieces = false;
    if (c->tune.denseMethod == 0 && opB_sorted(c) && c->products >= kHeavyP) {
        const int64_t cap = std::min<int64_t>({m, c->products / kHeavyP, 262144});
        CK(c, c->heavySlot.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1)));
        CK(c, c->slabCnt.ensure(sizeof(int32_t) * (size_t)kMaxSlabs * (size_t)cap));
        CK(c, cudaMemsetAsync(c->heavySlot.p, 0xff, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1), c->stream));
        sa.heavySlot = c->heavySlot.as<int32_t>();
        sa.slabCnt = c->slabCnt.as<int32_t>();
        sa.heavyCap = (int)cap;
        c->heavyCap = (int)cap;
    }
    // Keep the wide rows' column bitmaps (one slot of kRankWordsMax words per
    // wide row) for the numeric rank kernels when the store stays within an
    // eighth of the GPU budget.
    c->wideKept = false;
    {
        const int64_t nwide = c->symStart_h[SB_WIDE + 1] - c->symStart_h[SB_WIDE];
        const double bytes = 4.0 * (double)kRankWordsMax * (double)nwide;
        if (nwide > 0 && bytes <= c->cfg.gpu_gib * kGiB / 8) {
            CK(c, c->wideBits.ensure((size_t)bytes));
            CK(c, c->wideSlot.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1)));
            sa.wideBits = c->wideBits.as<uint32_t>();
            sa.wideSlot = c->wideSlot.as<int32_t>();
            c->wideKept = true;
        }
    }
    // Bins run concurrently, one stream each (heaviest first).
    static const int sorder[] = {SB_WIDE, SB_HCTA, SB_HWARP, SB_BITW, SB_TINY};
    Fork fk(c);
    for (int b : sorder) {
        const int32_t n = c->symStart_h[b + 1] - c->symStart_h[b];
        if (n <= 0) continue;
        cudaStream_t s = fk.stream(b);
        cudaEvent_t e0 = c->time_ev(s);
        launch_symbolic_bin(sa, b, c->symStart_h[b], n, s, &c->launches);
        if (e0) c->timed.push_back({0, b, e0, c->time_ev(s)});
    }
    fk.join();
    cudaEvent_t es = c->time_ev(c->stream);
    launch_row_scan(m, c->rowNnz.as<int32_t>(), c->part.as<int64_t>(), c->Cp.as<int64_t>(), c->stream);
    launch_num_bins(m, c->A.dev.ptr, row_info(c), c->rowNnz.as<int32_t>(), c->numBin.as<uint8_t>(), c->tune, c->stream,
                    c->num_sms);
    Binning nb{c->numBin.as<uint8_t>(), c->numList.as<int32_t>(), c->hist.as<int32_t>(),
               c->numTileOff.as<int32_t>(), c->numStart.as<int32_t>()};
    launch_bin_lists(m, nb, NB_COUNT, c->stream);
    if (es) c->timed.push_back({2, 0, es, c->time_ev(c->stream)});
    c->launches += 7;
    CK(c, cudaGetLastError());
    CK(c, cudaMemcpyAsync(&c->nnzC, c->Cp.as<int64_t>() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaMemcpyAsync(c->numStart_h, c->numStart.p, sizeof(c->numStart_h), cudaMemcpyDeviceToHost, c->stream));
    uint32_t heavy = 0;
    if (c->heavyCap > 0)
        CK(c, cudaMemcpyAsync(&heavy, c->ctrs.as<uint32_t>() + CTR_HEAVY, sizeof(heavy), cudaMemcpyDeviceToHost,
                              c->stream));
    c->numTileOff_h.assign((size_t)kMaxBins * (size_t)(c->ntiles + 1), 0);
    CK(c, cudaMemcpyAsync(c->numTileOff_h.data(), c->numTileOff.p, sizeof(int32_t) * c->numTileOff_h.size(),
                          cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaEventRecord(c->evSym, c->stream));
    int rc = check_device_err(c, "symbolic");
    if (rc) return rc;
    for (int q = 0; q < NB_COUNT; ++q) c->stats.rows_per_bin[q] = c->numStart_h[q + 1] - c->numStart_h[q];
    c->stats.nnz_c = c->nnzC;
    // Dense-bin work items: one per row plus the extra pieces of heavy rows
    // (at most kMaxSlabs per recorded row).
    const int64_t nDense = c->numStart_h[NB_DENSE + 1] - c->numStart_h[NB_DENSE];
    const int64_t nHeavy = std::min<int64_t>((int64_t)heavy, c->heavyCap);
    c->stats.heavy_rows = nHeavy;
    if (c->heavyCap > 0 && nHeavy > 0 && nDense > 0) {
        const int64_t icap = nDense + nHeavy * (kMaxSlabs - 1);
        if (icap < INT32_MAX) {
            CK(c, c->items.ensure(sizeof(DenseItem) * (size_t)icap));
            c->itemCap = (int)icap;
            c->pieces = true;
        }
    }
    if (c->nnzC > INT64_MAX / 16) return set_err(c, DBD_ERR_OVERFLOW, "nnz(C) too large");
    return DBD_OK;
}

// Numeric kernels of every bin restricted to rows [r0, r1).
void numeric_rows(dbd_ctx *c, int64_t r0, int64_t r1, int64_t outBase, int32_t *Ci, double *Cv) {
    NumArgs na;
    na.A = c->A.dev;
    na.B = opB(c);
    na.list = c->numList.as<int32_t>();
    na.Cp = c->Cp.as<int64_t>();
    na.outBase = outBase;
    na.Ci = Ci;
    na.Cv = Cv;
    na.state = c->cursor.as<int32_t>();
    na.bSorted = opB_sorted(c);
    na.err = c->err.as<int>();
    na.rowP = c->rowP.as<int64_t>();
    na.rowLo = c->rowLo.as<int32_t>();
    na.rowHi = c->rowHi.as<int32_t>();
    na.tune = c->tune;
    na.numSms = c->num_sms;
    na.ctr = c->ctrs.as<uint32_t>();
    if (c->gSlots > 0) {
        const size_t slot = gdense_slot_bytes(c->gStride);
        char *base = c->gdense.as<char>();
        na.gBits = reinterpret_cast<uint32_t *>(base);
        na.gWpre = reinterpret_cast<uint32_t *>(base + (size_t)c->gSlots * (c->gStride / 8));
        na.gStride = c->gStride;
        na.gSlots = c->gSlots;
        (void)slot;
    }
    if (c->pieces) {
        na.heavySlot = c->heavySlot.as<int32_t>();
        na.slabCnt = c->slabCnt.as<int32_t>();
        na.items = c->items.as<DenseItem>();
        na.itemCap = c->itemCap;
    }
    if (c->scrSlots > 0) {
        na.scr = c->dscr.as<double>();
        na.scrStride = c->scrStride;
        na.scrSlots = c->scrSlots;
    }
    if (c->wideKept) {
        na.wideBits = c->wideBits.as<uint32_t>();
        na.wideSlot = c->wideSlot.as<int32_t>();
    }
    if (c->batchCount > 0) na.colShift = c->rowShift.as<int32_t>();
    const int64_t t0 = r0 / kTileRows;
    const int64_t t1 = (r1 >= c->m) ? c->ntiles : r1 / kTileRows;
    // Bins run concurrently, one stream each; heaviest first so that their
    // long CTAs start early.
    static const int order[] = {NB_DENSE, NB_RANKL, NB_HCTA_L, NB_RANKS, NB_HCTA_S,
                                NB_HWARP, NB_RANKM, NB_RANKW, NB_DENSEW, NB_TINY};
    Fork fk(c);
    for (int b : order) {
        const int32_t lo = c->numTileOff_h[(size_t)t0 * kMaxBins + b];
        const int32_t hi = c->numTileOff_h[(size_t)t1 * kMaxBins + b];
        if (hi <= lo) continue;
        cudaStream_t s = fk.stream(b);
        cudaEvent_t e0 = c->time_ev(s);
        launch_numeric_bin(na, b, lo, hi, s, &c->launches);
        if (e0) c->timed.push_back({1, b, e0, c->time_ev(s)});
    }
    fk.join();
}

// Chunks of consecutive row blocks from block b0 on whose output fits cap_entries.
int plan_chunks(dbd_ctx *c, const std::vector<int64_t> &cpBlk, int64_t cap_entries, int64_t b0,
                std::vector<Chunk> &out) {
    out.clear();
    const int64_t nb = c->nblocks;
    const int64_t rpb = c->cfg.rows_per_block;
    int64_t b = b0;
    while (b < nb) {
        int64_t e = b + 1;
        if (cpBlk[(size_t)e] - cpBlk[(size_t)b] > cap_entries)
            return set_err(c, DBD_ERR_BUDGET, "one row block's output exceeds the device output buffer");
        while (e < nb && cpBlk[(size_t)e + 1] - cpBlk[(size_t)b] <= cap_entries) ++e;
        Chunk ch;
        ch.r0 = b * rpb;
        ch.r1 = std::min(c->m, e * rpb);
        ch.c0 = cpBlk[(size_t)b];
        ch.c1 = cpBlk[(size_t)e];
        out.push_back(ch);
        b = e;
    }
    return DBD_OK;
}

std::string join_path(const char *dir, const char *name) {
    std::string d = (dir && *dir) ? dir : ".";
    if (d.back() != '/') d += '/';
    return d + name;
}

// ---- host digest of C (the same per-row summary as k_digest.cu) ----------

uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void neumaier_add(double &s, double &c, double x) {
    const double t = s + x;
    if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// Digest of rows [r0, r1) of a host copy whose entries sit at Cp[r] - base,
// split over host threads by entries.
template <class V>
void host_digest_rows(dbd_ctx *c, const int64_t *Cp, int64_t r0, int64_t r1, int64_t base, const int32_t *ci,
                      const V *cv) {
    const int64_t ncols = c->ncols;
    auto run = [&](int64_t a, int64_t b) {
        int64_t bad = 0;
        for (int64_t r = a; r < b; ++r) {
            const int64_t e0 = Cp[r] - base, e1 = Cp[r + 1] - base;
            uint64_t h = 0, hv = 0;
            double s = 0, sc = 0, w = 0, wc = 0;
            bool rbad = false;
            for (int64_t i = e0; i < e1; ++i) {
                const int32_t col = ci[i];
                const double v = (double)cv[i];
                if (col < 0 || (int64_t)col >= ncols || (i > e0 && ci[i - 1] >= col)) rbad = true;
                uint64_t bits;
                memcpy(&bits, &v, sizeof(bits));
                h += mix64((uint64_t)(uint32_t)col);
                hv += mix64(bits + 0x9E3779B97F4A7C15ull * ((uint64_t)(uint32_t)col + 1));
                neumaier_add(s, sc, v);
                const double wt = 0.5 + (double)(mix64((uint64_t)(uint32_t)col) >> 11) * 0x1.0p-53;
                neumaier_add(w, wc, v * wt);
            }
            c->hdCount[(size_t)r] = e1 - e0;
            c->hdCol[(size_t)r] = h;
            c->hdVal[(size_t)r] = hv;
            c->hdSum[(size_t)r] = s + sc;
            c->hdWsum[(size_t)r] = w + wc;
            bad += rbad;
        }
        if (bad) c->hdBad += bad;
    };
    const int64_t entries = Cp[r1] - Cp[r0];
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)std::thread::hardware_concurrency(), 32,
                                                                entries / (1 << 20) + 1, r1 - r0}));
    if (nt <= 1) {
        run(r0, r1);
        return;
    }
    std::vector<std::thread> th;
    int64_t a = r0;
    for (int t = 1; t <= nt; ++t) {
        // First row whose start passes t/nt of the chunk's entries.
        const int64_t goal = Cp[r0] + entries * t / nt;
        int64_t b = t == nt ? r1 : (int64_t)(std::lower_bound(Cp + a, Cp + r1, goal) - Cp);
        b = std::max(b, a);
        if (b > a) th.emplace_back(run, a, b);
        a = b;
    }
    for (auto &x : th) x.join();
}

// Identity of the product for a resumable +I/O run: the operands' sizes,
// C's row pointers (host copy) and a device hash of the operands' arrays.
int product_fingerprint(dbd_ctx *c, uint64_t *out) {
    CK(c, c->hashOut.ensure(sizeof(uint64_t)));
    CK(c, cudaMemsetAsync(c->hashOut.p, 0, sizeof(uint64_t), c->stream));
    const CsrDev &A = c->A.dev, &B = opB(c);
    launch_hash_words(reinterpret_cast<const uint32_t *>(A.ptr), A.m + 1, 1, c->hashOut.as<uint64_t>(), c->stream);
    launch_hash_words(reinterpret_cast<const uint32_t *>(A.idx), A.nnz, 2, c->hashOut.as<uint64_t>(), c->stream);
    launch_hash_words(reinterpret_cast<const uint32_t *>(A.val), 2 * A.nnz, 3, c->hashOut.as<uint64_t>(), c->stream);
    launch_hash_words(reinterpret_cast<const uint32_t *>(B.ptr), B.m + 1, 4, c->hashOut.as<uint64_t>(), c->stream);
    launch_hash_words(reinterpret_cast<const uint32_t *>(B.idx), B.nnz, 5, c->hashOut.as<uint64_t>(), c->stream);
    launch_hash_words(reinterpret_cast<const uint32_t *>(B.val), 2 * B.nnz, 6, c->hashOut.as<uint64_t>(), c->stream);
    c->launches += 6;
    uint64_t h = 0;
    CK(c, cudaMemcpyAsync(&h, c->hashOut.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    const int64_t *cp = c->hCp.as<int64_t>();
    for (int64_t r = 0; r <= c->m; ++r) h += mix64((uint64_t)cp[r] ^ mix64((uint64_t)r));
    for (int64_t x : {c->m, c->ncols, c->nnzC, c->products, A.nnz, B.nnz}) h = mix64(h ^ (uint64_t)x);
    *out = h;
    return DBD_OK;
}

// ---- stage 3: the distributor --------------------------------------------

int distribute(dbd_ctx *c, dbd_scope scope, const char *out_dir) {
    if (!c->divided) {
        int rc = divide_blocks(c);
        if (rc) return rc;
    }
    c->divided = false;  // the bin lists are consumed by this multiply
    c->patternOk = false;
    c->replayOk = false;
    const auto t0 = Clock::now();
    int rc = symbolic(c);
    if (rc) return rc;
    // Global dense slots for the dense bin: up to two per SM, within an
    // eighth of the GPU budget; too few fit -> shared-memory windows.
    c->gSlots = 0;
    if (c->tune.denseMethod == 1 && c->numStart_h[NB_DENSE + 1] > c->numStart_h[NB_DENSE]) {
        const int64_t stride = (c->ncols + 1023) / 1024 * 1024;
        const size_t slot = gdense_slot_bytes(stride);
        const int64_t fit = (int64_t)(c->cfg.gpu_gib * kGiB / 8 / (double)slot);
        const int slots = (int)std::min<int64_t>(2 * (int64_t)c->num_sms, fit);
        if (slots >= c->num_sms / 2 && slots > 0 && stride / 1024 <= kGdenseSumMax) {
            CK(c, c->gdense.ensure(slot * (size_t)slots));
            CK(c, cudaMemsetAsync(c->gdense.p, 0, slot * (size_t)slots, c->stream));
            c->gSlots = slots;
            c->gStride = stride;
        }
    }
    // FP64 scratch rows of the one-pass dense kernel: one per SM, as wide as
    // 2^20 columns (at least the kernel's 2^19-column window) or C, within an
    // eighth of the GPU budget;
    // zeroed here, and the kernel leaves them zero behind every row.
    c->scrSlots = 0;
    if (c->tune.denseMethod == 3 && c->numStart_h[NB_DENSE + 1] > c->numStart_h[NB_DENSE]) {
        const int64_t stride = std::min<int64_t>((int64_t)1 << 20, (c->ncols + 31) / 32 * 32);
        const size_t bytes = sizeof(double) * (size_t)stride * (size_t)c->num_sms;
        if ((double)bytes <= c->cfg.gpu_gib * kGiB / 8) {
            CK(c, c->dscr.ensure(bytes));
            CK(c, cudaMemsetAsync(c->dscr.p, 0, bytes, c->stream));
            c->scrSlots = c->num_sms;
            c->scrStride = stride;
        }
    }
    const int64_t m = c->m, nnz = c->nnzC;
    const double gpu_budget = c->cfg.gpu_gib * kGiB;
    const double host_budget = c->cfg.host_gib * kGiB;
    size_t free_b = 0, total_b = 0;
    CK(c, cudaMemGetInfo(&free_b, &total_b));
    // Device memory already held by operands and work arrays.
    const double used = (double)(c->A.ptr.cap + c->A.idx.cap + c->A.val.cap + c->B.ptr.cap + c->B.idx.cap +
                                 c->B.val.cap + c->rowP.cap + c->symBin.cap + c->numBin.cap + c->rowNnz.cap +
                                 c->symList.cap + c->numList.cap + c->hist.cap + c->symTileOff.cap +
                                 c->numTileOff.cap + c->part.cap + c->Cp.cap + c->cursor.cap +
                                 (c->gSlots ? c->gdense.cap : 0) + (c->scrSlots ? c->dscr.cap : 0) +
                                 c->wideBits.cap + c->heavySlot.cap + c->slabCnt.cap + c->items.cap);
    const double dev_avail = std::min(gpu_budget - used, (double)free_b - 512.0 * 1024 * 1024);
    const bool copies = scope != DBD_SCOPE_KERNEL;
    // The reference's output layout (float32 values): the copying scopes
    // round each chunk's FP64 values once on the device, so 8 bytes per
    // entry cross the link instead of 12.  Device slots then hold 16 bytes
    // per entry (FP64 accumulators + their float32 copy).
    const bool f32out = copies && c->cfg.out_val_fp32 != 0;
    const double dev_bpe = f32out ? 16.0 : 12.0;
    const double host_bpe = f32out ? 8.0 : 12.0;
    const size_t hve = f32out ? sizeof(float) : sizeof(double);  // host bytes per value
    const double out_bytes = 12.0 * (double)nnz;
    const bool resident = out_bytes <= std::max(0.0, dev_avail) && scope == DBD_SCOPE_KERNEL;
    const bool host_fits = host_bpe * (double)nnz + 8.0 * (double)(m + 1) <= host_budget;

    int64_t bytes_d2h = 0;
    // The copying scopes bring all of C's row pointers to the host first:
    // Ptr.output, the host digest and a resumed run's start need them.
    if (copies) {
        CK(c, c->hCp.ensure(sizeof(int64_t) * (size_t)(m + 1)));
        CK(c, cudaMemcpyAsync(c->hCp.p, c->Cp.p, sizeof(int64_t) * (size_t)(m + 1), cudaMemcpyDeviceToHost,
                              c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        bytes_d2h += 8 * (m + 1);
    }
    // The +I/O writer opens before the chunks are planned: a resumed run
    // starts after the last row its files hold durably.
    struct WriterGuard {
        ChunkWriter *w = nullptr;
        ~WriterGuard() { writer_close(w); }
    } wg;
    int64_t resume_row = 0;
    if (scope == DBD_SCOPE_IO) {
        WriterOpts wo;
        wo.direct = c->cfg.io_buffered == 0;
        wo.val_fp32 = c->cfg.out_val_fp32 != 0;
        wo.src_fp32 = f32out;
        wo.ptr32 = c->cfg.out_ptr32 == 1 || (c->cfg.out_ptr32 == 2 && nnz <= INT32_MAX);
        wo.rotate_bytes = c->cfg.io_rotate_gib > 0 ? (int64_t)(c->cfg.io_rotate_gib * kGiB) : 0;
        wo.resume = c->cfg.io_resume != 0;
        wo.m = m;
        wo.nnz = nnz;
        if (wo.resume) {
            rc = product_fingerprint(c, &wo.fingerprint);
            if (rc) return rc;
        }
        std::string err;
        rc = writer_open(out_dir ? out_dir : ".", wo, &wg.w, &resume_row, &err);
        if (rc) return set_err(c, rc, err);
        if (resume_row % c->cfg.rows_per_block != 0 && resume_row != m)
            return set_err(c, DBD_ERR_INVALID, "the progress manifest does not end on a row block");
    }
    ChunkWriter *wr = wg.w;
    const int64_t b0 = resume_row / c->cfg.rows_per_block;

    std::vector<Chunk> chunks;
    int64_t cap_entries = nnz;
    // Chunks are large, so that the heaviest rows of a power-law matrix are
    // a small share of a launch's work.  The kernel scope copies nothing
    // out: one slot takes the whole remaining budget.  The copying scopes
    // keep two device slots (a chunk computes while the previous one is
    // copied) and two host ring slots, each a sixth of C's host bytes
    // clamped to [1, 6] GiB (and within both budgets): at least six chunks
    // overlap their copies with compute when C is small, and a large C
    // keeps its chunks large (slots of 11.5 GiB copied slower than 6 GiB
    // ones).
    const int nslots_dev = copies ? 2 : 1;
    if (resident) {
        Chunk ch{0, m, 0, nnz};
        chunks.push_back(ch);
    } else {
        double slot_entries_f = std::max(0.0, dev_avail) / nslots_dev / dev_bpe;
        if (copies) {
            double host_slot = std::min(6.0 * kGiB, std::max(1.0 * kGiB, host_bpe * (double)nnz / 6.0));
            if (!(scope == DBD_SCOPE_D2H && host_fits)) host_slot = std::min(host_slot, host_budget / 2.0);
            slot_entries_f = std::min(slot_entries_f, host_slot / host_bpe);
        }
        cap_entries = std::max<int64_t>((int64_t)slot_entries_f, 1);
        std::vector<int64_t> cpBlk((size_t)c->nblocks + 1);
        // Cp at block boundaries (from the host copy, or a strided copy of
        // one int64 per block).
        if (copies) {
            for (int64_t b = 0; b < c->nblocks; ++b)
                cpBlk[(size_t)b] = c->hCp.as<int64_t>()[b * c->cfg.rows_per_block];
        } else if (c->nblocks > 0) {
            const size_t pitch = sizeof(int64_t) * (size_t)c->cfg.rows_per_block;
            CK(c, cudaMemcpy2DAsync(cpBlk.data(), sizeof(int64_t), c->Cp.p, pitch, sizeof(int64_t),
                                    (size_t)c->nblocks, cudaMemcpyDeviceToHost, c->stream));
            CK(c, cudaStreamSynchronize(c->stream));
        }
        cpBlk[(size_t)c->nblocks] = nnz;
        int64_t maxblk = 0;
        for (int64_t b = b0; b < c->nblocks; ++b) maxblk = std::max(maxblk, cpBlk[(size_t)b + 1] - cpBlk[(size_t)b]);
        if (maxblk > cap_entries) {
            if ((double)maxblk * dev_bpe * nslots_dev > std::max(0.0, dev_avail))
                return set_err(c, DBD_ERR_BUDGET, "a row block's output does not fit the GPU budget");
            cap_entries = maxblk;
        }
        rc = plan_chunks(c, cpBlk, cap_entries, b0, chunks);
        if (rc) return rc;
    }
    c->stats.n_chunks = (int32_t)chunks.size();
    const int nslots = resident ? 1 : nslots_dev;
    const size_t slot_entries = resident ? (size_t)std::max<int64_t>(nnz, 1) : (size_t)cap_entries;
    CK(c, c->Ci.ensure(sizeof(int32_t) * slot_entries * nslots));
    CK(c, c->Cv.ensure(sizeof(double) * slot_entries * nslots));
    if (f32out) CK(c, c->Cf.ensure(sizeof(float) * slot_entries * nslots));
    c->dev_resident = resident;
    c->host_f32 = f32out;

    // Host side of D2H / IO.
    c->host_full = false;
    int nhslots = 0;
    // Ring slots leave 4 KiB of lead room on both sides of a chunk, so that
    // an O_DIRECT writer finds every chunk at its file offset modulo 4 KiB.
    const size_t si = (size_t)writer_slot_bytes((int64_t)slot_entries, 4);
    const size_t sv = (size_t)writer_slot_bytes((int64_t)slot_entries, (int64_t)hve);
    if (scope == DBD_SCOPE_D2H && host_fits) {
        CK(c, c->hCi.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1)));
        CK(c, c->hCv.ensure(hve * (size_t)std::max<int64_t>(nnz, 1)));
        c->host_full = true;
    } else if (scope != DBD_SCOPE_KERNEL) {
        nhslots = 2;
        const double ring = (double)nhslots * (double)(si + sv);
        if (ring > host_budget) return set_err(c, DBD_ERR_BUDGET, "host budget smaller than the output ring");
        CK(c, c->hCi.ensure(si * nhslots));
        CK(c, c->hCv.ensure(sv * nhslots));
    }

    // Digests of this multiply.
    c->dgDevOk = c->dgHostOk = false;
    const bool dev_dg = (c->digest & DBD_DIGEST_DEVICE) != 0;
    const bool host_dg = (c->digest & DBD_DIGEST_HOST) != 0 && scope != DBD_SCOPE_KERNEL;
    RowDigest rd;
    if (dev_dg) {
        const size_t mm = (size_t)std::max<int64_t>(m, 1);
        CK(c, c->dgCount.ensure(sizeof(int64_t) * mm));
        CK(c, c->dgCol.ensure(sizeof(uint64_t) * mm));
        CK(c, c->dgVal.ensure(sizeof(uint64_t) * mm));
        CK(c, c->dgSum.ensure(sizeof(double) * mm));
        CK(c, c->dgWsum.ensure(sizeof(double) * mm));
        CK(c, c->dgBad.ensure(sizeof(int64_t)));
        CK(c, cudaMemsetAsync(c->dgBad.p, 0, sizeof(int64_t), c->stream));
        rd.count = c->dgCount.as<int64_t>();
        rd.colHash = c->dgCol.as<uint64_t>();
        rd.valHash = c->dgVal.as<uint64_t>();
        rd.sum = c->dgSum.as<double>();
        rd.wsum = c->dgWsum.as<double>();
        rd.bad = c->dgBad.as<int64_t>();
    }
    if (host_dg) {
        c->hdCount.assign((size_t)m, 0);
        c->hdCol.assign((size_t)m, 0);
        c->hdVal.assign((size_t)m, 0);
        c->hdSum.assign((size_t)m, 0.0);
        c->hdWsum.assign((size_t)m, 0.0);
        c->hdBad = 0;
    }
    // Host slots are handed to a consumer thread (file writes, host digest)
    // unless the whole product lands in host memory.
    const bool consume = scope == DBD_SCOPE_IO || (host_dg && !c->host_full);

    // Consumer thread state.
    std::atomic<int> werr{0};
    std::string wmsg;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<WriteJob> jobs;
    std::vector<int64_t> slot_owner((size_t)std::max(nhslots, 1), -1);  // chunk using host slot, -1 free
    bool done = false;
    std::thread th;
    if (consume) {
        th = std::thread([&]() {
            for (;;) {
                WriteJob j;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return done || !jobs.empty(); });
                    if (jobs.empty()) return;
                    j = jobs.front();
                    jobs.pop_front();
                }
                if (cudaEventSynchronize(j.ready) != cudaSuccess && !werr) {
                    wmsg = "writer: copy event failed";
                    werr = DBD_ERR_CUDA;
                }
                char *ib = c->hCi.as<char>() + (size_t)j.slot * si;
                char *vb = c->hCv.as<char>() + (size_t)j.slot * sv;
                if (!werr && host_dg) {
                    const int32_t *ci = reinterpret_cast<const int32_t *>(ib + j.lead_i);
                    if (f32out)
                        host_digest_rows(c, c->hCp.as<int64_t>(), j.r0, j.r1, j.c0, ci,
                                         reinterpret_cast<const float *>(vb + j.lead_v));
                    else
                        host_digest_rows(c, c->hCp.as<int64_t>(), j.r0, j.r1, j.c0, ci,
                                         reinterpret_cast<const double *>(vb + j.lead_v));
                }
                if (!werr && wr) {
                    std::string err;
                    int e = writer_append(wr, ib, vb, j.n, j.r1, &err);
                    if (e) {
                        wmsg = err;
                        werr = e;
                    }
                }
                {
                    std::lock_guard<std::mutex> lk(mu);
                    slot_owner[(size_t)j.slot] = -1;
                }
                cv.notify_all();
            }
        });
    }

    // Events per chunk for the two-stream pipeline: the start and end of
    // each chunk's numeric work and of its copy (the ends also order the
    // streams).
    std::vector<cudaEvent_t> evNum(chunks.size()), evCopy(chunks.size()), evNum0(chunks.size()),
        evCopy0(chunks.size());
    for (size_t i = 0; i < chunks.size(); ++i) {
        cudaEventCreate(&evNum[i]);
        cudaEventCreate(&evCopy[i]);
        cudaEventCreate(&evNum0[i]);
        cudaEventCreate(&evCopy0[i]);
    }
    double t_d2h_issue = 0.0;
    CK(c, cudaEventRecord(c->evNumA, c->stream));
    int loop_rc = DBD_OK;
    for (size_t i = 0; i < chunks.size() && !loop_rc; ++i) {
        const Chunk &ch = chunks[i];
        const int ds = resident ? 0 : (int)(i % nslots);
        int32_t *dCi = c->Ci.as<int32_t>() + (resident ? 0 : (size_t)ds * slot_entries);
        double *dCv = c->Cv.as<double>() + (resident ? 0 : (size_t)ds * slot_entries);
        // The device slot is free once its previous chunk's copy finished.
        if (!resident && i >= (size_t)nslots && scope != DBD_SCOPE_KERNEL)
            cudaStreamWaitEvent(c->stream, evCopy[i - nslots], 0);
        cudaEventRecord(evNum0[i], c->stream);
        numeric_rows(c, ch.r0, ch.r1, ch.c0, dCi, dCv);
        float *dCf = f32out ? c->Cf.as<float>() + (size_t)ds * slot_entries : nullptr;
        if (f32out && ch.c1 > ch.c0) {
            launch_val_to_f32(dCv, dCf, ch.c1 - ch.c0, c->stream, c->num_sms);
            c->launches++;
        }
        if (dev_dg) {
            // The digest describes the values as they leave the device.
            if (f32out)
                launch_row_digest(ch.r0, ch.r1, c->Cp.as<int64_t>(), ch.c0, dCi, dCf, c->ncols, rd, c->stream,
                                  c->num_sms);
            else
                launch_row_digest(ch.r0, ch.r1, c->Cp.as<int64_t>(), ch.c0, dCi, dCv, c->ncols, rd, c->stream,
                                  c->num_sms);
            c->launches++;
        }
        cudaEventRecord(evNum[i], c->stream);
        if (scope == DBD_SCOPE_KERNEL) continue;
        const int64_t n = ch.c1 - ch.c0;
        int32_t *hCi;
        char *hCv;  // doubles, or floats with f32out
        int hs = 0;
        const int64_t lead_i = wr ? writer_lead_for(wr, ch.c0, 0) : 0;
        const int64_t lead_v = wr ? writer_lead_for(wr, ch.c0, 1) : 0;
        if (c->host_full) {
            hCi = c->hCi.as<int32_t>() + ch.c0;
            hCv = c->hCv.as<char>() + hve * (size_t)ch.c0;
        } else {
            hs = (int)(i % nhslots);
            if (consume) {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return slot_owner[(size_t)hs] < 0 || werr; });
                slot_owner[(size_t)hs] = (int64_t)i;
            } else if (i >= (size_t)nhslots) {
                // d2h scope with a ring: the host slot is overwritten, as the
                // reference's bin/d2h reuses one pinned buffer (preProc.cu:94-95).
            }
            hCi = reinterpret_cast<int32_t *>(c->hCi.as<char>() + (size_t)hs * si + lead_i);
            hCv = c->hCv.as<char>() + (size_t)hs * sv + lead_v;
        }
        const auto ti = Clock::now();
        cudaStreamWaitEvent(c->copy_stream, evNum[i], 0);
        cudaEventRecord(evCopy0[i], c->copy_stream);
        if (n > 0) {
            cudaError_t e1 = cudaMemcpyAsync(hCi, dCi, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost,
                                             c->copy_stream);
            cudaError_t e2 = f32out ? cudaMemcpyAsync(hCv, dCf, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost,
                                                      c->copy_stream)
                                    : cudaMemcpyAsync(hCv, dCv, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost,
                                                      c->copy_stream);
            if (e1 != cudaSuccess || e2 != cudaSuccess) loop_rc = cuda_fail(c, e1 != cudaSuccess ? e1 : e2, "D2H");
        }
        cudaEventRecord(evCopy[i], c->copy_stream);
        bytes_d2h += (int64_t)(4 + hve) * n;
        t_d2h_issue += seconds_since(ti);
        if (consume) {
            {
                std::lock_guard<std::mutex> lk(mu);
                jobs.push_back(WriteJob{(int64_t)i, hs, n, evCopy[i], ch.r0, ch.r1, ch.c0, lead_i, lead_v});
            }
            cv.notify_all();
        }
    }
    CK(c, cudaEventRecord(c->evNumB, c->stream));
    cudaError_t se = cudaStreamSynchronize(c->stream);
    cudaError_t ce = cudaStreamSynchronize(c->copy_stream);
    if (consume) {
        {
            std::lock_guard<std::mutex> lk(mu);
            done = true;
        }
        cv.notify_all();
        th.join();
    }
    double chunks_ms = 0.0, copy_ms = 0.0;
    for (size_t i = 0; i < chunks.size(); ++i) {
        float x = 0.f;
        if (!se && cudaEventElapsedTime(&x, evNum0[i], evNum[i]) == cudaSuccess) chunks_ms += x;
        if (!se && !ce && scope != DBD_SCOPE_KERNEL && cudaEventElapsedTime(&x, evCopy0[i], evCopy[i]) == cudaSuccess)
            copy_ms += x;
        cudaEventDestroy(evNum[i]);
        cudaEventDestroy(evCopy[i]);
        cudaEventDestroy(evNum0[i]);
        cudaEventDestroy(evCopy0[i]);
    }
    cudaGetLastError();  // events of chunks that a failed loop left unrecorded
    c->stats.t_chunks_ms = chunks_ms;
    c->stats.t_copy_ms = copy_ms;
    if (loop_rc) return loop_rc;
    if (se != cudaSuccess) return cuda_fail(c, se, "compute stream");
    if (ce != cudaSuccess) return cuda_fail(c, ce, "copy stream");
    if (host_dg && c->host_full && m > 0) {
        if (f32out) host_digest_rows(c, c->hCp.as<int64_t>(), 0, m, 0, c->hCi.as<int32_t>(), c->hCv.as<float>());
        else host_digest_rows(c, c->hCp.as<int64_t>(), 0, m, 0, c->hCi.as<int32_t>(), c->hCv.as<double>());
    }
    c->dgDevOk = dev_dg;
    c->dgHostOk = host_dg && !werr;
    rc = check_device_err(c, "numeric");
    if (rc) return rc;
    if (scope == DBD_SCOPE_IO) {
        int rc2 = werr;
        std::string msg = wmsg;
        if (!rc2) rc2 = writer_finish(wr, c->hCp.as<int64_t>(), &c->stats.t_fsync, &msg);
        c->stats.t_write_file = writer_busy(wr);
        c->stats.bytes_written = writer_bytes(wr);
        c->stats.io_direct = writer_is_direct(wr) ? 1 : 0;
        c->stats.resumed_from_row = resume_row;
        if (rc2) return set_err(c, rc2, msg.empty() ? "output write failed" : msg);
    }
    c->stats.t_kernel_exec = seconds_since(t0);
    c->stats.t_total = c->stats.t_preprocess + c->stats.t_kernel_exec;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->evStart, c->evNumB);
    c->stats.t_device_ms = ms;
    float msn = 0.f;
    cudaEventElapsedTime(&msn, c->evNumA, c->evNumB);
    c->stats.t_numeric_ms = msn;
    float mss = 0.f;
    cudaEventElapsedTime(&mss, c->evPre, c->evNumB);
    c->stats.t_compute_gpu = mss / 1000.0;
    c->stats.t_d2h = t_d2h_issue;
    c->stats.bytes_d2h = bytes_d2h;
    c->stats.gpu_launches = c->launches;
    float mta = 0.f;
    cudaEventElapsedTime(&mta, c->evStart, c->evPre);
    c->stats.t_analysis_ms = mta;
    for (const auto &t : c->timed) {
        float x = 0.f;
        if (cudaEventElapsedTime(&x, t.a, t.b) != cudaSuccess) continue;
        if (t.kind == 0) c->stats.t_sym_bin_ms[t.bin] += x;
        else if (t.kind == 1) c->stats.t_num_bin_ms[t.bin] += x;
        else c->stats.t_scan_ms += x;
    }
    c->last_scope = scope;
    c->replayOk = scope == DBD_SCOPE_KERNEL && resident;
    c->patternOk = c->replayOk && c->batchCount == 0;  // batched C has pair-local columns
    c->patA = c->A.dev.nnz;
    c->patB = opB(c).nnz;
    return DBD_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

void dbd_config_default(dbd_config *cfg) {
    memset(cfg, 0, sizeof(*cfg));
    cfg->host_gib = 28.0;
    cfg->gpu_gib = 22.0;
    cfg->rows_per_block = 4096;
    cfg->device = 0;
}

const char *dbd_error_string(int code) {
    switch (code) {
        case DBD_OK: return "ok";
        case DBD_ERR_INVALID: return "invalid argument";
        case DBD_ERR_OOM_DEVICE: return "out of device memory";
        case DBD_ERR_OOM_HOST: return "out of host memory";
        case DBD_ERR_BUDGET: return "does not fit the memory budget";
        case DBD_ERR_IO: return "I/O error";
        case DBD_ERR_CUDA: return "CUDA error";
        case DBD_ERR_TIMEOUT: return "timeout";
        case DBD_ERR_OVERFLOW: return "overflow";
        case DBD_ERR_DEVICE_CHECK: return "device consistency check failed";
        case DBD_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown error";
    }
}

const char *dbd_last_error(const dbd_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int dbd_create(const dbd_config *cfg_in, dbd_ctx **out) {
    if (!out) return DBD_ERR_INVALID;
    *out = nullptr;
    dbd_config cfg;
    if (cfg_in) cfg = *cfg_in; else dbd_config_default(&cfg);
    if (cfg.rows_per_block <= 0 || cfg.rows_per_block % kTileRows != 0 || cfg.host_gib <= 0 || cfg.gpu_gib <= 0)
        return DBD_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DBD_ERR_NO_DEVICE;
    if (cfg.device < 0 || cfg.device >= ndev) return DBD_ERR_INVALID;
    if (cudaSetDevice(cfg.device) != cudaSuccess) return DBD_ERR_CUDA;
    dbd_ctx *c = new (std::nothrow) dbd_ctx();
    if (!c) return DBD_ERR_OOM_HOST;
    c->cfg = cfg;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, cfg.device);
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return DBD_ERR_CUDA;
    }
    c->stream = c->own_stream;
    for (int b = 0; b < kMaxBins; ++b) {
        if (cudaStreamCreateWithFlags(&c->bin_streams[b], cudaStreamNonBlocking) != cudaSuccess) {
            dbd_destroy(c);
            return DBD_ERR_CUDA;
        }
    }
    cudaEventCreate(&c->evStart);
    cudaEventCreate(&c->evPre);
    cudaEventCreate(&c->evSym);
    cudaEventCreate(&c->evEnd);
    cudaEventCreate(&c->evNumA);
    cudaEventCreate(&c->evNumB);
    init_kernel_attributes();
    if (cudaGetLastError() != cudaSuccess) {
        dbd_destroy(c);
        return DBD_ERR_CUDA;
    }
    *out = c;
    return DBD_OK;
}

void dbd_destroy(dbd_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->cfg.device);
    if (c->own_stream) cudaStreamSynchronize(c->own_stream);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (DevBuf *b : {&c->A.ptr, &c->A.idx, &c->A.val, &c->A.tmp, &c->B.ptr, &c->B.idx, &c->B.val, &c->B.tmp,
                      &c->rowP, &c->symBin, &c->numBin, &c->rowNnz, &c->symList, &c->numList, &c->hist,
                      &c->symTileOff, &c->numTileOff, &c->symStart, &c->numStart, &c->part, &c->Cp, &c->cursor,
                      &c->err, &c->blockP, &c->flags, &c->Ci, &c->Cv, &c->wideBits, &c->wideSlot, &c->adjG,
                      &c->adjA, &c->adjB, &c->adjT, &c->rowLo, &c->rowHi, &c->A.bmin, &c->A.bmax, &c->B.bmin, &c->B.bmax,
                      &c->ctrs, &c->gdense, &c->dgCount, &c->dgCol, &c->dgVal, &c->dgSum, &c->dgWsum,
                      &c->dgBad, &c->hashOut, &c->dscr, &c->heavySlot, &c->slabCnt,
                      &c->items})
        b->release();
    c->hCp.release();
    c->hCi.release();
    c->hCv.release();
    for (cudaEvent_t e : {c->evStart, c->evPre, c->evSym, c->evEnd, c->evNumA, c->evNumB})
        if (e) cudaEventDestroy(e);
    drop_graph(c);
    c->batchDev.release();
    c->rowShift.release();
    c->batchHost.release();
    for (cudaEvent_t e : c->tpool) cudaEventDestroy(e);
    for (cudaEvent_t e : c->spool) cudaEventDestroy(e);
    for (int b = 0; b < kMaxBins; ++b) {
        if (c->bin_streams[b]) {
            cudaStreamSynchronize(c->bin_streams[b]);
            cudaStreamDestroy(c->bin_streams[b]);
        }
    }
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    delete c;
}

int dbd_set_stream(dbd_ctx *c, void *stream) {
    if (!c) return DBD_ERR_INVALID;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return DBD_OK;
}

int dbd_read_csr(const char *path, dbd_csr_host *out) {
    if (!path || !out) return DBD_ERR_INVALID;
    std::string err;
    int rc = read_csr_file(path, out, &err);
    if (rc) fprintf(stderr, "dbd_read_csr: %s\n", err.c_str());
    return rc;
}

int dbd_read_csr_gpu(const char *path, int device, dbd_csr_host *out) {
    if (!path || !out) return DBD_ERR_INVALID;
    std::string err;
    int rc = read_csr_file_gpu(path, device, out, &err);
    if (rc) fprintf(stderr, "dbd_read_csr_gpu: %s\n", err.c_str());
    return rc;
}

int dbd_write_csr(const char *path, const dbd_csr_view *m, int fp64) {
    if (!path || !m) return DBD_ERR_INVALID;
    std::string err;
    int rc = write_csr_file(path, m, fp64, &err);
    if (rc) fprintf(stderr, "dbd_write_csr: %s\n", err.c_str());
    return rc;
}

int dbd_load_a(dbd_ctx *c, const dbd_csr_view *a) {
    if (!c || !a) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    c->b_is_a = false;
    return load_operand(c, c->A, a, "A");
}

int dbd_load_b(dbd_ctx *c, const dbd_csr_view *b) {
    if (!c || !b) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    c->b_is_a = false;
    return load_operand(c, c->B, b, "B");
}

int dbd_divide_blocks(dbd_ctx *c, int64_t *num_blocks) {
    if (!c) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    int rc = divide_blocks(c);
    if (!rc && num_blocks) *num_blocks = c->nblocks;
    return rc;
}

int dbd_block_info(const dbd_ctx *c, int64_t *products, int32_t *category) {
    if (!c) return DBD_ERR_INVALID;
    for (size_t b = 0; b < c->blockP_h.size(); ++b) {
        if (products) products[b] = c->blockP_h[b];
        if (category) category[b] = c->blockCat_h[b];
    }
    return DBD_OK;
}

int dbd_distribute_workload(dbd_ctx *c, dbd_scope scope, const char *out_dir) {
    if (!c || scope < DBD_SCOPE_KERNEL || scope > DBD_SCOPE_IO) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    return distribute(c, scope, out_dir);
}

int dbd_result(dbd_ctx *c, dbd_csr_out *o) {
    if (!c || !o) return DBD_ERR_INVALID;
    memset(o, 0, sizeof(*o));
    o->n_rows = c->m;
    o->n_cols = c->ncols;
    o->nnz = c->nnzC;
    if (c->last_scope == DBD_SCOPE_KERNEL) {
        if (!c->dev_resident) return set_err(c, DBD_ERR_BUDGET, "the product was streamed, not kept on the device");
        o->row_ptr = c->Cp.as<int64_t>();
        o->col_idx = c->Ci.as<int32_t>();
        o->val = c->Cv.as<double>();
        o->on_device = 1;
        o->owner = 2;
        return DBD_OK;
    }
    if (!c->host_full) return set_err(c, DBD_ERR_BUDGET, "the product did not fit the host budget");
    o->row_ptr = c->hCp.as<int64_t>();
    o->col_idx = c->hCi.as<int32_t>();
    o->val = c->hCv.p;
    o->val_fp32 = c->host_f32 ? 1 : 0;
    o->owner = 2;
    return DBD_OK;
}

int dbd_result_copy(dbd_ctx *c, int64_t *row_ptr, int32_t *col_idx, double *val) {
    if (!c) return DBD_ERR_INVALID;
    if (!col_idx && !val && row_ptr) {
        // The row pointers stay on the device after any multiply, streamed or not.
        if (c->m <= 0 && c->nnzC == 0 && !c->Cp.p) return set_err(c, DBD_ERR_INVALID, "no multiply yet");
        cudaSetDevice(c->cfg.device);
        CK(c, cudaMemcpy(row_ptr, c->Cp.p, sizeof(int64_t) * (size_t)(c->m + 1), cudaMemcpyDefault));
        return DBD_OK;
    }
    dbd_csr_out o;
    int rc = dbd_result(c, &o);
    if (rc) return rc;
    const cudaMemcpyKind k = cudaMemcpyDefault;  // host or device destinations (unified addressing)
    if (row_ptr) CK(c, cudaMemcpy(row_ptr, o.row_ptr, sizeof(int64_t) * (size_t)(o.n_rows + 1), k));
    if (o.nnz > 0) {
        if (col_idx) CK(c, cudaMemcpy(col_idx, o.col_idx, sizeof(int32_t) * (size_t)o.nnz, k));
        if (val && o.val_fp32) {
            cudaPointerAttributes pa;
            if (cudaPointerGetAttributes(&pa, val) != cudaSuccess || pa.type == cudaMemoryTypeDevice) {
                cudaGetLastError();
                return set_err(c, DBD_ERR_INVALID, "float32 values widen into host memory only");
            }
            const float *f = static_cast<const float *>(o.val);
            for (int64_t i = 0; i < o.nnz; ++i) val[i] = (double)f[i];
        } else if (val) {
            CK(c, cudaMemcpy(val, o.val, sizeof(double) * (size_t)o.nnz, k));
        }
    }
    return DBD_OK;
}

int dbd_set_digest(dbd_ctx *c, int flags) {
    if (!c || (flags & ~(DBD_DIGEST_DEVICE | DBD_DIGEST_HOST))) return DBD_ERR_INVALID;
    c->digest = flags;
    return DBD_OK;
}

int dbd_digest_copy(dbd_ctx *c, int which, int64_t *count, uint64_t *col_hash, uint64_t *val_hash, double *sum,
                    double *wsum, int64_t *bad_rows) {
    if (!c || (which != DBD_DIGEST_DEVICE && which != DBD_DIGEST_HOST)) return DBD_ERR_INVALID;
    const size_t m = (size_t)c->m;
    if (which == DBD_DIGEST_HOST) {
        if (!c->dgHostOk) return set_err(c, DBD_ERR_INVALID, "the last multiply took no host digest");
        if (count) memcpy(count, c->hdCount.data(), sizeof(int64_t) * m);
        if (col_hash) memcpy(col_hash, c->hdCol.data(), sizeof(uint64_t) * m);
        if (val_hash) memcpy(val_hash, c->hdVal.data(), sizeof(uint64_t) * m);
        if (sum) memcpy(sum, c->hdSum.data(), sizeof(double) * m);
        if (wsum) memcpy(wsum, c->hdWsum.data(), sizeof(double) * m);
        if (bad_rows) *bad_rows = c->hdBad.load();
        return DBD_OK;
    }
    if (!c->dgDevOk) return set_err(c, DBD_ERR_INVALID, "the last multiply took no device digest");
    cudaSetDevice(c->cfg.device);
    const cudaMemcpyKind k = cudaMemcpyDefault;
    if (m) {
        if (count) CK(c, cudaMemcpy(count, c->dgCount.p, sizeof(int64_t) * m, k));
        if (col_hash) CK(c, cudaMemcpy(col_hash, c->dgCol.p, sizeof(uint64_t) * m, k));
        if (val_hash) CK(c, cudaMemcpy(val_hash, c->dgVal.p, sizeof(uint64_t) * m, k));
        if (sum) CK(c, cudaMemcpy(sum, c->dgSum.p, sizeof(double) * m, k));
        if (wsum) CK(c, cudaMemcpy(wsum, c->dgWsum.p, sizeof(double) * m, k));
    }
    if (bad_rows) CK(c, cudaMemcpy(bad_rows, c->dgBad.p, sizeof(int64_t), cudaMemcpyDeviceToHost));
    return DBD_OK;
}

int dbd_get_stats(const dbd_ctx *c, dbd_stats *st) {
    if (!c || !st) return DBD_ERR_INVALID;
    *st = c->stats;
    return DBD_OK;
}

int dbd_spgemm(dbd_ctx *c, const dbd_csr_view *a, const dbd_csr_view *b, dbd_scope scope, const char *out_dir,
               dbd_csr_out *out, dbd_stats *st) {
    if (!c || !a) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    int rc = load_operand(c, c->A, a, "A");
    if (rc) return rc;
    if (!b || b == a) {
        c->b_is_a = true;
    } else {
        c->b_is_a = false;
        rc = load_operand(c, c->B, b, "B");
        if (rc) return rc;
    }
    rc = divide_blocks(c);
    if (rc) return rc;
    rc = distribute(c, scope, out_dir);
    if (rc) return rc;
    if (st) *st = c->stats;
    if (out) {
        if (scope == DBD_SCOPE_IO) {
            memset(out, 0, sizeof(*out));
            out->n_rows = c->m;
            out->n_cols = c->ncols;
            out->nnz = c->nnzC;
            return DBD_OK;
        }
        return dbd_result(c, out);
    }
    return DBD_OK;
}

int dbd_spgemm_adjoint(dbd_ctx *c, const dbd_csr_view *a, const dbd_csr_view *b, const double *g, double *da,
                       double *db, int on_device, int flags) {
    if (!c || !a || !g || !da || !db || (flags & ~(DBD_ADJ_RECOMPUTE | DBD_ADJ_DETERMINISTIC)))
        return DBD_ERR_INVALID;
    const bool recompute_pattern = (flags & DBD_ADJ_RECOMPUTE) != 0;
    const bool det = (flags & DBD_ADJ_DETERMINISTIC) != 0;
    const dbd_csr_view *bb = (b && b != a) ? b : a;
    // Checked here too: the kept-pattern path below reloads the operands
    // without going through the multiply's own checks.
    if (a->n_cols != bb->n_rows) return set_err(c, DBD_ERR_INVALID, "inner dimensions differ (A.n_cols != B.n_rows)");
    cudaSetDevice(c->cfg.device);
    const bool have =c->patternOk && c->m == a->n_rows && c->ncols == bb->n_cols && c->patA == a->nnz &&
                      c->patB == bb->nnz;
    int rc;
    if (recompute_pattern || !have) {
        rc = dbd_spgemm(c, a, b, DBD_SCOPE_KERNEL, nullptr, nullptr, nullptr);
        if (rc) return rc;
        if (!c->patternOk) return set_err(c, DBD_ERR_BUDGET, "C's pattern does not fit the device budget");
    } else {
        // Same patterns as the last multiply: only the values may have changed.
        rc = load_operand(c, c->A, a, "A");
        if (rc) return rc;
        c->b_is_a = bb == a;
        if (!c->b_is_a) {
            rc = load_operand(c, c->B, bb, "B");
            if (rc) return rc;
        }
    }
    const CsrDev &A = c->A.dev;
    const CsrDev &B = opB(c);
    const int64_t nnzC = c->nnzC;
    const double *dG = g;
    double *dA = da, *dB = db;
    if (!on_device) {
        CK(c, c->adjG.ensure(sizeof(double) * (size_t)std::max<int64_t>(nnzC, 1)));
        CK(c, c->adjA.ensure(sizeof(double) * (size_t)std::max<int64_t>(A.nnz, 1)));
        CK(c, c->adjB.ensure(sizeof(double) * (size_t)std::max<int64_t>(B.nnz, 1)));
        if (nnzC > 0)
            CK(c, cudaMemcpyAsync(c->adjG.p, g, sizeof(double) * (size_t)nnzC, cudaMemcpyHostToDevice, c->stream));
        dG = c->adjG.as<double>();
        dA = c->adjA.as<double>();
        dB = c->adjB.as<double>();
    }
    if (A.nnz > 0) CK(c, cudaMemsetAsync(dA, 0, sizeof(double) * (size_t)A.nnz, c->stream));
    if (B.nnz > 0) CK(c, cudaMemsetAsync(dB, 0, sizeof(double) * (size_t)B.nnz, c->stream));
    CK(c, cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
    AdjArgs aa;
    aa.A = A;
    aa.B = B;
    aa.Cp = c->Cp.as<int64_t>();
    aa.Ci = c->Ci.as<int32_t>();
    aa.G = dG;
    aa.dA = dA;
    aa.dB = det ? nullptr : dB;  // deterministic: dB by its own pass below
    aa.order = c->numList.as<int32_t>();
    aa.nrows = c->m;
    aa.err = c->err.as<int>();
    int launches = 0;
    launch_adjoint(aa, c->stream, &launches);
    if (det && B.nnz > 0) {
        // A grouped by column (stably, so rows ascend in every column), then
        // dB by segments of every column (launch_adjoint_db).
        const size_t na = (size_t)std::max<int64_t>(A.nnz, 1);
        const size_t nb = (size_t)B.nnz;
        const int64_t cap = adjoint_db_part_cap(c->products);
        size_t bytes = 0;
        auto carve = [&bytes](size_t n) {
            const size_t at = bytes;
            bytes += (n + 15) / 16 * 16;
            return at;
        };
        const size_t oRow = carve(4 * na), oK0 = carve(4 * na), oV0 = carve(4 * na), oK1 = carve(4 * na),
                     oV1 = carve(4 * na), oCol = carve(sizeof(int32_t) * (size_t)(A.n + 1)),
                     oSort = carve((size_t)stable_sort_scratch_bytes(A.nnz)), oExtra = carve(4 * nb),
                     oStart = carve(8 * (nb + 1)), oScan = carve(8 * (size_t)(ceil_div(B.nnz, kScanTile) + 1)),
                     oPart = carve(8 * (size_t)cap);
        CK(c, c->adjT.ensure(bytes));
        char *p = c->adjT.as<char>();
        int32_t *colPtr = reinterpret_cast<int32_t *>(p + oCol);
        const uint32_t *perm = nullptr;
        launch_adjoint_transpose(A, reinterpret_cast<int32_t *>(p + oRow), reinterpret_cast<uint32_t *>(p + oK0),
                                 reinterpret_cast<uint32_t *>(p + oV0), reinterpret_cast<uint32_t *>(p + oK1),
                                 reinterpret_cast<uint32_t *>(p + oV1), p + oSort, colPtr, &perm, c->stream);
        AdjDbArgs ab;
        ab.B = B;
        ab.Aval = A.val;
        ab.colPtr = colPtr;
        ab.perm = perm;
        ab.rowOf = reinterpret_cast<int32_t *>(p + oRow);
        ab.Cp = c->Cp.as<int64_t>();
        ab.Ci = c->Ci.as<int32_t>();
        ab.G = dG;
        ab.dB = dB;
        ab.err = c->err.as<int>();
        ab.extra = reinterpret_cast<int32_t *>(p + oExtra);
        ab.xStart = reinterpret_cast<int64_t *>(p + oStart);
        ab.part = reinterpret_cast<double *>(p + oPart);
        ab.partCap = cap;
        launch_adjoint_db(ab, reinterpret_cast<int64_t *>(p + oScan), c->num_sms, c->stream);
    }
    CK(c, cudaGetLastError());
    if (!on_device) {
        if (A.nnz > 0)
            CK(c, cudaMemcpyAsync(da, dA, sizeof(double) * (size_t)A.nnz, cudaMemcpyDeviceToHost, c->stream));
        if (B.nnz > 0)
            CK(c, cudaMemcpyAsync(db, dB, sizeof(double) * (size_t)B.nnz, cudaMemcpyDeviceToHost, c->stream));
    }
    return check_device_err(c, "adjoint");
}

int dbd_spgemm_batched(dbd_ctx *c, int64_t count, const dbd_csr_view *a, const dbd_csr_view *b, dbd_scope scope,
                       int64_t *c_row_off, int64_t *c_nnz_off, dbd_csr_out *out, dbd_stats *st) {
    if (!c || !a || count <= 0) return DBD_ERR_INVALID;
    if (scope != DBD_SCOPE_KERNEL && scope != DBD_SCOPE_D2H)
        return set_err(c, DBD_ERR_INVALID, "batched products keep C on the device or in host memory (no file scope)");
    cudaSetDevice(c->cfg.device);
    c->batchCount = 0;
    c->replayOk = false;
    drop_graph(c);
    c->A.loaded = c->B.loaded = false;
    c->divided = false;
    const bool square = b == nullptr;
    const dbd_csr_view *bv = square ? a : b;
    const size_t n1 = (size_t)count + 1;
    // Pinned staging: pair descriptors of A and B, then rowOffA, nnzOffA,
    // rowOffB (= the inner offsets, A's column offsets), nnzOffB, colOffC.
    const size_t descBytes = sizeof(BatchPair) * 2 * (size_t)count;
    const size_t hostBytes = descBytes + sizeof(int64_t) * 5 * n1;
    CK(c, cudaStreamSynchronize(c->stream));  // the staging area may still feed an earlier copy
    CK(c, c->batchHost.ensure(hostBytes));
    BatchPair *pa = c->batchHost.as<BatchPair>();
    BatchPair *pb = pa + count;
    int64_t *rowA = reinterpret_cast<int64_t *>(c->batchHost.as<char>() + descBytes);
    int64_t *nnzA = rowA + n1, *rowB = nnzA + n1, *nnzB = rowB + n1, *colC = nnzB + n1;
    rowA[0] = nnzA[0] = rowB[0] = nnzB[0] = colC[0] = 0;
    for (int64_t q = 0; q < count; ++q) {
        const dbd_csr_view &x = a[q], &y = bv[q];
        const std::string tag = "pair " + std::to_string(q);
        for (const dbd_csr_view *v : {&x, &y}) {
            if (v->n_rows < 0 || v->n_cols < 0 || v->nnz < 0 || v->val_fp32 || !v->row_ptr ||
                (v->nnz > 0 && (!v->col_idx || !v->val)) || (v->n_rows == 0 && v->nnz > 0))
                return set_err(c, DBD_ERR_INVALID, tag + ": malformed operand (FP64 values and row_ptr required)");
        }
        if (x.n_cols != y.n_rows) return set_err(c, DBD_ERR_INVALID, tag + ": inner dimensions differ");
        rowA[q + 1] = rowA[q] + x.n_rows;
        nnzA[q + 1] = nnzA[q] + x.nnz;
        rowB[q + 1] = rowB[q] + y.n_rows;
        nnzB[q + 1] = nnzB[q] + y.nnz;
        colC[q + 1] = colC[q] + y.n_cols;
    }
    const int64_t lim = INT32_MAX - 1;
    if (rowA[count] > lim || rowB[count] > lim || colC[count] > lim || nnzA[count] > lim || nnzB[count] > lim)
        return set_err(c, DBD_ERR_INVALID, "the batch exceeds 2^31 rows, columns or entries; split it");

    // Concatenated operands.  Host pairs are copied raw into place (row
    // pointers into a staging area, since the gather rewrites them); device
    // pairs are read where they are.
    auto place = [&](Operand &op, const dbd_csr_view *views, const int64_t *rowOff, const int64_t *nnzOff,
                     const int64_t *colOff, const int64_t *shiftOff, BatchPair *desc) -> int {
        const int64_t rows = rowOff[count], ne = nnzOff[count];
        CK(c, op.ptr.ensure(sizeof(int32_t) * (size_t)(rows + 1)));
        CK(c, op.idx.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(ne, 1)));
        CK(c, op.val.ensure(sizeof(double) * (size_t)std::max<int64_t>(ne, 1)));
        bool anyHost = false;
        for (int64_t q = 0; q < count; ++q) anyHost = anyHost || !views[q].on_device;
        if (anyHost) CK(c, op.tmp.ensure(sizeof(int32_t) * (size_t)(rows + count)));
        for (int64_t q = 0; q < count; ++q) {
            const dbd_csr_view &v = views[q];
            BatchPair &d = desc[q];
            d.m = v.n_rows;
            d.nnz = v.nnz;
            d.ncols = v.n_cols;
            d.nnzOff = nnzOff[q];
            d.colOff = colOff[q];
            d.shift = shiftOff ? (int32_t)shiftOff[q] : 0;
            if (v.on_device) {
                d.ptr = v.row_ptr;
                d.idx = v.col_idx;
                d.val = (const double *)v.val;
                continue;
            }
            int32_t *sp = op.tmp.as<int32_t>() + rowOff[q] + q;
            int32_t *di = op.idx.as<int32_t>() + nnzOff[q];
            double *dv = op.val.as<double>() + nnzOff[q];
            CK(c, cudaMemcpyAsync(sp, v.row_ptr, sizeof(int32_t) * (size_t)(v.n_rows + 1), cudaMemcpyHostToDevice,
                                  c->stream));
            if (v.nnz > 0) {
                CK(c, cudaMemcpyAsync(di, v.col_idx, sizeof(int32_t) * (size_t)v.nnz, cudaMemcpyHostToDevice,
                                      c->stream));
                CK(c, cudaMemcpyAsync(dv, v.val, sizeof(double) * (size_t)v.nnz, cudaMemcpyHostToDevice, c->stream));
            }
            d.ptr = sp;
            d.idx = di;
            d.val = dv;
        }
        return DBD_OK;
    };
    int rc = place(c->A, a, rowA, nnzA, rowB, colC, pa);
    if (rc) return rc;
    if (!square) {
        rc = place(c->B, bv, rowB, nnzB, colC, nullptr, pb);
        if (rc) return rc;
    }
    CK(c, c->batchDev.ensure(hostBytes + sizeof(int64_t) * n1));
    CK(c, cudaMemcpyAsync(c->batchDev.p, c->batchHost.p, hostBytes, cudaMemcpyHostToDevice, c->stream));
    const BatchPair *dpa = c->batchDev.as<BatchPair>();
    const int64_t *drow = reinterpret_cast<const int64_t *>(c->batchDev.as<char>() + descBytes);
    const int64_t *dnnzA = drow + n1, *drowB = dnnzA + n1, *dnnzB = drowB + n1;
    int64_t *dCoff = const_cast<int64_t *>(dnnzB + 2 * n1);
    CK(c, c->rowShift.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(rowA[count], 1)));
    CK(c, c->flags.ensure(4 * sizeof(int)));
    CK(c, cudaMemsetAsync(c->flags.p, 0, sizeof(int), c->stream));
    launch_batch_gather(dpa, drow, dnnzA, count, rowA[count], nnzA[count], c->A.ptr.as<int32_t>(),
                        c->A.idx.as<int32_t>(), c->A.val.as<double>(), c->rowShift.as<int32_t>(), c->flags.as<int>(),
                        c->stream);
    if (!square)
        launch_batch_gather(dpa + count, drowB, dnnzB, count, rowB[count], nnzB[count], c->B.ptr.as<int32_t>(),
                            c->B.idx.as<int32_t>(), c->B.val.as<double>(), nullptr, c->flags.as<int>(), c->stream);
    CK(c, cudaGetLastError());
    int bad = 0;
    CK(c, cudaMemcpyAsync(&bad, c->flags.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (bad) return set_err(c, DBD_ERR_INVALID, (bad & 1) ? "a pair's row_ptr does not span [0, nnz] monotonically"
                                                          : "a pair's column index is out of range");
    CsrDev da;
    da.m = rowA[count];
    da.n = rowB[count];
    da.nnz = nnzA[count];
    da.ptr = c->A.ptr.as<int32_t>();
    da.idx = c->A.idx.as<int32_t>();
    da.val = c->A.val.as<double>();
    rc = finish_operand(c, c->A, da);
    if (rc) return rc;
    c->b_is_a = square;
    if (!square) {
        CsrDev db;
        db.m = rowB[count];
        db.n = colC[count];
        db.nnz = nnzB[count];
        db.ptr = c->B.ptr.as<int32_t>();
        db.idx = c->B.idx.as<int32_t>();
        db.val = c->B.val.as<double>();
        rc = finish_operand(c, c->B, db);
        if (rc) return rc;
    }
    c->batchCount = count;
    c->batchNnzA.assign(nnzA, nnzA + n1);
    c->batchNnzB.assign(nnzB, nnzB + n1);
    rc = divide_blocks(c);
    if (rc) return rc;
    rc = distribute(c, scope, nullptr);
    c->patternOk = false;  // C's columns are pair-local: no adjoint on this pattern
    if (rc) return rc;
    // Entry offsets of every pair's rows in C.
    launch_gather_i64(c->Cp.as<int64_t>(), drow, (int64_t)n1, dCoff, c->stream);
    int64_t *hCoff = colC;  // the host copy of the column offsets is no longer needed
    CK(c, cudaMemcpyAsync(hCoff, dCoff, sizeof(int64_t) * n1, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (c_row_off) memcpy(c_row_off, rowA, sizeof(int64_t) * n1);
    if (c_nnz_off) memcpy(c_nnz_off, hCoff, sizeof(int64_t) * n1);
    if (st) *st = c->stats;
    if (out) return dbd_result(c, out);
    return DBD_OK;
}

// ---- device-driven batched multiply ---------------------------------------

int dbd_batch_plan(dbd_ctx *c, int64_t count, const dbd_csr_view *a, const dbd_csr_view *b, int64_t c_capacity) {
    if (!c || !a || count <= 0 || c_capacity < 0) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    c->bpOk = false;
    c->batchCount = 0;
    c->replayOk = false;
    drop_graph(c);
    c->A.loaded = c->B.loaded = false;
    c->divided = false;
    const bool square = b == nullptr;
    const dbd_csr_view *bv = square ? a : b;
    const size_t n1 = (size_t)count + 1;
    std::vector<BatchPair> desc(2 * (size_t)count);
    std::vector<int64_t> off(5 * n1, 0);
    int64_t *rowA = off.data(), *nnzA = rowA + n1, *rowB = nnzA + n1, *nnzB = rowB + n1, *colC = nnzB + n1;
    for (int64_t q = 0; q < count; ++q) {
        const dbd_csr_view &x = a[q], &y = bv[q];
        const std::string tag = "pair " + std::to_string(q);
        for (const dbd_csr_view *v : {&x, &y}) {
            if (!v->on_device || v->val_fp32 || v->n_rows < 0 || v->n_cols < 0 || v->nnz < 0 || !v->row_ptr ||
                (v->nnz > 0 && (!v->col_idx || !v->val)) || (v->n_rows == 0 && v->nnz > 0))
                return set_err(c, DBD_ERR_INVALID, tag + ": device-resident FP64 operands required");
        }
        if (x.n_cols != y.n_rows) return set_err(c, DBD_ERR_INVALID, tag + ": inner dimensions differ");
        rowA[q + 1] = rowA[q] + x.n_rows;
        nnzA[q + 1] = nnzA[q] + x.nnz;
        rowB[q + 1] = rowB[q] + y.n_rows;
        nnzB[q + 1] = nnzB[q] + y.nnz;
        colC[q + 1] = colC[q] + y.n_cols;
    }
    const int64_t lim = INT32_MAX - 1;
    if (rowA[count] > lim || rowB[count] > lim || colC[count] > lim || nnzA[count] > lim || nnzB[count] > lim)
        return set_err(c, DBD_ERR_INVALID, "the batch exceeds 2^31 rows, columns or entries; split it");
    for (int side = 0; side < (square ? 1 : 2); ++side) {
        const dbd_csr_view *views = side ? bv : a;
        const int64_t *nOff = side ? nnzB : nnzA, *cOff = side ? colC : rowB;
        for (int64_t q = 0; q < count; ++q) {
            BatchPair &d = desc[(size_t)(side * count + q)];
            d.m = views[q].n_rows;
            d.nnz = views[q].nnz;
            d.ncols = views[q].n_cols;
            d.nnzOff = nOff[q];
            d.colOff = cOff[q];
            d.shift = side ? 0 : (int32_t)colC[q];
            d.ptr = views[q].row_ptr;
            d.idx = views[q].col_idx;
            d.val = (const double *)views[q].val;
        }
    }
    // Operands, descriptors, work arrays and C, all sized here.
    const int64_t m = rowA[count];
    const size_t descBytes = sizeof(BatchPair) * desc.size();
    CK(c, c->batchDev.ensure(descBytes + sizeof(int64_t) * 6 * n1));
    CK(c, cudaMemcpy(c->batchDev.p, desc.data(), descBytes, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->batchDev.as<char>() + descBytes, off.data(), sizeof(int64_t) * 5 * n1, cudaMemcpyHostToDevice));
    auto sized = [&](Operand &op, int64_t rows, int64_t ne) -> int {
        CK(c, op.ptr.ensure(sizeof(int32_t) * (size_t)(rows + 1)));
        CK(c, op.idx.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(ne, 1)));
        CK(c, op.val.ensure(sizeof(double) * (size_t)std::max<int64_t>(ne, 1)));
        CK(c, op.bmin.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(rows, 1)));
        CK(c, op.bmax.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(rows, 1)));
        return DBD_OK;
    };
    int rc = sized(c->A, m, nnzA[count]);
    if (!rc && !square) rc = sized(c->B, rowB[count], nnzB[count]);
    if (rc) return rc;
    CK(c, c->rowShift.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1)));
    CK(c, c->flags.ensure(4 * sizeof(int)));
    CsrDev da{}, db{};
    da.m = m;
    da.n = rowB[count];
    da.nnz = nnzA[count];
    da.ptr = c->A.ptr.as<int32_t>();
    da.idx = c->A.idx.as<int32_t>();
    da.val = c->A.val.as<double>();
    c->A.dev = da;
    c->A.sorted = 0;
    c->A.loaded = true;
    c->b_is_a = square;
    if (!square) {
        db.m = rowB[count];
        db.n = colC[count];
        db.nnz = nnzB[count];
        db.ptr = c->B.ptr.as<int32_t>();
        db.idx = c->B.idx.as<int32_t>();
        db.val = c->B.val.as<double>();
        c->B.dev = db;
        c->B.sorted = 0;
        c->B.loaded = true;
    }
    c->m = m;
    c->ncols = colC[count];
    c->ntiles = ceil_div(m, kTileRows);
    const size_t mm = (size_t)std::max<int64_t>(m, 1), nt = (size_t)c->ntiles;
    CK(c, c->rowP.ensure(sizeof(int64_t) * mm));
    CK(c, c->rowLo.ensure(sizeof(int32_t) * mm));
    CK(c, c->rowHi.ensure(sizeof(int32_t) * mm));
    CK(c, c->symBin.ensure(mm));
    CK(c, c->numBin.ensure(mm));
    CK(c, c->rowNnz.ensure(sizeof(int32_t) * mm));
    CK(c, c->symList.ensure(sizeof(int32_t) * mm));
    CK(c, c->numList.ensure(sizeof(int32_t) * mm));
    CK(c, c->hist.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->symTileOff.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->numTileOff.ensure(sizeof(int32_t) * kMaxBins * (nt + 1)));
    CK(c, c->symStart.ensure(sizeof(int32_t) * (kMaxBins + 1)));
    CK(c, c->numStart.ensure(sizeof(int32_t) * (kMaxBins + 1)));
    CK(c, c->part.ensure(sizeof(int64_t) * (size_t)(ceil_div(m, kScanTile) + 1)));
    CK(c, c->Cp.ensure(sizeof(int64_t) * (mm + 1)));
    CK(c, c->cursor.ensure(2 * sizeof(int32_t) * (size_t)std::max<int64_t>(nnzA[count], 1)));
    CK(c, c->err.ensure(sizeof(int)));
    CK(c, c->ctrs.ensure(sizeof(uint32_t) * CTR_COUNT));
    CK(c, c->Ci.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(c_capacity, 1)));
    CK(c, c->Cv.ensure(sizeof(double) * (size_t)std::max<int64_t>(c_capacity, 1)));
    // Every kernel of the run is loaded (and every grid looked up) now, so
    // that a capture of dbd_batch_enqueue loads and queries nothing.
    cudaError_t le = preload_analysis_kernels();
    if (le == cudaSuccess) le = preload_batch_kernels();
    if (le != cudaSuccess) return cuda_fail(c, le, "loading the kernels");
    prepare_dd_grids(c->tune, colC[count], c->num_sms);
    // The fork and join events of two forked phases, created now.
    c->sused = 0;
    for (int k = 0; k < 2 * (kMaxBins + 1); ++k) c->sync_ev();
    c->sused = 0;
    c->bpSquare = square;
    c->bpCount = count;
    c->bpCap = c_capacity;
    c->bpColsC = colC[count];
    c->bpRowsB = rowB[count];
    c->bpNnzB = nnzB[count];
    c->bpRowOff.assign(rowA, rowA + n1);
    c->bpOk = true;
    return DBD_OK;
}

int dbd_batch_enqueue(dbd_ctx *c, void *stream) {
    if (!c) return DBD_ERR_INVALID;
    if (!c->bpOk) return set_err(c, DBD_ERR_INVALID, "no batch planned (dbd_batch_plan)");
    cudaSetDevice(c->cfg.device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const int64_t count = c->bpCount, m = c->m;
    const size_t n1 = (size_t)count + 1;
    const size_t descBytes = sizeof(BatchPair) * 2 * (size_t)count;
    const BatchPair *dpa = c->batchDev.as<BatchPair>();
    const int64_t *drow = reinterpret_cast<const int64_t *>(c->batchDev.as<char>() + descBytes);
    const int64_t *dnnzA = drow + n1, *drowB = dnnzA + n1, *dnnzB = drowB + n1;
    int64_t *dCoff = const_cast<int64_t *>(dnnzB + 2 * n1);
    int *flags = c->flags.as<int>();
    CK(c, cudaMemsetAsync(flags, 0, 4 * sizeof(int), s));
    CK(c, cudaMemsetAsync(c->err.p, 0, sizeof(int), s));
    CK(c, cudaMemsetAsync(c->ctrs.p, 0, sizeof(uint32_t) * CTR_COUNT, s));
    CK(c, cudaMemsetAsync(c->rowNnz.p, 0, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1), s));
    // The pairs' current contents, gathered into the concatenated operands.
    launch_batch_gather(dpa, drow, dnnzA, count, m, c->A.dev.nnz, c->A.ptr.as<int32_t>(), c->A.idx.as<int32_t>(),
                        c->A.val.as<double>(), c->rowShift.as<int32_t>(), flags, s);
    if (!c->bpSquare)
        launch_batch_gather(dpa + count, drowB, dnnzB, count, c->bpRowsB, c->bpNnzB, c->B.ptr.as<int32_t>(),
                            c->B.idx.as<int32_t>(), c->B.val.as<double>(), nullptr, flags, s);
    launch_batch_guard(flags, c->A.ptr.as<int32_t>(), m + 1, c->bpSquare ? nullptr : c->B.ptr.as<int32_t>(),
                       c->bpSquare ? 0 : c->bpRowsB + 1, s, c->num_sms);
    const CsrDev &A = c->A.dev, &B = opB(c);
    const Operand &opb = c->bpSquare ? c->A : c->B;
    int launches = 0;
    launch_row_minmax(B, opb.bmin.as<int32_t>(), opb.bmax.as<int32_t>(), flags + 2, s, c->num_sms);
    launch_row_products(A, B.ptr, opb.bmin.as<int32_t>(), opb.bmax.as<int32_t>(), row_info(c), c->symBin.as<uint8_t>(),
                        c->err.as<int>(), c->tune, s, c->num_sms);
    Binning sb{c->symBin.as<uint8_t>(), c->symList.as<int32_t>(), c->hist.as<int32_t>(), c->symTileOff.as<int32_t>(),
               c->symStart.as<int32_t>()};
    launch_bin_lists(m, sb, SB_COUNT, s);
    SymArgs sa{};
    sa.A = A;
    sa.B = B;
    sa.list = c->symList.as<int32_t>();
    sa.binStart = c->symStart.as<int32_t>();
    sa.rowNnz = c->rowNnz.as<int32_t>();
    sa.ctr = c->ctrs.as<uint32_t>();
    sa.err = c->err.as<int>();
    sa.rowLo = c->rowLo.as<int32_t>();
    sa.rowHi = c->rowHi.as<int32_t>();
    sa.rowP = c->rowP.as<int64_t>();
    sa.tune = c->tune;
    sa.numSms = c->num_sms;
    sa.bSorted = 0;
    sa.bUnsorted = flags + 2;  // B's sortedness as the device found it in this run
    // Bins run concurrently, one stream each, forked from and joined to s
    // (a capture follows the forks).
    c->sused = 0;
    static const int sorder[] = {SB_WIDE, SB_HCTA, SB_HWARP, SB_BITW, SB_TINY};
    {
        Fork fk(c, s);
        for (int bin : sorder) launch_symbolic_bin_dd(sa, bin, fk.stream(bin), &launches);
        fk.join();
    }
    launch_row_scan(m, c->rowNnz.as<int32_t>(), c->part.as<int64_t>(), c->Cp.as<int64_t>(), s);
    launch_num_bins(m, A.ptr, row_info(c), c->rowNnz.as<int32_t>(), c->numBin.as<uint8_t>(), c->tune, s, c->num_sms);
    Binning nb{c->numBin.as<uint8_t>(), c->numList.as<int32_t>(), c->hist.as<int32_t>(), c->numTileOff.as<int32_t>(),
               c->numStart.as<int32_t>()};
    launch_bin_lists(m, nb, NB_COUNT, s);
    launch_numeric_guard(c->Cp.as<int64_t>() + m, c->bpCap, c->err.as<int>(), c->numStart.as<int32_t>(), NB_COUNT,
                         flags + 3, s);
    NumArgs na{};
    na.A = A;
    na.B = B;
    na.list = c->numList.as<int32_t>();
    na.binStart = c->numStart.as<int32_t>();
    na.Cp = c->Cp.as<int64_t>();
    na.outBase = 0;
    na.Ci = c->Ci.as<int32_t>();
    na.Cv = c->Cv.as<double>();
    na.state = c->cursor.as<int32_t>();
    na.bSorted = 0;
    na.bUnsorted = flags + 2;
    na.err = c->err.as<int>();
    na.rowP = c->rowP.as<int64_t>();
    na.rowLo = c->rowLo.as<int32_t>();
    na.rowHi = c->rowHi.as<int32_t>();
    na.colShift = c->rowShift.as<int32_t>();
    na.tune = c->tune;
    na.tune.denseMethod = 0;
    na.numSms = c->num_sms;
    na.ctr = c->ctrs.as<uint32_t>();
    static const int norder[] = {NB_DENSE, NB_RANKL, NB_HCTA_L, NB_RANKS, NB_HCTA_S,
                                 NB_HWARP, NB_RANKM, NB_RANKW, NB_DENSEW, NB_TINY};
    {
        Fork fk(c, s);
        for (int bin : norder) launch_numeric_bin_dd(na, bin, fk.stream(bin), &launches);
        fk.join();
    }
    launch_gather_i64(c->Cp.as<int64_t>(), drow, (int64_t)n1, dCoff, s);
    CK(c, cudaGetLastError());
    c->launches = launches + 10;
    c->last_scope = DBD_SCOPE_KERNEL;
    c->dev_resident = true;
    c->host_full = false;
    c->host_f32 = false;
    c->batchCount = count;
    c->patternOk = false;
    return DBD_OK;
}

int dbd_batch_result(dbd_ctx *c, int64_t *c_row_off, int64_t *c_nnz_off, dbd_csr_out *out) {
    if (!c) return DBD_ERR_INVALID;
    if (!c->bpOk) return set_err(c, DBD_ERR_INVALID, "no batch planned (dbd_batch_plan)");
    cudaSetDevice(c->cfg.device);
    const int64_t count = c->bpCount, m = c->m;
    const size_t n1 = (size_t)count + 1;
    int hf[4] = {0, 0, 0, 0}, derr = 0;
    int64_t nnz = 0;
    CK(c, cudaMemcpy(hf, c->flags.p, sizeof(hf), cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(&derr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(&nnz, c->Cp.as<int64_t>() + m, sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (hf[0]) return set_err(c, DBD_ERR_INVALID, (hf[0] & 1) ? "a pair's row_ptr does not span [0, nnz] monotonically"
                                                               : "a pair's column index is out of range");
    if (derr) return set_err(c, DBD_ERR_CUDA, "a device table overflowed in the batched multiply");
    c->nnzC = nnz;
    if (hf[3]) return set_err(c, DBD_ERR_BUDGET, "nnz(C) = " + std::to_string(nnz) + " exceeds the planned capacity");
    if (c_row_off) memcpy(c_row_off, c->bpRowOff.data(), sizeof(int64_t) * n1);
    if (c_nnz_off) {
        const size_t descBytes = sizeof(BatchPair) * 2 * (size_t)count;
        const int64_t *dCoff = reinterpret_cast<const int64_t *>(c->batchDev.as<char>() + descBytes) + 5 * n1;
        CK(c, cudaMemcpy(c_nnz_off, dCoff, sizeof(int64_t) * n1, cudaMemcpyDeviceToHost));
    }
    if (out) {
        memset(out, 0, sizeof(*out));
        out->n_rows = m;
        out->n_cols = c->bpColsC;
        out->nnz = nnz;
        out->row_ptr = c->Cp.as<int64_t>();
        out->col_idx = c->Ci.as<int32_t>();
        out->val = c->Cv.p;
        out->on_device = 1;
        out->owner = 2;
    }
    return DBD_OK;
}

int dbd_get_tuning(const dbd_ctx *c, dbd_tuning *t) {
    if (!c || !t) return DBD_ERR_INVALID;
    t->warp_span_words = c->tune.warpSpanWords;
    t->warp_max_nnz = c->tune.numWarpMax;
    t->sym_warp_max_products = c->tune.symWarpMax;
    t->rank_words_max = c->tune.rankWordsMax;
    t->rank_shared_max_nnz = c->tune.rankSharedMax;
    t->sym_hash_span_words = c->tune.symHashSpanWords;
    t->dense_warp_span_words = c->tune.denseWarpWords;
    t->mid_span_words = c->tune.midSpanWords;
    t->dense_method = c->tune.denseMethod;
    return DBD_OK;
}

int dbd_set_tuning(dbd_ctx *c, const dbd_tuning *t) {
    if (!c || !t) return DBD_ERR_INVALID;
    Tuning u;
    u.warpSpanWords = t->warp_span_words;
    u.numWarpMax = t->warp_max_nnz;
    u.symWarpMax = t->sym_warp_max_products;
    u.rankWordsMax = t->rank_words_max;
    u.rankSharedMax = t->rank_shared_max_nnz;
    u.symHashSpanWords = t->sym_hash_span_words;
    u.denseWarpWords = t->dense_warp_span_words;
    u.midSpanWords = t->mid_span_words;
    u.denseMethod = t->dense_method;
    const Tuning v = clamp_tuning(u);
    if (memcmp(&u, &v, sizeof(u)) != 0) return set_err(c, DBD_ERR_INVALID, "a tuning value is out of its range");
    c->tune = u;
    c->divided = false;  // bins depend on the thresholds
    return DBD_OK;
}

int dbd_autotune(dbd_ctx *c, int repeats, dbd_tuning *best, double *best_ms) {
    if (!c || repeats < 1) return DBD_ERR_INVALID;
    if (!c->A.loaded || (!c->b_is_a && !c->B.loaded))
        return set_err(c, DBD_ERR_INVALID, "load operands (or run a multiply) before autotuning");
    cudaSetDevice(c->cfg.device);
    auto run = [&](const Tuning &t, double *ms) -> int {
        c->tune = t;
        double bestt = 1e300;
        for (int r = 0; r < repeats; ++r) {
            const auto t0 = Clock::now();
            int rc = divide_blocks(c);
            if (!rc) rc = distribute(c, DBD_SCOPE_KERNEL, nullptr);
            if (rc) return rc;
            bestt = std::min(bestt, seconds_since(t0) * 1e3);
        }
        *ms = bestt;
        return DBD_OK;
    };
    // Candidates per knob; the current setting is always one of them.
    struct Knob {
        int32_t Tuning::*field;
        std::vector<int32_t> values;
    };
    const std::vector<Knob> knobs = {
        {&Tuning::warpSpanWords, {8, 16, 32, 64}},
        {&Tuning::numWarpMax, {64, 128, 256}},
        {&Tuning::rankWordsMax, {1024, 2048, 4096, 8192}},
        {&Tuning::rankSharedMax, {512, 1024, 2048, 4096}},
        {&Tuning::symWarpMax, {128, 256, 512}},
        {&Tuning::symHashSpanWords, {512, 2048, 8192}},
        {&Tuning::denseWarpWords, {0, 4, 8, 16}},
        {&Tuning::midSpanWords, {0, 256, 1024, 2048}},
        {&Tuning::denseMethod, {0, 1, 2, 3}},
    };
    const Tuning start = c->tune;
    Tuning cur = start;
    double cur_ms = 0.0;
    int rc = run(cur, &cur_ms);  // warms the context up; timed again below
    if (!rc) rc = run(cur, &cur_ms);
    for (int sweep = 0; sweep < 2 && !rc; ++sweep) {
        bool improved = false;
        for (const Knob &k : knobs) {
            for (int32_t v : k.values) {
                if (cur.*k.field == v) continue;
                Tuning t = cur;
                t.*k.field = v;
                t = clamp_tuning(t);
                double ms = 0.0;
                rc = run(t, &ms);
                if (rc) break;
                if (ms < cur_ms * 0.98) {  // keep a change only for a clear gain
                    cur = t;
                    cur_ms = ms;
                    improved = true;
                }
            }
            if (rc) break;
        }
        if (!improved) break;
    }
    c->tune = rc ? start : cur;
    c->divided = false;
    if (rc) return rc;
    if (best) dbd_get_tuning(c, best);
    if (best_ms) *best_ms = cur_ms;
    return DBD_OK;
}

int dbd_update_values(dbd_ctx *c, int64_t count, const double *const *a_val, const double *const *b_val,
                      int on_device) {
    if (!c || count <= 0 || !a_val) return DBD_ERR_INVALID;
    cudaSetDevice(c->cfg.device);
    if (!c->replayOk)
        return set_err(c, DBD_ERR_INVALID, "values can be updated after a kernel-scope multiply with C resident");
    const bool batch = c->batchCount > 0;
    if (batch ? count != c->batchCount : count != 1)
        return set_err(c, DBD_ERR_INVALID, "count differs from the last multiply's pair count");
    if (!c->b_is_a && !b_val) return set_err(c, DBD_ERR_INVALID, "b_val is required (the last multiply had a B)");
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    // Values go to context-owned arrays, whose addresses the graph holds.
    auto put = [&](Operand &op, const double *const *src, const std::vector<int64_t> &off) -> int {
        const int64_t ne = op.dev.nnz;
        if (op.dev.val != op.val.as<double>()) {
            CK(c, op.val.ensure(sizeof(double) * (size_t)std::max<int64_t>(ne, 1)));
            op.dev.val = op.val.as<double>();
            drop_graph(c);
        }
        for (int64_t q = 0; q < count; ++q) {
            const int64_t o = batch ? off[(size_t)q] : 0;
            const int64_t n = batch ? off[(size_t)q + 1] - o : ne;
            if (n > 0) {
                if (!src[q]) return set_err(c, DBD_ERR_INVALID, "null value array");
                CK(c, cudaMemcpyAsync(op.val.as<double>() + o, src[q], sizeof(double) * (size_t)n, kind, c->stream));
            }
        }
        return DBD_OK;
    };
    int rc = put(c->A, a_val, c->batchNnzA);
    if (rc) return rc;
    if (!c->b_is_a) {
        rc = put(c->B, b_val, c->batchNnzB);
        if (rc) return rc;
    }
    if (!c->numExec) {
        // Capture the numeric kernels of every bin (their fork/join across the
        // bin streams included) once; replays launch them with one call.
        c->tused = c->sused = 0;
        CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
        numeric_rows(c, 0, c->m, 0, c->Ci.as<int32_t>(), c->Cv.as<double>());
        c->capturing = false;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        c->numGraph = g;
        e = cudaGraphInstantiate(&c->numExec, g, 0);
        if (e != cudaSuccess) {
            drop_graph(c);
            return cuda_fail(c, e, "cudaGraphInstantiate");
        }
    }
    CK(c, cudaGraphLaunch(c->numExec, c->stream));
    return check_device_err(c, "update values");
}

int dbd_spgemm_files(dbd_ctx *c, const char *path_a, const char *path_b, dbd_scope scope, const char *out_dir,
                     dbd_stats *st) {
    if (!c || !path_a) return DBD_ERR_INVALID;
    dbd_csr_host ha, hb;
    memset(&hb, 0, sizeof(hb));
    int rc = dbd_read_csr_gpu(path_a, c->cfg.device, &ha);
    if (rc) return set_err(c, rc, std::string("cannot read ") + path_a);
    const bool same = !path_b || strcmp(path_a, path_b) == 0;
    if (!same) {
        rc = dbd_read_csr_gpu(path_b, c->cfg.device, &hb);
        if (rc) {
            dbd_csr_host_free(&ha);
            return set_err(c, rc, std::string("cannot read ") + path_b);
        }
    }
    if (c->cfg.verbose) {
        printf("Input: %s\n\tNumber of Rows:\t\t%lld\n\tNumber of Columns:\t%lld\n\tNumber of Edges:\t%lld\n\n",
               path_a, (long long)ha.n_rows, (long long)ha.n_cols, (long long)ha.nnz);
    }
    dbd_csr_view va{ha.n_rows, ha.n_cols, ha.nnz, ha.row_ptr, ha.col_idx, ha.val, 0, 0};
    dbd_csr_view vb{hb.n_rows, hb.n_cols, hb.nnz, hb.row_ptr, hb.col_idx, hb.val, 0, 0};
    rc = dbd_spgemm(c, &va, same ? nullptr : &vb, scope, out_dir, nullptr, st);
    dbd_csr_host_free(&ha);
    dbd_csr_host_free(&hb);
    return rc;
}

void dbd_csr_free(dbd_csr_out *o) {
    if (!o) return;
    if (o->owner == 1) {
        free(o->row_ptr);
        free(o->col_idx);
        free(o->val);
    }
    memset(o, 0, sizeof(*o));
}

}  // extern "C"
