// noalloc.cu -- dbd_spgemm_noalloc: the whole multiply without allocating.
//
// Some callers of this library cannot allocate device memory: code that runs
// while a caching allocator owns the device (an allocator hook, a framework
// that forbids allocation outside its pool), latency-critical loops where
// cudaMalloc/cudaFree's implicit device synchronisation is not acceptable,
// and processes whose device memory is fully reserved up front.  They pass
// device-resident A, B and the output arrays; every temporary array of the
// pipeline (row products, bins, row lists, per-tile offsets, row counts, scan
// partials, dense-window cursors and next columns, the error word) is carved out of the
// file-scope array below instead of cudaMalloc'ed, and the pipeline runs on
// the caller's stream without creating streams or events.
//
// The array is kDbdNoallocScratchBytes (32 MiB) per GPU, held by every GPU
// that loads this library until the process exits.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/dbd.h"
#include "dbd_internal.h"

namespace dbd {

namespace {

constexpr size_t kDbdNoallocScratchBytes = DBD_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kDbdNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
bool g_setup_done[kMaxDevices] = {};
unsigned char *g_scratch_addr[kMaxDevices] = {};
thread_local char g_msg[256];

// Failures are reported by the return code and one stderr line.
int report(int code) {
    fprintf(stderr, "dbd_spgemm_noalloc: %s\n", g_msg);
    return code;
}

int fail(int code, const char *msg) {
    snprintf(g_msg, sizeof(g_msg), "%s", msg);
    return report(code);
}

// Device address of the scratch array on the current device (set-up once
// per device: kernel attributes and cudaGetSymbolAddress).
int device_scratch(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(DBD_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_setup_done[dev]) {
        init_kernel_attributes();
        // Every kernel the pipeline launches is loaded here, so that no later
        // call has the CUDA driver load a module (and allocate) on first launch.
        cudaError_t le = preload_analysis_kernels();
        if (le == cudaSuccess) le = preload_spgemm_kernels();
        if (le != cudaSuccess) {
            snprintf(g_msg, sizeof(g_msg), "loading the kernels: %s", cudaGetErrorString(le));
            return report(DBD_ERR_CUDA);
        }
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            snprintf(g_msg, sizeof(g_msg), "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return report(DBD_ERR_CUDA);
        }
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
        g_setup_done[dev] = true;
    }
    *out = g_scratch_addr[dev];
    return DBD_OK;
}

struct Carver {
    unsigned char *base;
    size_t off = 0;
    template <class T> T *take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T *p = reinterpret_cast<T *>(base + off);
        off += sizeof(T) * (count > 0 ? count : 1);
        return p;
    }
};

// Bytes of scratch the pipeline needs for m rows and nnzA entries of A and
// mB rows of B; the carving below in dbd_spgemm_noalloc takes the same
// regions in this order.
size_t scratch_bytes(int64_t m, int64_t nnzA, int64_t mB) {
    Carver c{nullptr};
    const size_t nt = (size_t)ceil_div(m, kTileRows) + 1;
    c.take<int32_t>((size_t)mB);                   // bmin
    c.take<int32_t>((size_t)mB);                   // bmax
    c.take<int32_t>((size_t)m);                    // rowLo
    c.take<int32_t>((size_t)m);                    // rowHi
    c.take<int64_t>((size_t)m);                    // rowP
    c.take<uint8_t>((size_t)m);                    // symBin
    c.take<uint8_t>((size_t)m);                    // numBin
    c.take<int32_t>((size_t)m);                    // rowNnz
    c.take<int32_t>((size_t)m);                    // symList
    c.take<int32_t>((size_t)m);                    // numList
    c.take<int32_t>(kMaxBins * nt);                // hist
    c.take<int32_t>(kMaxBins * nt);                // symTileOff
    c.take<int32_t>(kMaxBins * nt);                // numTileOff
    c.take<int32_t>(kMaxBins + 1);                 // symStart
    c.take<int32_t>(kMaxBins + 1);                 // numStart
    c.take<int64_t>((size_t)ceil_div(m, kScanTile) + 1);  // part
    c.take<int32_t>(2 * (size_t)nnzA);             // dense-window state
    c.take<int>(4);                                // err + flags
    c.take<uint32_t>(CTR_COUNT);                   // persistent kernels' row counters
    return c.off;
}

#define NA_CK(call)                                                                  \
    do {                                                                             \
        cudaError_t _e = (call);                                                     \
        if (_e != cudaSuccess) {                                                     \
            snprintf(g_msg, sizeof(g_msg), "%s: %s", #call, cudaGetErrorString(_e)); \
            return report(_e == cudaErrorMemoryAllocation ? DBD_ERR_OOM_DEVICE : DBD_ERR_CUDA); \
        }                                                                            \
    } while (0)

}  // namespace

}  // namespace dbd

using namespace dbd;

extern "C" int dbd_spgemm_noalloc(const dbd_csr_view *a, const dbd_csr_view *b, int64_t *c_row_ptr,
                                  int32_t *c_col_idx, double *c_val, int64_t c_capacity, int64_t *c_nnz,
                                  void *stream_handle) {
    g_msg[0] = '\0';
    if (!a || !c_row_ptr || !c_nnz) return fail(DBD_ERR_INVALID, "null argument");
    if (!b) b = a;
    *c_nnz = -1;
    if (!a->on_device || !b->on_device) return fail(DBD_ERR_INVALID, "operands must be device-resident");
    if (a->val_fp32 || b->val_fp32) return fail(DBD_ERR_INVALID, "operands must hold FP64 values");
    if (a->n_cols != b->n_rows) return fail(DBD_ERR_INVALID, "inner dimensions differ");
    if (a->n_rows < 0 || a->n_rows >= INT32_MAX || b->n_cols > INT32_MAX || a->nnz < 0 || b->nnz < 0 ||
        a->nnz > INT32_MAX || b->nnz > INT32_MAX)
        return fail(DBD_ERR_INVALID, "size out of range");
    if ((a->nnz > 0 && (!a->col_idx || !a->val)) || (b->nnz > 0 && (!b->col_idx || !b->val)) || !a->row_ptr ||
        !b->row_ptr)
        return fail(DBD_ERR_INVALID, "null operand array");
    const int64_t m = a->n_rows;
    const size_t need = scratch_bytes(m, a->nnz, b->n_rows);
    if (need > kDbdNoallocScratchBytes) {
        snprintf(g_msg, sizeof(g_msg),
                 "needs %zu bytes of scratch for %lld rows and %lld entries of A; the limit is %zu bytes",
                 need, (long long)m, (long long)a->nnz, kDbdNoallocScratchBytes);
        return report(DBD_ERR_BUDGET);
    }
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    unsigned char *base = nullptr;
    int rc = device_scratch(dev, &base);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream_handle;
    // The call synchronises with the host twice (bin sizes, nnz(C)), which a
    // stream capture cannot hold: refuse it before anything is enqueued.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    if (cap != cudaStreamCaptureStatusNone)
        return fail(DBD_ERR_INVALID, "the stream is capturing: this call synchronises and cannot be captured");
    Carver c{base};  // the layout of scratch_bytes()
    const size_t nt = (size_t)ceil_div(m, kTileRows) + 1;
    int32_t *bmin = c.take<int32_t>((size_t)b->n_rows);
    int32_t *bmax = c.take<int32_t>((size_t)b->n_rows);
    RowInfo ri;
    ri.lo = c.take<int32_t>((size_t)m);
    ri.hi = c.take<int32_t>((size_t)m);
    int64_t *rowP = c.take<int64_t>((size_t)m);
    ri.rowP = rowP;
    uint8_t *symBin = c.take<uint8_t>((size_t)m);
    uint8_t *numBin = c.take<uint8_t>((size_t)m);
    int32_t *rowNnz = c.take<int32_t>((size_t)m);
    int32_t *symList = c.take<int32_t>((size_t)m);
    int32_t *numList = c.take<int32_t>((size_t)m);
    int32_t *hist = c.take<int32_t>(kMaxBins * nt);
    int32_t *symTileOff = c.take<int32_t>(kMaxBins * nt);
    int32_t *numTileOff = c.take<int32_t>(kMaxBins * nt);
    int32_t *symStart = c.take<int32_t>(kMaxBins + 1);
    int32_t *numStart = c.take<int32_t>(kMaxBins + 1);
    int64_t *part = c.take<int64_t>((size_t)ceil_div(m, kScanTile) + 1);
    int32_t *state = c.take<int32_t>(2 * (size_t)a->nnz);
    int *flags = c.take<int>(4);  // [0] device error word, [1] bad row_ptr, [2] bad index, [3] B unsorted
    uint32_t *ctrs = c.take<uint32_t>(CTR_COUNT);

    // The array keeps the previous call's contents: clear what starts at zero.
    NA_CK(cudaMemsetAsync(flags, 0, 4 * sizeof(int), s));
    NA_CK(cudaMemsetAsync(ctrs, 0, sizeof(uint32_t) * CTR_COUNT, s));
    NA_CK(cudaMemsetAsync(rowNnz, 0, sizeof(int32_t) * (size_t)(m > 0 ? m : 1), s));
    int hflags[4] = {0, 0, 0, 0};
    const dbd_csr_view *ops[2] = {a, b};
    // Indices are checked before any kernel gathers through them.
    for (const dbd_csr_view *v : ops) {
        launch_validate_ptr(v->row_ptr, v->n_rows, v->nnz, flags + 1, s);
        NA_CK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        if (hflags[1]) return fail(DBD_ERR_INVALID, "malformed row_ptr");
        launch_validate_idx(v->col_idx, v->nnz, v->n_cols, flags + 2, s);
        NA_CK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        if (hflags[2]) return fail(DBD_ERR_INVALID, "column index out of range");
    }
    CsrDev A, B;
    A.m = a->n_rows; A.n = a->n_cols; A.nnz = a->nnz;
    A.ptr = a->row_ptr; A.idx = a->col_idx; A.val = (const double *)a->val;
    B.m = b->n_rows; B.n = b->n_cols; B.nnz = b->nnz;
    B.ptr = b->row_ptr; B.idx = b->col_idx; B.val = (const double *)b->val;
    int sms = 0;
    NA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    launch_row_minmax(B, bmin, bmax, flags + 3, s, sms);
    // Analysis: products per row, symbolic bins, row lists.
    launch_row_products(A, B.ptr, bmin, bmax, ri, symBin, flags, Tuning{}, s, sms);
    Binning sb{symBin, symList, hist, symTileOff, symStart};
    launch_bin_lists(m, sb, SB_COUNT, s);
    int32_t symStart_h[kMaxBins + 1];
    NA_CK(cudaMemcpyAsync(symStart_h, symStart, sizeof(symStart_h), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    NA_CK(cudaGetLastError());
    if (hflags[0]) return fail(DBD_ERR_DEVICE_CHECK, "a row has more than 2^31 products");
    // Symbolic, row pointer, numeric bins.
    SymArgs sa;
    sa.A = A;
    sa.B = B;
    sa.list = symList;
    sa.binStart = symStart;
    sa.rowNnz = rowNnz;
    sa.ctr = ctrs;
    sa.numSms = sms;
    sa.bSorted = hflags[3] ? 0 : 1;
    sa.err = flags;
    sa.rowLo = ri.lo;
    sa.rowP = ri.rowP;
    sa.rowHi = ri.hi;
    int launches = 0;
    for (int bin = SB_TINY; bin < SB_COUNT; ++bin)
        launch_symbolic_bin(sa, bin, symStart_h[bin], symStart_h[bin + 1] - symStart_h[bin], s, &launches);
    launch_row_scan(m, rowNnz, part, c_row_ptr, s);
    launch_num_bins(m, A.ptr, ri, rowNnz, numBin, Tuning{}, s, sms);
    Binning nb{numBin, numList, hist, numTileOff, numStart};
    launch_bin_lists(m, nb, NB_COUNT, s);
    int64_t nnz = 0;
    int32_t numStart_h[kMaxBins + 1];
    NA_CK(cudaMemcpyAsync(&nnz, c_row_ptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaMemcpyAsync(numStart_h, numStart, sizeof(numStart_h), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    NA_CK(cudaGetLastError());
    if (hflags[0]) return fail(DBD_ERR_DEVICE_CHECK, "symbolic phase: device check failed");
    *c_nnz = nnz;
    if (nnz > c_capacity) {
        snprintf(g_msg, sizeof(g_msg), "output needs %lld entries, capacity is %lld", (long long)nnz,
                 (long long)c_capacity);
        return report(DBD_ERR_BUDGET);
    }
    if (nnz > 0 && (!c_col_idx || !c_val)) return fail(DBD_ERR_INVALID, "null output array");
    NumArgs na;
    na.A = A;
    na.B = B;
    na.list = numList;
    na.Cp = c_row_ptr;
    na.outBase = 0;
    na.Ci = c_col_idx;
    na.Cv = c_val;
    na.state = state;
    na.bSorted = hflags[3] ? 0 : 1;
    na.err = flags;
    na.rowP = rowP;
    na.rowLo = ri.lo;
    na.numSms = sms;
    na.rowHi = ri.hi;
    na.ctr = ctrs;
    for (int bin = NB_TINY; bin < NB_COUNT; ++bin)
        launch_numeric_bin(na, bin, numStart_h[bin], numStart_h[bin + 1], s, &launches);
    NA_CK(cudaMemcpyAsync(hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    NA_CK(cudaGetLastError());
    if (hflags[0]) return fail(DBD_ERR_DEVICE_CHECK, "numeric phase: device check failed");
    return DBD_OK;
}
