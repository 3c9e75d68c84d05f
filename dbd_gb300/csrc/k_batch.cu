// k_batch.cu -- assembly of a batch of independent products into one
// block-diagonal product.
//
// The operands of pair q are placed at row offset rowOff_q, entry offset
// nnzOff_q and column offset colOff_q of one concatenated CSR operand, so that
// diag(A_0, A_1, ...) * diag(B_0, B_1, ...) = diag(A_0 B_0, A_1 B_1, ...) is a
// single multiply whose row bins hold the rows of every pair.  The gather
// kernels below validate each pair's arrays while they copy them (row_ptr
// spans [0, nnz] and never decreases, every column is inside the pair's
// column range); they never trap, a bad pair sets a flag the host reads.
#include <algorithm>
#include <cstdint>

#include "dbd_internal.h"

namespace dbd {

namespace {

constexpr int kGatherThreads = 256;
constexpr int kGatherPerThread = 8;
constexpr int kGatherTile = kGatherThreads * kGatherPerThread;

// Pair of the first element of this CTA's tile: the last q with off[q] <= x.
__device__ __forceinline__ int64_t first_pair(const int64_t *off, int64_t count, int64_t x) {
    int64_t lo = 0, hi = count - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Row pointers (and the per-row column shift) of the concatenated operand.
// Element r < totalRows belongs to the pair q with rowOff[q] <= r < rowOff[q+1].
__global__ void __launch_bounds__(kGatherThreads)
k_batch_rows(const BatchPair *pairs, const int64_t *rowOff, int64_t count, int64_t totalRows, int64_t totalNnz,
             int32_t *outPtr, int32_t *rowShift, int *bad) {
    __shared__ int64_t q0;
    const int64_t t0 = (int64_t)blockIdx.x * kGatherTile;
    if (threadIdx.x == 0) q0 = first_pair(rowOff, count, t0);
    __syncthreads();
    int64_t q = q0;
    for (int k = 0; k < kGatherPerThread; ++k) {
        const int64_t r = t0 + threadIdx.x + (int64_t)k * kGatherThreads;
        if (r > totalRows) break;
        if (r == totalRows) {
            outPtr[r] = (int32_t)totalNnz;
            break;
        }
        while (rowOff[q + 1] <= r) ++q;
        const BatchPair &p = pairs[q];
        const int64_t lr = r - rowOff[q];
        const int32_t v = p.ptr[lr], w = p.ptr[lr + 1];
        const bool ok = (lr > 0 || v == 0) && w >= v && (lr + 1 < p.m || (int64_t)w == p.nnz);
        if (!ok) atomicOr(bad, 1);
        outPtr[r] = (int32_t)(v + p.nnzOff);
        if (rowShift) rowShift[r] = p.shift;
    }
}

// Column indices (shifted to the pair's column offset) and values.
__global__ void __launch_bounds__(kGatherThreads)
k_batch_entries(const BatchPair *pairs, const int64_t *nnzOff, int64_t count, int64_t totalNnz, int32_t *outIdx,
                double *outVal, int *bad) {
    __shared__ int64_t q0;
    const int64_t t0 = (int64_t)blockIdx.x * kGatherTile;
    if (threadIdx.x == 0) q0 = first_pair(nnzOff, count, t0);
    __syncthreads();
    int64_t q = q0;
    for (int k = 0; k < kGatherPerThread; ++k) {
        const int64_t e = t0 + threadIdx.x + (int64_t)k * kGatherThreads;
        if (e >= totalNnz) break;
        while (nnzOff[q + 1] <= e) ++q;
        const BatchPair &p = pairs[q];
        const int64_t le = e - nnzOff[q];
        const int32_t c = p.idx[le];
        if (c < 0 || (int64_t)c >= p.ncols) atomicOr(bad, 2);
        outIdx[e] = (int32_t)(c + p.colOff);
        const double *src = p.val + le;
        if (src != outVal + e) outVal[e] = *src;
    }
}

// Device-driven multiplies: a bad pair empties both concatenated operands
// (every row pointer 0), so that nothing downstream reads past an operand.
__global__ void __launch_bounds__(256) k_batch_guard(const int *bad, int32_t *ptrA, int64_t nA, int32_t *ptrB,
                                                     int64_t nB) {
    if (!*bad) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nA + nB; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nA) ptrA[i] = 0;
        else if (ptrB) ptrB[i - nA] = 0;
    }
}

// Device-driven multiplies: with an error in the symbolic pass or nnz(C)
// above the output's capacity, every numeric bin is emptied (and *over set
// in the second case), so the numeric kernels write nothing.
__global__ void k_numeric_guard(const int64_t *nnz, int64_t capacity, const int *err, int32_t *binStart, int nbins,
                                int *over) {
    if (threadIdx.x != 0) return;
    const bool full = *nnz > capacity;
    if (full) *over = 1;
    if (full || *err)
        for (int b = 0; b <= nbins; ++b) binStart[b] = 0;
}

__global__ void k_gather_i64(const int64_t *src, const int64_t *idx, int64_t n, int64_t *dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

}  // namespace

void launch_gather_i64(const int64_t *src, const int64_t *idx, int64_t n, int64_t *dst, cudaStream_t s) {
    if (n <= 0) return;
    k_gather_i64<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(src, idx, n, dst);
}

cudaError_t preload_batch_kernels() {
    const void *fns[] = {(const void *)k_batch_rows, (const void *)k_batch_entries, (const void *)k_batch_guard,
                         (const void *)k_numeric_guard, (const void *)k_gather_i64};
    for (const void *f : fns) {
        cudaFuncAttributes fa;
        const cudaError_t e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void launch_batch_guard(const int *bad, int32_t *ptrA, int64_t nA, int32_t *ptrB, int64_t nB, cudaStream_t s,
                        int num_sms) {
    const int64_t n = nA + nB;
    if (n <= 0) return;
    k_batch_guard<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), (int64_t)num_sms * 8), 256, 0, s>>>(bad, ptrA, nA,
                                                                                                     ptrB, nB);
}

void launch_numeric_guard(const int64_t *nnz, int64_t capacity, const int *err, int32_t *binStart, int nbins, int *over,
                          cudaStream_t s) {
    k_numeric_guard<<<1, 32, 0, s>>>(nnz, capacity, err, binStart, nbins, over);
}

void launch_batch_gather(const BatchPair *pairs, const int64_t *rowOff, const int64_t *nnzOff, int64_t count,
                         int64_t totalRows, int64_t totalNnz, int32_t *outPtr, int32_t *outIdx, double *outVal,
                         int32_t *rowShift, int *bad, cudaStream_t s) {
    if (count <= 0) return;
    const int64_t gr = ceil_div(totalRows + 1, kGatherTile);
    k_batch_rows<<<(unsigned)gr, kGatherThreads, 0, s>>>(pairs, rowOff, count, totalRows, totalNnz, outPtr,
                                                          rowShift, bad);
    if (totalNnz > 0) {
        const int64_t ge = ceil_div(totalNnz, kGatherTile);
        k_batch_entries<<<(unsigned)ge, kGatherThreads, 0, s>>>(pairs, nnzOff, count, totalNnz, outIdx, outVal,
                                                                 bad);
    }
}

}  // namespace dbd
