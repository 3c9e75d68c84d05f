// Adjoint kernels (no reference counterpart): gradients of a loss with
// respect to the values of A and B over their fixed patterns, given
// G = dL/dC on the pattern of C = A*B that the forward multiply left on the
// device (CSR, columns ascending in every row):
//   dA = mask_A(G * B^T)   dA(i,k) = sum_j G(i,j) * B(k,j)
//   dB = mask_B(A^T * G)   dB(k,j) = sum_i A(i,k) * G(i,j)
// k_adjoint takes both from A's rows (dB by FP64 reductions); with the
// deterministic option dB comes from its own pass over B's pattern
// (k_entry_rows, the stable radix sort of k_mtx.cu, k_col_ptr, then the
// k_adjoint_db kernels).
#include "dbd_internal.h"
#include "warp_chunk.cuh"

#include <algorithm>

namespace dbd {

namespace {

// Position of column k within C's sorted row [lo, hi), or hi.
__device__ __forceinline__ int64_t find_col(const int32_t *__restrict__ ci, int64_t lo, int64_t hi, int32_t k) {
    const int64_t end = hi;
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if (ci[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && ci[lo] == k) ? lo : end;
}

// One warp per row of A, rows in the forward's numeric order heaviest bins
// first.  Every product (e = (i,k), f = (k,j)) looks up g = G(i,j) in C's
// row i, adds A[e] * g to dB[f] (FP64 reduction at L2) and g * B[f] to dA[e]
// (summed over the adjacent lanes that share e first).
__global__ void __launch_bounds__(256) k_adjoint(AdjArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t item = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (item >= a.nrows) return;
    const int32_t row = a.order ? a.order[a.nrows - 1 - item] : (int32_t)item;
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const int64_t c0 = a.Cp[row], c1 = a.Cp[row + 1];
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
            const int32_t t = t0 + lane;
            const int o = chunk_owner(c, t);
            const int32_t incl_o = __shfl_sync(FULL, c.incl, o);
            const int32_t len_o = __shfl_sync(FULL, c.len, o);
            const int32_t bs_o = __shfl_sync(FULL, c.bs, o);
            const double av = __shfl_sync(FULL, c.a, o);
            const bool valid = t < c.total;
            double ga = 0.0;
            if (valid) {
                const int32_t pos = bs_o + (t - (incl_o - len_o));
                const int32_t k = a.B.idx[pos];
                const int64_t q = find_col(a.Ci, c0, c1, k);
                if (q < c1) {
                    const double g = a.G[q];
                    ga = __dmul_rn(g, a.B.val[pos]);
                    if (a.dB) atomicAdd(&a.dB[pos], __dmul_rn(av, g));
                } else {
                    raise(a.err, DEV_COUNT_MISMATCH);
                }
            }
            // Lanes of one entry are adjacent: sum ga over each run of equal o.
            const int key = valid ? o : -1 - lane;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int ok = __shfl_down_sync(FULL, key, d);
                const double og = __shfl_down_sync(FULL, ga, d);
                if (lane + d < 32 && ok == key) ga += og;
            }
            const int pk = __shfl_up_sync(FULL, key, 1);
            if (valid && (lane == 0 || pk != key)) atomicAdd(&a.dA[e + o], ga);
        }
    }
}

// Each A entry's row, and (column, entry) pairs to sort: one warp per row.
__global__ void __launch_bounds__(256) k_entry_rows(CsrDev A, int32_t *rowOf, uint32_t *keys, uint32_t *vals) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (r >= A.m) return;
    for (int32_t e = A.ptr[r] + lane; e < A.ptr[r + 1]; e += 32) {
        rowOf[e] = (int32_t)r;
        keys[e] = (uint32_t)A.idx[e];
        vals[e] = (uint32_t)e;
    }
}

// Column pointers from the entries sorted by column: column c starts at the
// first entry whose column is >= c.
__global__ void __launch_bounds__(256) k_col_ptr(const uint32_t *__restrict__ cols, int64_t n, int64_t ncols,
                                                 int32_t *__restrict__ colPtr) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = i == 0 ? 0 : (int64_t)cols[i - 1] + 1;
        const int64_t hi = i == n ? ncols : (int64_t)cols[i];
        for (int64_t c = lo; c <= hi; ++c) colPtr[c] = (int32_t)i;
    }
}

// dB = mask_B(A^T G) as its own pass over B's pattern.  Entry (k, j) of B
// sums A(i,k) * G(i,j) down column k of A in row order, each G(i,j) found by
// binary search of C's sorted row i.  The column is cut into segments of
// kAdjSeg entries: one thread per entry of B sums the first segment into
// dB and records how many segments follow; after a scan of those counts,
// k_adjoint_db_tail sums every further segment, one thread each, and
// k_adjoint_db_sum adds them to dB in segment order.  Every sum has a fixed
// order, so dB is identical run to run, and a long column of A (a
// power-law hub) no longer sets the pass's length: no thread sums more
// than kAdjSeg products.
constexpr int kAdjSeg = 32;

// Row of B holding entry f: the k with ptr[k] <= f < ptr[k + 1].
__device__ __forceinline__ int64_t b_row_of(const CsrDev &B, int64_t f) {
    int64_t lo = 0, hi = B.m;
    while (hi - lo > 1) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if ((int64_t)B.ptr[mid] <= f) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Sum of A(i,k) * G(i,j) over the entries [p, pe) of A's column grouping.
__device__ __forceinline__ double column_sum(const AdjDbArgs &a, int32_t p, int32_t pe, int32_t j) {
    double acc = 0.0;
    for (; p < pe; ++p) {
        const uint32_t e = a.perm[p];
        const int32_t i = a.rowOf[e];
        const int64_t c0 = a.Cp[i], c1 = a.Cp[i + 1];
        const int64_t q = find_col(a.Ci, c0, c1, j);
        if (q < c1) acc += __dmul_rn(a.Aval[e], a.G[q]);
        else raise(a.err, DEV_COUNT_MISMATCH);
    }
    return acc;
}

__global__ void __launch_bounds__(256) k_adjoint_db(AdjDbArgs a) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.B.nnz) return;
    const int64_t k = b_row_of(a.B, f);
    const int32_t p0 = a.colPtr[k], p1 = a.colPtr[k + 1];
    const int32_t len = p1 - p0;
    a.dB[f] = column_sum(a, p0, len > kAdjSeg ? p0 + kAdjSeg : p1, a.B.idx[f]);
    a.extra[f] = len > kAdjSeg ? (len - 1) / kAdjSeg : 0;
}

// Segments 1.. of every entry, one thread each (grid-stride over the total,
// which is read on the device), each into its own slot of part.
__global__ void __launch_bounds__(256) k_adjoint_db_tail(AdjDbArgs a) {
    const int64_t total = a.xStart[a.B.nnz];
    if (total > a.partCap) {  // the patterns are not the forward's
        if (blockIdx.x == 0 && threadIdx.x == 0) raise(a.err, DEV_COUNT_MISMATCH);
        return;
    }
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        // f: the entry with xStart[f] <= g < xStart[f + 1].
        int64_t lo = 0, hi = a.B.nnz;
        while (hi - lo > 1) {
            const int64_t mid = lo + ((hi - lo) >> 1);
            if (a.xStart[mid] <= g) lo = mid;
            else hi = mid;
        }
        const int64_t f = lo;
        const int64_t k = b_row_of(a.B, f);
        const int32_t p1 = a.colPtr[k + 1];
        const int64_t pb = (int64_t)a.colPtr[k] + (1 + (g - a.xStart[f])) * kAdjSeg;
        a.part[g] = column_sum(a, (int32_t)pb, (int32_t)min((int64_t)p1, pb + kAdjSeg), a.B.idx[f]);
    }
}

__global__ void __launch_bounds__(256) k_adjoint_db_sum(AdjDbArgs a) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.B.nnz || a.xStart[a.B.nnz] > a.partCap) return;
    const int64_t x0 = a.xStart[f], x1 = a.xStart[f + 1];
    if (x1 == x0) return;
    double acc = a.dB[f];
    for (int64_t g = x0; g < x1; ++g) acc += a.part[g];
    a.dB[f] = acc;
}

}  // namespace

void launch_adjoint_transpose(const CsrDev &A, int32_t *rowOf, uint32_t *keys0, uint32_t *vals0, uint32_t *keys1,
                              uint32_t *vals1, void *scratch, int32_t *colPtr, const uint32_t **perm, cudaStream_t s) {
    if (A.m > 0) k_entry_rows<<<(unsigned)ceil_div(A.m, 8), 256, 0, s>>>(A, rowOf, keys0, vals0);
    int bits = 0;
    while (bits < 32 && ((uint64_t)std::max<int64_t>(A.n - 1, 0) >> bits) != 0) ++bits;
    uint32_t *ks = keys0, *vs = vals0;
    launch_stable_sort_u32(keys0, vals0, keys1, vals1, A.nnz, bits, scratch, s, &ks, &vs);
    const int64_t grid = std::min<int64_t>(ceil_div(A.nnz + 1, 256), 65535);
    k_col_ptr<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, s>>>(ks, A.nnz, A.n, colPtr);
    *perm = vs;
}

int64_t adjoint_db_part_cap(int64_t products) { return products / kAdjSeg + 1; }

void launch_adjoint_db(const AdjDbArgs &a, int64_t *scanPart, int num_sms, cudaStream_t s) {
    if (a.B.nnz <= 0) return;
    const unsigned grid = (unsigned)ceil_div(a.B.nnz, 256);
    k_adjoint_db<<<grid, 256, 0, s>>>(a);
    launch_row_scan(a.B.nnz, a.extra, scanPart, a.xStart, s);
    k_adjoint_db_tail<<<(unsigned)std::max(num_sms, 1) * 8, 256, 0, s>>>(a);
    k_adjoint_db_sum<<<grid, 256, 0, s>>>(a);
}

void launch_adjoint(const AdjArgs &a, cudaStream_t s, int *launches) {
    if (a.nrows <= 0) return;
    k_adjoint<<<(unsigned)ceil_div(a.nrows, 8), 256, 0, s>>>(a);
    ++*launches;
}

}  // namespace dbd
