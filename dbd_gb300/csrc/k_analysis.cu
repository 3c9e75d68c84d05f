// k_analysis.cu -- work estimate, row categorisation, per-bin row lists and
// the int64 row_ptr scan.
//
// Replaces calculate_UpperBound + get_UpperBound
// (dbd/for_small_datasets/src/preProc.cu:142-179): the reference launches one
// 32-thread CTA per row with a global atomicAdd per A entry, copies the
// counts to the host, scans them sequentially there and copies them back.
// Here eight lanes share a row and reduce with shuffles (no atomics), the
// counts are int64 (the reference's int32 wraps past 2^31 products), and all
// scans stay on the device.
#include "dbd_internal.h"

#include <algorithm>

namespace dbd {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// First and last column of every B row (one warp per row, any column order).
__global__ void k_row_minmax(CsrDev B, int32_t *__restrict__ bmin, int32_t *__restrict__ bmax,
                             int *__restrict__ unsorted) {
    const int lane = threadIdx.x & 31;
    int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t stride = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool down = false;  // some column not above its predecessor
    for (; row < B.m; row += stride) {
        int32_t lo = INT32_MAX, hi = -1;
        const int32_t s = B.ptr[row], e = B.ptr[row + 1];
        for (int32_t i = s + lane; i < e; i += 32) {
            const int32_t c = B.idx[i];
            lo = min(lo, c);
            hi = max(hi, c);
            if (i > s && c <= B.idx[i - 1]) down = true;
        }
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            lo = min(lo, __shfl_xor_sync(FULL, lo, d));
            hi = max(hi, __shfl_xor_sync(FULL, hi, d));
        }
        if (lane == 0) {
            bmin[row] = lo;
            bmax[row] = hi;
        }
    }
    if (down) atomicExch(unsorted, 1);
}

// Products per row, P_r = sum over k in A_r of |B_k|, and the row's column
// window [lo, hi] from the B rows' first and last columns.  Eight lanes per
// row; rows of more than kLongRow entries (power-law hubs, whose serial walk
// by eight lanes would set the kernel's duration) are left to a second
// stage in which a whole CTA takes each of them.
constexpr int kLongRow = 256;

__device__ __forceinline__ void row_products_out(const CsrDev &A, int64_t row, int64_t sum, int32_t lo, int32_t hi,
                                                 RowInfo &ri, uint8_t *symBin, int *err, const Tuning &tune) {
    const int32_t n = A.ptr[row + 1] - A.ptr[row];
    ri.rowP[row] = sum;
    ri.lo[row] = lo;
    ri.hi[row] = hi;
    symBin[row] = sym_bin_of(sum, n, span_words(lo, hi), tune);
    if (sum > 0x7fffffffLL) atomicCAS(err, 0, (int)DEV_ROW_TOO_LONG);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_row_products(CsrDev A, const int32_t *__restrict__ Bp,
                                                          const int32_t *__restrict__ bmin,
                                                          const int32_t *__restrict__ bmax, RowInfo ri,
                                                          uint8_t *__restrict__ symBin, int *err, Tuning tune) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int sub = lane & 7;
    const unsigned gmask = 0xffu << (lane & 24);
    const int64_t stride = ((int64_t)gridDim.x * THREADS) >> 3;
    for (int64_t row = (blockIdx.x * (int64_t)THREADS + tid) >> 3; row < A.m; row += stride) {
        const int32_t s = A.ptr[row], e = A.ptr[row + 1];
        if (e - s > kLongRow) continue;  // the whole group skips together
        int64_t sum = 0;
        int32_t lo = INT32_MAX, hi = -1;
        for (int32_t i = s + sub; i < e; i += 8) {
            const int32_t k = A.idx[i];
            sum += (int64_t)(Bp[k + 1] - Bp[k]);
            lo = min(lo, bmin[k]);
            hi = max(hi, bmax[k]);
        }
#pragma unroll
        for (int d = 4; d; d >>= 1) {
            sum += __shfl_xor_sync(gmask, sum, d, 8);
            lo = min(lo, __shfl_xor_sync(gmask, lo, d, 8));
            hi = max(hi, __shfl_xor_sync(gmask, hi, d, 8));
        }
        if (sub == 0) row_products_out(A, row, sum, lo, hi, ri, symBin, err, tune);
    }

    // Long rows: CTA b takes the long rows r with r = b (mod gridDim.x), one
    // by one with all its threads.  Hubs sit close together in row order
    // (power-law generators put them at small indices), so the modular
    // assignment spreads them over the CTAs.
    __shared__ int32_t longRows[THREADS];
    __shared__ int nLong;
    __shared__ int64_t rs[THREADS / 32];
    __shared__ int32_t rlo[THREADS / 32], rhi[THREADS / 32];
    for (int64_t t0 = 0; t0 < A.m; t0 += (int64_t)gridDim.x * THREADS) {
        if (tid == 0) nLong = 0;
        __syncthreads();
        const int64_t row = t0 + blockIdx.x + (int64_t)gridDim.x * tid;
        if (row < A.m && A.ptr[row + 1] - A.ptr[row] > kLongRow) longRows[atomicAdd(&nLong, 1)] = (int32_t)row;
        __syncthreads();
        const int nl = nLong;
        for (int j = 0; j < nl; ++j) {
            const int32_t r = longRows[j];
            const int32_t s = A.ptr[r], e = A.ptr[r + 1];
            int64_t sum = 0;
            int32_t lo = INT32_MAX, hi = -1;
            for (int32_t i = s + tid; i < e; i += THREADS) {
                const int32_t k = A.idx[i];
                sum += (int64_t)(Bp[k + 1] - Bp[k]);
                lo = min(lo, bmin[k]);
                hi = max(hi, bmax[k]);
            }
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                sum += __shfl_xor_sync(FULL, sum, d);
                lo = min(lo, __shfl_xor_sync(FULL, lo, d));
                hi = max(hi, __shfl_xor_sync(FULL, hi, d));
            }
            if (lane == 0) {
                rs[warp] = sum;
                rlo[warp] = lo;
                rhi[warp] = hi;
            }
            __syncthreads();
            if (tid == 0) {
                for (int w = 1; w < THREADS / 32; ++w) {
                    sum += rs[w];
                    lo = min(lo, rlo[w]);
                    hi = max(hi, rhi[w]);
                }
                row_products_out(A, r, sum, lo, hi, ri, symBin, err, tune);
            }
            __syncthreads();
        }
    }
}

// Products per row block (block_Info of divide_Blocks, ZIP:dbd/src/main.cpp:276-296).
__global__ void k_block_products(int64_t m, const int64_t *__restrict__ rowP,
                                 int64_t rows_per_block, int64_t *__restrict__ blockP) {
    __shared__ int64_t red[32];
    const int64_t b = blockIdx.x;
    const int64_t r0 = b * rows_per_block;
    const int64_t r1 = min(m, r0 + rows_per_block);
    int64_t s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) s += rowP[r];
    for (int d = 16; d; d >>= 1) s += __shfl_xor_sync(FULL, s, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
        for (int d = 16; d; d >>= 1) s += __shfl_xor_sync(FULL, s, d);
        if (threadIdx.x == 0) blockP[b] = s;
    }
}

__global__ void k_num_bins(int64_t m, const int32_t *__restrict__ Ap, RowInfo ri,
                           const int32_t *__restrict__ rowNnz, uint8_t *__restrict__ numBin, Tuning tune) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x)
        numBin[r] = num_bin_of(ri.rowP[r], Ap[r + 1] - Ap[r], rowNnz[r], span_words(ri.lo[r], ri.hi[r]), tune);
}

// Per-tile (kTileRows rows) counts of each bin.
__global__ void k_bin_hist(int64_t m, const uint8_t *__restrict__ bin, int nbins,
                           int32_t *__restrict__ hist) {
    __shared__ int32_t wc[kTileRows / 32][kMaxBins];
    const int64_t r = (int64_t)blockIdx.x * kTileRows + threadIdx.x;
    const int b = r < m ? (int)bin[r] : -1;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = 0; q < nbins; ++q) {
        const unsigned mk = __ballot_sync(FULL, b == q);
        if (lane == 0) wc[w][q] = __popc(mk);
    }
    __syncthreads();
    if (threadIdx.x < nbins) {
        int32_t s = 0;
        for (int i = 0; i < kTileRows / 32; ++i) s += wc[i][threadIdx.x];
        hist[(int64_t)blockIdx.x * kMaxBins + threadIdx.x] = s;
    }
}

// Block-wide exclusive scan of one int per thread (blockDim.x == 1024).
__device__ __forceinline__ int32_t block_excl_scan_1024(int32_t v, int32_t *total, int32_t *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t t = sh[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t y = __shfl_up_sync(FULL, t, d);
            if (lane >= d) t += y;
        }
        sh[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    const int32_t base = w ? sh[w - 1] : 0;
    *total = sh[31];
    __syncthreads();
    return base + x - v;
}

// Exclusive scan of every bin's column of hist over tiles, then absolute
// offsets (bin start + within-bin offset) into tileOff; one CTA of 1024.
__global__ void k_bin_scan(int64_t ntiles, int nbins, const int32_t *__restrict__ hist,
                           int32_t *__restrict__ tileOff, int32_t *__restrict__ binStart) {
    __shared__ int32_t sh[32];
    __shared__ int32_t totals[kMaxBins];
    for (int q = 0; q < nbins; ++q) {
        int32_t carry = 0;
        for (int64_t t0 = 0; t0 < ntiles; t0 += 1024) {
            const int64_t t = t0 + threadIdx.x;
            const int32_t v = t < ntiles ? hist[t * kMaxBins + q] : 0;
            int32_t tot;
            const int32_t ex = block_excl_scan_1024(v, &tot, sh);
            if (t < ntiles) tileOff[t * kMaxBins + q] = carry + ex;
            carry += tot;
        }
        if (threadIdx.x == 0) totals[q] = carry;
        __syncthreads();
    }
    __shared__ int32_t starts[kMaxBins + 1];
    if (threadIdx.x == 0) {
        int32_t s = 0;
        for (int q = 0; q < kMaxBins; ++q) {
            starts[q] = s;
            if (q < nbins) s += totals[q];
        }
        starts[kMaxBins] = s;
        for (int q = 0; q <= kMaxBins; ++q) binStart[q] = starts[q];
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < ntiles * kMaxBins; i += blockDim.x) {
        const int q = (int)(i % kMaxBins);
        if (q < nbins) tileOff[i] += starts[q];
        else tileOff[i] = starts[kMaxBins];
    }
    if (threadIdx.x < kMaxBins)
        tileOff[ntiles * kMaxBins + threadIdx.x] =
            threadIdx.x < nbins ? starts[threadIdx.x] + totals[threadIdx.x] : starts[kMaxBins];
}

// Stable scatter of row ids into their bin's list.
__global__ void k_bin_scatter(int64_t m, const uint8_t *__restrict__ bin, int nbins,
                              const int32_t *__restrict__ tileOff, int32_t *__restrict__ list) {
    __shared__ int32_t wc[kTileRows / 32][kMaxBins];
    const int64_t r = (int64_t)blockIdx.x * kTileRows + threadIdx.x;
    const int b = r < m ? (int)bin[r] : -1;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int rank = 0;
    for (int q = 0; q < nbins; ++q) {
        const unsigned mk = __ballot_sync(FULL, b == q);
        if (b == q) rank = __popc(mk & ((1u << lane) - 1u));
        if (lane == 0) wc[w][q] = __popc(mk);
    }
    __syncthreads();
    if (b >= 0) {
        int32_t pos = tileOff[(int64_t)blockIdx.x * kMaxBins + b] + rank;
        for (int i = 0; i < w; ++i) pos += wc[i][b];
        list[pos] = (int32_t)r;
    }
}

// ---- int32 row counts -> int64 exclusive scan (row_ptr of C) ----

__device__ __forceinline__ int64_t block_excl_scan_i64(int64_t v, int64_t *total, int64_t *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t t = lane < nw ? sh[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(FULL, t, d);
            if (lane >= d) t += y;
        }
        sh[lane] = t;
    }
    __syncthreads();
    const int64_t base = w ? sh[w - 1] : 0;
    *total = sh[nw - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void k_scan_reduce(int64_t m, const int32_t *__restrict__ cnt, int64_t *__restrict__ part) {
    __shared__ int64_t sh[32];
    const int64_t r0 = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        const int64_t r = r0 + i;
        if (r < m) s += cnt[r];
    }
    int64_t tot;
    block_excl_scan_i64(s, &tot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void k_scan_parts(int64_t nparts, int64_t *__restrict__ part) {
    __shared__ int64_t sh[32];
    int64_t carry = 0;
    for (int64_t i0 = 0; i0 < nparts; i0 += blockDim.x) {
        const int64_t i = i0 + threadIdx.x;
        const int64_t v = i < nparts ? part[i] : 0;
        int64_t tot;
        const int64_t ex = block_excl_scan_i64(v, &tot, sh);
        if (i < nparts) part[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) part[nparts] = carry;
}

// blockDim.x == kScanTile / 4: four consecutive rows per thread.
__global__ void k_scan_final(int64_t m, const int32_t *__restrict__ cnt,
                             const int64_t *__restrict__ part, int64_t nparts,
                             int64_t *__restrict__ Cp) {
    __shared__ int64_t sh[32];
    const int64_t r0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * 4;
    int32_t c[4];
    int64_t s = 0;
    for (int j = 0; j < 4; ++j) {
        c[j] = (r0 + j < m) ? cnt[r0 + j] : 0;
        s += c[j];
    }
    int64_t tot;
    int64_t run = part[blockIdx.x] + block_excl_scan_i64(s, &tot, sh);
    for (int j = 0; j < 4; ++j) {
        if (r0 + j < m) Cp[r0 + j] = run;
        run += c[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) Cp[m] = part[nparts];
}

// Widens float32 values (a view with val_fp32) into the FP64 operand copy.
__global__ void k_f32_to_f64(const float *__restrict__ src, double *__restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

// flag <- 1 unless ptr[0] == 0, ptr[m] == nnz and ptr is non-decreasing.
__global__ void k_validate_ptr(const int32_t *__restrict__ ptr, int64_t m, int64_t nnz, int *flag) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= m; r += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ptr[r];
        bool bad = v < 0 || v > nnz;
        if (r == 0) bad |= v != 0;
        if (r == m) bad |= v != nnz;
        if (r < m) bad |= ptr[r + 1] < v;
        if (bad) atomicExch(flag, 1);
    }
}

// flag <- 1 if any column index lies outside [0, ncols).
__global__ void k_validate_idx(const int32_t *__restrict__ idx, int64_t nnz, int64_t ncols, int *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = idx[i];
        if (c < 0 || c >= ncols) atomicExch(flag, 1);
    }
}

}  // namespace

void launch_row_minmax(const CsrDev &B, int32_t *bmin, int32_t *bmax, int *unsorted, cudaStream_t s, int num_sms) {
    if (B.m == 0) return;
    const int grid = (int)std::min<int64_t>(ceil_div(B.m * 32, 256), (int64_t)num_sms * 8);
    k_row_minmax<<<grid, 256, 0, s>>>(B, bmin, bmax, unsorted);
}

void launch_row_products(const CsrDev &A, const int32_t *Bp, const int32_t *bmin, const int32_t *bmax,
                         const RowInfo &ri, uint8_t *symBin, int *err, const Tuning &t, cudaStream_t s,
                         int num_sms) {
    if (A.m == 0) return;
    constexpr int threads = 256;
    const int64_t need = ceil_div(A.m * 8, threads);
    const int grid = (int)std::min<int64_t>(need, (int64_t)num_sms * 8);
    k_row_products<threads><<<grid, threads, 0, s>>>(A, Bp, bmin, bmax, ri, symBin, err, t);
}

void launch_block_products(int64_t m, const int64_t *rowP, int64_t rows_per_block, int64_t *blockP,
                           cudaStream_t s) {
    const int64_t nb = ceil_div(m, rows_per_block);
    if (nb == 0) return;
    k_block_products<<<(unsigned)nb, 256, 0, s>>>(m, rowP, rows_per_block, blockP);
}

void launch_bin_lists(int64_t m, const Binning &b, int nbins, cudaStream_t s) {
    const int64_t ntiles = ceil_div(m, kTileRows);
    if (ntiles > 0) k_bin_hist<<<(unsigned)ntiles, kTileRows, 0, s>>>(m, b.bin, nbins, b.hist);
    k_bin_scan<<<1, 1024, 0, s>>>(ntiles, nbins, b.hist, b.tileOff, b.binStart);
    if (ntiles > 0) k_bin_scatter<<<(unsigned)ntiles, kTileRows, 0, s>>>(m, b.bin, nbins, b.tileOff, b.list);
}

void launch_num_bins(int64_t m, const int32_t *Ap, const RowInfo &ri, const int32_t *rowNnz,
                     uint8_t *numBin, const Tuning &t, cudaStream_t s, int num_sms) {
    if (m == 0) return;
    const int grid = (int)std::min<int64_t>(ceil_div(m, 256), (int64_t)num_sms * 8);
    k_num_bins<<<grid, 256, 0, s>>>(m, Ap, ri, rowNnz, numBin, t);
}

void launch_row_scan(int64_t m, const int32_t *rowNnz, int64_t *part, int64_t *Cp, cudaStream_t s) {
    const int64_t nparts = ceil_div(m, kScanTile);
    if (nparts > 0) k_scan_reduce<<<(unsigned)nparts, 1024, 0, s>>>(m, rowNnz, part);
    k_scan_parts<<<1, 1024, 0, s>>>(nparts, part);
    if (nparts > 0) {
        k_scan_final<<<(unsigned)nparts, kScanTile / 4, 0, s>>>(m, rowNnz, part, nparts, Cp);
    } else {
        cudaMemsetAsync(Cp, 0, sizeof(int64_t), s);
    }
}

void launch_f32_to_f64(const float *src, double *dst, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    k_f32_to_f64<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 4096), 256, 0, s>>>(src, dst, n);
}

void launch_validate_ptr(const int32_t *ptr, int64_t m, int64_t nnz, int *flag, cudaStream_t s) {
    k_validate_ptr<<<(unsigned)std::min<int64_t>(ceil_div(m + 1, 256), 4096), 256, 0, s>>>(ptr, m, nnz, flag);
}

void launch_validate_idx(const int32_t *idx, int64_t nnz, int64_t ncols, int *flag, cudaStream_t s) {
    if (nnz <= 0) return;
    k_validate_idx<<<(unsigned)std::min<int64_t>(ceil_div(nnz, 256), 4096), 256, 0, s>>>(idx, nnz, ncols, flag);
}

// Loads every kernel of this file now (CUDA loads kernels lazily, on first
// launch, by default).  Returns the first error.
cudaError_t preload_analysis_kernels() {
    const void *fns[] = {
        (const void *)k_row_minmax, (const void *)k_row_products<256>, (const void *)k_block_products,
        (const void *)k_num_bins, (const void *)k_bin_hist, (const void *)k_bin_scan, (const void *)k_bin_scatter,
        (const void *)k_scan_reduce, (const void *)k_scan_parts, (const void *)k_scan_final,
        (const void *)k_f32_to_f64, (const void *)k_validate_ptr, (const void *)k_validate_idx,
    };
    for (const void *f : fns) {
        cudaFuncAttributes fa;
        const cudaError_t e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace dbd
