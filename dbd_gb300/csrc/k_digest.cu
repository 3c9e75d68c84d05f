// k_digest.cu -- per-row digest of C, taken on the device while a chunk of C
// is resident (no reference counterpart: the reference verifies nothing).
//
// An out-of-core product is never whole in any memory: the kernel scope
// overwrites its one device slot chunk after chunk, and the copying scopes
// recycle their host ring.  The digest summarises every row of C while its
// chunk is on the device, so the complete product can be checked afterwards:
//
//   count[r]    entries of row r
//   colHash[r]  sum over the row's entries of mix64(col)          (mod 2^64)
//   valHash[r]  sum of mix64(bits(val) + G * (col + 1)), G = 0x9E3779B97F4A7C15
//               (the golden-ratio increment of SplitMix64)          (mod 2^64)
//   sum[r]      sum of the row's values            (compensated: Neumaier)
//   wsum[r]     sum of val * w(col), w(col) = 0.5 + u(col) in [0.5, 1.5),
//               u(col) = (mix64(col) >> 11) * 2^-53               (compensated)
//   *bad        rows whose columns are not strictly ascending or leave
//               [0, ncols)
//
// The two hashes are order-independent integer sums, so any implementation
// that sees the same entries (the host digest of the pinned copy, the oracle)
// reproduces them bit for bit.  sum and wsum check the values against
// A*(B*1) and A*(B*w), which the oracle gets in O(nnz) without forming C.
// mix64 is the output function of SplitMix64 (Steele, Lea and Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014).
#include <algorithm>
#include <cstdint>

#include "dbd_internal.h"

namespace dbd {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double col_weight(int32_t col) {
    return 0.5 + (double)(mix64((uint64_t)(uint32_t)col) >> 11) * 0x1.0p-53;
}

// Neumaier's compensated sum: (s, c) += x.
__device__ __forceinline__ void neumaier_add(double &s, double &c, double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// (s, c) += (s2, c2), exact in s by Knuth's TwoSum.
__device__ __forceinline__ void two_sum_merge(double &s, double &c, double s2, double c2) {
    const double t = s + s2;
    const double bp = t - s;
    const double e = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = c + c2 + e;
}

// One warp per row of [r0, r1), persistent over the rows.  V is the type the
// values leave the device in (FP64, or float32 for the reference's layout);
// either is hashed and summed as the FP64 number it holds.
template <class V>
__global__ void __launch_bounds__(256) k_row_digest(int64_t r0, int64_t r1, const int64_t *__restrict__ Cp,
                                                    int64_t outBase, const int32_t *__restrict__ Ci,
                                                    const V *__restrict__ Cv, int64_t ncols, RowDigest d) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = r0 + warp; row < r1; row += nwarps) {
        const int64_t b = Cp[row] - outBase, e = Cp[row + 1] - outBase;
        uint64_t h = 0, hv = 0;
        double s = 0.0, sc = 0.0, w = 0.0, wc = 0.0;
        int bad = 0;
        for (int64_t i = b + lane; i < e; i += 32) {
            const int32_t col = __ldcs(Ci + i);
            const double v = (double)__ldcs(Cv + i);
            if (col < 0 || (int64_t)col >= ncols) bad = 1;
            if (i > b && __ldg(Ci + i - 1) >= col) bad = 1;
            const uint64_t mc = mix64((uint64_t)(uint32_t)col);
            h += mc;
            hv += mix64((uint64_t)__double_as_longlong(v) + 0x9E3779B97F4A7C15ull * ((uint64_t)(uint32_t)col + 1));
            neumaier_add(s, sc, v);
            neumaier_add(w, wc, __dmul_rn(v, col_weight(col)));
        }
        for (int o = 16; o > 0; o >>= 1) {
            h += __shfl_xor_sync(0xffffffffu, h, o);
            hv += __shfl_xor_sync(0xffffffffu, hv, o);
            const double s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, sc, o);
            const double w2 = __shfl_xor_sync(0xffffffffu, w, o), d2 = __shfl_xor_sync(0xffffffffu, wc, o);
            two_sum_merge(s, sc, s2, c2);
            two_sum_merge(w, wc, w2, d2);
        }
        bad = __any_sync(0xffffffffu, bad);
        if (lane == 0) {
            d.count[row] = e - b;
            d.colHash[row] = h;
            d.valHash[row] = hv;
            d.sum[row] = s + sc;
            d.wsum[row] = w + wc;
            if (bad) atomicAdd(reinterpret_cast<unsigned long long *>(d.bad), 1ull);
        }
    }
}

// C's values rounded once to float32 (the reference's output type), after
// the FP64 accumulation: dst[i] = src[i] to nearest.
__global__ void __launch_bounds__(256) k_val_to_f32(const double *__restrict__ src, float *__restrict__ dst,
                                                    int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        __stcs(dst + i, __double2float_rn(__ldcs(src + i)));
}

__global__ void __launch_bounds__(256) k_hash_words(const uint32_t *__restrict__ w, int64_t n, uint64_t salt,
                                                    uint64_t *acc) {
    uint64_t h = 0;
    const uint64_t key = salt * 0x9E3779B97F4A7C15ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        h += mix64((((uint64_t)i << 32) | __ldg(w + i)) ^ key);
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(reinterpret_cast<unsigned long long *>(acc), (unsigned long long)h);
}

}  // namespace

void launch_hash_words(const uint32_t *w, int64_t n, uint64_t salt, uint64_t *acc, cudaStream_t s) {
    if (n <= 0 || !w) return;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
    k_hash_words<<<(unsigned)blocks, 256, 0, s>>>(w, n, salt, acc);
}

template <class V>
static void row_digest(int64_t r0, int64_t r1, const int64_t *Cp, int64_t outBase, const int32_t *Ci, const V *Cv,
                       int64_t ncols, const RowDigest &d, cudaStream_t s, int num_sms) {
    if (r1 <= r0) return;
    const int64_t warps = r1 - r0;
    const int64_t blocks = std::min<int64_t>((warps + 7) / 8, (int64_t)num_sms * 8);
    k_row_digest<V><<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(r0, r1, Cp, outBase, Ci, Cv, ncols, d);
}

void launch_row_digest(int64_t r0, int64_t r1, const int64_t *Cp, int64_t outBase, const int32_t *Ci,
                       const double *Cv, int64_t ncols, const RowDigest &d, cudaStream_t s, int num_sms) {
    row_digest(r0, r1, Cp, outBase, Ci, Cv, ncols, d, s, num_sms);
}

void launch_row_digest(int64_t r0, int64_t r1, const int64_t *Cp, int64_t outBase, const int32_t *Ci,
                       const float *Cv, int64_t ncols, const RowDigest &d, cudaStream_t s, int num_sms) {
    row_digest(r0, r1, Cp, outBase, Ci, Cv, ncols, d, s, num_sms);
}

void launch_val_to_f32(const double *src, float *dst, int64_t n, cudaStream_t s, int num_sms) {
    if (n <= 0) return;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 8);
    k_val_to_f32<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n);
}

}  // namespace dbd
