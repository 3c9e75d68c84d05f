// k_spgemm.cu -- symbolic and numeric SpGEMM kernels per row category.
//
// Replaces the reference's expansion kernels rowproduct_{sparse,dense,ddense}
// (dbd/for_small_datasets/src/computeGPU.cu:135-294), its global-memory dense
// merge (:296-329) and its compaction kernel collect (:331-341).  The
// reference writes every intermediate product to HBM and re-reads it for an
// FP32 atomic merge into a dense global row, deciding structure by value
// (|partial sum| < 1e-4).  Here no intermediate product touches HBM; each
// bin of rows (by products, size and column window) has its own kernels:
//
//   tiny rows   (P_r <= 32)     one warp per row, products held one per lane,
//                               duplicates found with __match_any_sync and
//                               summed in Gustavson order (bit-exact FP64)
//   narrow rows (small window)  one warp per row over a window of flag bytes
//                               and FP64 accumulators (symbolic: the length of
//                               the union of the B rows' column runs when
//                               each is one run); warp bitmap ranks
//   short rows  (<= 256 nnz)    one warp per row: symbolic by a shared hash
//                               table; numeric by expand-sort-compress for
//                               rows of at most 256 products, else by the
//                               table, compaction and a bucket sort
//   CTA rows                    the row's A entries staged in shared memory,
//                               warps over consecutive products with several
//                               B loads in flight (warp_range_ld): hash
//                               tables for narrow-span rows, bitmap + word
//                               ranks for rows within 2^18 columns (values in
//                               shared memory or reduced into C in place)
//   wide rows   (symbolic)      persistent CTAs, a shared bitmap over windows
//                               of up to 2^19 columns that stays zero between
//                               rows, kept for the numeric rank kernels
//   dense rows  (numeric)       persistent CTAs, bitmap ranks over 2^19-column
//                               windows in shared memory, work per window
//                               over its non-empty words only, products
//                               reduced into C in place
//
// Structure is decided by index only (a column belongs to a row as soon as a
// product lands on it).  GB300's FP64 pipe is narrow (about two FP64
// instructions per SM per clock), so the numeric kernels spend one FP64
// instruction per product: a fused multiply-add into the accumulator (plain,
// or inside a compare-and-swap loop where lanes may collide), or a multiply
// whose sum the L2 performs (global reductions).  The tiny path rounds each
// product (__dmul_rn) and adds in the oracle's order, reproducing it bit for
// bit; the other paths differ from it by summation order and by the fused
// roundings, well inside the 1e-12 tolerance.
#include "dbd_internal.h"
#include "warp_chunk.cuh"

#include <algorithm>
#include <mutex>
#include <vector>
#include <climits>

namespace dbd {

namespace {

constexpr int32_t EMPTY = -1;

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

__device__ __forceinline__ uint32_t hslot(int32_t c, int shift) {
    return ((uint32_t)c * 0x9E3779B1u) >> shift;
}

// *acc += a * b with one rounding, atomically (a compare-and-swap loop around
// one DFMA; shared or global memory).
__device__ __forceinline__ void atomic_fma(double *acc, double a, double b) {
    unsigned long long *p = reinterpret_cast<unsigned long long *>(acc);
    unsigned long long old = *reinterpret_cast<volatile unsigned long long *>(p), seen;
    do {
        seen = old;
        old = atomicCAS(p, seen, (unsigned long long)__double_as_longlong(
                                     __fma_rn(a, b, __longlong_as_double((long long)seen))));
    } while (old != seen);
}

// A column's offset in its row's window: true when inside [0, limit), else
// records DEV_OUT_OF_WINDOW (the window came from B's row ranges, so this
// only fires when B changed after it was loaded) and the product is skipped.
__device__ __forceinline__ bool in_window(uint32_t rel, uint32_t limit, int *err) {
    if (rel < limit) return true;
    raise(err, DEV_OUT_OF_WINDOW);
    return false;
}

// ---------------------------------------------------------------------------
// Warp-level enumeration of the products of up to 32 consecutive A entries
// (Chunk, load_chunk and chunk_owner in warp_chunk.cuh): product t
// (0 <= t < total) comes from the lane whose inclusive length prefix first
// exceeds t.
// ---------------------------------------------------------------------------
// Steps of B loads a wide-row warp keeps in flight on rows past the touch list.
constexpr int kWideLoads = 4;
// Steps of B loads a warp-hash row keeps in flight.
constexpr int kHashWarpLoads = 2;

// Position in B of product t (all lanes call; result valid when t < total).
__device__ __forceinline__ int32_t chunk_pos(const Chunk &c, int32_t t, double *a_out) {
    const int o = chunk_owner(c, t);
    const int32_t incl_o = __shfl_sync(FULL, c.incl, o);
    const int32_t len_o = __shfl_sync(FULL, c.len, o);
    const int32_t bs_o = __shfl_sync(FULL, c.bs, o);
    if (a_out) *a_out = __shfl_sync(FULL, c.a, o);
    return bs_o + (t - (incl_o - len_o));
}

// ---------------------------------------------------------------------------
// Block-level helpers.
// ---------------------------------------------------------------------------
template <int THREADS>
__device__ __forceinline__ int32_t block_excl_scan(int32_t v, int32_t *total, int32_t *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    int32_t base = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < THREADS / 32; ++i) {
        const int32_t s = sh[i];
        if (i < w) base += s;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return base + x - v;
}

template <int THREADS>
__device__ __forceinline__ int32_t block_min_i32(int32_t v, int32_t *sh) {
#pragma unroll
    for (int d = 16; d; d >>= 1) v = min(v, __shfl_xor_sync(FULL, v, d));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    int32_t r = INT_MAX;
#pragma unroll
    for (int i = 0; i < THREADS / 32; ++i) r = min(r, sh[i]);
    __syncthreads();
    return r;
}

template <int THREADS>
__device__ __forceinline__ int block_sum_i(int v, int *sh) {
#pragma unroll
    for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    int r = 0;
#pragma unroll
    for (int i = 0; i < THREADS / 32; ++i) r += sh[i];
    __syncthreads();
    return r;
}

// Lower bound of target in the ascending bi (the first index whose column
// is >= target), known to lie in [l, h], found by the group of m aligned
// lanes this lane belongs to (m a power of two, lg = log2 m): each step the
// m lanes probe the midpoints of m equal slices of [l, h) at once and the
// range shrinks about m times.  m = 1 is a binary search.  Every lane of
// the warp calls; lanes with l == h wait for their warp.
__device__ __forceinline__ int32_t group_lower_bound(const int32_t *bi, int32_t l, int32_t h, int64_t target,
                                                    int lg) {
    const int lane = threadIdx.x & 31;
    const int m = 1 << lg;
    const int j = lane & (m - 1);
    const int base = lane & ~(m - 1);
    const uint32_t gm = m == 32 ? FULL : (1u << m) - 1u;
    while (__any_sync(FULL, l < h)) {
        const int64_t n = h - l;
        const bool act = l < h;
        const int32_t p = l + (int32_t)((n * (2 * j + 1)) >> (lg + 1));
        const bool below = act && (int64_t)__ldg(&bi[p]) < target;
        const int c = __popc((__ballot_sync(FULL, below) >> base) & gm);
        if (act) {
            // The group's first c probes are below target (bi ascends).
            const int32_t nl = c > 0 ? l + (int32_t)((n * (2 * c - 1)) >> (lg + 1)) + 1 : l;
            const int32_t nh = c < m ? l + (int32_t)((n * (2 * c + 1)) >> (lg + 1)) : h;
            l = nl;
            h = nh;
        }
    }
    return l;
}

// A batch of up to THREADS entries of one A row staged in shared memory,
// keeping only entries whose B row is non-empty: pre[i] = exclusive prefix
// of |B_k| (pre[*nb] = the batch's products), bst[i] = first position of B_k,
// av[i] = A value.  Every staged entry has at least one product, so 32
// consecutive products span at most 32 entries.  Returns the products.
// With clip (B's rows ascending), each entry keeps only the part of its B
// row inside the column window [cLo, cHi), so a row walked window by window
// enumerates each product once.  The two ends of each part are lower-bound
// searches over the B row, which are dependent L2 loads: an entry gets
// as many lanes as the batch leaves free (up to 32), half searching each
// end, so that the CTA waits a few probes instead of two binary searches.
// With cur (a row walked through consecutive windows with the same batch),
// cur[i] carries where entry i's part of the previous window ended, which
// is where this window's starts (carry), and all the entry's lanes search
// the other end.
template <int THREADS, bool VALS>
__device__ __forceinline__ int32_t stage_entries(const CsrDev &A, const CsrDev &B, int32_t eb, int n_in,
                                                 int32_t *pre, int32_t *bst, double *av, int *nb,
                                                 int32_t *sh, bool clip = false, int64_t cLo = 0,
                                                 int64_t cHi = 0, int32_t *cur = nullptr, bool carry = false) {
    const int tid = threadIdx.x;
    int32_t len = 0, s = 0;
    double a = 0.0;
    if (!clip) {
        if (tid < n_in) {
            const int32_t k = A.idx[eb + tid];
            s = B.ptr[k];
            len = B.ptr[k + 1] - s;
            if constexpr (VALS) a = A.val[eb + tid];
        }
    } else {
        // Lanes per entry: L = 2^lgL, the largest with n_in L <= THREADS.
        int lgL = 0;
        while (lgL < 5 && n_in * (2 << lgL) <= THREADS) ++lgL;
        const int L = 1 << lgL;
        const int ent = tid >> lgL, sub = tid & (L - 1);
        int32_t rs = 0, rl = 0;
        if (ent < n_in) {
            const int32_t k = A.idx[eb + ent];
            rs = B.ptr[k];
            rl = B.ptr[k + 1] - rs;
        }
        const int32_t *bi = B.idx + rs;
        bool needLo = false, needHi = false;
        int32_t a0 = 0;
        if (rl > 0) {
            if (carry) a0 = cur[ent] - rs;
            else needLo = (int64_t)__ldg(&bi[0]) < cLo;
            needHi = (int64_t)__ldg(&bi[rl - 1]) >= cHi;
        }
        int32_t lo, hi;
        if (carry || L == 1) {
            // One search per group of L lanes (L == 1: both ends in turn);
            // the lanes of a group reach the same bounds.
            int32_t r0 = a0;
            if (!carry) r0 = group_lower_bound(bi, needLo ? 1 : 0, needLo ? rl : 0, cLo, 0);
            lo = r0;
            hi = group_lower_bound(bi, needHi ? r0 : rl, needHi ? rl - 1 : rl, cHi, lgL);
        } else {
            // Lanes [0, L/2) of the group find the start, [L/2, L) the end
            // (one call site: the searches hold warp votes).
            const bool upper = sub >= L / 2;
            const int32_t l0 = upper ? (needHi ? 0 : rl) : (needLo ? 1 : 0);
            const int32_t h0 = upper ? (needHi ? rl - 1 : rl) : (needLo ? rl : 0);
            const int32_t r = group_lower_bound(bi, l0, h0, upper ? cHi : cLo, lgL - 1);
            const int g0 = (tid & 31) & ~(L - 1);
            lo = __shfl_sync(FULL, r, g0);
            hi = __shfl_sync(FULL, r, g0 + L / 2);
        }
        if (ent < n_in && sub == 0) {
            s = rs + lo;
            len = max(0, hi - lo);
            if (cur) cur[ent] = rs + max(hi, lo);
            if constexpr (VALS) a = A.val[eb + ent];
        }
    }
    int32_t total, kept;
    const int32_t ex = block_excl_scan<THREADS>(len, &total, sh);
    const int32_t slot = block_excl_scan<THREADS>(len > 0 ? 1 : 0, &kept, sh);
    if (len > 0) {
        pre[slot] = ex;
        bst[slot] = s;
        if constexpr (VALS) av[slot] = a;
    }
    if (tid == 0) pre[kept] = total;
    *nb = kept;
    __syncthreads();
    return total;
}

// B's rows ascend strictly: the host's flag, or for a device-driven launch
// the flag the device computed for this run (bUnsorted).
template <class Args>
__device__ __forceinline__ bool b_sorted(const Args &a) {
    return a.bUnsorted ? *a.bUnsorted == 0 : a.bSorted != 0;
}

// Largest i in [0, nb) with pre[i] <= t.
__device__ __forceinline__ int find_entry(const int32_t *pre, int nb, int32_t t) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One warp walks products [tb, te) of a staged batch, 32 per step, in
// groups of U steps whose B loads are all issued before any is used:
// ld(pos) reads what a product needs from B (read-only loads), use(valid, x,
// e) consumes it on every lane (e = staged entry; meaningful when valid).
// A warp keeps U loads in flight instead of one, which hides the L2 latency
// of B's rows.  A step whose products all lie in the current entry (long B
// rows) takes their positions from registers; otherwise each lane finds its
// entry by a 5-step shuffle search among the 32 entry starts after the
// step's first entry.  use is called by all lanes for each step, so it may
// hold warp collectives.
template <int U, class LD, class USE>
__device__ __forceinline__ void warp_range_ld(const int32_t *pre, const int32_t *bst, int nb, int32_t tb,
                                              int32_t te, LD &&ld, USE &&use) {
    if (tb >= te) return;
    const int lane = threadIdx.x & 31;
    int e0 = find_entry(pre, nb, tb);
    int32_t p0 = pre[e0], b0 = bst[e0], p1 = e0 + 1 < nb ? pre[e0 + 1] : INT_MAX;
    for (int32_t g0 = tb; g0 < te; g0 += 32 * U) {
        int32_t pos[U];
        int ent[U];
        bool val[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int32_t t0 = g0 + 32 * u;
            const int32_t t = t0 + lane;
            val[u] = t < te;
            ent[u] = e0;
            pos[u] = b0 + (t - p0);
            if (t0 >= te || p1 > t0 + 31) continue;  // past the range, or all in entry e0
            const int ej = e0 + 1 + lane;
            const int32_t bnd = ej <= nb ? pre[ej] : INT_MAX;
            int o = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int32_t v = __shfl_sync(FULL, bnd, o + step - 1);
                if (v <= t) o += step;
            }
            const int e = min(e0 + o, nb - 1);
            ent[u] = e;
            pos[u] = bst[e] + (t - pre[e]);
            e0 = __shfl_sync(FULL, e, 31);
            p0 = pre[e0];
            b0 = bst[e0];
            p1 = e0 + 1 < nb ? pre[e0 + 1] : INT_MAX;
        }
        using T = decltype(ld(0));
        T x[U];
#pragma unroll
        for (int u = 0; u < U; ++u) x[u] = val[u] ? ld(pos[u]) : T{};
#pragma unroll
        for (int u = 0; u < U; ++u) use(val[u], x[u], ent[u]);
    }
}

// Column and value of a product, as loaded by warp_range_ld.
struct ColVal {
    int32_t c;
    double v;
};

// Sets bit rel of a shared bitmap on lanes with v, one atomicOr per lane.
// Lanes that share a word serialise on it; a segmented OR over runs of such
// lanes (one atomic per run) costs more instructions than that saves, on
// sparse and dense power-law windows alike.
__device__ __forceinline__ void or_bit(uint32_t *bm, bool v, uint32_t rel) {
    if (v) atomicOr(&bm[rel >> 5], 1u << (rel & 31));
}

// Writes the columns of a ranked bitmap with the work balanced by output
// position: thread t writes out[r] = colbase + 32 w + b for the output ranks
// r in [t tot / T, (t + 1) tot / T) below lim, a contiguous run.  The bitmap
// is cut into THREADS groups of G consecutive words (G <= 32); tbase[g] is
// the rank of group g's first column and tmask[g] the mask of its non-empty
// words (both in shared memory).  A thread finds the group holding its
// first rank by binary search, then walks words and bits in order.  (When
// the columns are written by the thread that owns their words instead, a
// thread over a dense stretch of the row writes up to 32 G columns while
// its neighbours write few, and the CTA waits for it.)  The run goes out in
// aligned 16-byte stores, its ragged ends one column at a time: each lane
// of a warp writes its own run, so per-column stores would cost a memory
// transaction per column.
template <int THREADS>
__device__ __forceinline__ void write_columns_balanced(const uint32_t *bits, const int32_t *tbase,
                                                       const uint32_t *tmask, int G, int32_t tot, int32_t *out,
                                                       int64_t lim, int64_t colbase) {
    const int tid = threadIdx.x;
    const int32_t r0 = (int32_t)((int64_t)tot * tid / THREADS);
    const int32_t r1 = (int32_t)min((int64_t)tot * (tid + 1) / THREADS, lim);
    if (r0 >= r1) return;
    // The last group whose first rank is at most r0 holds rank r0 (the
    // next group starts above it, so this one is not empty).
    int lo = 0, hi = THREADS - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tbase[mid] <= r0) lo = mid;
        else hi = mid - 1;
    }
    int g = lo;
    uint32_t m = tmask[g];
    int32_t p = tbase[g];
    int w = G * g + __ffs(m) - 1;
    uint32_t word = bits[w];
    while (p + __popc(word) <= r0) {
        p += __popc(word);
        m &= m - 1u;
        w = G * g + __ffs(m) - 1;
        word = bits[w];
    }
    for (; p < r0; ++p) word &= word - 1u;  // drop the bits before rank r0
    // out + r is 16-byte aligned when (k0 + r) % 4 == 0.
    const uint32_t k0 = (uint32_t)(reinterpret_cast<uintptr_t>(out) >> 2) & 3u;
    int32_t q0 = 0, q1 = 0, q2 = 0, q3 = 0;
    for (; p < r1; ++p) {
        while (!word) {
            m &= m - 1u;
            while (!m) m = tmask[++g];
            w = G * g + __ffs(m) - 1;
            word = bits[w];
        }
        const int b = __ffs(word) - 1;
        word &= word - 1u;
        const int32_t c = (int32_t)(colbase + (w << 5) + b);
        const uint32_t k = (k0 + (uint32_t)p) & 3u;
        if (k == 0) q0 = c;
        else if (k == 1) q1 = c;
        else if (k == 2) q2 = c;
        else q3 = c;
        if (k == 3 || p + 1 == r1) {
            const int32_t first = p - (int32_t)k;  // the quad's first rank
            if (k == 3 && first >= r0) {
                __stcs(reinterpret_cast<int4 *>(out + first), make_int4(q0, q1, q2, q3));
            } else {
                for (int32_t t = max(first, r0); t <= p; ++t) {
                    const uint32_t kt = (k0 + (uint32_t)t) & 3u;
                    __stcs(out + t, kt == 0 ? q0 : (kt == 1 ? q1 : (kt == 2 ? q2 : q3)));
                }
            }
        }
    }
}

// Contiguous share of [0, total) for this warp, in multiples of 32 products.
template <int THREADS>
__device__ __forceinline__ void warp_share(int32_t total, int32_t *tb, int32_t *te) {
    constexpr int NW = THREADS / 32;
    const int64_t per = ((int64_t)total + NW * 32 - 1) / (NW * 32) * 32;
    const int64_t b = (int64_t)(threadIdx.x >> 5) * per;
    *tb = (int32_t)(b < total ? b : (int64_t)total);
    *te = (int32_t)(b + per < total ? b + per : (int64_t)total);
}

template <int GROUP, int ROWS>
__device__ __forceinline__ void group_sync() {
    if constexpr (ROWS > 1) {
        static_assert(GROUP == 32, "multi-row CTAs use one warp per row");
        __syncwarp();
    } else {
        __syncthreads();
    }
}

template <int TABLE>
__device__ __forceinline__ int hash_insert_key(int32_t *keys, int32_t col, int *err) {
    constexpr int SHIFT = 32 - ilog2(TABLE);
    uint32_t h = hslot(col, SHIFT);
#pragma unroll 1
    for (int probe = 0; probe < TABLE; ++probe) {
        const int32_t k = ((volatile int32_t *)keys)[h];
        if (k == col) return 0;
        if (k == EMPTY) {
            const int32_t old = atomicCAS(&keys[h], EMPTY, col);
            if (old == EMPTY) return 1;
            if (old == col) return 0;
        }
        h = (h + 1) & (TABLE - 1);
    }
    raise(err, DEV_TABLE_FULL);
    return 0;
}

template <int TABLE>
__device__ __forceinline__ int hash_insert_slot(int32_t *keys, int32_t col, int *err) {
    constexpr int SHIFT = 32 - ilog2(TABLE);
    uint32_t h = hslot(col, SHIFT);
#pragma unroll 1
    for (int probe = 0; probe < TABLE; ++probe) {
        const int32_t k = ((volatile int32_t *)keys)[h];
        if (k == col) return (int)h;
        if (k == EMPTY) {
            const int32_t old = atomicCAS(&keys[h], EMPTY, col);
            if (old == EMPTY || old == col) return (int)h;
        }
        h = (h + 1) & (TABLE - 1);
    }
    raise(err, DEV_TABLE_FULL);
    return -1;
}

__device__ __forceinline__ int warp_sum_i(int v) {
#pragma unroll
    for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    return v;
}

// Shared-memory layout of the staged entries (after an 8-aligned prefix).
template <int ECAP>
struct StageLayout {
    static constexpr size_t pre = 0;                              // int32[ECAP + 1]
    static constexpr size_t bst = ((4 * (ECAP + 1)) + 7) / 8 * 8;  // int32[ECAP]
    static constexpr size_t av = bst + ((4 * ECAP) + 7) / 8 * 8;  // double[ECAP]
    static constexpr size_t bytes = av + 8 * ECAP;
};

// ======================================================================
// Symbolic kernels: rowNnz[row] = number of distinct columns of C's row.
// ======================================================================

// Tiny rows: one warp per row, all products at once (P_r <= 32, |A_r| <= 32).
__device__ __forceinline__ void sym_tiny_rows(const SymArgs &a, int32_t begin, int32_t count, int64_t vb) {
    const int lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * 8 + (threadIdx.x >> 5);
    if (item >= count) return;
    const int32_t row = a.list[begin + item];
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const Chunk c = load_chunk(a.A, a.B, e0, e1, lane);
    const bool valid = lane < c.total;
    const int32_t j = chunk_pos(c, lane, nullptr);
    const uint32_t key = valid ? (uint32_t)a.B.idx[j] : (0x80000000u | (uint32_t)lane);
    const unsigned grp = __match_any_sync(FULL, key);
    const bool leader = valid && (lane == __ffs(grp) - 1);
    const unsigned lm = __ballot_sync(FULL, leader);
    if (lane == 0) a.rowNnz[row] = __popc(lm);
}

__global__ void __launch_bounds__(256) k_sym_tiny(SymArgs a, int32_t begin, int32_t count) {
    sym_tiny_rows(a, begin, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
__global__ void __launch_bounds__(256) k_sym_tiny_dd(SymArgs a, int bin) {
    const int32_t begin = a.binStart[bin], count = a.binStart[bin + 1] - begin;
    for (int64_t vb = blockIdx.x; vb * 8 < count; vb += gridDim.x) {
        sym_tiny_rows(a, begin, count, vb);
        __syncthreads();
    }
}

// Warp hash rows: one warp per row, ROWS rows per CTA, TABLE keys per row.
template <int ROWS, int TABLE>
__device__ __forceinline__ void sym_hash_warp_rows(const SymArgs &a, int32_t begin, int32_t count, int64_t vb) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * ROWS + g;
    if (item >= count) return;
    int32_t *keys = reinterpret_cast<int32_t *>(smem) + (size_t)g * TABLE;
    const int32_t row = a.list[begin + item];
    for (int i = lane; i < TABLE; i += 32) keys[i] = EMPTY;
    __syncwarp();
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    int cnt = 0;
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32 * kHashWarpLoads) {
            int32_t col[kHashWarpLoads];
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                col[u] = -1;
                const int32_t t = t0 + 32 * u + lane;
                if (t0 + 32 * u < c.total) {
                    const int32_t j = chunk_pos(c, t, nullptr);
                    if (t < c.total) col[u] = __ldg(&a.B.idx[j]);
                }
            }
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u)
                if (col[u] >= 0) cnt += hash_insert_key<TABLE>(keys, col[u], a.err);
        }
    }
    cnt = warp_sum_i(cnt);
    if (lane == 0) a.rowNnz[row] = cnt;
}

template <int ROWS, int TABLE>
__global__ void __launch_bounds__(32 * ROWS) k_sym_hash_warp(SymArgs a, int32_t begin, int32_t count) {
    sym_hash_warp_rows<ROWS, TABLE>(a, begin, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int ROWS, int TABLE>
__global__ void __launch_bounds__(32 * ROWS) k_sym_hash_warp_dd(SymArgs a, int bin) {
    const int32_t begin = a.binStart[bin], count = a.binStart[bin + 1] - begin;
    for (int64_t vb = blockIdx.x; vb * ROWS < count; vb += gridDim.x) {
        sym_hash_warp_rows<ROWS, TABLE>(a, begin, count, vb);
        __syncthreads();
    }
}

// CTA hash rows: one CTA per row, products spread over all threads.
template <int THREADS, int TABLE>
__device__ __forceinline__ void sym_hash_cta_rows(const SymArgs &a, int32_t begin, int64_t vb) {
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    __shared__ int32_t sh[THREADS / 32];
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    int32_t *keys = reinterpret_cast<int32_t *>(smem + L::bytes);
    const int tid = threadIdx.x;
    const int32_t row = a.list[begin + vb];
    for (int i = tid; i < TABLE; i += THREADS) keys[i] = EMPTY;
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    int cnt = 0;
    for (int32_t eb = e0; eb < e1; eb += THREADS) {
        int nb;
        const int32_t total =
            stage_entries<THREADS, false>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, nullptr, &nb, sh);
        int32_t tb, te;
        warp_share<THREADS>(total, &tb, &te);
        warp_range_ld<4>(
            pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
            [&](bool v, int32_t col, int) {
                if (v) cnt += hash_insert_key<TABLE>(keys, col, a.err);
            });
        __syncthreads();
    }
    cnt = block_sum_i<THREADS>(cnt, sh);
    if (tid == 0) a.rowNnz[row] = cnt;
}

template <int THREADS, int TABLE>
__global__ void __launch_bounds__(THREADS) k_sym_hash_cta(SymArgs a, int32_t begin) {
    sym_hash_cta_rows<THREADS, TABLE>(a, begin, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int THREADS, int TABLE>
__global__ void __launch_bounds__(THREADS) k_sym_hash_cta_dd(SymArgs a, int bin) {
    const int32_t begin = a.binStart[bin], count = a.binStart[bin + 1] - begin;
    for (int64_t vb = blockIdx.x; vb < count; vb += gridDim.x) {
        sym_hash_cta_rows<THREADS, TABLE>(a, begin, vb);
        __syncthreads();
    }
}

// or_bit that also counts and records: returns the number of bits this
// lane newly set (its bit, if the word's old value lacked it), and appends
// every word it finds zero to touched[] (through *nt; entries past cap are
// dropped, *nt still counts them).  Lanes that share a bit or a word
// serialise on its atomic, so exactly one of them counts the bit and one
// records the word.
__device__ __forceinline__ int or_bits_count(uint32_t *bm, bool v, uint32_t rel, int32_t *touched, int *nt,
                                             int cap) {
    if (!v) return 0;
    const uint32_t bit = 1u << (rel & 31);
    const uint32_t old = atomicOr(&bm[rel >> 5], bit);
    if (cap > 0 && old == 0u) {
        const int k = atomicAdd(nt, 1);
        if (k < cap) touched[k] = (int32_t)(rel >> 5);
    }
    return (old & bit) ? 0 : 1;
}

// Words a wide-row window clears one by one: past a quarter of the window a
// full clear is as cheap.
__host__ __device__ __forceinline__ int wide_touch_cap(int winBits) {
    return min(kWideTouchMax, (winBits >> 5) / 4);
}

// Wide rows: persistent CTAs take rows from a counter (heavy rows spread
// over the whole grid).  A shared bitmap over windows of winBits columns
// stays zero between rows: every window records the words it touched and
// clears only those (the whole window when more than kWideTouchMax were
// touched).  The row's size is the sum of newly set bits, so no popcount
// pass over the window either: a row costs its products, not its span.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_sym_wide(SymArgs a, int32_t begin, int32_t count, int winBits) {
    if (begin < 0) {  // device-driven: the bin's rows from the bin table
        begin = a.binStart[SB_WIDE];
        count = a.binStart[SB_WIDE + 1] - begin;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    __shared__ int32_t sh[THREADS / 32];
    __shared__ int nt;
    __shared__ int32_t next;
    __shared__ int32_t slot;
    __shared__ int32_t slabSh[kWideWindowBitsMax >> kSlabShift];
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    uint32_t *bm = reinterpret_cast<uint32_t *>(smem + L::bytes);
    int32_t *touched = reinterpret_cast<int32_t *>(bm + (winBits >> 5));
    const int cap = wide_touch_cap(winBits);
    int32_t *cur = touched + cap;  // per staged entry: its B cursor across windows
    const int tid = threadIdx.x;
    for (int i = tid; i < (winBits >> 5); i += THREADS) bm[i] = 0u;
    for (;;) {
        if (tid == 0) next = (int32_t)atomicAdd(&a.ctr[CTR_SYM_WIDE], 1u);
        __syncthreads();
        const int32_t item = next;
        if (item >= count) break;
        const int32_t row = a.list[begin + item];
        const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
        // The row's window [lo, hi], in windows of winBits columns from lo's word.
        const int32_t rlo = a.rowLo[row], rhi = a.rowHi[row];
        const int sw = span_words(rlo, rhi);
        const int64_t base = (int64_t)(rlo >> 5) << 5;
        const int64_t end = (int64_t)rhi + 1;
        // Rows with more products than the list holds touch more words than
        // it holds as a rule: they set their bits with plain ORs (no old
        // values, no bookkeeping) and count, keep and clear the window in one
        // sweep over its words.
        const int rowCap = a.rowP[row] <= cap ? cap : 0;
        const bool keep = a.wideBits && sw <= kRankWordsMax;
        // Heavy rows record their entries per slab of 2^kSlabShift columns
        // (from `base`), for the numeric pass to cut them into pieces.
        if (tid == 0) {
            int32_t sl = -1;
            const int64_t nslabs = ((end - base) + (1 << kSlabShift) - 1) >> kSlabShift;
            if (a.slabCnt && !rowCap && a.rowP[row] >= kHeavyP && winBits >= (1 << kSlabShift) &&
                nslabs <= kMaxSlabs) {
                sl = (int32_t)atomicAdd(&a.ctr[CTR_HEAVY], 1u);
                if (sl >= a.heavyCap) sl = -1;
            }
            slot = sl;
            if (a.heavySlot) a.heavySlot[row] = sl;
        }
        int cnt = 0;
        // Rows over several windows enumerate, per window, only the part of
        // each B row inside it (B's rows ascending).
        const bool clip = b_sorted(a) && end - base > (int64_t)winBits;
        const bool once = e1 - e0 <= THREADS;  // one batch: its cursors carry over the windows
        for (int64_t c_lo = base; c_lo < end; c_lo += winBits) {
            const int words = (int)min((int64_t)winBits, end - c_lo + 31) >> 5;
            if (tid == 0) nt = rowCap ? 0 : cap + 1;
            if (tid < (kWideWindowBitsMax >> kSlabShift)) slabSh[tid] = 0;
            __syncthreads();
            for (int32_t eb = e0; eb < e1; eb += THREADS) {
                int nb;
                const int32_t total =
                    stage_entries<THREADS, false>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, nullptr, &nb, sh, clip,
                                                  c_lo, c_lo + winBits, once ? cur : nullptr, once && c_lo != base);
                int32_t tb, te;
                warp_share<THREADS>(total, &tb, &te);
                if (rowCap) {
                    warp_range_ld<kWideLoads>(
                        pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
                        [&](bool v, int32_t col, int) {
                            const int64_t rel = v ? (int64_t)col - c_lo : -1;
                            const bool in = rel >= 0 && rel < winBits;
                            cnt += or_bits_count(bm, in, in ? (uint32_t)rel : 0u, touched, &nt, rowCap);
                        });
                } else {
                    warp_range_ld<kWideLoads>(
                        pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
                        [&](bool v, int32_t col, int) {
                            const int64_t rel = v ? (int64_t)col - c_lo : -1;
                            if (rel >= 0 && rel < winBits) atomicOr(&bm[rel >> 5], 1u << (rel & 31));
                        });
                }
                __syncthreads();
            }
            if (!rowCap) {
                uint32_t *dst = keep ? a.wideBits + (size_t)item * kRankWordsMax : nullptr;
                const int32_t sl = slot;
                if (sl < 0) {
                    for (int i = tid; i < words; i += THREADS) {
                        const uint32_t x = bm[i];
                        cnt += __popc(x);
                        if (dst) __stcs(&dst[i], x);
                        bm[i] = 0u;
                    }
                } else {
                    // Groups of 32 consecutive words per thread (a slab is 64
                    // groups); lanes start at different words of their group
                    // so that a warp's loads hit 32 banks.
                    const int lane = tid & 31;
                    for (int g = tid; 32 * g < words; g += THREADS) {
                        int c = 0;
                        for (int k = 0; k < 32; ++k) {
                            const int i = 32 * g + ((k + lane) & 31);
                            if (i < words) {
                                const uint32_t x = bm[i];
                                c += __popc(x);
                                if (dst) __stcs(&dst[i], x);
                                bm[i] = 0u;
                            }
                        }
                        cnt += c;
                        if (c) atomicAdd(&slabSh[(32 * g) >> (kSlabShift - 5)], c);
                    }
                    __syncthreads();
                    const int s0 = (int)((c_lo - base) >> kSlabShift);
                    const int ns = (words + (1 << (kSlabShift - 5)) - 1) >> (kSlabShift - 5);
                    for (int t = tid; t < ns; t += THREADS) a.slabCnt[(size_t)sl * kMaxSlabs + s0 + t] = slabSh[t];
                }
                if (keep && tid == 0) a.wideSlot[row] = item;
                __syncthreads();
                continue;
            }
            if (keep) {
                // One window covers the row here; keep its bitmap for the numeric pass.
                uint32_t *dst = a.wideBits + (size_t)item * kRankWordsMax;
                for (int i = tid; i < sw; i += THREADS) __stcs(&dst[i], bm[i]);
                if (tid == 0) a.wideSlot[row] = item;
                __syncthreads();
            }
            const int n = nt;
            if (n <= cap) {
                for (int i = tid; i < n; i += THREADS) bm[touched[i]] = 0u;
            } else {
                for (int i = tid; i < words; i += THREADS) bm[i] = 0u;
            }
            __syncthreads();
        }
        cnt = block_sum_i<THREADS>(cnt, sh);
        if (tid == 0) a.rowNnz[row] = cnt;
    }
}

// Size of a row of C whose B rows are each one contiguous run of columns
// (banded and stencil matrices), with the runs' first columns non-decreasing
// in A's entry order: the length of the union of the runs, by a prefix
// maximum of the runs' last columns (the run of entry i adds the part of
// [first_i, last_i] beyond every earlier run's end).  One warp, 32 entries a
// step, no per-column work.  Returns false (count unset) when some B row is
// not one run or the first columns decrease; B's rows must ascend strictly.
__device__ __forceinline__ bool interval_union_count(const CsrDev &A, const CsrDev &B, int32_t e0, int32_t e1,
                                                     int lane, int *count) {
    int32_t endMax = INT32_MIN, firstMax = INT32_MIN;  // over the entries of earlier steps
    int cnt = 0;
    for (int32_t eb = e0; eb < e1; eb += 32) {
        bool has = false;
        int32_t f = INT32_MIN, l = INT32_MIN;
        bool run = true;
        if (eb + lane < e1) {
            const int32_t k = A.idx[eb + lane];
            const int32_t bs = B.ptr[k], len = B.ptr[k + 1] - bs;
            if (len > 0) {
                has = true;
                f = __ldg(&B.idx[bs]);
                l = __ldg(&B.idx[bs + len - 1]);
                run = l - f == len - 1;
            }
        }
        // Inclusive prefix maxima of the first and last columns over lanes.
        int32_t fm = f, lm = l;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t yf = __shfl_up_sync(FULL, fm, d), yl = __shfl_up_sync(FULL, lm, d);
            if (lane >= d) {
                fm = max(fm, yf);
                lm = max(lm, yl);
            }
        }
        int32_t fPrev = __shfl_up_sync(FULL, fm, 1), lPrev = __shfl_up_sync(FULL, lm, 1);
        if (lane == 0) {
            fPrev = INT32_MIN;
            lPrev = INT32_MIN;
        }
        fPrev = max(fPrev, firstMax);
        lPrev = max(lPrev, endMax);
        if (!__all_sync(FULL, run && (!has || f >= fPrev))) return false;
        int add = 0;
        if (has) add = (int)max(0LL, (long long)l - max((long long)f - 1, (long long)lPrev));
        cnt += warp_sum_i(add);
        firstMax = max(firstMax, __shfl_sync(FULL, fm, 31));
        endMax = max(endMax, __shfl_sync(FULL, lm, 31));
    }
    *count = cnt;
    return true;
}

// Products of one row for one warp, calling f(j, av) for every product (B
// position j, A value av) on the lane that owns it: 32 products of up to 32
// A entries per step (Chunk).  Callers with long B rows walk them row-wise
// themselves.
template <class F>
__device__ __forceinline__ void warp_products(const CsrDev &A, const CsrDev &B, int32_t e0, int32_t e1, int lane,
                                              F &&f) {
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(A, B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
            const int32_t t = t0 + lane;
            double av;
            const int32_t j = chunk_pos(c, t, &av);
            if (t < c.total) f(j, av);
        }
    }
}

// Average B row length from which a row is enumerated row-wise.
constexpr int kRowwiseMinLen = 16;

// Narrow rows (window of at most kWarpSpanWords words): one warp per row,
// one flag byte per column of the window in shared memory; the row's size is
// the number of flags set.
template <int ROWS>
__device__ __forceinline__ void sym_flagw_rows(const SymArgs &a, int32_t begin, int32_t count, int64_t vb) {
    constexpr int kWords = kWarpSpanWords * 8;  // 32 flag bytes per window word
    __shared__ uint32_t fls[ROWS][kWords];
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * ROWS + g;
    if (item >= count) return;
    uint32_t *fw = fls[g];
    uint8_t *fb = reinterpret_cast<uint8_t *>(fw);
    const int32_t row = a.list[begin + item];
    const int32_t rlo = a.rowLo[row];
    const int32_t base = (rlo >> 5) << 5;
    const int sw = min(span_words(rlo, a.rowHi[row]), kWarpSpanWords);
    const uint32_t nb = (uint32_t)sw * 32u;
    for (int i = lane; i < sw * 8; i += 32) fw[i] = 0u;
    __syncwarp();
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const bool rowwise = a.rowP[row] >= (int64_t)kRowwiseMinLen * (e1 - e0);
    int *err = a.err;
    const int32_t *bidx = a.B.idx;
    if (rowwise && b_sorted(a)) {
        int cnt;
        if (interval_union_count(a.A, a.B, e0, e1, lane, &cnt)) {
            if (lane == 0) a.rowNnz[row] = cnt;
            return;
        }
    }
    if (rowwise) {
        // One A entry at a time.  A B row whose columns form one contiguous
        // run (banded and stencil matrices) flags its run a word (4 columns)
        // per lane; any other B row flags a column per lane.
        for (int32_t eb = e0; eb < e1; eb += 32) {
            // Each lane loads its entry's B row bounds and first and last
            // columns up front, so the entries below need no loads of their
            // own before flagging.
            int32_t bs = 0, len = 0, fc = 0, lc = 0;
            if (eb + lane < e1) {
                const int32_t k = a.A.idx[eb + lane];
                bs = a.B.ptr[k];
                len = a.B.ptr[k + 1] - bs;
                if (len > 0) {
                    fc = __ldg(&bidx[bs]);
                    lc = __ldg(&bidx[bs + len - 1]);
                }
            }
            const int n = min(32, e1 - eb);
            for (int q = 0; q < n; ++q) {
                const int32_t bq = __shfl_sync(FULL, bs, q);
                const int32_t lq = __shfl_sync(FULL, len, q);
                const int32_t first = __shfl_sync(FULL, fc, q), last = __shfl_sync(FULL, lc, q);
                if (lq == 0) continue;
                const uint32_t r0 = (uint32_t)(first - base), r1 = (uint32_t)(last - base);
                if (b_sorted(a) && last - first == lq - 1 && r0 < nb && r1 < nb) {
                    for (uint32_t w = (r0 >> 2) + lane; w <= (r1 >> 2); w += 32) {
                        uint32_t m = 0x01010101u;
                        if (w == (r0 >> 2)) m &= 0xffffffffu << (8 * (r0 & 3));
                        if (w == (r1 >> 2)) m &= 0xffffffffu >> (8 * (3 - (r1 & 3)));
                        atomicOr(&fw[w], m);
                    }
                } else {
                    for (int32_t i = lane; i < lq; i += 32) {
                        const uint32_t rel = (uint32_t)(bidx[bq + i] - base);
                        if (in_window(rel, nb, err)) fb[rel] = 1;
                    }
                }
                __syncwarp();
            }
        }
    } else {
        warp_products(a.A, a.B, e0, e1, lane, [&](int32_t j, double) {
            const uint32_t rel = (uint32_t)(bidx[j] - base);
            if (in_window(rel, nb, err)) fb[rel] = 1;
        });
    }
    __syncwarp();
    int cnt = 0;
    for (int i = lane; i < sw * 8; i += 32) cnt += __popc(fw[i]);
    cnt = warp_sum_i(cnt);
    if (lane == 0) a.rowNnz[row] = cnt;
}

template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_sym_flagw(SymArgs a, int32_t begin, int32_t count) {
    sym_flagw_rows<ROWS>(a, begin, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_sym_flagw_dd(SymArgs a, int bin) {
    const int32_t begin = a.binStart[bin], count = a.binStart[bin + 1] - begin;
    for (int64_t vb = blockIdx.x; vb * ROWS < count; vb += gridDim.x) {
        sym_flagw_rows<ROWS>(a, begin, count, vb);
        __syncthreads();
    }
}

// ======================================================================
// Numeric kernels: columns ascending, values in FP64.
// ======================================================================

// Amount subtracted from the columns a row writes (0 unless batched).
__device__ __forceinline__ int32_t col_shift(const NumArgs &a, int32_t row) {
    return a.colShift ? a.colShift[row] : 0;
}

__device__ __forceinline__ void num_tiny_rows(const NumArgs &a, int32_t lo, int32_t count, int64_t vb) {
    const int lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * 8 + (threadIdx.x >> 5);
    if (item >= count) return;
    const int32_t row = a.list[lo + item];
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const Chunk c = load_chunk(a.A, a.B, e0, e1, lane);
    const bool valid = lane < c.total;
    double av;
    const int32_t j = chunk_pos(c, lane, &av);
    int32_t col = -1;
    double p = 0.0;
    if (valid) {
        col = a.B.idx[j];
        p = __dmul_rn(av, a.B.val[j]);
    }
    const uint32_t key = valid ? (uint32_t)col : (0x80000000u | (uint32_t)lane);
    const unsigned grp = __match_any_sync(FULL, key);
    const bool leader = valid && (lane == __ffs(grp) - 1);
    const unsigned lm = __ballot_sync(FULL, leader);
    double acc = 0.0;
    int rank = 0;
#pragma unroll
    for (int q = 0; q < 32; ++q) {
        const double pq = __shfl_sync(FULL, p, q);
        const int32_t cq = __shfl_sync(FULL, col, q);
        if ((grp >> q) & 1u) acc = __dadd_rn(acc, pq);
        if (((lm >> q) & 1u) && cq < col) ++rank;
    }
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    const int64_t base = a.Cp[row] - a.outBase;
    if (leader && rank < expect) {
        a.Ci[base + rank] = col - col_shift(a, row);
        a.Cv[base + rank] = acc;
    }
    if (lane == 0 && __popc(lm) != expect) raise(a.err, DEV_COUNT_MISMATCH);
}

__global__ void __launch_bounds__(256) k_num_tiny(NumArgs a, int32_t lo, int32_t count) {
    num_tiny_rows(a, lo, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
__global__ void __launch_bounds__(256) k_num_tiny_dd(NumArgs a, int bin) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb * 8 < count; vb += gridDim.x) {
        num_tiny_rows(a, lo, count, vb);
        __syncthreads();
    }
}

// Bitonic sort of buf[0, N) ascending by GROUP threads (N a power of two).
template <int GROUP, int ROWS>
__device__ __forceinline__ void group_bitonic(uint64_t *buf, int N, int gt) {
    for (int k = 2; k <= N; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int i = gt; i < N; i += GROUP) {
                const int ixj = i ^ jj;
                if (ixj > i) {
                    const uint64_t x = buf[i], y = buf[ixj];
                    const bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        buf[i] = y;
                        buf[ixj] = x;
                    }
                }
            }
            group_sync<GROUP, ROWS>();
        }
    }
}

// One warp orders n <= kBucketN packed (column << 32 | slot) entries of a
// row whose columns lie in [lo, lo + span): a counting sort by bucket
// (256 buckets of equal column width, each lane owning 8), then insertion
// sort inside each bucket.  Rows of uniform columns put a few entries in
// each bucket, so this costs a few operations per entry instead of a
// bitonic network.  Returns false (nothing written) when a bucket holds
// more than 32 entries (clustered columns); the caller sorts otherwise.
constexpr int kBuckets = 256;
__device__ __forceinline__ bool warp_bucket_order(const uint64_t *in, int n, int32_t lo, int64_t span, int *cnts,
                                                  uint64_t *out) {
    const int lane = threadIdx.x & 31;
    for (int b = lane; b < kBuckets; b += 32) cnts[b] = 0;
    __syncwarp();
    constexpr int PER = kNumWarpMax / 32;  // entries per lane
    uint64_t key[PER];
    int bk[PER], rk[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int i = lane + 32 * u;
        bk[u] = -1;
        if (i < n) {
            key[u] = in[i];
            const int64_t rel = (int64_t)(int32_t)(key[u] >> 32) - lo;
            bk[u] = (int)min((int64_t)kBuckets - 1, max((int64_t)0, rel * kBuckets / span));
            rk[u] = atomicAdd(&cnts[bk[u]], 1);
        }
    }
    __syncwarp();
    // Lane l owns buckets [8 l, 8 l + 8): counts -> starts.
    int c8[8], mine = 0, mx = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        c8[q] = cnts[8 * lane + q];
        mine += c8[q];
        mx = max(mx, c8[q]);
    }
#pragma unroll
    for (int d = 16; d; d >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, d));
    if (mx > 32) return false;
    int incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    int st = incl - mine;
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        cnts[8 * lane + q] = st;
        st += c8[q];
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < PER; ++u)
        if (bk[u] >= 0) out[cnts[bk[u]] + rk[u]] = key[u];
    __syncwarp();
    // Insertion sort inside each of this lane's buckets (by column).
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int s0 = cnts[8 * lane + q], c = c8[q];
        for (int i = 1; i < c; ++i) {
            const uint64_t v = out[s0 + i];
            int j = i - 1;
            while (j >= 0 && (out[s0 + j] >> 32) > (v >> 32)) {
                out[s0 + j + 1] = out[s0 + j];
                --j;
            }
            out[s0 + j + 1] = v;
        }
    }
    __syncwarp();
    return true;
}

// Compacts the occupied slots of a (keys, vals) table into sbuf (which
// aliases keys) as packed (column, slot) pairs, sorts them and writes the
// row.  GROUP threads per row; all of them call.  One-warp rows pass
// bucket buffers (cnts, bbuf) and are ordered by warp_bucket_order when
// their columns spread evenly.
template <int GROUP, int ROWS, int TABLE>
__device__ __forceinline__ void table_write_sorted(const NumArgs &a, int32_t row, int32_t *keys, const double *vals,
                                                   int *gcnt, int gt, int *cnts = nullptr,
                                                   uint64_t *bbuf = nullptr) {
    constexpr int KPT = TABLE / GROUP;
    constexpr int NMAX = TABLE / 2;
    const int lane = threadIdx.x & 31;
    uint64_t *sbuf = reinterpret_cast<uint64_t *>(keys);
    int32_t mk[KPT];
#pragma unroll
    for (int q = 0; q < KPT; ++q) mk[q] = keys[gt + q * GROUP];
    group_sync<GROUP, ROWS>();
#pragma unroll
    for (int q = 0; q < KPT; ++q) {
        const bool occ = mk[q] != EMPTY;
        const unsigned bal = __ballot_sync(FULL, occ);
        int wbase = 0;
        if (lane == 0 && bal) wbase = atomicAdd(gcnt, __popc(bal));
        wbase = __shfl_sync(FULL, wbase, 0);
        if (occ) {
            const int pos = wbase + __popc(bal & ((1u << lane) - 1u));
            if (pos < NMAX) sbuf[pos] = ((uint64_t)(uint32_t)mk[q] << 32) | (uint32_t)(gt + q * GROUP);
        }
    }
    group_sync<GROUP, ROWS>();
    const int n = *gcnt;
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    if (gt == 0 && (n != expect || n > NMAX)) raise(a.err, DEV_COUNT_MISMATCH);
    const int nn = min(n, NMAX);
    const uint64_t *sorted = sbuf;
    bool done = false;
    if constexpr (GROUP == 32 && ROWS > 1 && NMAX <= kNumWarpMax) {
        if (cnts) {
            const int32_t lo = a.rowLo[row];
            const int64_t span = max((int64_t)1, (int64_t)a.rowHi[row] - lo + 1);
            done = warp_bucket_order(sbuf, nn, lo, span, cnts, bbuf);
            if (done) sorted = bbuf;
        }
    }
    if (!done) {
        int N = 1;
        while (N < nn) N <<= 1;
        for (int i = nn + gt; i < N; i += GROUP) sbuf[i] = ~0ull;
        group_sync<GROUP, ROWS>();
        group_bitonic<GROUP, ROWS>(sbuf, N, gt);
    }
    const int64_t obase = a.Cp[row] - a.outBase;
    const int32_t shift = col_shift(a, row);
    const int wn = (int)min((int64_t)nn, expect);
    for (int i = gt; i < wn; i += GROUP) {
        const uint64_t v = sorted[i];
        a.Ci[obase + i] = (int32_t)(v >> 32) - shift;
        a.Cv[obase + i] = vals[(uint32_t)v];
    }
}

// Shared bytes per warp of the warp hash kernel: keys, values and the bucket
// counters.  Rows of at most kNumWarpMax products (expand-sort-compress) sort
// into the upper half of the values, which they do not use; the table path
// sorts its compacted keys in place (bitonic).  7 KB per warp.
constexpr size_t warp_hash_bytes(int table) { return 12 * (size_t)table + 4 * (size_t)kBuckets; }

// Warp hash rows: keys int32[TABLE] then values double[TABLE] per row.
// A row of at most kNumWarpMax products, by one warp without a hash table
// (expand, sort, compress): every product's column and value go to shared
// memory, a bucket counting sort (or a bitonic sort when columns cluster)
// orders them by column, and each run of equal columns is summed by the lane
// holding its first entry and written at the run's rank.  pk holds
// kNumWarpMax packed (column << 32 | product) keys, pv the products' values.
template <int ROWS>
__device__ __forceinline__ void esc_row(const NumArgs &a, int32_t row, int32_t e0, int32_t e1, int n, uint64_t *pk,
                                        double *pv, int *cnts, uint64_t *bbuf) {
    const int lane = threadIdx.x & 31;
    int32_t tb = 0;  // products of the earlier chunks
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32 * kHashWarpLoads) {
            int32_t j[kHashWarpLoads];
            double av[kHashWarpLoads];
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                j[u] = -1;
                av[u] = 0.0;
                const int32_t t = t0 + 32 * u + lane;
                if (t0 + 32 * u < c.total) {
                    const int32_t jj = chunk_pos(c, t, &av[u]);
                    if (t < c.total && tb + t < n) j[u] = jj;
                }
            }
            int32_t col[kHashWarpLoads];
            double bv[kHashWarpLoads];
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                col[u] = j[u] >= 0 ? __ldg(&a.B.idx[j[u]]) : 0;
                bv[u] = j[u] >= 0 ? __ldg(&a.B.val[j[u]]) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                if (j[u] >= 0) {
                    const int t = tb + t0 + 32 * u + lane;
                    pk[t] = ((uint64_t)(uint32_t)col[u] << 32) | (uint32_t)t;
                    pv[t] = __dmul_rn(av[u], bv[u]);
                }
            }
        }
        tb += c.total;
    }
    __syncwarp();
    const int32_t rlo = a.rowLo[row];
    const int64_t span = max((int64_t)1, (int64_t)a.rowHi[row] - rlo + 1);
    const uint64_t *sorted = bbuf;
    if (!warp_bucket_order(pk, n, rlo, span, cnts, bbuf)) {
        int N = 1;
        while (N < n) N <<= 1;
        for (int i = n + lane; i < N; i += 32) pk[i] = ~0ull;
        __syncwarp();
        group_bitonic<32, ROWS>(pk, N, lane);
        sorted = pk;
    }
    // Lane l takes sorted entries [8 l, 8 l + 8): the first entry of each
    // run of equal columns is a head; heads before it give its rank.
    constexpr int PER = kNumWarpMax / 32;
    uint32_t headMask = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int i = PER * lane + q;
        if (i < n && (i == 0 || (sorted[i] >> 32) != (sorted[i - 1] >> 32))) headMask |= 1u << q;
    }
    const int mine = __popc(headMask);
    int incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    if (lane == 0 && total != expect) raise(a.err, DEV_COUNT_MISMATCH);
    const int64_t obase = a.Cp[row] - a.outBase;
    const int32_t shift = col_shift(a, row);
    int64_t pos = incl - mine;
    for (uint32_t m = headMask; m; m &= m - 1u) {
        const int i = PER * lane + __ffs(m) - 1;
        const uint64_t k0 = sorted[i];
        double sum = pv[(uint32_t)k0];
        for (int jx = i + 1; jx < n && (sorted[jx] >> 32) == (k0 >> 32); ++jx) sum = __dadd_rn(sum, pv[(uint32_t)sorted[jx]]);
        if (pos < expect) {
            a.Ci[obase + pos] = (int32_t)(k0 >> 32) - shift;
            a.Cv[obase + pos] = sum;
        }
        ++pos;
    }
}

template <int ROWS, int TABLE>
__device__ __forceinline__ void num_hash_warp_rows(const NumArgs &a, int32_t lo, int32_t count, int64_t vb) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int gcnt[ROWS];
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * ROWS + g;
    if (item >= count) return;
    unsigned char *base_ptr = smem + (size_t)g * warp_hash_bytes(TABLE);
    int32_t *keys = reinterpret_cast<int32_t *>(base_ptr);
    double *vals = reinterpret_cast<double *>(base_ptr + 4 * (size_t)TABLE);
    int *cnts = reinterpret_cast<int *>(base_ptr + 12 * (size_t)TABLE);
    const int32_t row = a.list[lo + item];
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    if (a.rowP[row] <= kNumWarpMax && TABLE >= 2 * kNumWarpMax) {
        esc_row<ROWS>(a, row, e0, e1, (int)a.rowP[row], reinterpret_cast<uint64_t *>(keys), vals, cnts,
                      reinterpret_cast<uint64_t *>(vals + kNumWarpMax));
        return;
    }
    for (int i = lane; i < TABLE; i += 32) {
        keys[i] = EMPTY;
        vals[i] = 0.0;
    }
    if (lane == 0) gcnt[g] = 0;
    __syncwarp();
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        // kHashWarpLoads steps at a time: positions first, then all their B
        // loads, then the inserts.
        for (int32_t t0 = 0; t0 < c.total; t0 += 32 * kHashWarpLoads) {
            int32_t j[kHashWarpLoads], col[kHashWarpLoads];
            double av[kHashWarpLoads], bv[kHashWarpLoads];
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                j[u] = -1;
                av[u] = 0.0;
                const int32_t t = t0 + 32 * u + lane;
                if (t0 + 32 * u < c.total) {
                    const int32_t jj = chunk_pos(c, t, &av[u]);
                    if (t < c.total) j[u] = jj;
                }
            }
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                col[u] = j[u] >= 0 ? __ldg(&a.B.idx[j[u]]) : 0;
                bv[u] = j[u] >= 0 ? __ldg(&a.B.val[j[u]]) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kHashWarpLoads; ++u) {
                if (j[u] >= 0) {
                    const int s = hash_insert_slot<TABLE>(keys, col[u], a.err);
                    if (s >= 0) atomic_fma(&vals[s], av[u], bv[u]);
                }
            }
        }
    }
    __syncwarp();
    table_write_sorted<32, ROWS, TABLE>(a, row, keys, vals, &gcnt[g], lane);
}

template <int ROWS, int TABLE>
__global__ void __launch_bounds__(32 * ROWS) k_num_hash_warp(NumArgs a, int32_t lo, int32_t count) {
    num_hash_warp_rows<ROWS, TABLE>(a, lo, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int ROWS, int TABLE>
__global__ void __launch_bounds__(32 * ROWS) k_num_hash_warp_dd(NumArgs a, int bin) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb * ROWS < count; vb += gridDim.x) {
        num_hash_warp_rows<ROWS, TABLE>(a, lo, count, vb);
        __syncthreads();
    }
}

// CTA hash rows: one CTA per row, products spread over all threads.
template <int THREADS, int TABLE>
__device__ __forceinline__ void num_hash_cta_rows(const NumArgs &a, int32_t lo, int64_t vb) {
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    __shared__ int32_t sh[THREADS / 32];
    __shared__ int gcnt;
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    double *av = reinterpret_cast<double *>(smem + L::av);
    int32_t *keys = reinterpret_cast<int32_t *>(smem + L::bytes);
    double *vals = reinterpret_cast<double *>(smem + L::bytes + 4 * (size_t)TABLE);
    const int tid = threadIdx.x;
    const int32_t row = a.list[lo + vb];
    for (int i = tid; i < TABLE; i += THREADS) {
        keys[i] = EMPTY;
        vals[i] = 0.0;
    }
    if (tid == 0) gcnt = 0;
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    for (int32_t eb = e0; eb < e1; eb += THREADS) {
        int nb;
        const int32_t total =
            stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av, &nb, sh);
        int32_t tb, te;
        warp_share<THREADS>(total, &tb, &te);
        warp_range_ld<4>(
            pre, bst, nb, tb, te,
            [&](int32_t pos) { return ColVal{__ldg(&a.B.idx[pos]), __ldg(&a.B.val[pos])}; },
            [&](bool v, const ColVal &x, int e) {
                if (v) {
                    const int s = hash_insert_slot<TABLE>(keys, x.c, a.err);
                    if (s >= 0) atomic_fma(&vals[s], av[e], x.v);
                }
            });
        __syncthreads();
    }
    table_write_sorted<THREADS, 1, TABLE>(a, row, keys, vals, &gcnt, tid);
}

template <int THREADS, int TABLE>
__global__ void __launch_bounds__(THREADS) k_num_hash_cta(NumArgs a, int32_t lo) {
    num_hash_cta_rows<THREADS, TABLE>(a, lo, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int THREADS, int TABLE>
__global__ void __launch_bounds__(THREADS) k_num_hash_cta_dd(NumArgs a, int bin) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb < count; vb += gridDim.x) {
        num_hash_cta_rows<THREADS, TABLE>(a, lo, vb);
        __syncthreads();
    }
}

// Rank rows (C has at most 2^18 columns): one CTA per row.  Pass 1 sets the
// row's columns in a shared bitmap over all of C's columns; a scan of the
// words' popcounts gives every column its rank among the row's columns, which
// is its position in C's row.  Pass 2 accumulates every product into
// vals[rank].  The output is in column order without hashing or sorting.
// Rows with more than vcap entries accumulate vcap ranks per pass 2.  With
// GLOBAL_ACC the row's slice of C's values is zeroed and accumulated in place
// by FP64 reductions at L2 (no shared value array, no slices).
template <int THREADS, bool GLOBAL_ACC>
__device__ __forceinline__ void num_rank_rows(const NumArgs &a, int32_t lo, int maxWords, int vcap, int64_t vb) {
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    constexpr int NW = THREADS / 32;
    __shared__ int32_t sh[NW];
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    double *av = reinterpret_cast<double *>(smem + L::av);
    uint32_t *bits = reinterpret_cast<uint32_t *>(smem + L::bytes);
    int32_t *wpre = reinterpret_cast<int32_t *>(bits + maxWords);
    double *vals = reinterpret_cast<double *>(wpre + maxWords);
    // Per thread, the rank of its first column and its non-empty words, kept
    // in the staging area (idle between the passes).
    static_assert(8 * THREADS <= L::bytes && kRankWordsMax <= 32 * THREADS, "rank groups");
    int32_t *tbase = pre;
    uint32_t *tmask = reinterpret_cast<uint32_t *>(pre + THREADS);
    const int tid = threadIdx.x, lane = tid & 31;
    const int32_t row = a.list[lo + vb];
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    const int64_t obase = a.Cp[row] - a.outBase;
    // The row's window: words [rw0, rw0 + nwords) of C's columns.
    const int32_t rlo = a.rowLo[row];
    const int32_t rw0 = rlo >> 5;
    const int nwords = min(span_words(rlo, a.rowHi[row]), maxWords);
    const int32_t cbase = rw0 << 5;
    const int32_t obc = cbase - col_shift(a, row);  // column written for bit 0

    if (a.wideBits && sym_bin_of(a.rowP[row], e1 - e0, nwords, a.tune) == SB_WIDE) {
        // The symbolic pass kept this row's bitmap.
        const uint32_t *src = a.wideBits + (size_t)a.wideSlot[row] * kRankWordsMax;
        for (int i = tid; i < nwords; i += THREADS) bits[i] = __ldcs(&src[i]);
        __syncthreads();
    } else {
        for (int i = tid; i < nwords; i += THREADS) bits[i] = 0u;
        for (int32_t eb = e0; eb < e1; eb += THREADS) {
            int nb;
            const int32_t total =
                stage_entries<THREADS, false>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, nullptr, &nb, sh);
            int32_t tb, te;
            warp_share<THREADS>(total, &tb, &te);
            warp_range_ld<4>(
                pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
                [&](bool v, int32_t col, int) {
                    const uint32_t rel = v ? (uint32_t)(col - cbase) : 0u;
                    or_bit(bits, v && in_window(rel, (uint32_t)nwords * 32u, a.err), rel);
                });
            __syncthreads();
        }
    }

    // Ranks, per thread over its own wpt consecutive words (wpt a power of
    // two, THREADS * wpt >= nwords): one sweep gives the thread the mask of
    // its non-empty words and their bit count, a block scan the rank of its
    // first column; then only the non-empty words are ranked.  Lanes start
    // their sweeps at different words so that a warp's loads hit 32 banks.
    // C's columns are then written balanced by output position.
    int wpt = 1;
    while (wpt * THREADS < nwords) wpt <<= 1;
    const int w0 = tid * wpt;
    const int rot = (lane * wpt) >> 5;
    uint32_t mask = 0u;
    int32_t cnt = 0;
    for (int k = 0; k < wpt; ++k) {
        const int q = (k + rot) & (wpt - 1);
        if (w0 + q < nwords) {
            const uint32_t x = bits[w0 + q];
            if (x) mask |= 1u << q;
            cnt += __popc(x);
        }
    }
    int32_t tot;
    const int32_t base = block_excl_scan<THREADS>(cnt, &tot, sh);
    if (tid == 0 && tot != expect) raise(a.err, DEV_COUNT_MISMATCH);
    {
        int32_t p = base;
        for (uint32_t m = mask; m; m &= m - 1u) {
            const int w = w0 + __ffs(m) - 1;
            wpre[w] = p;
            p += __popc(bits[w]);
        }
        tbase[tid] = base;
        tmask[tid] = mask;
    }
    __syncthreads();
    write_columns_balanced<THREADS>(bits, tbase, tmask, wpt, tot, a.Ci + obase, expect, obc);
    __syncthreads();

    if constexpr (GLOBAL_ACC) {
        double *cv = a.Cv + obase;
        for (int64_t i = tid; i < expect; i += THREADS) cv[i] = 0.0;
        __syncthreads();
        for (int32_t eb = e0; eb < e1; eb += THREADS) {
            int nb;
            const int32_t total =
                stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av, &nb, sh);
            int32_t tb, te;
            warp_share<THREADS>(total, &tb, &te);
            warp_range_ld<4>(
                pre, bst, nb, tb, te,
                [&](int32_t pos) { return ColVal{__ldg(&a.B.idx[pos]), __ldg(&a.B.val[pos])}; },
                [&](bool v, const ColVal &x, int e) {
                    const int32_t c = x.c - cbase;
                    if (v && (uint32_t)c < (uint32_t)nwords * 32u) {
                        const int w = c >> 5;
                        const int64_t r = (int64_t)wpre[w] + __popc(bits[w] & ((1u << (c & 31)) - 1u));
                        if (r < expect) atomicAdd(&cv[r], __dmul_rn(av[e], x.v));
                    }
                });
            __syncthreads();
        }
    } else {
        // Values, vcap ranks per pass.
        for (int64_t s0 = 0; s0 < expect; s0 += vcap) {
            const int ns = (int)min((int64_t)vcap, expect - s0);
            for (int i = tid; i < ns; i += THREADS) vals[i] = 0.0;
            for (int32_t eb = e0; eb < e1; eb += THREADS) {
                int nb;
                const int32_t total =
                    stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av, &nb, sh);
                int32_t tb, te;
                warp_share<THREADS>(total, &tb, &te);
                warp_range_ld<4>(
                    pre, bst, nb, tb, te,
                    [&](int32_t pos) { return ColVal{__ldg(&a.B.idx[pos]), __ldg(&a.B.val[pos])}; },
                    [&](bool v, const ColVal &x, int e) {
                        const int32_t c = x.c - cbase;
                        if (v && (uint32_t)c < (uint32_t)nwords * 32u) {
                            const int w = c >> 5;
                            const int64_t r = (int64_t)wpre[w] + __popc(bits[w] & ((1u << (c & 31)) - 1u)) - s0;
                            if (r >= 0 && r < ns) atomic_fma(&vals[r], av[e], x.v);
                        }
                    });
                __syncthreads();
            }
            for (int i = tid; i < ns; i += THREADS) a.Cv[obase + s0 + i] = vals[i];
            __syncthreads();
        }
    }
}

template <int THREADS, bool GLOBAL_ACC>
__global__ void __launch_bounds__(THREADS, GLOBAL_ACC ? 3 : 1) k_num_rank(NumArgs a, int32_t lo, int maxWords, int vcap) {
    num_rank_rows<THREADS, GLOBAL_ACC>(a, lo, maxWords, vcap, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int THREADS, bool GLOBAL_ACC>
__global__ void __launch_bounds__(THREADS, GLOBAL_ACC ? 3 : 1) k_num_rank_dd(NumArgs a, int bin, int maxWords, int vcap) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb < count; vb += gridDim.x) {
        num_rank_rows<THREADS, GLOBAL_ACC>(a, lo, maxWords, vcap, vb);
        __syncthreads();
    }
}

// Narrowest rows (window of at most kDenseWarpWords words): one warp per row
// with a dense FP64 accumulator and a flag byte per column of the window in
// shared memory.  Row-wise enumeration over strictly ascending B rows adds
// each column's products in A's entry order with plain fused multiply-adds
// (deterministic); otherwise atomic ones.  The flags give the columns in
// order: no bitmap ranks, no sorting.
template <int ROWS>
__device__ __forceinline__ void num_densew_rows(const NumArgs &a, int32_t lo, int32_t count, int64_t vb) {
    constexpr int kCols = kDenseWarpWords * 32;
    __shared__ double vs[ROWS][kCols];
    __shared__ __align__(16) uint32_t fls[ROWS][kCols / 4];
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * ROWS + g;
    if (item >= count) return;
    double *vals = vs[g];
    uint32_t *fw = fls[g];
    uint8_t *fb = reinterpret_cast<uint8_t *>(fw);
    const int32_t row = a.list[lo + item];
    const int32_t rlo = a.rowLo[row];
    const int32_t cbase = (rlo >> 5) << 5;
    const int sw = min(span_words(rlo, a.rowHi[row]), kDenseWarpWords);
    const uint32_t nb = (uint32_t)sw * 32u;
    const int32_t obc = cbase - col_shift(a, row);  // column written for flag 0
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    const int64_t obase = a.Cp[row] - a.outBase;
    for (int i = lane; i < (int)nb; i += 32) vals[i] = 0.0;
    for (int i = lane; i < sw * 8; i += 32) fw[i] = 0u;
    __syncwarp();
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const bool rowwise = a.rowP[row] >= (int64_t)kRowwiseMinLen * (e1 - e0);
    const bool plain = rowwise && b_sorted(a);
    int *err = a.err;
    const int32_t *bidx = a.B.idx;
    const double *bval = a.B.val;
    auto add = [&](uint32_t rel, double av, double bv) {
        if (in_window(rel, nb, err)) {
            if (plain) vals[rel] = __fma_rn(av, bv, vals[rel]);
            else atomic_fma(&vals[rel], av, bv);
            fb[rel] = 1;
        }
    };
    if (rowwise) {
        // One A entry at a time; each lane loads up to four of the B row's
        // products before using any, so their loads are in flight together.
        for (int32_t eb = e0; eb < e1; eb += 32) {
            int32_t bs = 0, len = 0;
            double avl = 0.0;
            if (eb + lane < e1) {
                const int32_t k = a.A.idx[eb + lane];
                bs = a.B.ptr[k];
                len = a.B.ptr[k + 1] - bs;
                avl = a.A.val[eb + lane];
            }
            const int n = min(32, e1 - eb);
            for (int q = 0; q < n; ++q) {
                const int32_t bq = __shfl_sync(FULL, bs, q);
                const int32_t lq = __shfl_sync(FULL, len, q);
                const double aq = __shfl_sync(FULL, avl, q);
                for (int32_t i0 = 0; i0 < lq; i0 += 128) {
                    int32_t c[4];
                    double v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int32_t i = i0 + 32 * u + lane;
                        c[u] = i < lq ? bidx[bq + i] : INT_MIN;
                        v[u] = i < lq ? bval[bq + i] : 0.0;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (c[u] != INT_MIN) add((uint32_t)(c[u] - cbase), aq, v[u]);
                }
                __syncwarp();
            }
        }
    } else {
        warp_products(a.A, a.B, e0, e1, lane,
                      [&](int32_t j, double av) { add((uint32_t)(bidx[j] - cbase), av, bval[j]); });
    }
    __syncwarp();
    // Lane l owns columns [16 l, 16 l + 16) of the window.
    const uint4 f4 = reinterpret_cast<const uint4 *>(fw)[lane];
    const bool mine = lane * 16 < (int)nb;
    const int cnt = mine ? __popc(f4.x) + __popc(f4.y) + __popc(f4.z) + __popc(f4.w) : 0;
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    if (lane == 0 && total != expect) raise(a.err, DEV_COUNT_MISMATCH);
    if (mine) {
        int64_t p = incl - cnt;
        const uint32_t wv[4] = {f4.x, f4.y, f4.z, f4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                if ((wv[q] >> (8 * b)) & 0xffu) {
                    const int col = lane * 16 + q * 4 + b;
                    if (p < expect) {
                        a.Ci[obase + p] = obc + col;
                        a.Cv[obase + p] = vals[col];
                    }
                    ++p;
                }
            }
        }
    }
}

template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_num_densew(NumArgs a, int32_t lo, int32_t count) {
    num_densew_rows<ROWS>(a, lo, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_num_densew_dd(NumArgs a, int bin) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb * ROWS < count; vb += gridDim.x) {
        num_densew_rows<ROWS>(a, lo, count, vb);
        __syncthreads();
    }
}

// Narrow rows (window of at most kWarpSpanWords words, at most kNumWarpMax
// entries): one warp per row with the window's bitmap, word ranks and the
// row's values in shared memory; the rank kernel's method at warp scale.
template <int ROWS>
__device__ __forceinline__ void num_rankw_rows(const NumArgs &a, int32_t lo, int32_t count, int64_t vb) {
    static_assert(kWarpSpanWords == 64, "two bitmap words per lane");
    __shared__ uint32_t bms[ROWS][kWarpSpanWords];
    __shared__ int32_t wps[ROWS][kWarpSpanWords];
    __shared__ double vs[ROWS][kNumWarpMax];
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t item = (int64_t)vb * ROWS + g;
    if (item >= count) return;
    uint32_t *bm = bms[g];
    int32_t *wp = wps[g];
    double *vals = vs[g];
    const int32_t row = a.list[lo + item];
    const int32_t cbase = (a.rowLo[row] >> 5) << 5;
    const int32_t obc = cbase - col_shift(a, row);  // column written for bit 0
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    const int64_t obase = a.Cp[row] - a.outBase;
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    for (int i = lane; i < kWarpSpanWords; i += 32) bm[i] = 0u;
    for (int i = lane; i < kNumWarpMax; i += 32) vals[i] = 0.0;
    __syncwarp();
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
            const int32_t t = t0 + lane;
            const int32_t j = chunk_pos(c, t, nullptr);
            const uint32_t rel = t < c.total ? (uint32_t)(a.B.idx[j] - cbase) : 0u;
            const bool v = t < c.total && in_window(rel, kWarpSpanWords * 32, a.err);
            or_bit(bm, v, rel);
        }
    }
    __syncwarp();
    const int32_t p0 = __popc(bm[lane]), p1 = __popc(bm[lane + 32]);
    int32_t i0 = p0, i1 = p1;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t y0 = __shfl_up_sync(FULL, i0, d), y1 = __shfl_up_sync(FULL, i1, d);
        if (lane >= d) {
            i0 += y0;
            i1 += y1;
        }
    }
    const int32_t half = __shfl_sync(FULL, i0, 31);
    const int32_t total = half + __shfl_sync(FULL, i1, 31);
    wp[lane] = i0 - p0;
    wp[lane + 32] = half + i1 - p1;
    if (lane == 0 && total != expect) raise(a.err, DEV_COUNT_MISMATCH);
    __syncwarp();
    for (int w = lane; w < kWarpSpanWords; w += 32) {
        uint32_t word = bm[w];
        int64_t p = wp[w];
        while (word) {
            const int b = __ffs(word) - 1;
            word &= word - 1u;
            if (p < expect) a.Ci[obase + p] = obc + (w << 5) + b;
            ++p;
        }
    }
    for (int32_t e = e0; e < e1; e += 32) {
        const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
        for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
            const int32_t t = t0 + lane;
            double av;
            const int32_t j = chunk_pos(c, t, &av);
            const int32_t col = t < c.total ? a.B.idx[j] - cbase : 0;
            if (t < c.total && (uint32_t)col < (uint32_t)(kWarpSpanWords * 32)) {
                const int w = col >> 5;
                const int r = wp[w] + __popc(bm[w] & ((1u << (col & 31)) - 1u));
                if (r < kNumWarpMax) atomic_fma(&vals[r], av, a.B.val[j]);
            }
        }
    }
    __syncwarp();
    const int64_t nout = min(expect, (int64_t)kNumWarpMax);
    for (int64_t i = lane; i < nout; i += 32) a.Cv[obase + i] = vals[i];
}

template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_num_rankw(NumArgs a, int32_t lo, int32_t count) {
    num_rankw_rows<ROWS>(a, lo, count, blockIdx.x);
}

// The same rows launched device-driven: the bin's rows from the bin table
// on the device, covered by a grid-stride loop.
template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_num_rankw_dd(NumArgs a, int bin) {
    const int32_t lo = a.binStart[bin], count = a.binStart[bin + 1] - lo;
    for (int64_t vb = blockIdx.x; vb * ROWS < count; vb += gridDim.x) {
        num_rankw_rows<ROWS>(a, lo, count, vb);
        __syncthreads();
    }
}

// A segmented OR over runs of lanes that share a word that also marks, in a summary bitmap (one bit per word),
// every word it finds zero.  All lanes call.
__device__ __forceinline__ void or_bits_mark(uint32_t *bm, uint32_t *sum, bool v, uint32_t rel) {
    const int lane = threadIdx.x & 31;
    const int32_t w = v ? (int32_t)(rel >> 5) : -1 - lane;
    uint32_t acc = v ? 1u << (rel & 31) : 0u;
    bool head = v;
    if (__any_sync(FULL, __shfl_up_sync(FULL, w, 1) == w && lane > 0)) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t ow = __shfl_down_sync(FULL, w, d);
            const uint32_t ob = __shfl_down_sync(FULL, acc, d);
            if (lane + d < 32 && ow == w) acc |= ob;
        }
        const int32_t pw = __shfl_up_sync(FULL, w, 1);
        head = v && (lane == 0 || pw != w);
    }
    if (head && atomicOr(&bm[w], acc) == 0u) atomicOr(&sum[w >> 5], 1u << (w & 31));
}

// Rows of at most kNumWarpMax entries whose window spans at most
// kMidSpanWords words: persistent warps, one row at a time, the rank method
// over the row's own window.  A summary bitmap (one bit per window word)
// lists the words the row touched, so word ranks, output and the clean-up
// for the next row visit only those words: a row costs its products and
// entries, not its span.  No hash table, no sort.
template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_num_rankm(NumArgs a, int32_t lo, int32_t count) {
    if (lo < 0) {  // device-driven: the bin's rows from the bin table
        lo = a.binStart[NB_RANKM];
        count = a.binStart[NB_RANKM + 1] - lo;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int kSumWords = kMidSpanWords / 32;
    constexpr size_t kWarpBytes =
        8 * (size_t)kNumWarpMax + 4 * (size_t)kMidSpanWords + 4 * (size_t)kSumWords + 2 * (size_t)kMidSpanWords;
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *vals = reinterpret_cast<double *>(smem + g * kWarpBytes);
    uint32_t *bm = reinterpret_cast<uint32_t *>(vals + kNumWarpMax);
    uint32_t *sum = bm + kMidSpanWords;
    uint16_t *wp = reinterpret_cast<uint16_t *>(sum + kSumWords);
    for (int i = lane; i < kMidSpanWords; i += 32) bm[i] = 0u;
    for (int i = lane; i < kSumWords; i += 32) sum[i] = 0u;
    for (int i = lane; i < kNumWarpMax; i += 32) vals[i] = 0.0;
    __syncwarp();
    const int64_t warps = (int64_t)gridDim.x * ROWS;
    for (int64_t item = (int64_t)blockIdx.x * ROWS + g; item < count; item += warps) {
        const int32_t row = a.list[lo + item];
        const int32_t rlo = a.rowLo[row];
        const int32_t cbase = (rlo >> 5) << 5;
        const int nw = min(span_words(rlo, a.rowHi[row]), kMidSpanWords);
        const uint32_t nbits = (uint32_t)nw * 32u;
        const int32_t obc = cbase - col_shift(a, row);  // column written for bit 0
        const int64_t expect = a.Cp[row + 1] - a.Cp[row];
        const int64_t obase = a.Cp[row] - a.outBase;
        const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
        for (int32_t e = e0; e < e1; e += 32) {
            const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
            for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
                const int32_t t = t0 + lane;
                const int32_t j = chunk_pos(c, t, nullptr);
                const uint32_t rel = t < c.total ? (uint32_t)(a.B.idx[j] - cbase) : 0u;
                const bool v = t < c.total && in_window(rel, nbits, a.err);
                or_bits_mark(bm, sum, v, rel);
            }
        }
        __syncwarp();
        // Lane l owns window words [64 l, 64 l + 64): summary words 2l, 2l + 1.
        const uint32_t s0 = sum[2 * lane], s1 = sum[2 * lane + 1];
        int cnt = 0;
        for (uint32_t m = s0; m; m &= m - 1u) cnt += __popc(bm[64 * lane + __ffs(m) - 1]);
        for (uint32_t m = s1; m; m &= m - 1u) cnt += __popc(bm[64 * lane + 32 + __ffs(m) - 1]);
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, d);
            if (lane >= d) incl += y;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        if (lane == 0 && total != expect) raise(a.err, DEV_COUNT_MISMATCH);
        int64_t p = incl - cnt;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            for (uint32_t m = h ? s1 : s0; m; m &= m - 1u) {
                const int w = 64 * lane + 32 * h + __ffs(m) - 1;
                wp[w] = (uint16_t)p;
                uint32_t word = bm[w];
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1u;
                    if (p < expect) a.Ci[obase + p] = obc + (w << 5) + b;
                    ++p;
                }
            }
        }
        __syncwarp();
        for (int32_t e = e0; e < e1; e += 32) {
            const Chunk c = load_chunk(a.A, a.B, e, e1, lane);
            for (int32_t t0 = 0; t0 < c.total; t0 += 32) {
                const int32_t t = t0 + lane;
                double av;
                const int32_t j = chunk_pos(c, t, &av);
                const int32_t col = t < c.total ? a.B.idx[j] - cbase : 0;
                if (t < c.total && (uint32_t)col < nbits) {
                    const int w = col >> 5;
                    const int r = wp[w] + __popc(bm[w] & ((1u << (col & 31)) - 1u));
                    if (r < kNumWarpMax) atomic_fma(&vals[r], av, a.B.val[j]);
                }
            }
        }
        __syncwarp();
        const int nout = (int)min(expect, (int64_t)kNumWarpMax);
        for (int i = lane; i < nout; i += 32) {
            a.Cv[obase + i] = vals[i];
            vals[i] = 0.0;
        }
        // Leave the bitmap and summary clean for the next row.
        for (uint32_t m = s0; m; m &= m - 1u) bm[64 * lane + __ffs(m) - 1] = 0u;
        for (uint32_t m = s1; m; m &= m - 1u) bm[64 * lane + 32 + __ffs(m) - 1] = 0u;
        sum[2 * lane] = 0u;
        sum[2 * lane + 1] = 0u;
        __syncwarp();
    }
}

// Work items of the dense bin for list[lo, lo + n): one per row, except that
// a row of more than kPieceNnz entries whose slab counts the symbolic pass
// recorded (B's rows ascending) is cut at slab boundaries into pieces of
// about kPieceNnz entries and at most kPieceSlabs slabs.  Every item is
// independent: it knows its columns and where its entries start in C's row.
__global__ void __launch_bounds__(256) k_dense_items(NumArgs a, int32_t lo, int32_t n) {
    const int32_t i = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const int32_t row = a.list[lo + i];
    const int64_t nnz = a.Cp[row + 1] - a.Cp[row];
    const int32_t sl = a.heavySlot[row];
    auto put = [&](int s0, int s1, int32_t cnt, int64_t off) {
        const uint32_t k = atomicAdd(&a.ctr[CTR_ITEMS], 1u);
        if (k >= (uint32_t)a.itemCap) {
            raise(a.err, DEV_TABLE_FULL);
            return;
        }
        a.items[k] = DenseItem{row, (int16_t)s0, (int16_t)s1, cnt, off};
    };
    if (sl < 0 || !b_sorted(a) || nnz <= kPieceNnz) {
        put(-1, -1, (int32_t)min(nnz, (int64_t)INT32_MAX), 0);
        return;
    }
    const int64_t base = (int64_t)(a.rowLo[row] >> 5) << 5;
    const int ns = (int)((((int64_t)a.rowHi[row] + 1 - base) + (1 << kSlabShift) - 1) >> kSlabShift);
    const int32_t *sc = a.slabCnt + (size_t)sl * kMaxSlabs;
    int s0 = 0;
    int32_t acc = 0;
    int64_t off = 0;
    for (int s = 0; s < ns; ++s) {
        const int32_t c = sc[s];
        if (s > s0 && (acc + c > kPieceNnz || s - s0 == kPieceSlabs)) {
            put(s0, s, acc, off);
            off += acc;
            acc = 0;
            s0 = s;
        }
        acc += c;
    }
    put(s0, ns, acc, off);
}

// Dense rows (windows wider than the CTA rank kernel's): persistent CTAs,
// two per SM, take rows from a counter and apply the rank method over
// windows of WIN words of the row's span (2^19 columns in shared memory).
// Per window: a pass over the row's products sets the bits inside the
// window; a sweep gives each thread the non-empty-word mask and bit count
// of its 32 words (one summary word), and a scan of the counts gives every
// thread the rank of its first column.  From there everything visits only
// the non-empty words: their ranks (a 16-bit offset from a 32-bit base per
// 256 words), C's columns (each thread writes a contiguous run of them), and
// the clean-up that leaves the bitmap zero for the next window.  A second
// pass adds every product inside the window into C's row in place at its
// rank (FP64 L2 reductions).  Power-law rows spread thinly over millions of
// columns pay for their entries, not for their span, past the one sweep.
template <int THREADS, int WIN>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) k_num_rankwin(NumArgs a, int32_t lo, int32_t count) {
    static_assert(WIN == 32 * THREADS, "one summary word of 32 bitmap words per thread");
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    constexpr int NW = THREADS / 32;
    __shared__ int32_t sh[NW];
    __shared__ int32_t next;
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    double *av = reinterpret_cast<double *>(smem + L::av);
    uint32_t *bits = reinterpret_cast<uint32_t *>(smem + L::bytes);
    uint16_t *wpre = reinterpret_cast<uint16_t *>(bits + WIN);
    int32_t *gbase = reinterpret_cast<int32_t *>(wpre + WIN);
    int32_t *tbase = gbase + WIN / 256;                          // per thread: rank of its first column
    uint32_t *tmask = reinterpret_cast<uint32_t *>(tbase + THREADS);  // per thread: its non-empty words
    int32_t *cur = reinterpret_cast<int32_t *>(tmask + THREADS);      // per staged entry: its B cursor
    const int tid = threadIdx.x, lane = tid & 31;
    for (int i = tid; i < WIN; i += THREADS) bits[i] = 0u;
    // With work items (heavy rows cut into pieces), the items the builder
    // wrote before this launch; otherwise the bin's rows.
    if (lo < 0) {  // device-driven: the bin's rows from the bin table
        lo = a.binStart[NB_DENSE];
        count = a.binStart[NB_DENSE + 1] - lo;
    }
    const int32_t nitems = a.items ? (int32_t)min(*(volatile uint32_t *)&a.ctr[CTR_ITEMS], (uint32_t)a.itemCap)
                                   : count;
    for (;;) {
        if (tid == 0) next = (int32_t)atomicAdd(&a.ctr[CTR_NUM_RANKWIN], 1u);
        __syncthreads();
        if (next >= nitems) break;
        const int32_t item = next;
        DenseItem it{0, -1, -1, 0, 0};
        if (a.items) it = a.items[item];
        const int32_t row = a.items ? it.row : a.list[lo + item];
        const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
        const int64_t expect = a.Cp[row + 1] - a.Cp[row];
        const int64_t obase = a.Cp[row] - a.outBase;
        const int32_t shift = col_shift(a, row);
        int64_t end = (int64_t)a.rowHi[row] + 1;
        int64_t start = (int64_t)(a.rowLo[row] >> 5) << 5;
        int64_t run = 0, expectEnd = expect;
        if (it.s0 >= 0) {
            // A piece: the row's columns [start + s0 slabs, start + s1 slabs).
            const int64_t b = start;
            start = b + ((int64_t)it.s0 << kSlabShift);
            end = min(end, b + ((int64_t)it.s1 << kSlabShift));
            run = it.off;
            expectEnd = it.off + it.cnt;
        }
        // Rows over several windows and pieces enumerate, per window, only
        // the part of each B row inside it (B's rows ascending).
        const bool clip = b_sorted(a) && (it.s0 >= 0 || end - start > (int64_t)WIN * 32);
        for (int64_t c_lo = start; c_lo < end; c_lo += (int64_t)WIN * 32) {
            const int nwords = (int)min((int64_t)WIN, (end - c_lo + 31) >> 5);
            const uint32_t nbits = (uint32_t)nwords * 32u;
            const int64_t c_hi = c_lo + nbits;
            // Pass 1: the window's bits.  A row (or piece) of at most THREADS
            // entries is staged once, with its A values, and pass 2 reuses
            // the staging (no second round of loads and clipping searches).
            const bool once = e1 - e0 <= THREADS;
            int nb1 = 0;
            int32_t total1 = 0;
            for (int32_t eb = e0; eb < e1; eb += THREADS) {
                int nb;
                const int32_t total =
                    once ? stage_entries<THREADS, true>(a.A, a.B, eb, e1 - eb, pre, bst, av, &nb, sh, clip, c_lo, c_hi,
                                                        cur, c_lo != start)
                         : stage_entries<THREADS, false>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, nullptr, &nb,
                                                         sh, clip, c_lo, c_hi);
                nb1 = nb;
                total1 = total;
                int32_t tb, te;
                warp_share<THREADS>(total, &tb, &te);
                warp_range_ld<4>(
                    pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
                    [&](bool v, int32_t col, int) {
                        const uint32_t rel = v ? (uint32_t)((int64_t)col - c_lo) : 0u;
                        or_bit(bits, v && rel < nbits, rel);
                    });
                __syncthreads();
            }
            // This thread's 32 words [32 tid, 32 tid + 32): which are
            // non-empty and how many bits they hold.  Lanes start at
            // different words so that a warp's loads hit 32 banks.
            uint32_t mask = 0;
            int32_t cnt = 0;
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const int q = (k + lane) & 31;
                const uint32_t x = bits[32 * tid + q];
                if (x) mask |= 1u << q;
                cnt += __popc(x);
            }
            int32_t tot;
            const int32_t base = block_excl_scan<THREADS>(cnt, &tot, sh);
            // 256-word groups are 8 threads: the group's base is its first
            // thread's.
            const int32_t gb = __shfl_sync(FULL, base, lane & ~7);
            if ((lane & 7) == 0) gbase[tid >> 3] = base;
            {
                int32_t p = base;
                for (uint32_t m = mask; m; m &= m - 1u) {
                    const int w = 32 * tid + __ffs(m) - 1;
                    wpre[w] = (uint16_t)(p - gb);
                    p += __popc(bits[w]);
                }
                tbase[tid] = base;
                tmask[tid] = mask;
            }
            __syncthreads();
            // C's columns, balanced over the threads by output position.
            write_columns_balanced<THREADS>(bits, tbase, tmask, 32, tot, a.Ci + obase + run, expect - run,
                                            c_lo - shift);
            for (int64_t i = tid; i < tot && run + i < expect; i += THREADS) a.Cv[obase + run + i] = 0.0;
            __syncthreads();
            // Pass 2: the window's products into C's row in place.
            for (int32_t eb = e0; eb < e1; eb += THREADS) {
                int nb = nb1;
                const int32_t total =
                    once ? total1
                         : stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av, &nb, sh,
                                                        clip, c_lo, c_hi);
                int32_t tb, te;
                warp_share<THREADS>(total, &tb, &te);
                warp_range_ld<4>(
                    pre, bst, nb, tb, te,
                    [&](int32_t pos) { return ColVal{__ldg(&a.B.idx[pos]), __ldg(&a.B.val[pos])}; },
                    [&](bool v, const ColVal &x, int e) {
                        const uint32_t c = v ? (uint32_t)((int64_t)x.c - c_lo) : 0u;
                        if (v && c < nbits) {
                            const int w = (int)(c >> 5);
                            const int64_t r = run + (int64_t)gbase[w >> 8] + wpre[w] +
                                              __popc(bits[w] & ((1u << (c & 31)) - 1u));
                            if (r < expect) atomicAdd(&a.Cv[obase + r], __dmul_rn(av[e], x.v));
                        }
                    });
                __syncthreads();
            }
            // Leave the bitmap zero: only this thread's non-empty words.
            for (uint32_t m = mask; m; m &= m - 1u) bits[32 * tid + __ffs(m) - 1] = 0u;
            __syncthreads();
            run += tot;
        }
        if (tid == 0 && run != expectEnd) raise(a.err, DEV_COUNT_MISMATCH);
        __syncthreads();  // every thread has read `next` before it changes
    }
}

// Dense rows in one product pass: persistent CTAs (one per scratch row) take
// rows from a counter; per window of WIN words of the row's span (2^19 columns)
// one pass over the row's products sets each product's column bit in a
// shared bitmap and adds the product into the CTA's FP64 scratch row in
// global memory, indexed by column (an L2 reduction whose result is not
// read back).  Then each warp compacts its 1024 words of the window, word
// by word in column order: the 32 lanes are the word's 32 columns, so C's
// columns and values go out as contiguous runs (coalesced), the values read
// from the scratch row at the same 32 consecutive columns, which the warp
// zeroes behind it, leaving the scratch row and the bitmap zero for the next
// window.  Compared with the rank method this enumerates every product once
// instead of twice and writes C once, coalesced, instead of zeroing it and
// reducing into it in place.
template <int THREADS, int WIN>
__global__ void __launch_bounds__(THREADS) k_num_dscr(NumArgs a, int32_t lo, int32_t count) {
    static_assert(WIN == 32 * THREADS, "one 32-word group per thread");
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    constexpr int NW = THREADS / 32;
    __shared__ int32_t sh[NW];
    __shared__ int32_t next;
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    double *av = reinterpret_cast<double *>(smem + L::av);
    uint32_t *bits = reinterpret_cast<uint32_t *>(smem + L::bytes);
    double *scr = a.scr + (size_t)blockIdx.x * (size_t)a.scrStride;
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t lt = (1u << lane) - 1u;
    for (int i = tid; i < WIN; i += THREADS) bits[i] = 0u;
    for (;;) {
        if (tid == 0) next = (int32_t)atomicAdd(&a.ctr[CTR_NUM_DSCR], 1u);
        __syncthreads();
        if (next >= count) break;
        const int32_t item = next;
        const int32_t row = a.list[lo + item];
        const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
        const int64_t expect = a.Cp[row + 1] - a.Cp[row];
        const int64_t obase = a.Cp[row] - a.outBase;
        const int32_t shift = col_shift(a, row);
        const int64_t end = (int64_t)a.rowHi[row] + 1;
        const int64_t start = (int64_t)(a.rowLo[row] >> 5) << 5;
        const bool clip = b_sorted(a) && end - start > (int64_t)WIN * 32;
        int64_t run = 0;
        for (int64_t c_lo = start; c_lo < end; c_lo += (int64_t)WIN * 32) {
            const int nwords = (int)min((int64_t)WIN, (end - c_lo + 31) >> 5);
            const uint32_t nbits = min((uint32_t)nwords * 32u, (uint32_t)a.scrStride);
            const int64_t c_hi = c_lo + nbits;
            // The pass: bits in shared memory, products into the scratch row.
            for (int32_t eb = e0; eb < e1; eb += THREADS) {
                int nb;
                const int32_t total = stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av,
                                                                   &nb, sh, clip, c_lo, c_hi);
                int32_t tb, te;
                warp_share<THREADS>(total, &tb, &te);
                warp_range_ld<4>(
                    pre, bst, nb, tb, te,
                    [&](int32_t pos) { return ColVal{__ldg(&a.B.idx[pos]), __ldg(&a.B.val[pos])}; },
                    [&](bool v, const ColVal &x, int e) {
                        const uint32_t rel = v ? (uint32_t)((int64_t)x.c - c_lo) : 0u;
                        const bool in = v && rel < nbits;
                        or_bit(bits, in, rel);
                        if (in) atomicAdd(&scr[rel], __dmul_rn(av[e], x.v));
                    });
                __syncthreads();
            }
            // Word counts: thread t holds words [32 t, 32 t + 32).
            uint32_t mask = 0;
            int32_t cnt = 0;
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const int q = (k + lane) & 31;
                const uint32_t x = bits[32 * tid + q];
                if (x) mask |= 1u << q;
                cnt += __popc(x);
            }
            int32_t tot;
            const int32_t base = block_excl_scan<THREADS>(cnt, &tot, sh);
            // Compaction: the warp walks its lanes' non-empty words in column
            // order; lane b takes column 32 w + b of word w.
            for (int src = 0; src < 32; ++src) {
                uint32_t m = __shfl_sync(FULL, mask, src);
                int64_t p = run + __shfl_sync(FULL, base, src);
                while (m) {
                    const int w = 32 * (32 * (tid >> 5) + src) + __ffs(m) - 1;
                    m &= m - 1u;
                    const uint32_t word = bits[w];
                    const int64_t q = p + __popc(word & lt);
                    if ((word >> lane) & 1u) {
                        double *s = &scr[32 * w + lane];
                        if (q < expect) {
                            __stcs(&a.Ci[obase + q], (int32_t)(c_lo + 32 * w + lane - shift));
                            __stcs(&a.Cv[obase + q], __ldcg(s));
                        }
                        __stcg(s, 0.0);
                    }
                    p += __popc(word);
                }
            }
            __syncthreads();  // every warp has read its words before they clear
            for (uint32_t m = mask; m; m &= m - 1u) bits[32 * tid + __ffs(m) - 1] = 0u;
            __syncthreads();
            run += tot;
        }
        if (tid == 0 && run != expect) raise(a.err, DEV_COUNT_MISMATCH);
        __syncthreads();  // every thread has read `next` before it changes
    }
}

// Dense rows with a global slot: persistent CTAs, one slot each, take rows
// from a counter; the rank method over the whole row, its bitmap and word
// ranks in the slot (two bits per column of C, so the slots of all CTAs stay
// in L2 for millions of columns) and the summary bitmap (one bit per bitmap
// word) in shared memory.  Pass 1 sets every product's column bit by an L2
// reduction (no round trip) and its word's summary bit in shared memory.  The word ranks are computed over the summary
// bits of the row's window in order (the row's entries plus its span / 1024),
// which also writes C's columns.  Pass 2 adds every product into C's row in
// place at its rank (FP64 L2 reductions).  The clean-up clears the words it
// set.  Reads after reductions go to L2 (__ldcg), past the SM's L1.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_num_gdense(NumArgs a, int32_t lo, int32_t count) {
    extern __shared__ __align__(16) unsigned char smem[];
    using L = StageLayout<THREADS>;
    constexpr int NW = THREADS / 32;
    __shared__ int32_t sh[NW];
    __shared__ int32_t next;
    int32_t *pre = reinterpret_cast<int32_t *>(smem + L::pre);
    int32_t *bst = reinterpret_cast<int32_t *>(smem + L::bst);
    double *av = reinterpret_cast<double *>(smem + L::av);
    uint32_t *sum = reinterpret_cast<uint32_t *>(smem + L::bytes);
    const int tid = threadIdx.x;
    uint32_t *bits = a.gBits + (size_t)blockIdx.x * (a.gStride >> 5);
    uint32_t *wpre = a.gWpre + (size_t)blockIdx.x * (a.gStride >> 5);
    const uint32_t ncols = (uint32_t)min(a.gStride, a.B.n);
    int *err = a.err;
    for (int i = tid; i < (int)(a.gStride >> 10); i += THREADS) sum[i] = 0u;
    for (;;) {
        if (tid == 0) next = (int32_t)atomicAdd(&a.ctr[CTR_NUM_GDENSE], 1u);
        __syncthreads();
        const int32_t item = next;
        if (item >= count) break;
        const int32_t row = a.list[lo + item];
        const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
        const int64_t expect = a.Cp[row + 1] - a.Cp[row];
        const int64_t obase = a.Cp[row] - a.outBase;
        const int32_t shift = col_shift(a, row);
        // Pass 1: bits.
        for (int32_t eb = e0; eb < e1; eb += THREADS) {
            int nb;
            const int32_t total =
                stage_entries<THREADS, false>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, nullptr, &nb, sh);
            int32_t tb, te;
            warp_share<THREADS>(total, &tb, &te);
            warp_range_ld<4>(
                pre, bst, nb, tb, te, [&](int32_t pos) { return __ldg(&a.B.idx[pos]); },
                [&](bool v, int32_t col, int) {
                    if (v) {
                        const uint32_t c = (uint32_t)col;
                        if (in_window(c, ncols, err)) {
                            atomicOr(&bits[c >> 5], 1u << (c & 31));
                            atomicOr(&sum[c >> 10], 1u << ((c >> 5) & 31));  // shared
                        }
                    }
                });
            __syncthreads();
        }
        __threadfence();
        __syncthreads();
        // Word ranks and C's columns; thread t owns a contiguous run of the
        // window's summary words.
        const int32_t s0 = a.rowLo[row] >> 10, s1 = a.rowHi[row] >> 10;
        const int nsum = s1 - s0 + 1;
        const int per = (nsum + THREADS - 1) / THREADS;
        const int q0 = s0 + min(nsum, tid * per), q1 = s0 + min(nsum, tid * per + per);
        int cnt = 0;
        for (int q = q0; q < q1; ++q)
            for (uint32_t m = sum[q]; m; m &= m - 1u) cnt += __popc(__ldcg(&bits[q * 32 + __ffs(m) - 1]));
        int32_t tot;
        int64_t pos = block_excl_scan<THREADS>(cnt, &tot, sh);
        if (tid == 0 && tot != expect) raise(a.err, DEV_COUNT_MISMATCH);
        for (int q = q0; q < q1; ++q) {
            for (uint32_t m = sum[q]; m; m &= m - 1u) {
                const int w = q * 32 + __ffs(m) - 1;
                __stcg(&wpre[w], (uint32_t)pos);
                uint32_t word = __ldcg(&bits[w]);
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1u;
                    if (pos < expect) a.Ci[obase + pos] = w * 32 + b - shift;
                    ++pos;
                }
            }
        }
        for (int64_t i = tid; i < expect; i += THREADS) __stcg(&a.Cv[obase + i], 0.0);
        __threadfence();
        __syncthreads();
        // Pass 2: values in place at their ranks.
        for (int32_t eb = e0; eb < e1; eb += THREADS) {
            int nb;
            const int32_t total =
                stage_entries<THREADS, true>(a.A, a.B, eb, min(THREADS, e1 - eb), pre, bst, av, &nb, sh);
            int32_t tb, te;
            warp_share<THREADS>(total, &tb, &te);
            warp_range_ld<4>(
                pre, bst, nb, tb, te,
                [&](int32_t p) { return ColVal{__ldg(&a.B.idx[p]), __ldg(&a.B.val[p])}; },
                [&](bool v, const ColVal &x, int e) {
                    if (v) {
                        const uint32_t c = (uint32_t)x.c;
                        if (c < ncols) {
                            const int w = (int)(c >> 5);
                            const int64_t r =
                                (int64_t)__ldcg(&wpre[w]) + __popc(__ldcg(&bits[w]) & ((1u << (c & 31)) - 1u));
                            if (r < expect) atomicAdd(&a.Cv[obase + r], __dmul_rn(av[e], x.v));
                        }
                    }
                });
            __syncthreads();
        }
        // Clean-up: the words this row set, then its summary words.
        for (int q = q0; q < q1; ++q) {
            for (uint32_t m = sum[q]; m; m &= m - 1u) __stcg(&bits[q * 32 + __ffs(m) - 1], 0u);
            sum[q] = 0u;
        }
        __threadfence();
        __syncthreads();
    }
}

// Dense rows: one CTA per row sweeps windows of W columns.  Every A entry
// keeps a cursor into its B row and the next column at or past it, in shared
// memory for rows of at most ECAP entries and in a.state otherwise.  Per
// window, each warp reads the next columns of 32 entries at a time (one
// coalesced load), and only entries with products inside the window are
// worked on: the warp scans that entry's B row from its cursor 32 products
// per step (with B rows ascending the products inside the window are a
// prefix, found by ballot).  No block barrier runs per entry, only per
// window.  Without sorted B rows every window rescans whole B rows and
// filters.  The window is zeroed once and every written column is zeroed as
// it is written out, so a window costs its products and C entries, not its
// width.
template <int THREADS, int W, int ECAP, bool SORTED>
__global__ void __launch_bounds__(THREADS) k_num_dense(NumArgs a, int32_t lo) {
    extern __shared__ __align__(16) unsigned char smem[];
    static_assert(W / 32 <= THREADS, "one bitmap word per thread");
    constexpr int NW = THREADS / 32;
    double *dense = reinterpret_cast<double *>(smem);
    uint32_t *bits = reinterpret_cast<uint32_t *>(smem + 8 * (size_t)W);
    int32_t *scur = reinterpret_cast<int32_t *>(smem + 8 * (size_t)W + W / 8);
    int32_t *snext = scur + ECAP;
    __shared__ int32_t sh[NW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t row = a.list[lo + blockIdx.x];
    const int32_t e0 = a.A.ptr[row], e1 = a.A.ptr[row + 1];
    const int32_t nA = e1 - e0;
    const bool resident = nA <= ECAP;
    int32_t *cur_of = resident ? scur : a.state + e0;              // cursor per A entry
    int32_t *next_of = resident ? snext : a.state + a.A.nnz + e0;  // next column per A entry
    const int64_t expect = a.Cp[row + 1] - a.Cp[row];
    const int64_t obase = a.Cp[row] - a.outBase;
    const int32_t shift = col_shift(a, row);
    for (int i = tid; i < W; i += THREADS) dense[i] = 0.0;
    for (int i = tid; i < W / 32; i += THREADS) bits[i] = 0u;

    // Initial state of every entry.
    int32_t mymin = INT_MAX;
    for (int32_t i = tid; i < nA; i += THREADS) {
        const int32_t k = a.A.idx[e0 + i];
        const int32_t s = a.B.ptr[k], t = a.B.ptr[k + 1];
        int32_t nx = INT_MAX;
        if constexpr (SORTED) {
            if (s < t) nx = a.B.idx[s];
        } else {
            for (int32_t q = s; q < t; ++q) nx = min(nx, a.B.idx[q]);
        }
        mymin = min(mymin, nx);
        cur_of[i] = s;
        next_of[i] = nx;
    }
    int32_t cmin = block_min_i32<THREADS>(mymin, sh);
    int64_t run = 0;
    while (cmin != INT_MAX) {
        const int32_t c_lo = (cmin / W) * W;
        const int64_t c_hi = (int64_t)c_lo + W;
        mymin = INT_MAX;
        for (int32_t g = warp * 32; g < nA; g += NW * 32) {
            const int32_t nxl = g + lane < nA ? next_of[g + lane] : INT_MAX;
            unsigned act = __ballot_sync(FULL, nxl < c_hi);
            if (nxl >= c_hi) mymin = min(mymin, nxl);
            while (act) {
                const int q = __ffs(act) - 1;
                act &= act - 1u;
                const int32_t i = g + q;
                const int32_t k = a.A.idx[e0 + i];
                const int32_t end = a.B.ptr[k + 1];
                const double av = a.A.val[e0 + i];
                int32_t cur = SORTED ? cur_of[i] : a.B.ptr[k];
                int32_t nxt = INT_MAX;
                if constexpr (SORTED) {
                    for (;;) {
                        const int32_t p = cur + lane;
                        const int32_t c = p < end ? a.B.idx[p] : INT_MAX;
                        const bool v = c < c_hi;
                        const unsigned m = __ballot_sync(FULL, v);
                        // cursors never point below the window (it starts at the
                        // smallest next column); the guard keeps a malformed row
                        // inside shared memory all the same
                        const int rel = v ? max(c - c_lo, 0) : 0;
                        if (v) atomic_fma(&dense[rel], av, a.B.val[p]);
                        or_bit(bits, v, (uint32_t)rel);
                        const int n = __popc(m);
                        cur += n;
                        if (n < 32) {
                            nxt = __shfl_sync(FULL, c, n);
                            break;
                        }
                    }
                } else {
                    for (int32_t q0 = cur; q0 < end; q0 += 32) {
                        const int32_t p = q0 + lane;
                        const int32_t c = p < end ? a.B.idx[p] : INT_MAX;
                        const bool v = c >= c_lo && c < c_hi;
                        const int rel = v ? c - c_lo : 0;
                        if (v) atomic_fma(&dense[rel], av, a.B.val[p]);
                        or_bit(bits, v, (uint32_t)rel);
                        if (!v && c >= c_hi) nxt = min(nxt, c);
                    }
#pragma unroll
                    for (int d = 16; d; d >>= 1) nxt = min(nxt, __shfl_xor_sync(FULL, nxt, d));
                }
                mymin = min(mymin, nxt);
                if (lane == 0) {
                    if constexpr (SORTED) cur_of[i] = cur;
                    next_of[i] = nxt;
                }
            }
        }
        __syncthreads();
        uint32_t word = tid < W / 32 ? bits[tid] : 0u;
        if (tid < W / 32) bits[tid] = 0u;
        int32_t tot;
        const int32_t off = block_excl_scan<THREADS>(__popc(word), &tot, sh);
        int64_t pos = run + off;
        while (word) {
            const int b = __ffs(word) - 1;
            word &= word - 1u;
            const int rel = tid * 32 + b;
            if (pos < expect) {
                a.Ci[obase + pos] = c_lo - shift + rel;
                a.Cv[obase + pos] = dense[rel];
            }
            dense[rel] = 0.0;
            ++pos;
        }
        run += tot;
        cmin = block_min_i32<THREADS>(mymin, sh);
    }
    if (tid == 0 && run != expect) raise(a.err, DEV_COUNT_MISMATCH);
}

// Configurations and their dynamic shared memory.
constexpr int kSymWarpRows = 8;
constexpr int kNumWarpRows = 4;
constexpr int kSymCtaThreads = 256;
constexpr int kNumCtaSThreads = 256;
constexpr int kNumCtaLThreads = 512;
constexpr int kDenseThreads = 512;
constexpr int kDenseStage = 1024;  // entries whose cursors stay in shared memory
constexpr int kWideThreads = 512;       // two or more CTAs per SM
constexpr size_t kSmemSymWarp = (size_t)kSymWarpRows * kSymWarpTable * 4;
constexpr size_t kSmemSymCta = StageLayout<kSymCtaThreads>::bytes + (size_t)kSymCtaTable * 4;
constexpr size_t kSmemNumWarp = (size_t)kNumWarpRows * warp_hash_bytes(kNumWarpTable);
constexpr size_t kSmemNumCtaS = StageLayout<kNumCtaSThreads>::bytes + (size_t)kNumCtaSTable * 12;
constexpr size_t kSmemNumCtaL = StageLayout<kNumCtaLThreads>::bytes + (size_t)kNumCtaLTable * 12;
constexpr size_t kSmemDense = (size_t)kDenseWindow * 8 + kDenseWindow / 8 + (size_t)kDenseStage * 8;
constexpr size_t kSmemWideBase = StageLayout<kWideThreads>::bytes;
constexpr int kRankSThreads = 256, kRankSVcap = kNumCtaLMax;
constexpr int kRankLThreads = 512;  // global accumulation: staging + bitmap + ranks only
constexpr size_t kSmemRankSMax = StageLayout<kRankSThreads>::bytes + 8 * (size_t)kRankWordsMax + 8 * (size_t)kRankSVcap;
constexpr size_t kSmemRankLMax = StageLayout<kRankLThreads>::bytes + 8 * (size_t)kRankWordsMax;
constexpr int kBitwRows = 8;
constexpr int kRankwRows = 8;
constexpr int kDensewRows = 8;
constexpr int kGdenseThreads = 512;
constexpr int kRankWinThreads = 512;  // two CTAs per SM: one works while the other waits at a barrier
constexpr int kRankWinWords = 16384;  // 2^19 columns per window
constexpr size_t kSmemRankWin = StageLayout<kRankWinThreads>::bytes + 6 * (size_t)kRankWinWords +
                                4 * (size_t)(kRankWinWords / 256) + 12 * (size_t)kRankWinThreads;
constexpr size_t kSmemGdenseBase = StageLayout<kGdenseThreads>::bytes;
constexpr size_t kSmemDscr = StageLayout<kRankWinThreads>::bytes + 4 * (size_t)kRankWinWords;
constexpr int kRankmRows = 5;  // 14.6 KiB per warp: three CTAs (15 warps) per SM
constexpr size_t kSmemRankm =
    (size_t)kRankmRows * (6 * (size_t)kMidSpanWords + 4 * (size_t)(kMidSpanWords / 32) + 8 * (size_t)kNumWarpMax);

}  // namespace

void init_kernel_attributes() {
    cudaFuncSetAttribute(k_sym_hash_warp<kSymWarpRows, kSymWarpTable>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemSymWarp);
    cudaFuncSetAttribute(k_sym_hash_cta<kSymCtaThreads, kSymCtaTable>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemSymCta);
    cudaFuncSetAttribute(k_sym_wide<kWideThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kSmemWideBase + kWideWindowBitsMax / 8 + 4 * (size_t)kWideTouchMax + 4 * kWideThreads));
    cudaFuncSetAttribute(k_num_hash_warp<kNumWarpRows, kNumWarpTable>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNumWarp);
    cudaFuncSetAttribute(k_num_hash_cta<kNumCtaSThreads, kNumCtaSTable>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNumCtaS);
    cudaFuncSetAttribute(k_num_hash_cta<kNumCtaLThreads, kNumCtaLTable>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNumCtaL);
    cudaFuncSetAttribute(k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, true>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDense);
    cudaFuncSetAttribute(k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, false>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDense);
    cudaFuncSetAttribute(k_num_rank<kRankSThreads, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemRankSMax);
    cudaFuncSetAttribute(k_num_rank<kRankLThreads, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemRankLMax);
    cudaFuncSetAttribute(k_num_rankm<kRankmRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemRankm);
    cudaFuncSetAttribute(k_num_rankwin<kRankWinThreads, kRankWinWords>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemRankWin);
    cudaFuncSetAttribute(k_num_dscr<kRankWinThreads, kRankWinWords>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemDscr);
    cudaFuncSetAttribute(k_num_gdense<kGdenseThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kSmemGdenseBase + 4 * (size_t)kGdenseSumMax));
    // The device-driven forms of the same kernels.
    cudaFuncSetAttribute(k_sym_hash_warp_dd<kSymWarpRows, kSymWarpTable>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemSymWarp);
    cudaFuncSetAttribute(k_sym_hash_cta_dd<kSymCtaThreads, kSymCtaTable>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemSymCta);
    cudaFuncSetAttribute(k_num_hash_warp_dd<kNumWarpRows, kNumWarpTable>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemNumWarp);
    cudaFuncSetAttribute(k_num_hash_cta_dd<kNumCtaSThreads, kNumCtaSTable>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemNumCtaS);
    cudaFuncSetAttribute(k_num_hash_cta_dd<kNumCtaLThreads, kNumCtaLTable>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemNumCtaL);
    cudaFuncSetAttribute(k_num_rank_dd<kRankSThreads, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemRankSMax);
    cudaFuncSetAttribute(k_num_rank_dd<kRankLThreads, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemRankLMax);
}

// Loads every symbolic and numeric kernel of this file now.  CUDA loads
// kernels lazily (on first launch) by default; a caller that must not have
// the CUDA driver allocate during a later call (the allocation-free entry point)
// has them loaded at its set-up instead.  Returns the first error.
cudaError_t preload_spgemm_kernels() {
    const void *fns[] = {
        (const void *)k_sym_tiny,
        (const void *)k_sym_flagw<kBitwRows>,
        (const void *)k_sym_hash_warp<kSymWarpRows, kSymWarpTable>,
        (const void *)k_sym_hash_cta<kSymCtaThreads, kSymCtaTable>,
        (const void *)k_sym_wide<kWideThreads>,
        (const void *)k_num_tiny,
        (const void *)k_num_hash_warp<kNumWarpRows, kNumWarpTable>,
        (const void *)k_num_densew<kDensewRows>,
        (const void *)k_num_rankm<kRankmRows>,
        (const void *)k_num_rankw<kRankwRows>,
        (const void *)k_num_rank<kRankSThreads, false>,
        (const void *)k_num_rank<kRankLThreads, true>,
        (const void *)k_num_hash_cta<kNumCtaSThreads, kNumCtaSTable>,
        (const void *)k_num_hash_cta<kNumCtaLThreads, kNumCtaLTable>,
        (const void *)k_num_rankwin<kRankWinThreads, kRankWinWords>,
        (const void *)k_dense_items,
        (const void *)k_num_dscr<kRankWinThreads, kRankWinWords>,
        (const void *)k_num_gdense<kGdenseThreads>,
        (const void *)k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, true>,
        (const void *)k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, false>,
    };
    for (const void *f : fns) {
        cudaFuncAttributes fa;
        const cudaError_t e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Dynamic shared memory of the rank kernel: staging, bitmap and word ranks of
// maxWords words, vcap shared values.
static size_t smem_rank(int threads, int maxWords, int vcap) {
    const size_t stage = threads == kRankSThreads ? StageLayout<kRankSThreads>::bytes : StageLayout<kRankLThreads>::bytes;
    return stage + 8 * (size_t)maxWords + 8 * (size_t)vcap;
}

static int wide_window_bits(int64_t ncols) {
    int64_t w = 32;
    while (w < ncols && w < kWideWindowBitsMax) w <<= 1;
    return (int)w;
}

// Symbolic kernel of bin b over list[begin, begin + n).
void launch_symbolic_bin(const SymArgs &a, int bin, int32_t begin, int32_t n, cudaStream_t s,
                         int *launches) {
    if (n <= 0) return;
    switch (bin) {
        case SB_TINY:
            k_sym_tiny<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(a, begin, n);
            break;
        case SB_BITW:
            k_sym_flagw<kBitwRows><<<(unsigned)ceil_div(n, kBitwRows), 32 * kBitwRows, 0, s>>>(a, begin, n);
            break;
        case SB_HWARP:
            k_sym_hash_warp<kSymWarpRows, kSymWarpTable>
                <<<(unsigned)ceil_div(n, kSymWarpRows), 32 * kSymWarpRows, kSmemSymWarp, s>>>(a, begin, n);
            break;
        case SB_HCTA:
            k_sym_hash_cta<kSymCtaThreads, kSymCtaTable><<<(unsigned)n, kSymCtaThreads, kSmemSymCta, s>>>(a, begin);
            break;
        case SB_WIDE: {
            // Persistent: as many CTAs as fit on the GPU at once (two per SM
            // with the widest window), rows taken from a counter.
            const int wb = wide_window_bits(a.B.n);
            const size_t smem = kSmemWideBase + (size_t)wb / 8 + 4 * (size_t)wide_touch_cap(wb) + 4 * kWideThreads;
            const int per_sm = std::max(1, std::min(2048 / kWideThreads, (int)((227 * 1024) / (smem + 1024))));
            const int grid = (int)std::min<int64_t>(n, (int64_t)std::max(a.numSms, 1) * per_sm);
            k_sym_wide<kWideThreads><<<(unsigned)grid, kWideThreads, smem, s>>>(a, begin, n, wb);
            break;
        }
        default:
            return;
    }
    ++*launches;
}

// Resident CTAs of kernel fn on the whole GPU (the grid of a device-driven
// launch, which strides over however many rows its bin holds).
// The occupancy is looked up once per kernel and shared-memory size, so
// that launches inside a stream capture query nothing.
static int resident_grid(const void *fn, int threads, size_t smem, int sms) {
    struct Entry {
        const void *fn;
        size_t smem;
        int per_sm;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    std::lock_guard<std::mutex> lk(mu);
    for (const Entry &e : cache)
        if (e.fn == fn && e.smem == smem) return e.per_sm * std::max(sms, 1);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    cache.push_back(Entry{fn, smem, per_sm});
    return per_sm * std::max(sms, 1);
}

void launch_symbolic_bin_dd(const SymArgs &a, int bin, cudaStream_t s, int *launches) {
    switch (bin) {
        case SB_TINY: {
            const void *fn = (const void *)k_sym_tiny_dd;
            k_sym_tiny_dd<<<resident_grid(fn, 256, 0, a.numSms), 256, 0, s>>>(a, bin);
            break;
        }
        case SB_BITW: {
            const void *fn = (const void *)k_sym_flagw_dd<kBitwRows>;
            k_sym_flagw_dd<kBitwRows><<<resident_grid(fn, 32 * kBitwRows, 0, a.numSms), 32 * kBitwRows, 0, s>>>(a, bin);
            break;
        }
        case SB_HWARP: {
            const void *fn = (const void *)k_sym_hash_warp_dd<kSymWarpRows, kSymWarpTable>;
            k_sym_hash_warp_dd<kSymWarpRows, kSymWarpTable>
                <<<resident_grid(fn, 32 * kSymWarpRows, kSmemSymWarp, a.numSms), 32 * kSymWarpRows, kSmemSymWarp, s>>>(
                    a, bin);
            break;
        }
        case SB_HCTA: {
            const void *fn = (const void *)k_sym_hash_cta_dd<kSymCtaThreads, kSymCtaTable>;
            k_sym_hash_cta_dd<kSymCtaThreads, kSymCtaTable>
                <<<resident_grid(fn, kSymCtaThreads, kSmemSymCta, a.numSms), kSymCtaThreads, kSmemSymCta, s>>>(a, bin);
            break;
        }
        case SB_WIDE: {
            const int wb = wide_window_bits(a.B.n);
            const size_t smem = kSmemWideBase + (size_t)wb / 8 + 4 * (size_t)wide_touch_cap(wb) + 4 * kWideThreads;
            const int grid = resident_grid((const void *)k_sym_wide<kWideThreads>, kWideThreads, smem, a.numSms);
            k_sym_wide<kWideThreads><<<(unsigned)grid, kWideThreads, smem, s>>>(a, -1, 0, wb);
            break;
        }
        default:
            return;
    }
    ++*launches;
}

// Device-driven numeric launch of bin `bin` (rows from a.binStart on the
// device): persistent grids, the dense bin on rank windows without pieces.
void launch_numeric_bin_dd(const NumArgs &a, int bin, cudaStream_t s, int *launches) {
    switch (bin) {
        case NB_TINY: {
            k_num_tiny_dd<<<resident_grid((const void *)k_num_tiny_dd, 256, 0, a.numSms), 256, 0, s>>>(a, bin);
            break;
        }
        case NB_HWARP: {
            const void *fn = (const void *)k_num_hash_warp_dd<kNumWarpRows, kNumWarpTable>;
            k_num_hash_warp_dd<kNumWarpRows, kNumWarpTable>
                <<<resident_grid(fn, 32 * kNumWarpRows, kSmemNumWarp, a.numSms), 32 * kNumWarpRows, kSmemNumWarp, s>>>(
                    a, bin);
            break;
        }
        case NB_DENSEW: {
            const void *fn = (const void *)k_num_densew_dd<kDensewRows>;
            k_num_densew_dd<kDensewRows><<<resident_grid(fn, 32 * kDensewRows, 0, a.numSms), 32 * kDensewRows, 0, s>>>(
                a, bin);
            break;
        }
        case NB_RANKM: {
            const int grid = std::max(a.numSms, 1) * 3;
            k_num_rankm<kRankmRows><<<(unsigned)grid, 32 * kRankmRows, kSmemRankm, s>>>(a, -1, 0);
            break;
        }
        case NB_RANKW: {
            const void *fn = (const void *)k_num_rankw_dd<kRankwRows>;
            k_num_rankw_dd<kRankwRows><<<resident_grid(fn, 32 * kRankwRows, 0, a.numSms), 32 * kRankwRows, 0, s>>>(
                a, bin);
            break;
        }
        case NB_RANKS: {
            const size_t smem = smem_rank(kRankSThreads, a.tune.rankWordsMax, a.tune.rankSharedMax);
            const void *fn = (const void *)k_num_rank_dd<kRankSThreads, false>;
            k_num_rank_dd<kRankSThreads, false><<<resident_grid(fn, kRankSThreads, smem, a.numSms), kRankSThreads, smem,
                                                  s>>>(a, bin, a.tune.rankWordsMax, a.tune.rankSharedMax);
            break;
        }
        case NB_RANKL: {
            const size_t smem = smem_rank(kRankLThreads, a.tune.rankWordsMax, 0);
            const void *fn = (const void *)k_num_rank_dd<kRankLThreads, true>;
            k_num_rank_dd<kRankLThreads, true><<<resident_grid(fn, kRankLThreads, smem, a.numSms), kRankLThreads, smem,
                                                 s>>>(a, bin, a.tune.rankWordsMax, 0);
            break;
        }
        case NB_HCTA_S: {
            const void *fn = (const void *)k_num_hash_cta_dd<kNumCtaSThreads, kNumCtaSTable>;
            k_num_hash_cta_dd<kNumCtaSThreads, kNumCtaSTable>
                <<<resident_grid(fn, kNumCtaSThreads, kSmemNumCtaS, a.numSms), kNumCtaSThreads, kSmemNumCtaS, s>>>(a,
                                                                                                               bin);
            break;
        }
        case NB_HCTA_L: {
            const void *fn = (const void *)k_num_hash_cta_dd<kNumCtaLThreads, kNumCtaLTable>;
            k_num_hash_cta_dd<kNumCtaLThreads, kNumCtaLTable>
                <<<resident_grid(fn, kNumCtaLThreads, kSmemNumCtaL, a.numSms), kNumCtaLThreads, kSmemNumCtaL, s>>>(a,
                                                                                                               bin);
            break;
        }
        case NB_DENSE: {
            cudaMemsetAsync(a.ctr + CTR_NUM_RANKWIN, 0, sizeof(uint32_t), s);
            const void *fn = (const void *)k_num_rankwin<kRankWinThreads, kRankWinWords>;
            k_num_rankwin<kRankWinThreads, kRankWinWords>
                <<<resident_grid(fn, kRankWinThreads, kSmemRankWin, a.numSms), kRankWinThreads, kSmemRankWin, s>>>(a, -1,
                                                                                                              0);
            break;
        }
        default:
            return;
    }
    ++*launches;
}

// Looks up the grids of every device-driven launch for these thresholds and
// B's column count ahead of any stream capture.
void prepare_dd_grids(const Tuning &t, int64_t bcols, int sms) {
    const int wb = wide_window_bits(bcols);
    resident_grid((const void *)k_sym_tiny_dd, 256, 0, sms);
    resident_grid((const void *)k_sym_flagw_dd<kBitwRows>, 32 * kBitwRows, 0, sms);
    resident_grid((const void *)k_sym_hash_warp_dd<kSymWarpRows, kSymWarpTable>, 32 * kSymWarpRows, kSmemSymWarp, sms);
    resident_grid((const void *)k_sym_hash_cta_dd<kSymCtaThreads, kSymCtaTable>, kSymCtaThreads, kSmemSymCta, sms);
    resident_grid((const void *)k_sym_wide<kWideThreads>, kWideThreads,
                  kSmemWideBase + (size_t)wb / 8 + 4 * (size_t)wide_touch_cap(wb) + 4 * kWideThreads, sms);
    resident_grid((const void *)k_num_tiny_dd, 256, 0, sms);
    resident_grid((const void *)k_num_hash_warp_dd<kNumWarpRows, kNumWarpTable>, 32 * kNumWarpRows, kSmemNumWarp, sms);
    resident_grid((const void *)k_num_densew_dd<kDensewRows>, 32 * kDensewRows, 0, sms);
    resident_grid((const void *)k_num_rankw_dd<kRankwRows>, 32 * kRankwRows, 0, sms);
    resident_grid((const void *)k_num_rank_dd<kRankSThreads, false>, kRankSThreads,
                  smem_rank(kRankSThreads, t.rankWordsMax, t.rankSharedMax), sms);
    resident_grid((const void *)k_num_rank_dd<kRankLThreads, true>, kRankLThreads,
                  smem_rank(kRankLThreads, t.rankWordsMax, 0), sms);
    resident_grid((const void *)k_num_hash_cta_dd<kNumCtaSThreads, kNumCtaSTable>, kNumCtaSThreads, kSmemNumCtaS, sms);
    resident_grid((const void *)k_num_hash_cta_dd<kNumCtaLThreads, kNumCtaLTable>, kNumCtaLThreads, kSmemNumCtaL, sms);
    resident_grid((const void *)k_num_rankwin<kRankWinThreads, kRankWinWords>, kRankWinThreads, kSmemRankWin, sms);
    resident_grid((const void *)k_num_rankm<kRankmRows>, 32 * kRankmRows, kSmemRankm, sms);
}

void launch_numeric_bin(const NumArgs &a, int bin, int32_t lo, int32_t hi, cudaStream_t s,
                        int *launches) {
    const int32_t n = hi - lo;
    if (n <= 0) return;
    switch (bin) {
        case NB_TINY:
            k_num_tiny<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(a, lo, n);
            break;
        case NB_HWARP:
            k_num_hash_warp<kNumWarpRows, kNumWarpTable>
                <<<(unsigned)ceil_div(n, kNumWarpRows), 32 * kNumWarpRows, kSmemNumWarp, s>>>(a, lo, n);
            break;
        case NB_DENSEW:
            k_num_densew<kDensewRows><<<(unsigned)ceil_div(n, kDensewRows), 32 * kDensewRows, 0, s>>>(a, lo, n);
            break;
        case NB_RANKM: {
            // Persistent: three CTAs of kRankmRows warps per SM.
            const int grid = (int)std::min<int64_t>(ceil_div(n, kRankmRows), (int64_t)std::max(a.numSms, 1) * 3);
            k_num_rankm<kRankmRows><<<(unsigned)grid, 32 * kRankmRows, kSmemRankm, s>>>(a, lo, n);
            break;
        }
        case NB_RANKW:
            k_num_rankw<kRankwRows><<<(unsigned)ceil_div(n, kRankwRows), 32 * kRankwRows, 0, s>>>(a, lo, n);
            break;
        case NB_RANKS:
            k_num_rank<kRankSThreads, false>
                <<<(unsigned)n, kRankSThreads, smem_rank(kRankSThreads, a.tune.rankWordsMax, a.tune.rankSharedMax), s>>>(
                    a, lo, a.tune.rankWordsMax, a.tune.rankSharedMax);
            break;
        case NB_RANKL:
            k_num_rank<kRankLThreads, true><<<(unsigned)n, kRankLThreads, smem_rank(kRankLThreads, a.tune.rankWordsMax, 0),
                                             s>>>(a, lo, a.tune.rankWordsMax, 0);
            break;
        case NB_HCTA_S:
            k_num_hash_cta<kNumCtaSThreads, kNumCtaSTable><<<(unsigned)n, kNumCtaSThreads, kSmemNumCtaS, s>>>(a, lo);
            break;
        case NB_HCTA_L:
            k_num_hash_cta<kNumCtaLThreads, kNumCtaLTable><<<(unsigned)n, kNumCtaLThreads, kSmemNumCtaL, s>>>(a, lo);
            break;
        case NB_DENSE:
            if (a.tune.denseMethod == 0) {
                cudaMemsetAsync(a.ctr + CTR_NUM_RANKWIN, 0, sizeof(uint32_t), s);
                const int per_sm = std::max(1, (int)((227 * 1024) / (kSmemRankWin + 1024)));
                int64_t work = n;
                if (a.items) {
                    // Heavy rows cut into pieces: the items are built on the
                    // device, so the grid is the persistent one.
                    cudaMemsetAsync(a.ctr + CTR_ITEMS, 0, sizeof(uint32_t), s);
                    k_dense_items<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(a, lo, n);
                    ++*launches;
                    work = (int64_t)a.itemCap;
                }
                const int grid = (int)std::min<int64_t>(work, (int64_t)std::max(a.numSms, 1) * per_sm);
                k_num_rankwin<kRankWinThreads, kRankWinWords>
                    <<<(unsigned)grid, kRankWinThreads, kSmemRankWin, s>>>(a, lo, n);
            } else if (a.tune.denseMethod == 3 && a.scr) {
                cudaMemsetAsync(a.ctr + CTR_NUM_DSCR, 0, sizeof(uint32_t), s);
                const int grid = (int)std::min<int64_t>(n, a.scrSlots);
                k_num_dscr<kRankWinThreads, kRankWinWords><<<(unsigned)grid, kRankWinThreads, kSmemDscr, s>>>(a, lo, n);
            } else if (a.tune.denseMethod == 1 && a.gBits) {
                cudaMemsetAsync(a.ctr + CTR_NUM_GDENSE, 0, sizeof(uint32_t), s);
                const int grid = (int)std::min<int64_t>(n, a.gSlots);
                const size_t smem = kSmemGdenseBase + 4 * (size_t)(a.gStride >> 10);
                k_num_gdense<kGdenseThreads><<<(unsigned)grid, kGdenseThreads, smem, s>>>(a, lo, n);
            } else if (a.bSorted)
                k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, true>
                    <<<(unsigned)n, kDenseThreads, kSmemDense, s>>>(a, lo);
            else
                k_num_dense<kDenseThreads, kDenseWindow, kDenseStage, false>
                    <<<(unsigned)n, kDenseThreads, kSmemDense, s>>>(a, lo);
            break;
        default:
            return;
    }
    ++*launches;
}

}  // namespace dbd
