// dbd_internal.h -- declarations shared by the host engine and the CUDA
// kernels of libdbd.  Not part of the public ABI (include/dbd.h is).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dbd {

// Device view of a CSR operand: int32 row_ptr/col_idx, FP64 values.
struct CsrDev {
    int64_t m = 0, n = 0, nnz = 0;
    const int32_t *ptr = nullptr;
    const int32_t *idx = nullptr;
    const double *val = nullptr;
};

// Row categories.  Each row of C spans the columns [lo, hi] (the smallest
// and largest column its products reach, from the first and last column of
// every B row it references); "span words" below is the number of 32-column
// words that range covers.  The symbolic pass bins rows by their product
// count P_r (an upper bound of the row's output size) and span, the numeric
// pass by the exact output size nnz_r and span.  Lists of rows per bin keep
// row order, so the rows of any run of row blocks form one contiguous range
// of every bin.
enum SymBin : uint8_t { SB_EMPTY = 0, SB_TINY, SB_BITW, SB_HWARP, SB_HCTA, SB_WIDE, SB_COUNT };
enum NumBin : uint8_t {
    NB_EMPTY = 0, NB_TINY, NB_RANKW, NB_HWARP, NB_RANKS, NB_RANKL, NB_HCTA_S, NB_HCTA_L, NB_DENSE, NB_DENSEW, NB_RANKM,
    NB_COUNT
};
constexpr int kMaxBins = 12;
constexpr int kTileRows = 256;     // granularity of the per-bin offset tables
constexpr int kScanTile = 4096;    // rows per CTA of the row_ptr scan

// Compile-time table sizes of the accumulators; the bin thresholds below
// must keep every row inside its table at load factor <= 1/2.
constexpr int kTinyMax = 32;                 // products held one per lane
constexpr int kSymWarpTable = 1024, kSymWarpMax = 512;
constexpr int kSymCtaTable = 8192, kSymCtaMax = 4096;
constexpr int kNumWarpTable = 512, kNumWarpMax = 256;
constexpr int kNumCtaSTable = 2048, kNumCtaSMax = 1024;
constexpr int kNumCtaLTable = 8192, kNumCtaLMax = 4096;
constexpr int kDenseWindow = 8192;           // FP64 columns per dense window (64 KiB)
constexpr int kWideWindowBitsMax = 1 << 19;  // symbolic bitmap window (64 KiB: two CTAs per SM)
constexpr int kWarpSpanWords = 64;           // warp-level bitmap rows: span <= 2048 columns
constexpr int kDenseWarpWords = 16;          // warp dense-window rows: span <= 512 columns
constexpr int kMidSpanWords = 2048;          // warp rank rows over their own window: span <= 2^16 columns
constexpr int kRankWordsMax = 8192;          // CTA rank rows: span <= 2^18 columns
constexpr int kWideHashSpanWords = 2048;     // symbolic: P <= kSymCtaMax rows hash above this span
constexpr int kWideTouchMax = 8192;          // words a wide-row window clears one by one
// Heavy rows of the dense bin are cut into pieces by column.  The symbolic
// pass records, for rows with at least kHeavyP products, the entries of C's
// row in every slab of 2^kSlabShift columns (from the row's first word);
// the numeric pass cuts dense rows of more than kPieceNnz entries at slab
// boundaries into pieces of about kPieceNnz entries and at most
// kPieceSlabs slabs (2^20 columns, two windows of the dense-bin kernel),
// each an independent work item.
constexpr int kSlabShift = 16;
constexpr int kMaxSlabs = 64;                // rows spanning up to 2^22 columns
constexpr int64_t kHeavyP = 65536;
constexpr int kPieceNnz = 65536;
constexpr int kPieceSlabs = 16;

__host__ __device__ __forceinline__ int span_words(int32_t lo, int32_t hi) {
    return hi >= lo ? (hi >> 5) - (lo >> 5) + 1 : 0;
}

// Runtime bin thresholds (the autotuner's knobs).  Each is capped by the
// compile-time size it selects against, so every choice keeps every row
// inside its kernel's tables: warpSpanWords <= kWarpSpanWords, numWarpMax <=
// kNumWarpMax, symWarpMax <= kSymWarpMax, rankWordsMax <= kRankWordsMax,
// rankSharedMax <= kNumCtaLMax (the shared value array of the rank kernel).
struct Tuning {
    int32_t warpSpanWords = kWarpSpanWords;   // narrow rows: warp bitmap / warp rank kernels
    int32_t numWarpMax = kNumWarpMax;         // numeric rows on one warp (rank or hash)
    int32_t symWarpMax = kSymWarpMax;         // symbolic rows on a warp hash table
    int32_t rankWordsMax = kRankWordsMax;     // CTA rank kernels for windows up to this many words
    int32_t rankSharedMax = kNumCtaLMax;      // rank rows accumulating in shared memory
    int32_t symHashSpanWords = kWideHashSpanWords;  // symbolic CTA rows hash above this span
    int32_t denseWarpWords = kDenseWarpWords; // numeric rows on one warp's dense window
    int32_t midSpanWords = 0;                 // numeric rows on one warp's rank window (off: the
                                              // bucket-sorted warp hash measures faster)
    int32_t denseMethod = 0;                  // dense bin: 0 rank windows, 1 global slots, 2 FP64 windows,
                                              // 3 one pass into FP64 scratch rows
};

__host__ __device__ __forceinline__ uint8_t sym_bin_of(int64_t P, int32_t nA, int sw, const Tuning &t) {
    if (P == 0) return SB_EMPTY;
    if (P <= kTinyMax && nA <= 32) return SB_TINY;
    if (sw <= t.warpSpanWords) return SB_BITW;
    if (P <= t.symWarpMax) return SB_HWARP;
    if (P <= kSymCtaMax && sw > t.symHashSpanWords) return SB_HCTA;
    return SB_WIDE;
}

__host__ __device__ __forceinline__ uint8_t num_bin_of(int64_t P, int32_t nA, int32_t nnz, int sw,
                                                       const Tuning &t) {
    if (nnz == 0) return NB_EMPTY;
    if (P <= kTinyMax && nA <= 32) return NB_TINY;
    if (sw <= t.denseWarpWords) return NB_DENSEW;
    if (sw <= t.warpSpanWords && nnz <= t.numWarpMax) return NB_RANKW;
    if (sw <= t.midSpanWords && nnz <= t.numWarpMax) return NB_RANKM;
    if (nnz <= t.numWarpMax) return NB_HWARP;
    if (sw <= t.rankWordsMax) return nnz <= t.rankSharedMax ? NB_RANKS : NB_RANKL;
    if (nnz <= kNumCtaSMax) return NB_HCTA_S;
    if (nnz <= kNumCtaLMax) return NB_HCTA_L;
    return NB_DENSE;
}

// Clamps t into its caps (minimums keep each bin meaningful).
inline Tuning clamp_tuning(Tuning t) {
    auto cl = [](int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); };
    t.warpSpanWords = cl(t.warpSpanWords, 1, kWarpSpanWords);
    t.numWarpMax = cl(t.numWarpMax, 1, kNumWarpMax);
    t.symWarpMax = cl(t.symWarpMax, kTinyMax, kSymWarpMax);
    t.rankWordsMax = cl(t.rankWordsMax, 1, kRankWordsMax);
    t.rankSharedMax = cl(t.rankSharedMax, 1, kNumCtaLMax);
    t.symHashSpanWords = cl(t.symHashSpanWords, 0, 1 << 26);
    t.denseWarpWords = cl(t.denseWarpWords, 0, kDenseWarpWords);
    t.midSpanWords = cl(t.midSpanWords, 0, kMidSpanWords);
    t.denseMethod = cl(t.denseMethod, 0, 3);
    return t;
}

// Per-row analysis of A*B: products and the column window of each row.
struct RowInfo {
    int64_t *rowP = nullptr;  // products
    int32_t *lo = nullptr;    // smallest column reached (INT32_MAX if none)
    int32_t *hi = nullptr;    // largest column reached (-1 if none)
};

// Device-side error word values (kernels never trap; the host reads this).
enum DevErr : int { DEV_OK = 0, DEV_TABLE_FULL = 1, DEV_COUNT_MISMATCH = 2, DEV_ROW_TOO_LONG = 3, DEV_OUT_OF_WINDOW = 4 };

// Counter slots for dynamically scheduled kernels (zeroed per multiply).
enum CounterSlot : int {
    CTR_SYM_TINY = 0, CTR_SYM_HWARP, CTR_SYM_HCTA, CTR_SYM_WIDE, CTR_NUM_GDENSE, CTR_NUM_RANKWIN, CTR_NUM_DSCR,
    CTR_HEAVY, CTR_ITEMS, CTR_COUNT = 16
};

struct Binning {
    uint8_t *bin = nullptr;     // m bin ids
    int32_t *list = nullptr;    // m row ids grouped by bin
    int32_t *hist = nullptr;    // ntiles * kMaxBins counts
    int32_t *tileOff = nullptr; // (ntiles + 1) * kMaxBins absolute offsets into list
    int32_t *binStart = nullptr;// kMaxBins + 1
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---- launchers (k_analysis.cu) ----
// First and last column of every row of B (bmin = INT32_MAX, bmax = -1 for
// empty rows; any column order).
void launch_row_minmax(const CsrDev &B, int32_t *bmin, int32_t *bmax, int *unsorted, cudaStream_t s, int num_sms);
void launch_row_products(const CsrDev &A, const int32_t *Bp, const int32_t *bmin, const int32_t *bmax,
                         const RowInfo &ri, uint8_t *symBin, int *err, const Tuning &t, cudaStream_t s,
                         int num_sms);
void launch_block_products(int64_t m, const int64_t *rowP, int64_t rows_per_block,
                           int64_t *blockP, cudaStream_t s);
void launch_bin_lists(int64_t m, const Binning &b, int nbins, cudaStream_t s);
void launch_num_bins(int64_t m, const int32_t *Ap, const RowInfo &ri, const int32_t *rowNnz,
                     uint8_t *numBin, const Tuning &t, cudaStream_t s, int num_sms);
void launch_row_scan(int64_t m, const int32_t *rowNnz, int64_t *part, int64_t *Cp, cudaStream_t s);

// ---- launchers (k_spgemm.cu) ----
struct SymArgs {
    CsrDev A, B;
    const int32_t *list;
    const int32_t *binStart;
    int32_t *rowNnz;
    uint32_t *ctr;
    int *err;
    const int32_t *rowLo = nullptr;  // per-row column window (RowInfo)
    const int32_t *rowHi = nullptr;
    const int64_t *rowP = nullptr;   // per-row products (RowInfo)
    // Optional store of the wide rows' column bitmaps for the numeric rank
    // kernel (null: not kept): kRankWordsMax words per wide row (the row's
    // window from word lo/32 on), at the row's position in the wide bin;
    // wideSlot[row] receives that position.
    uint32_t *wideBits = nullptr;
    int32_t *wideSlot = nullptr;
    Tuning tune;
    int numSms = 0;  // persistent kernels size their grid by it; ctr holds their zeroed row counters
    int bSorted = 0; // B's rows have strictly ascending columns
    const int *bUnsorted = nullptr;  // device-driven launches: the device's flag instead (nonzero: not ascending)
    // Slab counts of heavy rows (null: not recorded): heavySlot[row] = -1 or
    // the row's slot (taken from ctr[CTR_HEAVY], below heavyCap); slabCnt
    // holds kMaxSlabs counts per slot.
    int32_t *heavySlot = nullptr;
    int32_t *slabCnt = nullptr;
    int heavyCap = 0;
};
// Launches the symbolic kernel of bin `bin` over list[begin, begin + n).
void launch_symbolic_bin(const SymArgs &a, int bin, int32_t begin, int32_t n, cudaStream_t s, int *launches);
// Device-driven launch of a symbolic bin: its rows from a.binStart on the
// device, a grid of resident CTAs striding over them (no host read of the
// bin sizes, so a stream capture holds it).
void launch_symbolic_bin_dd(const SymArgs &a, int bin, cudaStream_t s, int *launches);
void launch_f32_to_f64(const float *src, double *dst, int64_t n, cudaStream_t s);
void launch_validate_ptr(const int32_t *ptr, int64_t m, int64_t nnz, int *flag, cudaStream_t s);
void launch_validate_idx(const int32_t *idx, int64_t nnz, int64_t ncols, int *flag, cudaStream_t s);

// One work item of the dense bin: row, or the piece of it over the column
// slabs [s0, s1) whose entries start `off` entries into C's row (s0 < 0:
// the whole row).
struct DenseItem {
    int32_t row;
    int16_t s0, s1;
    int32_t cnt;   // entries of the piece
    int64_t off;
};

struct NumArgs {
    CsrDev A, B;
    const int32_t *list;
    const int32_t *binStart = nullptr;  // device-driven launches: each bin's [start, end) in list
    const int64_t *Cp;
    int64_t outBase;      // Cp value stored at out[0]
    int32_t *Ci;
    double *Cv;
    int32_t *state;       // 2 * nnz(A) scratch for the dense windows (cursor, next column)
    int bSorted;          // B's rows have ascending columns
    const int *bUnsorted = nullptr;  // device-driven launches: the device's flag instead (nonzero: not ascending)
    int *err;
    const int64_t *rowP = nullptr;   // per-row products and column window (RowInfo)
    const int32_t *rowLo = nullptr;
    const int32_t *rowHi = nullptr;
    // Optional per-row amount subtracted from the columns written to Ci
    // (batched products: each pair's columns start at 0).
    const int32_t *colShift = nullptr;
    // Column bitmaps of the wide rows kept by the symbolic pass (null: the
    // rank kernels rebuild them); a row's is kept when its symbolic bin is
    // SB_WIDE and its window has at most kRankWordsMax words.
    const uint32_t *wideBits = nullptr;
    const int32_t *wideSlot = nullptr;
    Tuning tune;
    int numSms = 0;  // persistent kernels size their grid by it
    // Global slots for the dense bin (null: shared-memory windows): gSlots
    // slots of gStride columns, each a bitmap and its word ranks; bitmaps
    // are zero between rows.
    uint32_t *gBits = nullptr;
    uint32_t *gWpre = nullptr;
    int64_t gStride = 0;   // multiple of 1024
    int gSlots = 0;
    uint32_t *ctr = nullptr;  // row counters of the persistent dense-row kernels (zeroed per launch)
    // FP64 scratch rows of the one-pass dense kernel (dense_method 3): one of
    // scrStride doubles per CTA (scrSlots of them), zero between rows.
    double *scr = nullptr;
    int64_t scrStride = 0;
    int scrSlots = 0;
    // Work items of the dense bin (null: one item per row).  Built on the
    // device per launch from the bin's rows: a heavy row with slab counts
    // becomes several pieces; the count is ctr[CTR_ITEMS].
    const int32_t *heavySlot = nullptr;
    const int32_t *slabCnt = nullptr;
    DenseItem *items = nullptr;
    int itemCap = 0;
};

// Bytes of one global dense slot of `stride` columns.
inline size_t gdense_slot_bytes(int64_t stride) { return (size_t)stride / 4; }
constexpr int kGdenseSumMax = 8192;  // summary words in shared memory: C up to 2^23 columns
// Runs the numeric kernels of bin b over list[lo, hi).
// Device-driven launch of a numeric bin (rows from a.binStart on the
// device; the dense bin on rank windows without pieces).
void launch_numeric_bin_dd(const NumArgs &a, int bin, cudaStream_t s, int *launches);
// Looks up the grids of the device-driven launches ahead of a stream capture.
void prepare_dd_grids(const Tuning &t, int64_t bcols, int sms);
void launch_numeric_bin(const NumArgs &a, int bin, int32_t lo, int32_t hi, cudaStream_t s,
                        int *launches);

// Adjoint of C = A*B over fixed patterns: given G = dL/dC on C's pattern
// (Cp, Ci), dA[e] = sum_k G(i,k) B(j,k) for e = (i,j) in A and
// dB[f] += A(i,j) G(i,k) for f = (j,k) in B.  dA and dB start at zero.
struct AdjArgs {
    CsrDev A, B;
    const int64_t *Cp;
    const int32_t *Ci;
    const double *G;
    double *dA;
    double *dB;
    const int32_t *order;  // rows of A in the forward's numeric bin order (null: 0..m-1)
    int64_t nrows;
    int *err;
};
void launch_adjoint(const AdjArgs &a, cudaStream_t s, int *launches);
// dB = mask_B(A^T G) on its own: one warp per row k of B, each lane one
// entry (k, j), summing A(i,k) * G(i,j) over column k of A in row order
// (colPtr / perm / rowOf: A's entries grouped by column, stably).
struct AdjDbArgs {
    CsrDev B;
    const double *Aval;
    const int32_t *colPtr;  // A.n + 1
    const uint32_t *perm;   // A's entry indices by column, rows ascending
    const int32_t *rowOf;   // row of each A entry
    const int64_t *Cp;
    const int32_t *Ci;
    const double *G;
    double *dB;
    int *err;
    int32_t *extra;         // nnz(B): segments after the first, per entry
    int64_t *xStart;        // nnz(B) + 1: their exclusive scan
    double *part;           // partCap: one partial sum per further segment
    int64_t partCap;
};
// Entry rows and the column grouping of A for launch_adjoint_db (keys and
// vals: two pairs of nnz(A) uint32 buffers; scratch: stable_sort_scratch_bytes).
void launch_adjoint_transpose(const CsrDev &A, int32_t *rowOf, uint32_t *keys0, uint32_t *vals0, uint32_t *keys1,
                              uint32_t *vals1, void *scratch, int32_t *colPtr, const uint32_t **perm, cudaStream_t s);
// partCap for a.part: the further segments number at most the forward's
// products over the segment length.  scanPart: ceil(nnz(B) / kScanTile) + 1
// int64 for the scan of the segment counts.
int64_t adjoint_db_part_cap(int64_t products);
void launch_adjoint_db(const AdjDbArgs &a, int64_t *scanPart, int num_sms, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs by the low `bits` of the key
// (k_mtx.cu): k0/v0 in, k1/v1 scratch; *keys / *vals receive whichever pair
// holds the result.
int64_t stable_sort_scratch_bytes(int64_t n);
void launch_stable_sort_u32(uint32_t *k0, uint32_t *v0, uint32_t *k1, uint32_t *v1, int64_t n, int bits,
                            void *scratch, cudaStream_t s, uint32_t **keys, uint32_t **vals);

// ---- batched products (k_batch.cu) ----
// One operand of one pair and its place in the concatenated operand.
struct BatchPair {
    const int32_t *ptr;     // m + 1 row pointers (device-accessible)
    const int32_t *idx;     // nnz columns in [0, ncols)
    const double *val;      // nnz values (may alias the output at nnzOff)
    int64_t m, nnz, ncols;
    int64_t nnzOff;         // first entry in the concatenated operand
    int64_t colOff;         // added to every column
    int32_t shift;          // per-row column shift recorded for the product's rows
};
// Concatenates count pairs' operands: rows [rowOff[q], rowOff[q+1]) and
// entries [nnzOff[q], nnzOff[q+1]) of the output come from pair q.  rowShift
// (may be null) receives pairs[q].shift for every row of pair q.  *bad gets
// bit 0 for a malformed row_ptr and bit 1 for a column out of range.
void launch_batch_gather(const BatchPair *pairs, const int64_t *rowOff, const int64_t *nnzOff, int64_t count,
                         int64_t totalRows, int64_t totalNnz, int32_t *outPtr, int32_t *outIdx, double *outVal,
                         int32_t *rowShift, int *bad, cudaStream_t s);

// dst[i] = src[idx[i]] for i < n.
void launch_gather_i64(const int64_t *src, const int64_t *idx, int64_t n, int64_t *dst, cudaStream_t s);
// Guards of the device-driven (capturable) batched multiply: a bad pair
// (*bad) empties both operands (nA / nB row pointers); a symbolic error or
// nnz(C) above capacity empties every numeric bin (the latter sets *over).
void launch_batch_guard(const int *bad, int32_t *ptrA, int64_t nA, int32_t *ptrB, int64_t nB, cudaStream_t s,
                        int num_sms);
void launch_numeric_guard(const int64_t *nnz, int64_t capacity, const int *err, int32_t *binStart, int nbins, int *over,
                          cudaStream_t s);

// ---- output digest (k_digest.cu) ----
// Per-row digest arrays of C (m entries each) and the count of rows whose
// columns are not strictly ascending or out of range.
struct RowDigest {
    int64_t *count = nullptr;
    uint64_t *colHash = nullptr;
    uint64_t *valHash = nullptr;
    double *sum = nullptr;
    double *wsum = nullptr;
    int64_t *bad = nullptr;
};
// Digest of rows [r0, r1) whose entries sit at Cp[r] - outBase in Ci / Cv
// (FP64 values, or the float32 values of the reference's output layout).
void launch_row_digest(int64_t r0, int64_t r1, const int64_t *Cp, int64_t outBase, const int32_t *Ci,
                       const double *Cv, int64_t ncols, const RowDigest &d, cudaStream_t s, int num_sms);
void launch_row_digest(int64_t r0, int64_t r1, const int64_t *Cp, int64_t outBase, const int32_t *Ci,
                       const float *Cv, int64_t ncols, const RowDigest &d, cudaStream_t s, int num_sms);
// dst[i] = src[i] rounded to float32, i < n.
void launch_val_to_f32(const double *src, float *dst, int64_t n, cudaStream_t s, int num_sms);

// *acc += sum over i < n of mix64(((uint64)i << 32 | w[i]) ^ (salt * G)) (an
// order-dependent hash of a device array of 32-bit words).
void launch_hash_words(const uint32_t *w, int64_t n, uint64_t salt, uint64_t *acc, cudaStream_t s);

// One-time kernel attribute setup (dynamic shared memory limits).
void init_kernel_attributes();
// Load the kernels of k_analysis.cu / k_spgemm.cu now instead of at their
// first launch (cudaFuncGetAttributes on each); the first error is returned.
cudaError_t preload_analysis_kernels();
cudaError_t preload_spgemm_kernels();
cudaError_t preload_batch_kernels();

}  // namespace dbd
