/*
 * dbd.h -- C ABI of libdbd, a GB300-native (sm_103a) out-of-core row-block
 * SpGEMM, C = A*B in CSR, that stands in for DBD's SSpMM / compute / d2h path.
 *
 * The reference is a program, not a library: its interface is the argv
 * contract of bin/SSpMM, bin/compute, bin/d2h (ZIP:dbd/src/main.cpp:152-187),
 * the .csr input and Ptr/Idx/Val.output files, and the process-global
 * function set of ZIP:dbd/src/SSpMM.hpp:126-149.  Each entry point below names
 * the reference function it replaces.  The CLI binaries built with this
 * library (bin/SSpMM, bin/compute, bin/d2h, bin/debug) are thin callers of
 * dbd_spgemm_files().
 *
 * Conventions
 *   - Every function returns int: DBD_OK (0) or a negative DBD_ERR_* code;
 *     dbd_error_string() names it and dbd_last_error() gives the message of the
 *     last failure on a context.
 *   - Input CSR: int32 row_ptr (n_rows+1) and col_idx (nnz), values FP64 or
 *     FP32 (val_fp32 = 1, the reference's .csr layout; promoted to FP64 on
 *     upload).  Columns inside a row need not be sorted.  Pointers are host
 *     memory unless on_device = 1.
 *   - Output CSR: int64 row_ptr, int32 col_idx, FP64 values; columns of each
 *     row ascending and unique; structure decided by index only.
 *   - A context owns its device memory, pinned host buffers, streams and the
 *     writer thread; it is not thread-safe (use one per host thread).  Every
 *     call returns with all its device work and file writes complete.
 */
#ifndef DBD_H
#define DBD_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes.  The reference returns -1 with a stderr line for budget and
 * allocation failures (ZIP:dbd/src/main.cpp:211-226, preProc.cu:57-60) and
 * checks no CUDA or I/O return code; here every failure is reported. */
#define DBD_OK                 0
#define DBD_ERR_INVALID       -1  /* bad argument or malformed CSR */
#define DBD_ERR_OOM_DEVICE    -2  /* cudaMalloc failed */
#define DBD_ERR_OOM_HOST      -3  /* malloc / cudaMallocHost failed */
#define DBD_ERR_BUDGET        -4  /* the product does not fit the GPU/host budgets */
#define DBD_ERR_IO            -5  /* open/read/write/fsync failed or short */
#define DBD_ERR_CUDA          -6  /* a CUDA runtime call failed */
#define DBD_ERR_TIMEOUT       -7  /* a bounded wait gave up */
#define DBD_ERR_OVERFLOW      -8  /* an index or count does not fit its type */
#define DBD_ERR_DEVICE_CHECK  -9  /* a kernel's own consistency check fired */
#define DBD_ERR_NO_DEVICE    -10  /* no CUDA device / library built without one */

/* Timing scopes of the reference's three binaries (README "Result"):
 * KERNEL = bin/compute, D2H = bin/d2h, IO = bin/SSpMM. */
typedef enum {
    DBD_SCOPE_KERNEL = 0,
    DBD_SCOPE_D2H = 1,
    DBD_SCOPE_IO = 2
} dbd_scope;

typedef struct dbd_ctx dbd_ctx;

/* Read-only CSR operand (struct csr, ZIP:dbd/src/SSpMM.hpp:36-44, with FP64
 * values and an explicit placement flag). */
typedef struct {
    int64_t n_rows;
    int64_t n_cols;
    int64_t nnz;
    const int32_t *row_ptr;   /* n_rows + 1 entries */
    const int32_t *col_idx;   /* nnz entries */
    const void *val;          /* nnz doubles, or floats when val_fp32 */
    int32_t val_fp32;
    int32_t on_device;        /* 1: the three arrays are device pointers */
} dbd_csr_view;

/* Product matrix.  The library fills it; arrays it allocated are released by
 * dbd_csr_free().  For DBD_SCOPE_KERNEL the arrays are device pointers owned
 * by the context and valid until its next multiply (on_device = 1). */
typedef struct {
    int64_t n_rows;
    int64_t n_cols;
    int64_t nnz;
    int64_t *row_ptr;         /* n_rows + 1 */
    int32_t *col_idx;         /* nnz */
    void *val;                /* nnz doubles, or floats when val_fp32 */
    int32_t on_device;
    int32_t owner;            /* 0: caller, 1: library host allocation, 2: context device memory */
    int32_t val_fp32;         /* 1: val holds floats (a D2H product with out_val_fp32) */
} dbd_csr_out;

/* Budgets and layout (the argv of ZIP:dbd/src/main.cpp:152-187 plus the
 * compile-time ROWS_IN_BLOCK of SSpMM.hpp:16-23). */
typedef struct {
    double host_gib;          /* host DRAM budget for result buffers; reference default 28 */
    double gpu_gib;           /* device budget; reference default 22 */
    int64_t rows_per_block;   /* 4096 (for_small_datasets) or 512 (for_large_datasets) */
    int32_t device;           /* CUDA device ordinal */
    int32_t out_val_fp32;     /* C's values as float32, the reference's layout: in the D2H and IO
                                 scopes each chunk's FP64 values are rounded once on the device, so
                                 8 bytes per entry cross the link (not 12); Val.output is float32 and
                                 a D2H product kept in host memory holds floats (dbd_csr_out.val_fp32).
                                 The kernel scope keeps FP64 on the device. */
    int32_t out_ptr32;        /* Ptr.output as int32 (reference layout): 1 always (fails if nnz(C) >= 2^31),
                                 2 when nnz(C) < 2^31 and int64 otherwise */
    int32_t verbose;          /* print the reference's progress lines */
    int32_t time_kernels;     /* record CUDA events around every kernel family (dbd_stats.t_*_bin_ms);
                                 the bins then run one after another on the context's stream, so
                                 each time is that kernel's own duration (for profiling runs) */
    double io_rotate_gib;     /* > 0: +I/O output files wrap after this many GiB (disk smaller than C) */
    int32_t io_buffered;      /* +I/O through the page cache instead of aligned O_DIRECT writes */
    int32_t io_resume;        /* +I/O keeps a progress manifest and continues an interrupted run
                                 (DBD_WRITER_RESUME; not with io_rotate_gib) */
} dbd_config;

/* Number of row bins the categoriser produces for the symbolic and numeric
 * kernels (see dbd_stats.rows_per_bin). */
#define DBD_NUM_BINS 12

/* Counters and times of the last multiply.  Times are seconds. */
typedef struct {
    double t_preprocess;      /* work estimate + segmentation + categorisation ("Preprocessing", main.cpp:101) */
    double t_compute_gpu;     /* device time of the multiply ("Compute GPU", main.cpp:103) */
    double t_write_file;      /* writer thread busy time ("Write File", main.cpp:104) */
    double t_kernel_exec;     /* distributor wall time of the scope ("Kernel Execution", main.cpp:105) */
    double t_total;           /* t_preprocess + t_kernel_exec ("Total Execution", main.cpp:106) */
    double t_d2h;             /* device->host copy busy time */
    double t_fsync;           /* time spent in fsync at the end of +I/O */
    double t_device_ms;       /* CUDA-event time of the whole device pipeline, ms */
    double t_numeric_ms;      /* CUDA-event time of the numeric kernels, ms */
    int64_t products;         /* intermediate products P = sum |B_k| over A's entries */
    int64_t nnz_c;
    int64_t n_blocks;
    int64_t max_block_products;
    int32_t criteria;         /* categoriser threshold (distributeWorkload.cpp:249-264) */
    int32_t n_chunks;         /* device output chunks streamed */
    int64_t blocks_per_category[3]; /* 0 dense, 1 light, 2 either (distributeWorkload.cpp:266-270) */
    int64_t rows_per_bin[DBD_NUM_BINS];   /* numeric bins: empty, tiny, warp rank, warp hash, CTA rank (shared),
                                             CTA rank (in place), CTA hash S, CTA hash L, dense windows,
                                             warp dense window, warp rank window */
    int64_t sym_rows_per_bin[DBD_NUM_BINS]; /* symbolic bins: empty, tiny, warp flags, warp hash, CTA hash, CTA bitmap */
    int64_t bytes_d2h;
    int64_t bytes_written;
    int64_t gpu_launches;     /* kernels this library launched for the multiply */
    double t_analysis_ms;     /* with time_kernels: work estimate + binning kernels */
    double t_sym_bin_ms[DBD_NUM_BINS];  /* with time_kernels: symbolic kernel of each bin */
    double t_scan_ms;         /* with time_kernels: row_ptr scan + numeric binning */
    double t_num_bin_ms[DBD_NUM_BINS];  /* with time_kernels: numeric kernels of each bin, summed over chunks */
    int64_t io_direct;        /* +I/O: 1 when the files were written with O_DIRECT */
    int64_t resumed_from_row; /* +I/O with io_resume: the row an earlier run's manifest let this one start at */
    int64_t heavy_rows;       /* rows whose per-slab counts the symbolic pass kept, so that the dense bin
                                 could cut them into column pieces */
    double t_chunks_ms;       /* device time of the chunks' numeric work (kernels, float32 rounding,
                                 digest), summed over chunks: t_numeric_ms minus this is time the
                                 compute stream waited for a device slot to be copied out */
    double t_copy_ms;         /* copying scopes: device time of the D2H copies, summed over chunks */
} dbd_stats;

/* ---- lifecycle ---------------------------------------------------------- */

/* Default budgets: host 28 GiB, GPU 22 GiB, 4096 rows per block, device 0. */
void dbd_config_default(dbd_config *cfg);

/* Creates a context on cfg->device and warms it up.
 * Replaces initialize + initialize_GPU (ZIP:dbd/src/main.cpp:152-187,
 * dbd/for_small_datasets/src/preProc.cu:23-26). */
int dbd_create(const dbd_config *cfg, dbd_ctx **out);

/* Releases everything the context owns.
 * Replaces free_Resource + free_GPU (main.cpp:123-150, computeGPU.cu:101-132). */
void dbd_destroy(dbd_ctx *ctx);

/* Uses this CUDA stream (a cudaStream_t cast to void*) for the device
 * pipeline instead of the context's own; NULL restores the context's. */
int dbd_set_stream(dbd_ctx *ctx, void *stream);

const char *dbd_error_string(int code);
const char *dbd_last_error(const dbd_ctx *ctx);

/* ---- files -------------------------------------------------------------- */

/* Host CSR read from disk; free with dbd_csr_host_free(). */
typedef struct {
    int64_t n_rows, n_cols, nnz;
    int32_t *row_ptr;
    int32_t *col_idx;
    double *val;
    int32_t src_fp32;         /* 1: the file held float32 values */
} dbd_csr_host;

/* Reads <path>.dcsr (FP64 layout of this library) or <path>.csr (the
 * reference layout: int32 nr, nc, ne; int32 ptr[nr+1]; int32 idx[ne];
 * float32 val[ne]); if neither exists, converts the Matrix Market / .dat file
 * at <path> the way the reference does and caches it as <path>.csr.
 * Replaces read_CSR / make_CSR (ZIP:dbd/src/readInput.cpp:18-176). */
int dbd_read_csr(const char *path, dbd_csr_host *out);
/* dbd_read_csr with the Matrix Market / .dat conversion done on GPU `device`
 * (the text is parsed, its entries stably sorted by row and the CSR built
 * there): the same CSR and the same <path>.csr cache, byte for byte, as the
 * host conversion.  dbd_spgemm_files converts on its context's GPU. */
int dbd_read_csr_gpu(const char *path, int device, dbd_csr_host *out);
void dbd_csr_host_free(dbd_csr_host *m);

/* Writes <path> in the reference .csr layout (fp64 = 0, values rounded to
 * float32) or the .dcsr FP64 layout (fp64 = 1).
 * Replaces the cache write of make_CSR (readInput.cpp:166-175). */
int dbd_write_csr(const char *path, const dbd_csr_view *m, int fp64);

/* ---- the reference's stage functions ------------------------------------ */

/* Uploads A (resp. B) to the device; device views are used in place.
 * Replaces initialize_A / initialize_B (preProc.cu:28-46). */
int dbd_load_a(dbd_ctx *ctx, const dbd_csr_view *a);
int dbd_load_b(dbd_ctx *ctx, const dbd_csr_view *b);

/* Work estimate, row-block segmentation and categorisation of the loaded
 * A*B.  Returns the number of row blocks in *num_blocks.
 * Replaces divide_Blocks + get_UpperBound (main.cpp:259-310,
 * preProc.cu:142-156). */
int dbd_divide_blocks(dbd_ctx *ctx, int64_t *num_blocks);

/* Per-block products (block_Info, main.cpp:279) and category
 * (analyze_Block, distributeWorkload.cpp:266-270) of the last
 * dbd_divide_blocks; arrays of num_blocks entries (either may be NULL). */
int dbd_block_info(const dbd_ctx *ctx, int64_t *products, int32_t *category);

/* Runs the multiply over all row blocks in the given scope: the device
 * result (KERNEL), plus the complete C in pinned host memory (D2H), plus
 * Ptr.output / Idx.output / Val.output in out_dir (IO).
 * Replaces distribute_Workload + compute_GPU + write_File + write_Ptr
 * (distributeWorkload.cpp:25-223, computeGPU.cu:15-98,
 * writeFile.cpp:13-196). */
int dbd_distribute_workload(dbd_ctx *ctx, dbd_scope scope, const char *out_dir);

/* The product of the last dbd_distribute_workload: device arrays for KERNEL,
 * pinned host arrays for D2H when C fit the host budget.  Owned by the
 * context (valid until its next multiply). */
int dbd_result(dbd_ctx *ctx, dbd_csr_out *c);

/* Copies the product of the last multiply (device- or host-resident) into
 * caller-provided arrays, host or device memory, sized from dbd_result:
 * row_ptr n_rows+1, col_idx and val nnz entries; any of them may be NULL.
 * Float32 values (dbd_csr_out.val_fp32) are widened exactly into a host val
 * (DBD_ERR_INVALID for a device val: copy them from dbd_result instead).
 * For FFI callers that cannot read the context's memory; the reference hands
 * results back only through Ptr/Idx/Val.output.  With col_idx and val both
 * NULL, row_ptr is copied after any multiply, including one whose C was
 * streamed out in chunks (the row pointers stay on the device). */
int dbd_result_copy(dbd_ctx *ctx, int64_t *row_ptr, int32_t *col_idx, double *val);

int dbd_get_stats(const dbd_ctx *ctx, dbd_stats *st);

/* ---- one-shot entry points ----------------------------------------------- */

/* C = A*B: load, divide, distribute, and (c != NULL) hand back the product:
 * for DBD_SCOPE_KERNEL a device view owned by the context, for D2H/IO a host
 * copy the caller frees with dbd_csr_free() (when C fits host memory). */
int dbd_spgemm(dbd_ctx *ctx, const dbd_csr_view *a, const dbd_csr_view *b,
               dbd_scope scope, const char *out_dir, dbd_csr_out *c, dbd_stats *st);

/* The argv-equivalent of bin/SSpMM | compute | d2h: path_b may be NULL for
 * A*A (main.cpp:152-176). */
int dbd_spgemm_files(dbd_ctx *ctx, const char *path_a, const char *path_b,
                     dbd_scope scope, const char *out_dir, dbd_stats *st);

void dbd_csr_free(dbd_csr_out *c);

/* ---- adjoint (no reference counterpart) ----------------------------------- */

/* Gradients of a scalar loss L(C), C = A*B, with respect to the values of A
 * and B over their fixed patterns:  dA = mask_A(G * B^T),
 * dB = mask_B(A^T * G), where g holds G = dL/dC on C's pattern in the order
 * of the product's col_idx (nnz(C) values).  The reference has no
 * differentiation.  The adjoint is a pair of sampled products: by default one
 * SDDMM-style kernel over A's rows in the forward's numeric row order, or
 * (DBD_ADJ_DETERMINISTIC) that kernel for dA and a second SDDMM over B's
 * pattern for dB.
 *
 * C's pattern is the one the last multiply on this context left on the
 * device (DBD_SCOPE_KERNEL, resident).  flags:
 *   DBD_ADJ_RECOMPUTE      recompute C's pattern from a and b instead, for
 *                          callers that dropped it to save memory;
 *   DBD_ADJ_DETERMINISTIC  dB by a pass of its own over B's pattern (A
 *                          grouped by column on the device, each entry of B
 *                          summed down its column of A in segments of 32
 *                          entries, added in a fixed order): run-to-run
 *                          identical, where the default adds each product
 *                          into dB by an FP64 reduction from A's rows (any
 *                          order; one pass over the products instead of two).
 * dA is summed in a fixed order either way.  on_device = 1: g, da, db are
 * device pointers; 0: host arrays.  da has nnz(A) entries, db nnz(B); both
 * are overwritten. */
#define DBD_ADJ_RECOMPUTE 1
#define DBD_ADJ_DETERMINISTIC 2
int dbd_spgemm_adjoint(dbd_ctx *ctx, const dbd_csr_view *a, const dbd_csr_view *b, const double *g,
                       double *da, double *db, int on_device, int flags);

/* ---- batched products (no reference counterpart) -------------------------- */

/* C_q = A_q * B_q for q in [0, count) -- hundreds of independent, uneven
 * products in one multiply.  The reference runs one product per process
 * (main.cpp:152-176).  The pairs are
 * placed block-diagonally, diag(A_q) * diag(B_q) = diag(C_q), so that one set
 * of binned kernel launches covers the rows of every pair.
 *
 * a[q], b[q]: host or device views (each its own residency) with FP64 values;
 * b == NULL multiplies every A_q by itself.  Sums over the batch (rows, inner
 * and output columns, entries of A and of B) must stay below 2^31.
 * scope: DBD_SCOPE_KERNEL (C stays on the device) or DBD_SCOPE_D2H.
 *
 * C is returned as one CSR (the same forms as dbd_spgemm's c): pair q owns
 * rows [c_row_off[q], c_row_off[q+1]) and entries [c_nnz_off[q],
 * c_nnz_off[q+1]); its row pointers are global (subtract c_nnz_off[q]) and
 * its column indices are local to C_q (0 .. b[q].n_cols - 1).  c_row_off and
 * c_nnz_off are host arrays of count + 1 entries (either may be NULL).
 * Invalid pairs (row_ptr not spanning [0, nnz] monotonically, a column out of
 * range, mismatched inner dimensions) return DBD_ERR_INVALID before any
 * multiply.  dbd_spgemm_adjoint does not apply to a batched product. */
int dbd_spgemm_batched(dbd_ctx *ctx, int64_t count, const dbd_csr_view *a, const dbd_csr_view *b,
                       dbd_scope scope, int64_t *c_row_off, int64_t *c_nnz_off, dbd_csr_out *c,
                       dbd_stats *st);

/* The batched multiply as device work a CUDA graph can hold: no host
 * synchronisation and no allocation once planned.
 *
 * dbd_batch_plan fixes the batch's shapes -- count pairs of device-resident
 * FP64 views (b == NULL: A_q * A_q), each pair's dimensions and entry counts
 * -- and sizes everything for them, C with room for c_capacity entries.  The
 * pairs' arrays must stay where they are; their contents (row pointers,
 * columns, values: the sparsity pattern too) may change between runs as
 * long as every count stays the same.
 *
 * dbd_batch_enqueue puts the whole multiply on `stream` (NULL: the
 * context's): gathering the pairs' current contents, validating them, the
 * per-row analysis, the symbolic bins, C's row pointers, the numeric bins
 * and the pairs' entry offsets.  Every bin is launched device-driven (its
 * rows counted on the device, a grid of resident CTAs striding over them),
 * so nothing is read back: the call can be captured into a CUDA graph
 * (cudaStreamBeginCapture ... cudaStreamEndCapture) and the graph replayed.
 *
 * dbd_batch_result, once the stream's work has completed, returns the
 * status of the last run: DBD_ERR_INVALID for a malformed pair (the run then
 * computed an empty product), DBD_ERR_BUDGET when nnz(C) exceeded
 * c_capacity (no values were written), DBD_ERR_CUDA for a device table
 * overflow; else C (device arrays owned by the context, as dbd_spgemm_batched
 * returns them) and the pairs' row and entry offsets (host arrays of
 * count + 1, either may be NULL). */
int dbd_batch_plan(dbd_ctx *ctx, int64_t count, const dbd_csr_view *a, const dbd_csr_view *b, int64_t c_capacity);
int dbd_batch_enqueue(dbd_ctx *ctx, void *stream);
int dbd_batch_result(dbd_ctx *ctx, int64_t *c_row_off, int64_t *c_nnz_off, dbd_csr_out *c);

/* ---- tuning (no reference counterpart) ------------------------------------ */

/* Row-bin thresholds of the categoriser: which kernel (and so which table
 * size and how many threads) each row of C gets.  The reference fixes its
 * block categories at compile time (distributeWorkload.cpp:249-270); these
 * are runtime knobs, each capped by the size of the tables it selects:
 *   warp_span_words        rows whose column window spans at most this many
 *                          32-column words use the one-warp bitmap kernels (1..64)
 *   warp_max_nnz           numeric rows with at most this many entries stay
 *                          on one warp (1..256)
 *   sym_warp_max_products  symbolic rows with at most this many products use a
 *                          one-warp hash table (32..512)
 *   rank_words_max         CTA rank kernels take windows up to this many words;
 *                          wider rows use CTA hash tables or dense windows (1..8192)
 *   rank_shared_max_nnz    rank rows up to this size accumulate in shared
 *                          memory, larger ones in place in C (1..4096)
 *   sym_hash_span_words    symbolic rows with at most 4096 products hash
 *                          (instead of a bitmap) above this span (>= 0)
 *   dense_warp_span_words  numeric rows whose window spans at most this many
 *                          words accumulate in one warp's dense window (0..16)
 *   mid_span_words         numeric rows of at most warp_max_nnz entries whose
 *                          window spans at most this many words use one warp's
 *                          rank window instead of a hash table (0..2048)
 *   dense_method           rows of the dense bin: 0 rank windows of 2^19 columns in
 *                          shared memory, 1 rank over the whole row in global slots,
 *                          2 FP64 windows of 8192 columns swept by cursors, 3 one pass
 *                          per 2^19-column window into an FP64 scratch row per SM */
typedef struct {
    int32_t warp_span_words;
    int32_t warp_max_nnz;
    int32_t sym_warp_max_products;
    int32_t rank_words_max;
    int32_t rank_shared_max_nnz;
    int32_t sym_hash_span_words;
    int32_t dense_warp_span_words;
    int32_t mid_span_words;
    int32_t dense_method;
} dbd_tuning;

int dbd_get_tuning(const dbd_ctx *ctx, dbd_tuning *t);
/* Values outside the ranges above return DBD_ERR_INVALID. */
int dbd_set_tuning(dbd_ctx *ctx, const dbd_tuning *t);

/* Autotuner: times the multiply of the operands currently loaded on the
 * context (after dbd_load_a/b, dbd_spgemm or dbd_spgemm_batched) in the
 * kernel scope under candidate thresholds, one knob at a time (coordinate
 * descent, best of `repeats` runs per candidate), and keeps the fastest
 * setting on the context.  *best and *best_ms (either may be NULL) receive it
 * and its time.  The context's product afterwards is that of the last trial
 * (the same C as any other setting gives). */
int dbd_autotune(dbd_ctx *ctx, int repeats, dbd_tuning *best, double *best_ms);

/* ---- new values on the same patterns (no reference counterpart) ----------- */

/* Recomputes C's values for new values of A and B on the patterns of the last
 * multiply on this context, which must have run in DBD_SCOPE_KERNEL with C
 * resident (dbd_spgemm or dbd_spgemm_batched).  Only the numeric kernels run:
 * the first call captures them (every bin, across the bin streams) into a
 * CUDA graph, later calls copy the values and replay it with one launch.  C's
 * structure and the plan stay as they were; C's values are overwritten in
 * place (dbd_result gives them).
 *
 * count: 1 after dbd_spgemm, the pair count after dbd_spgemm_batched.
 * a_val[q]: nnz(A_q) values in A_q's entry order; b_val[q] likewise for B_q
 * (b_val is ignored when the last multiply squared A).  on_device: the value
 * arrays are device (1) or host (0) memory.  Device operands of the last
 * multiply must still hold their row pointers and column indices.  A new
 * multiply, dbd_load_a/b or dbd_spgemm_adjoint's reload drops the graph. */
int dbd_update_values(dbd_ctx *ctx, int64_t count, const double *const *a_val, const double *const *b_val,
                      int on_device);

/* ---- output digest (no reference counterpart) ----------------------------- */

/* Per-row digest of C, for checking a product that is never whole in any
 * memory (out-of-core: the device slot and the host ring are recycled chunk
 * by chunk; the reference checks nothing).  With DBD_DIGEST_DEVICE set, every
 * multiply summarises each row of C on the device right after its chunk's
 * numeric kernels; with DBD_DIGEST_HOST set, the D2H and IO scopes summarise
 * each row again from its pinned host copy (a host thread takes every chunk
 * before its ring slot is reused).  Per row r:
 *   count[r]     entries
 *   col_hash[r]  sum of mix64(col) over the row's entries, mod 2^64
 *   val_hash[r]  sum of mix64(bits(val) + G * (col + 1)), mod 2^64,
 *                G = 0x9E3779B97F4A7C15
 *   sum[r]       sum of the values (compensated summation)
 *   wsum[r]      sum of val * w(col), w(col) = 0.5 + (mix64(col) >> 11) * 2^-53
 * where mix64 is SplitMix64's output function.  The hashes do not depend on
 * entry order, so two digests of the same C agree bit for bit; sum and wsum
 * equal A*(B*1) and A*(B*w) up to rounding.  *bad_rows counts rows whose
 * columns are not strictly ascending or fall outside [0, n_cols).  Off by
 * default; the digest costs one read of C per multiply (device) and host
 * threads at the copy rate (host). */
#define DBD_DIGEST_DEVICE 1
#define DBD_DIGEST_HOST   2
int dbd_set_digest(dbd_ctx *ctx, int flags);

/* Copies the digest of the last multiply (which = DBD_DIGEST_DEVICE or
 * DBD_DIGEST_HOST) into host arrays of n_rows entries (any may be NULL). */
int dbd_digest_copy(dbd_ctx *ctx, int which, int64_t *count, uint64_t *col_hash, uint64_t *val_hash,
                    double *sum, double *wsum, int64_t *bad_rows);

/* ---- output writer ------------------------------------------------------- */

/* The writer of the +I/O scope on the caller's own chunks: Idx.output and
 * Val.output appended in row order, Ptr.output at the end.  Replaces
 * write_File / flush_Buffer / write_Ptr (ZIP:dbd/src/writeFile.cpp:13-196;
 * the coalescing variant writeFile_binding.cpp:60-160).  dbd_spgemm's IO
 * scope drives the same writer from its pinned host ring without copies.
 *
 * By default every write is 4 KiB-aligned O_DIRECT (the page cache is
 * bypassed, so the data reaches the device as it is written and the final
 * fsync is short); filesystems that refuse O_DIRECT get page-cache writes
 * (dbd_writer_is_direct tells which).  DBD_WRITER_RESUME keeps a progress
 * manifest (DBD.progress in out_dir): after every append the data is
 * fdatasync'ed and the manifest records the rows written; opening the same
 * product again (same n_rows, nnz, fingerprint and flags, files still
 * holding the recorded bytes) continues there, and *resume_row receives the
 * first row still to be appended (0 otherwise).  A resumed caller appends
 * from that row on.  rotate_gib > 0 wraps the two data files at that total
 * size (disks smaller than C; not with DBD_WRITER_RESUME).  Errors
 * (ENOSPC, EIO, a short write off the 4 KiB grid) return DBD_ERR_IO with the
 * message in dbd_writer_error(). */
typedef struct dbd_writer dbd_writer;
#define DBD_WRITER_BUFFERED 1   /* page-cache writes instead of O_DIRECT */
#define DBD_WRITER_VAL_FP32 2   /* Val.output as float32 (the reference layout) */
#define DBD_WRITER_PTR32    4   /* Ptr.output as int32 (the reference layout; fails if nnz >= 2^31) */
#define DBD_WRITER_RESUME   8   /* progress manifest; reopening continues after the last durable row */
int dbd_writer_open(const char *out_dir, int64_t n_rows, int64_t nnz, uint64_t fingerprint, int flags,
                    double rotate_gib, dbd_writer **w, int64_t *resume_row);
/* Appends the n entries of the next rows, which end at row row_end. */
int dbd_writer_append(dbd_writer *w, int64_t row_end, const int32_t *col_idx, const double *val, int64_t n);
/* Writes Ptr.output (n_rows + 1 row pointers), makes all three files
 * durable (*t_fsync: seconds in fsync) and removes the manifest. */
int dbd_writer_finish(dbd_writer *w, const int64_t *row_ptr, double *t_fsync);
int dbd_writer_is_direct(const dbd_writer *w);
const char *dbd_writer_error(const dbd_writer *w);
void dbd_writer_close(dbd_writer *w);

/* ---- allocation-free multiply --------------------------------------------- */

/* Bytes of device scratch that dbd_spgemm_noalloc owns per GPU. */
#define DBD_NOALLOC_SCRATCH_BYTES (32u << 20)

/* C = A*B (b == NULL: A*A) without allocating anything, for callers that
 * cannot allocate device memory -- code running inside a caching allocator's
 * hooks or a framework that forbids allocation outside its own pool, loops
 * that cannot afford cudaMalloc/cudaFree's implicit device synchronisation,
 * processes that reserved all device memory up front.  No counterpart in the
 * reference (which cudaMallocs per run, preProc.cu:29-106).
 *
 * a, b: device-resident CSR (on_device = 1) with FP64 values.  The caller
 * passes the outputs in device memory: c_row_ptr (n_rows + 1 int64) and
 * c_col_idx / c_val with room for c_capacity entries.  *c_nnz receives
 * nnz(C); when it exceeds c_capacity the call returns DBD_ERR_BUDGET with
 * c_row_ptr filled, so the caller can size its buffers and call again.
 * Work runs on `stream` (a cudaStream_t; NULL = the legacy default stream)
 * and the call returns when it is complete.
 *
 * Every temporary array lives in one file-scope device array of
 * DBD_NOALLOC_SCRATCH_BYTES (32 MiB), which each GPU that loads the library
 * holds until the process exits.  Inputs whose scratch would exceed it --
 * about 31 bytes per row of A, 8 per row of B and 8 per entry of A, so a
 * square A with 2 entries per row fits up to about 610k rows (31 + 8 + 16 =
 * 55 bytes per row) -- are rejected with DBD_ERR_BUDGET.  The first call on a
 * device sets that device up (its kernel attributes, the loading of every
 * kernel the pipeline launches, and the array's device address), so make the
 * first call on each device before reserving the device's memory.
 * The call reads bin sizes and nnz(C) back to the host, so it cannot be
 * captured into a CUDA graph: on a capturing stream it returns
 * DBD_ERR_INVALID before enqueueing anything (dbd_batch_plan /
 * dbd_batch_enqueue is the capturable form).
 * All calls share the array: calls that overlap on the GPU (other threads or
 * streams) race and must be serialised by the caller.  On failure the
 * message is printed to stderr. */
int dbd_spgemm_noalloc(const dbd_csr_view *a, const dbd_csr_view *b, int64_t *c_row_ptr,
                       int32_t *c_col_idx, double *c_val, int64_t c_capacity, int64_t *c_nnz,
                       void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DBD_H */
