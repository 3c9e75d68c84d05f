/*
 * oracle.c -- CPU restatement of DBD's SpGEMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libdbd, the CLI
 * binaries, the Python host package) links, loads or calls this file.  It is
 * used by tests/ as the checker, by __graft_entry__.smoke() to check one small
 * GPU result, and by bench.py's cpu_baseline / --impl reference legs as the
 * timed CPU implementation of the reference's algorithm.
 *
 * Parity pin: the FP32 restatement of the reference's CPU worker
 * (orc_ref_cpu_rows) is checked bit-for-bit against the reference's own
 * computeCPU.cpp compiled from its sources (oracle/build_ref.py ->
 * oracle/_ref/libdbdref.so), and the FP64 oracle of record is checked against
 * the reference's known-answer vectors (bhsparse/main.cu:182-279) and against
 * the canonicalised reference output on quirk-inert inputs (tests/golden).
 *
 * Arithmetic convention of the FP64 oracle (what "exact" means in the tests):
 * every product is rounded to double (p = fl(a*b), no fused multiply-add),
 * and every column accumulator starts at 0.0 and adds the products of its
 * column in Gustavson order (A's row entries in storage order, then B's row
 * entries in storage order).  Build with -ffp-contract=off so that no
 * compiler contracts a*b+c into an FMA on either x86-64 or aarch64.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Work estimate ("upper bound").                                            */
/* ------------------------------------------------------------------------ */

/* Products per row of A: rowP[r] = sum over k in A[r] of |B[k]|.
 * Follows calculate_UpperBound (dbd/for_small_datasets/src/preProc.cu:170-179),
 * which accumulates ptrB[k+1]-ptrB[k] per A entry with atomicAdd.  Deviation:
 * int64 counts (the reference's int32 d_Upp wraps for 5.5e10 products).
 * Returns the total number of products. */
int64_t orc_row_products(int64_t m, const int32_t *Ap, const int32_t *Ai,
                         const int32_t *Bp, int64_t *rowP)
{
    int64_t total = 0;
    for (int64_t r = 0; r < m; ++r) {
        int64_t s = 0;
        for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
            int32_t k = Ai[e];
            s += (int64_t)Bp[k + 1] - Bp[k];
        }
        rowP[r] = s;
        total += s;
    }
    return total;
}

/* Exclusive scan, out[0] = 0, out[n] = total.
 * Follows get_UpperBound's host scan (preProc.cu:149-154).  Deviation: the
 * reference copies only n of the n+1 entries back to the device (:155), so
 * d_Upp[n] stays 0 on the GPU; here all n+1 are produced. */
void orc_exclusive_scan_i64(int64_t n, const int64_t *in, int64_t *out)
{
    int64_t s = 0;
    for (int64_t i = 0; i < n; ++i) { out[i] = s; s += in[i]; }
    out[n] = s;
}

/* Fixed row blocks of rows_per_block rows (the last one may be short).
 * Follows divide_Blocks (ZIP:dbd/src/main.cpp:259-310): block_ptr[b] is the
 * first row of block b, block_info[b] the products in block b, *max_block the
 * largest block_info.  Returns the number of blocks. */
int64_t orc_divide_blocks(int64_t m, const int64_t *upp, int64_t rows_per_block,
                          int64_t *block_ptr, int64_t *block_info, int64_t *max_block)
{
    int64_t nb = m > 0 ? (m - 1) / rows_per_block + 1 : 0;
    int64_t mx = 0;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t r0 = b * rows_per_block;
        int64_t r1 = r0 + rows_per_block < m ? r0 + rows_per_block : m;
        block_ptr[b] = r0;
        block_info[b] = upp[r1] - upp[r0];
        if (block_info[b] > mx) mx = block_info[b];
    }
    block_ptr[nb] = m;
    *max_block = mx;
    return nb;
}

/* Categoriser threshold: int(1.28 * sigma) + avg over per-block average
 * products per row.  Follows calculate_Criteria
 * (ZIP:dbd/src/distributeWorkload.cpp:249-264): avg is
 * (neC / num_Blocks) / ROWS_IN_BLOCK in integer arithmetic, each block's
 * average is block_Info / ROWS_IN_BLOCK (integer division), sigma is the
 * float population standard deviation.  Deviation: the squared difference is
 * formed in int64 (the reference's int product overflows once a block
 * averages more than ~46k products per row). */
int32_t orc_criteria(int64_t nblocks, const int64_t *block_info,
                     int64_t rows_per_block, int64_t neC)
{
    if (nblocks <= 0) return 0;
    int64_t avg = (neC / nblocks) / rows_per_block;
    float var = 0.0f;
    for (int64_t b = 0; b < nblocks; ++b) {
        int64_t d = avg - block_info[b] / rows_per_block;
        var += (float)(d * d);
    }
    var /= (float)nblocks;
    float sd = sqrtf(var);
    return (int32_t)(1.28f * sd) + (int32_t)avg;
}

/* Block category: 0 = dense (GPU-only in the reference), 1 = light
 * (<= 64 products per row, CPU-preferred), 2 = either.  Follows analyze_Block
 * (ZIP:dbd/src/distributeWorkload.cpp:266-270). */
int32_t orc_analyze_block(int32_t criteria, int64_t avg_products_per_row)
{
    if (avg_products_per_row > criteria) return 0;
    if (avg_products_per_row <= 64) return 1;
    return 2;
}

/* Threads per A row chosen from the block's total products: <=128 -> 64,
 * <=512 -> 256, else 1024.  Follows analyze_Block
 * (dbd/for_small_datasets/src/computeGPU.cu:9-13). */
int32_t orc_threads_per_row(int64_t block_products)
{
    if (block_products <= 128) return 64;
    if (block_products <= 512) return 256;
    return 1024;
}

/* ------------------------------------------------------------------------ */
/* FP64 Gustavson oracle of record (sorted, duplicate-free, index-determined) */
/* ------------------------------------------------------------------------ */

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* Symbolic phase: Cp[r+1]-Cp[r] = number of distinct columns reached by row
 * r's products.  Structure is decided by index only: a column belongs to C's
 * row as soon as one product lands on it, whatever the value (the reference
 * decides by value, |partial sum| < 1e-4 at computeCPU.cpp:48 and
 * computeGPU.cu:312; that quirk is restated separately below).
 * Cp has m+1 entries; returns nnz(C). */
int64_t orc_spgemm_symbolic(int64_t m, int64_t ncols,
                            const int32_t *Ap, const int32_t *Ai,
                            const int32_t *Bp, const int32_t *Bi,
                            int64_t *Cp)
{
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    #pragma omp parallel
    {
        int32_t *mark = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ncols > 0 ? ncols : 1));
        for (int64_t c = 0; c < ncols; ++c) mark[c] = -1;
        #pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < m; ++r) {
            int64_t nz = 0;
            for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
                int32_t k = Ai[e];
                for (int64_t f = Bp[k]; f < Bp[k + 1]; ++f) {
                    int32_t c = Bi[f];
                    if (mark[c] != (int32_t)r) { mark[c] = (int32_t)r; ++nz; }
                }
            }
            cnt[r] = nz;
        }
        free(mark);
    }
    orc_exclusive_scan_i64(m, cnt, Cp);
    free(cnt);
    return Cp[m];
}

/* Numeric phase into the structure made by orc_spgemm_symbolic: columns of
 * each row ascending, values accumulated in Gustavson order with fl(a*b)
 * products.  Follows the arithmetic of compute_CPU
 * (ZIP:dbd/src/computeCPU.cpp:43-59) in FP64 without the value-based
 * first-touch test.  Cabs (nullable) receives sum |a*b| per entry, the scale
 * used by the tolerance |c - oracle| <= tol * sum|a*b|. */
void orc_spgemm_numeric(int64_t m, int64_t ncols,
                        const int32_t *Ap, const int32_t *Ai, const double *Av,
                        const int32_t *Bp, const int32_t *Bi, const double *Bv,
                        const int64_t *Cp, int32_t *Ci, double *Cv, double *Cabs)
{
    #pragma omp parallel
    {
        double *acc = (double *)calloc((size_t)(ncols > 0 ? ncols : 1), sizeof(double));
        double *aab = Cabs ? (double *)calloc((size_t)(ncols > 0 ? ncols : 1), sizeof(double)) : NULL;
        int32_t *mark = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ncols > 0 ? ncols : 1));
        for (int64_t c = 0; c < ncols; ++c) mark[c] = -1;
        #pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < m; ++r) {
            int64_t base = Cp[r], nz = 0;
            for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
                int32_t k = Ai[e];
                double a = Av[e];
                for (int64_t f = Bp[k]; f < Bp[k + 1]; ++f) {
                    int32_t c = Bi[f];
                    double p = a * Bv[f];
                    if (mark[c] != (int32_t)r) {
                        mark[c] = (int32_t)r;
                        Ci[base + nz++] = c;
                        acc[c] = 0.0;
                        if (aab) aab[c] = 0.0;
                    }
                    acc[c] = acc[c] + p;
                    if (aab) aab[c] = aab[c] + fabs(p);
                }
            }
            qsort(Ci + base, (size_t)nz, sizeof(int32_t), cmp_i32);
            for (int64_t j = 0; j < nz; ++j) {
                int32_t c = Ci[base + j];
                Cv[base + j] = acc[c];
                if (Cabs) Cabs[base + j] = aab[c];
            }
        }
        free(acc); free(aab); free(mark);
    }
}

/* ------------------------------------------------------------------------ */
/* Restatement of the reference's CPU worker (FP32, value-based structure)   */
/* ------------------------------------------------------------------------ */

/* Row-by-row FP32 dense-accumulator Gustavson exactly as compute_CPU
 * (ZIP:dbd/src/computeCPU.cpp:32-62) computes it: a column is appended to the
 * row's list whenever its running float sum lies strictly inside
 * (-0.0001, 0.0001) before the product is added (:48-50), so exact
 * cancellation or tiny values produce duplicate entries; values are gathered
 * in list order and the accumulator reset (:55-59), so a duplicate reads 0.
 * Output of row r is written at slot offset slot_off[r] - slot_off[row0] like
 * h_IdxC/h_ValC (:38-40), with its count in rowcnt[r].  slot_off is the
 * exclusive scan of products (h_Upp).  Rows are independent, so the result
 * does not depend on nthreads (the reference uses 8 OpenMP threads,
 * SSpMM.hpp CPU_DENSE). */
void orc_ref_cpu_rows(int64_t row0, int64_t row1, int64_t ncols,
                      const int32_t *Ap, const int32_t *Ai, const float *Av,
                      const int32_t *Bp, const int32_t *Bi, const float *Bv,
                      const int64_t *slot_off, int32_t *rowcnt,
                      int32_t *idx_slots, float *val_slots, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    #pragma omp parallel num_threads(nthreads)
    {
        float *sub = (float *)calloc((size_t)(ncols > 0 ? ncols : 1), sizeof(float));
        #pragma omp for schedule(dynamic, 1)
        for (int64_t r = row0; r < row1; ++r) {
            int64_t base = slot_off[r] - slot_off[row0];
            int32_t *ic = idx_slots + base;
            float *vc = val_slots + base;
            int32_t nz = 0;
            for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
                float a = Av[e];
                int32_t k = Ai[e];
                for (int64_t f = Bp[k]; f < Bp[k + 1]; ++f) {
                    int32_t c = Bi[f];
                    if ((double)sub[c] < 0.0001 && (double)sub[c] > -0.0001) ic[nz++] = c;
                    float p = a * Bv[f];
                    sub[c] = sub[c] + p;
                }
            }
            for (int32_t j = 0; j < nz; ++j) {
                int32_t c = ic[j];
                vc[j] = sub[c];
                sub[c] = 0.0f;
            }
            rowcnt[r] = nz;
        }
        free(sub);
    }
}

/* ------------------------------------------------------------------------ */
/* Adjoint of C = A*B over fixed patterns (no reference counterpart)         */
/* ------------------------------------------------------------------------ */

/* Position of column c in C's sorted row r, or -1. */
static int64_t find_col(const int64_t *Cp, const int32_t *Ci, int64_t r, int32_t c)
{
    int64_t lo = Cp[r], hi = Cp[r + 1];
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (Ci[mid] < c) lo = mid + 1; else hi = mid;
    }
    return (lo < Cp[r + 1] && Ci[lo] == c) ? lo : -1;
}

/* Given G = dL/dC on C's pattern (Cp, Ci sorted), computes
 *   dA[e] for e=(i,j) in A:  sum over (j,k) in B of G(i,k) * B(j,k)
 *   dB[f] for f=(j,k) in B:  sum over (i,j) in A of A(i,j) * G(i,k)
 * i.e. dA = mask_A(G * B^T), dB = mask_B(A^T * G), sequentially in FP64
 * with fl() products and storage-order accumulation. */
void orc_adjoint(int64_t m,
                 const int32_t *Ap, const int32_t *Ai, const double *Av,
                 const int32_t *Bp, const int32_t *Bi, const double *Bv,
                 int64_t nnzB,
                 const int64_t *Cp, const int32_t *Ci, const double *G,
                 double *dA, double *dB)
{
    for (int64_t f = 0; f < nnzB; ++f) dB[f] = 0.0;
    for (int64_t i = 0; i < m; ++i) {
        for (int64_t e = Ap[i]; e < Ap[i + 1]; ++e) {
            int32_t j = Ai[e];
            double s = 0.0;
            for (int64_t f = Bp[j]; f < Bp[j + 1]; ++f) {
                int64_t q = find_col(Cp, Ci, i, Bi[f]);
                double g = q >= 0 ? G[q] : 0.0;
                double p = g * Bv[f];
                s = s + p;
                double t = Av[e] * g;
                dB[f] = dB[f] + t;
            }
            dA[e] = s;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Digest of C without forming C (checks of out-of-core products)           */
/* ------------------------------------------------------------------------ */

/* SplitMix64's output function (Steele, Lea and Flood, OOPSLA 2014): the
 * column hash of the library's per-row digest of C. */
static uint64_t orc_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Column weight w(c) = 0.5 + (mix64(c) >> 11) * 2^-53, in [0.5, 1.5). */
double orc_col_weight(int32_t c)
{
    return 0.5 + (double)(orc_mix64((uint64_t)(uint32_t)c) >> 11) * 0x1.0p-53;
}

/* Per row r in [r0, r1) of A*B: cnt[r - r0] = distinct columns its products
 * reach (nnz of C's row in the index-determined structure of
 * orc_spgemm_symbolic) and hash[r - r0] = sum of mix64(col) over those
 * columns, mod 2^64 -- the count and column hash of the library's digest,
 * without forming or sorting C.  O(products) with one marker array per
 * thread. */
void orc_row_col_digest(int64_t r0, int64_t r1, int64_t ncols,
                        const int32_t *Ap, const int32_t *Ai,
                        const int32_t *Bp, const int32_t *Bi,
                        int64_t *cnt, uint64_t *hash)
{
    #pragma omp parallel
    {
        int64_t *mark = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncols > 0 ? ncols : 1));
        for (int64_t c = 0; c < ncols; ++c) mark[c] = -1;
        #pragma omp for schedule(dynamic, 16)
        for (int64_t r = r0; r < r1; ++r) {
            int64_t nz = 0;
            uint64_t h = 0;
            for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
                int32_t k = Ai[e];
                for (int64_t f = Bp[k]; f < Bp[k + 1]; ++f) {
                    int32_t c = Bi[f];
                    if (mark[c] != r) {
                        mark[c] = r;
                        ++nz;
                        h += orc_mix64((uint64_t)(uint32_t)c);
                    }
                }
            }
            cnt[r - r0] = nz;
            hash[r - r0] = h;
        }
        free(mark);
    }
}

/* Neumaier's compensated summation. */
static void orc_neumaier(double *s, double *c, double x)
{
    double t = *s + x;
    if (fabs(*s) >= fabs(x)) *c += (*s - t) + x;
    else *c += (x - t) + *s;
    *s = t;
}

/* Row sums of C = A*B weighted by column, without forming C:
 *   y = B * w (w = 1 when weighted == 0, else w(c) = orc_col_weight(c)),
 *   out[r] = (A * y)[r],  out_abs[r] = (|A| * (|B| * w))[r],
 * each dot product by compensated summation, so its error stays within a
 * few units of the last place of out_abs.  These are the library digest's
 * sum (weighted == 0) and wsum (weighted == 1) up to C's own rounding. */
void orc_row_sums(int64_t m, const int32_t *Ap, const int32_t *Ai, const double *Av,
                  int64_t mb, const int32_t *Bp, const int32_t *Bi, const double *Bv,
                  int weighted, double *out, double *out_abs)
{
    double *y = (double *)malloc(sizeof(double) * (size_t)(mb > 0 ? mb : 1));
    double *ya = (double *)malloc(sizeof(double) * (size_t)(mb > 0 ? mb : 1));
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t k = 0; k < mb; ++k) {
        double s = 0, c = 0, sa = 0, ca = 0;
        for (int64_t f = Bp[k]; f < Bp[k + 1]; ++f) {
            double w = weighted ? orc_col_weight(Bi[f]) : 1.0;
            double p = Bv[f] * w;
            orc_neumaier(&s, &c, p);
            orc_neumaier(&sa, &ca, fabs(p));
        }
        y[k] = s + c;
        ya[k] = sa + ca;
    }
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < m; ++r) {
        double s = 0, c = 0, sa = 0, ca = 0;
        for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
            int32_t k = Ai[e];
            orc_neumaier(&s, &c, Av[e] * y[k]);
            orc_neumaier(&sa, &ca, fabs(Av[e]) * ya[k]);
        }
        out[r] = s + c;
        out_abs[r] = sa + ca;
    }
    free(y);
    free(ya);
}
