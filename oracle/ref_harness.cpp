// ref_harness.cpp -- drives the reference's own host code, compiled from its
// sources, so that the oracle's restatement can be pinned against it.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file together
// with the reference's main.cpp, distributeWorkload.cpp, computeCPU.cpp and
// readInput.cpp (DBD_FULL.zip:dbd/src, built with -DCOMPUTE as the
// reference's `compute` target does, ZIP:dbd/Makefile:30-31; main is renamed)
// into oracle/_ref/libdbdref.so.  The reference's GPU translation units cannot
// run without a GPU, so the few functions of preProc.cu / computeGPU.cu that
// the host files call are stubbed here; get_UpperBound's stub computes h_Upp
// on the CPU (the products per row of calculate_UpperBound,
// preProc.cu:170-179, then the host scan of :149-154).
//
// Entry points:
//   ref_read_csr     -> read_CSR (ZIP:dbd/src/readInput.cpp:18-176)
//   ref_divide       -> divide_Blocks (ZIP:dbd/src/main.cpp:259-310)
//   ref_criteria     -> calculate_Criteria (ZIP:dbd/src/distributeWorkload.cpp:249-264)
//   ref_cpu_spgemm   -> compute_CPU (ZIP:dbd/src/computeCPU.cpp:10-98) over all
//                       row blocks, driven through the reference's own
//                       threadArgs flag protocol (SSpMM.hpp:53-59)
//   ref_cpu_blocks   -> the same worker block by block, each block's output
//                       canonicalised and handed to a callback (products too
//                       large to hold whole)
#include "SSpMM.hpp"

#include <algorithm>
#include <vector>

// Defined by the reference's main.cpp / distributeWorkload.cpp (compiled in).
extern long int neC;
extern int *block_Info;

int calculate_Criteria(int);
int divide_Blocks();

// ---- stubs of the GPU-side functions the host files reference ----------
void initialize_GPU() {}
void initialize_A() {}
void initialize_B() {}
int initialize_C(int) { return 0; }
void free_GPU() {}
void *compute_GPU(void *) { return NULL; }
void get_UpperBound() {
    h_Upp = (int *)malloc(sizeof(int) * (A.nr + 1));
    h_Upp[0] = 0;
    for (int r = 0; r < A.nr; ++r) {
        int s = 0;
        for (int e = A.ptr[r]; e < A.ptr[r + 1]; ++e) s += B.ptr[A.idx[e] + 1] - B.ptr[A.idx[e]];
        h_Upp[r + 1] = h_Upp[r] + s;
    }
}

static void flag_store(bool *p, bool v) { __atomic_store_n(p, v, __ATOMIC_SEQ_CST); }
static bool flag_load(bool *p) { return __atomic_load_n(p, __ATOMIC_SEQ_CST); }

static void set_operands(int nrA, int ncA, const int *Ap, const int *Ai, const float *Av, int nrB, int ncB,
                         const int *Bp, const int *Bi, const float *Bv) {
    // compute_CPU sizes its dense rows by A.nc (computeCPU.cpp:41 with
    // main.cpp:232) and indexes them by B's columns; A.nc = B.nc keeps that
    // in bounds for rectangular products.
    (void)ncA;
    A.nr = nrA; A.nc = ncB; A.ne = Ap[nrA];
    A.ptr = const_cast<int *>(Ap); A.idx = const_cast<int *>(Ai); A.val = const_cast<float *>(Av);
    B.nr = nrB; B.nc = ncB; B.ne = Bp[nrB];
    B.ptr = const_cast<int *>(Bp); B.idx = const_cast<int *>(Bi); B.val = const_cast<float *>(Bv);
}

extern "C" int ref_read_csr(const char *path, int *nr, int *nc, int *ne, int **ptr, int **idx, float **val) {
    csr m;
    memset(&m, 0, sizeof(m));
    read_CSR(std::string(path), &m);
    *nr = m.nr; *nc = m.nc; *ne = m.ne;
    *ptr = m.ptr; *idx = m.idx; *val = m.val;
    return 0;
}

extern "C" void ref_free(void *p) { free(p); }

extern "C" int ref_rows_in_block(void) { return ROWS_IN_BLOCK; }

// divide_Blocks on A*B: returns num_Blocks; block_info/block_ptr receive
// num_Blocks (+1) entries, *total the accumulated neC.
extern "C" int ref_divide(int nrA, int ncA, const int *Ap, const int *Ai, int nrB, int ncB, const int *Bp,
                          int *block_info, int *block_ptr, long long *total) {
    std::vector<float> dummyA(Ap[nrA] > 0 ? Ap[nrA] : 1), dummyB(Bp[nrB] > 0 ? Bp[nrB] : 1);
    set_operands(nrA, ncA, Ap, Ai, dummyA.data(), nrB, ncB, Bp, Ai, dummyB.data());
    neC = 0;
    int nb = divide_Blocks();
    if (nb > 0) {
        memcpy(block_info, block_Info, sizeof(int) * nb);
        memcpy(block_ptr, block_Ptr, sizeof(int) * (nb + 1));
    }
    *total = neC;
    free(h_Upp); free(block_Ptr); free(block_Info);
    if (h_IdxC) free(h_IdxC);
    if (h_ValC) free(h_ValC);
    h_Upp = NULL; block_Ptr = NULL; block_Info = NULL; h_IdxC = NULL; h_ValC = NULL;
    return nb;
}

extern "C" int ref_criteria(int num_blocks, const int *block_info, long long total) {
    block_Info = const_cast<int *>(block_info);
    neC = total;
    int c = calculate_Criteria(num_blocks);
    block_Info = NULL;
    return c;
}

// Runs the reference CPU worker over all rows of A*B.  Row r's entries are
// returned at slot offset slot_off[r] (the exclusive scan of products, i.e.
// h_Upp), its count in rowcnt[r].  slot_off has nrA+1 entries.
extern "C" int ref_cpu_spgemm(int nrA, int ncA, const int *Ap, const int *Ai, const float *Av,
                              int nrB, int ncB, const int *Bp, const int *Bi, const float *Bv,
                              long long *slot_off, int *rowcnt, int *idx_slots, float *val_slots)
{
    set_operands(nrA, ncA, Ap, Ai, Av, nrB, ncB, Bp, Bi, Bv);
    get_UpperBound();
    slot_off[0] = 0;
    for (int r = 0; r < nrA; ++r) {
        long long s = 0;
        for (int e = Ap[r]; e < Ap[r + 1]; ++e) s += Bp[Ai[e] + 1] - Bp[Ai[e]];
        slot_off[r + 1] = slot_off[r] + s;
    }
    int nb = (nrA - 1) / ROWS_IN_BLOCK + 1;
    block_Ptr = (int *)malloc(sizeof(int) * (nb + 1));
    long long max_blk = 0;
    for (int b = 0; b < nb; ++b) {
        block_Ptr[b] = b * ROWS_IN_BLOCK;
        int r1 = (b + 1) * ROWS_IN_BLOCK < nrA ? (b + 1) * ROWS_IN_BLOCK : nrA;
        long long p = slot_off[r1] - slot_off[b * ROWS_IN_BLOCK];
        if (p > max_blk) max_blk = p;
    }
    block_Ptr[nb] = nrA;
    h_IdxC = (int *)malloc(sizeof(int) * (max_blk > 0 ? max_blk : 1));
    h_ValC = (float *)malloc(sizeof(float) * (max_blk > 0 ? max_blk : 1));
    cpu_Dense = (float *)calloc((size_t)A.nc * CPU_DENSE, sizeof(float));
    ptrC = (int *)calloc(nrA + 1, sizeof(int));
    cpu_Args = (threadArgs *)malloc(sizeof(threadArgs));
    *cpu_Args = {0, false, true, false};

    pthread_t th;
    pthread_create(&th, NULL, compute_CPU, NULL);
    for (int b = 0; b < nb; ++b) {
        cpu_Args->block_Index = b;
        flag_store(&cpu_Args->working, true);
        while (flag_load(&cpu_Args->working)) usleep(50);
        int r0 = block_Ptr[b], r1 = block_Ptr[b + 1];
        for (int r = r0; r < r1; ++r) {
            int cnt = ptrC[r + 1];
            rowcnt[r] = cnt;
            long long src = (long long)h_Upp[r] - h_Upp[r0];
            memcpy(idx_slots + slot_off[r], h_IdxC + src, sizeof(int) * cnt);
            memcpy(val_slots + slot_off[r], h_ValC + src, sizeof(float) * cnt);
        }
    }
    usleep(2000);
    flag_store(&cpu_Args->finished, true);
    pthread_join(th, NULL);

    free(h_Upp); free(block_Ptr); free(h_IdxC); free(h_ValC);
    free(cpu_Dense); free(ptrC); free(cpu_Args);
    h_Upp = NULL; block_Ptr = NULL; h_IdxC = NULL; h_ValC = NULL;
    cpu_Dense = NULL; ptrC = NULL; cpu_Args = NULL;
    return 0;
}

// Runs the reference CPU worker over A*B in blocks of rows_per_block rows and
// hands each block's output to cb, canonicalised: every row's columns sorted
// (duplicates kept and counted).  Only the largest block's products are held
// at a time, so products with billions of entries can be checked.  h_Upp is
// the reference's int32 exclusive scan of products (get_UpperBound,
// preProc.cu:142-156), wrapping mod 2^32 past 2^31 products as the
// reference's own does; compute_CPU only takes differences of it within a
// block (computeCPU.cpp:38), which are exact while a block holds fewer than
// 2^31 products (checked here).  Returns -2 when a block holds more.
typedef void (*ref_block_cb)(int r0, int r1, const int *cnt, const unsigned long long *hash, const int *idx,
                             long long n, long long dups, void *user);

// SplitMix64's output function: hash[r] = sum of mix64(col) over the row's
// entries (mod 2^64), the column hash of libdbd's per-row digest.
static unsigned long long harness_mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

extern "C" int ref_cpu_blocks(int nrA, int ncA, const int *Ap, const int *Ai, const float *Av,
                              int nrB, int ncB, const int *Bp, const int *Bi, const float *Bv,
                              int rows_per_block, ref_block_cb cb, void *user)
{
    if (nrA <= 0 || rows_per_block <= 0) return -1;
    set_operands(nrA, ncA, Ap, Ai, Av, nrB, ncB, Bp, Bi, Bv);
    std::vector<long long> off((size_t)nrA + 1, 0);
    h_Upp = (int *)malloc(sizeof(int) * (nrA + 1));
    unsigned int wrapped = 0;
    h_Upp[0] = 0;
    for (int r = 0; r < nrA; ++r) {
        long long s = 0;
        for (int e = Ap[r]; e < Ap[r + 1]; ++e) s += Bp[Ai[e] + 1] - Bp[Ai[e]];
        off[r + 1] = off[r] + s;
        wrapped += (unsigned int)s;
        h_Upp[r + 1] = (int)wrapped;
    }
    const int nb = (nrA - 1) / rows_per_block + 1;
    block_Ptr = (int *)malloc(sizeof(int) * (nb + 1));
    long long max_blk = 0;
    for (int b = 0; b <= nb; ++b) block_Ptr[b] = b < nb ? b * rows_per_block : nrA;
    for (int b = 0; b < nb; ++b) {
        const long long p = off[block_Ptr[b + 1]] - off[block_Ptr[b]];
        if (p > max_blk) max_blk = p;
    }
    if (max_blk >= (1ll << 31)) {
        free(h_Upp); free(block_Ptr);
        h_Upp = NULL; block_Ptr = NULL;
        return -2;
    }
    h_IdxC = (int *)malloc(sizeof(int) * (max_blk > 0 ? max_blk : 1));
    h_ValC = (float *)malloc(sizeof(float) * (max_blk > 0 ? max_blk : 1));
    cpu_Dense = (float *)calloc((size_t)A.nc * CPU_DENSE, sizeof(float));
    ptrC = (int *)calloc(nrA + 1, sizeof(int));
    cpu_Args = (threadArgs *)malloc(sizeof(threadArgs));
    *cpu_Args = {0, false, true, false};

    pthread_t th;
    pthread_create(&th, NULL, compute_CPU, NULL);
    std::vector<int> cnt((size_t)rows_per_block);
    std::vector<unsigned long long> hash((size_t)rows_per_block);
    std::vector<int> canon;
    for (int b = 0; b < nb; ++b) {
        cpu_Args->block_Index = b;
        flag_store(&cpu_Args->working, true);
        while (flag_load(&cpu_Args->working)) usleep(50);
        const int r0 = block_Ptr[b], r1 = block_Ptr[b + 1];
        long long n = 0;
        for (int r = r0; r < r1; ++r) n += (cnt[r - r0] = ptrC[r + 1]);
        canon.resize((size_t)(n > 0 ? n : 1));
        long long at = 0, dups = 0;
        for (int r = r0; r < r1; ++r) {
            const int c = cnt[r - r0];
            int *row = canon.data() + at;
            memcpy(row, h_IdxC + (off[r] - off[r0]), sizeof(int) * c);
            std::sort(row, row + c);
            unsigned long long h = 0;
            for (int j = 0; j < c; ++j) {
                h += harness_mix64((unsigned long long)(unsigned int)row[j]);
                if (j) dups += row[j] == row[j - 1];
            }
            hash[r - r0] = h;
            at += c;
        }
        cb(r0, r1, cnt.data(), hash.data(), canon.data(), n, dups, user);
    }
    usleep(2000);
    flag_store(&cpu_Args->finished, true);
    pthread_join(th, NULL);

    free(h_Upp); free(block_Ptr); free(h_IdxC); free(h_ValC);
    free(cpu_Dense); free(ptrC); free(cpu_Args);
    h_Upp = NULL; block_Ptr = NULL; h_IdxC = NULL; h_ValC = NULL;
    cpu_Dense = NULL; ptrC = NULL; cpu_Args = NULL;
    return 0;
}
