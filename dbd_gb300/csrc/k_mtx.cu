// k_mtx.cu -- Matrix Market / .dat text to CSR on the device: the GPU side of
// the reference's input conversion (make_CSR, ZIP:dbd/src/readInput.cpp:48-176,
// with its base-10 LSD radix sort by row, :192-215).
//
// The output equals the host conversion (csr_io.cpp, itself byte-identical to
// make_CSR) byte for byte, quirks included:
//
//  * the text is read as fgets(line, 200) reads it: a line longer than 199
//    characters is taken in pieces of 199, each parsed as a line of its own;
//  * tokens are split on "\t, " (strtok), so '\r' and '\n' stay inside the
//    last token; a piece without tokens is skipped, one with a single token
//    is an error; a missing third token reads as 1.0;
//  * indices are atoi (strtol semantics: leading white space, sign,
//    saturation to the range of long, then truncation to int) and values are
//    (float)atof: the decimal text correctly rounded to double, then rounded
//    to float, so values that round twice come out as the reference's;
//  * "symmetric" in the first line mirrors every off-diagonal entry right
//    after it; entries are stably ordered by row.
//
// Pipeline: the host reads the file and parses the header (first line, the
// comment lines and the size line); the body goes to the device, where
// per-tile newline counts and a scan give every line's start, one thread
// per line counts its entries, a scan gives their positions, the same
// threads write the entries (row, column, float value), the rare values
// that the fast decimal path cannot convert exactly are finished by a
// second kernel with an exact decimal algorithm, and a stable LSD radix sort
// (8 bits per pass, one warp per tile of 2048 keys) orders the entries by
// row.  Row pointers come from the sorted rows directly.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dbd_internal.h"
#include "dbd_io.h"
#include "mtx_parse.h"

namespace dbd {
namespace {

using namespace mtx;

constexpr int kPiece = 199;        // characters fgets(line, 200) returns at most
constexpr int kTextTile = 4096;    // bytes per CTA of the newline passes (256 threads x 16)
constexpr int kSortTile = 2048;    // keys per warp of the radix sort
// ---- lines ---------------------------------------------------------------

__global__ void __launch_bounds__(256) k_nl_count(const char *__restrict__ t, int64_t n, int32_t *__restrict__ cnt) {
    const int64_t i0 = (int64_t)blockIdx.x * kTextTile + threadIdx.x * 16;
    int c = 0;
    for (int j = 0; j < 16; ++j)
        if (i0 + j < n && t[i0 + j] == '\n') ++c;
    c = __reduce_add_sync(0xffffffffu, (unsigned)c);
    __shared__ int sh[8];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < 8; ++w) s += sh[w];
        cnt[blockIdx.x] = s;
    }
}

// starts[1 + k] = one past the k-th newline; starts[0] = 0.
__global__ void __launch_bounds__(256) k_line_starts(const char *__restrict__ t, int64_t n,
                                                     const int64_t *__restrict__ tileOff,
                                                     int64_t *__restrict__ starts) {
    const int64_t i0 = (int64_t)blockIdx.x * kTextTile + threadIdx.x * 16;
    int c = 0;
    for (int j = 0; j < 16; ++j)
        if (i0 + j < n && t[i0 + j] == '\n') ++c;
    // Exclusive scan of the per-thread counts over the CTA.
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = c;
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    __shared__ int sh[8];
    if (lane == 31) sh[w] = x;
    __syncthreads();
    int base = 0;
    for (int k = 0; k < w; ++k) base += sh[k];
    int64_t k = tileOff[blockIdx.x] + base + x - c;
    for (int j = 0; j < 16; ++j)
        if (i0 + j < n && t[i0 + j] == '\n') starts[1 + k++] = i0 + j + 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) starts[0] = 0;
}

struct LineArgs {
    const char *t;        // body text
    int64_t n;            // its bytes
    const int64_t *starts;  // nlines + 1
    int64_t nlines;
    int symmetric;
    int32_t *edgeCnt;     // per line (count pass)
    const int64_t *edgeOff;  // per line (emit pass)
    int32_t *from, *to;
    float *val;
    unsigned long long *slowN;
    int64_t *slowEdge, *slowTok;  // slow values: first edge, token offset << 8 | length
    unsigned long long *badLine;  // set when a piece holds a single token
};

// One line, piece by piece: the edges it holds; EMIT writes them.
template <bool EMIT>
__global__ void __launch_bounds__(256) k_lines(LineArgs a) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= a.nlines) return;
    const int64_t s0 = a.starts[line], s1 = line + 1 < a.nlines ? a.starts[line + 1] : a.n;
    int32_t cnt = 0;
    int slow = 0;
    int64_t out = EMIT ? a.edgeOff[line] : 0;
    for (int64_t ps = s0; ps < s1; ps += kPiece) {
        const char *pb = a.t + ps, *pe = a.t + min(s1, ps + kPiece);
        const char *s = pb, *t1s, *t1e, *t2s, *t2e, *t3s, *t3e;
        if (!next_tok(s, pe, t1s, t1e)) continue;
        if (!next_tok(s, pe, t2s, t2e)) {
            *a.badLine = 1ull;
            return;
        }
        const bool has3 = next_tok(s, pe, t3s, t3e);
        const int32_t from = parse_atoi(t1s, t1e), to = parse_atoi(t2s, t2e);
        const bool mirror = a.symmetric && from != to;
        ValueScan v{1.0f, false};
        if (has3) v = parse_value_fast(t3s, t3e);
        if (EMIT) {
            a.from[out] = from;
            a.to[out] = to;
            a.val[out] = v.v;
            if (mirror) {
                a.from[out + 1] = to;
                a.to[out + 1] = from;
                a.val[out + 1] = v.v;
            }
            if (v.slow) {
                const unsigned long long k = atomicAdd(a.slowN, 1ull);
                a.slowEdge[k] = out | (mirror ? (1ll << 62) : 0);
                a.slowTok[k] = ((int64_t)(t3s - a.t) << 8) | (int64_t)(t3e - t3s);
            }
            out += mirror ? 2 : 1;
        }
        cnt += mirror ? 2 : 1;
        slow += v.slow;
    }
    if (!EMIT) {
        a.edgeCnt[line] = cnt;
        if (slow) atomicAdd(a.slowN, (unsigned long long)slow);
    }
}

__global__ void __launch_bounds__(64) k_slow_values(const char *__restrict__ t, const int64_t *__restrict__ edge,
                                                    const int64_t *__restrict__ tok, int64_t n, float *val) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Decimal a;
    const int64_t off = tok[i] >> 8;
    const int len = (int)(tok[i] & 255);
    const float v = parse_value_exact(t + off, t + off + len, a);
    const int64_t e = edge[i] & ((1ll << 62) - 1);
    val[e] = v;
    if (edge[i] >> 62) val[e + 1] = v;
}

__global__ void __launch_bounds__(256) k_check_edges(const int32_t *__restrict__ from, const int32_t *__restrict__ to,
                                                     int64_t n, int64_t nr, int64_t nc, uint32_t *keys,
                                                     uint32_t *idx, int *bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t f = from[i], c = to[i];
        if (f < 0 || f >= nr || c < 0 || c >= nc) *bad = 1;
        keys[i] = (uint32_t)f;
        idx[i] = (uint32_t)i;
    }
}

// ---- stable LSD radix sort by row (one warp per tile of kSortTile keys) ----

__global__ void __launch_bounds__(32) k_sort_hist(const uint32_t *__restrict__ keys, int64_t n, int shift,
                                                  int32_t *__restrict__ hist, int64_t ntiles) {
    __shared__ int cnt[256];
    const int lane = threadIdx.x;
    for (int d = lane; d < 256; d += 32) cnt[d] = 0;
    __syncwarp();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int j = lane; j < kSortTile; j += 32)
        if (base + j < n) atomicAdd(&cnt[(keys[base + j] >> shift) & 255], 1);
    __syncwarp();
    for (int d = lane; d < 256; d += 32) hist[(int64_t)d * ntiles + blockIdx.x] = cnt[d];
}

__global__ void __launch_bounds__(32) k_sort_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                     uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                     int64_t n, int shift, const int64_t *__restrict__ off,
                                                     int64_t ntiles) {
    __shared__ int64_t pos[256];
    const int lane = threadIdx.x;
    for (int d = lane; d < 256; d += 32) pos[d] = off[(int64_t)d * ntiles + blockIdx.x];
    __syncwarp();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortTile / 32; ++r) {
        const int64_t i = base + r * 32 + lane;
        const bool valid = i < n;
        const uint32_t k = valid ? kin[i] : 0u;
        const int d = valid ? (int)((k >> shift) & 255) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid) {
            const int64_t p = pos[d] + __popc(peers & lt);
            kout[p] = k;
            vout[p] = vin[i];
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) pos[d] += __popc(peers);
        __syncwarp();
    }
}

// CSR from the sorted edges: columns and values gathered, row pointers from
// the sorted rows (row r starts at the first edge of a row >= r).
__global__ void __launch_bounds__(256) k_build_csr(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ perm,
                                                   const int32_t *__restrict__ to, const float *__restrict__ val,
                                                   int64_t n, int64_t nr, int32_t *__restrict__ ptr,
                                                   int32_t *__restrict__ col, float *__restrict__ v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = i == 0 ? 0 : (int64_t)rows[i - 1] + 1;
        const int64_t hi = i == n ? nr : (int64_t)rows[i];
        for (int64_t r = lo; r <= hi; ++r) ptr[r] = (int32_t)i;
        if (i < n) {
            const uint32_t e = perm[i];
            col[i] = to[e];
            v[i] = val[e];
        }
    }
}

// ---- host ----------------------------------------------------------------

struct Dev {
    void *p = nullptr;
    ~Dev() {
        if (p) cudaFree(p);
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

int cuda_err(std::string *err, cudaError_t e, const char *what) {
    if (err) *err = std::string("GPU conversion: ") + what + ": " + cudaGetErrorString(e);
    return DBD_ERR_CUDA;
}

#define MTX_CK(call, what)                                 \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_err(err, e_, what); \
    } while (0)

// fgets(line, 200) over a buffer: the next piece [pos, end).
bool host_piece(const char *b, int64_t n, int64_t &pos, int64_t &p0, int64_t &p1) {
    if (pos >= n) return false;
    p0 = pos;
    while (pos < n && pos - p0 < kPiece) {
        if (b[pos++] == '\n') break;
    }
    p1 = pos;
    return true;
}

}  // namespace

int64_t stable_sort_scratch_bytes(int64_t n) {
    const int64_t tiles = std::max<int64_t>((n + kSortTile - 1) / kSortTile, 1);
    const int64_t parts = (256 * tiles + kScanTile - 1) / kScanTile + 2;
    return 4 * 256 * tiles + 8 * (256 * tiles + 1) + 8 * parts + 64;
}

void launch_stable_sort_u32(uint32_t *k0, uint32_t *v0, uint32_t *k1, uint32_t *v1, int64_t n, int bits,
                            void *scratch, cudaStream_t s, uint32_t **keys, uint32_t **vals) {
    const int64_t tiles = std::max<int64_t>((n + kSortTile - 1) / kSortTile, 1);
    char *p = static_cast<char *>(scratch);
    int32_t *hist = reinterpret_cast<int32_t *>(p);
    p += (4 * 256 * tiles + 15) / 16 * 16;
    int64_t *off = reinterpret_cast<int64_t *>(p);
    p += (8 * (256 * tiles + 1) + 15) / 16 * 16;
    int64_t *part = reinterpret_cast<int64_t *>(p);
    for (int shift = 0; shift < bits && n > 0; shift += 8) {
        k_sort_hist<<<(unsigned)tiles, 32, 0, s>>>(k0, n, shift, hist, tiles);
        launch_row_scan(256 * tiles, hist, part, off, s);
        k_sort_scatter<<<(unsigned)tiles, 32, 0, s>>>(k0, v0, k1, v1, n, shift, off, tiles);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    *keys = k0;
    *vals = v0;
}

int convert_matrix_file_gpu(const std::string &path, int device, dbd_csr_host *m, std::string *err) {
    memset(m, 0, sizeof(*m));
    MTX_CK(cudaSetDevice(device), "set device");
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) {
        if (err) *err = "cannot open " + path + ": " + strerror(errno);
        return DBD_ERR_IO;
    }
    fseek(f, 0, SEEK_END);
    const int64_t size = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *text = nullptr;
    cudaError_t ce = cudaMallocHost(&text, (size_t)size + 1);
    if (ce != cudaSuccess) {
        fclose(f);
        return cuda_err(err, ce, "pinned text buffer");
    }
    struct HostFree {
        char *p;
        ~HostFree() { cudaFreeHost(p); }
    } hf{text};
    const bool read_ok = size == 0 || fread(text, 1, (size_t)size, f) == (size_t)size;
    fclose(f);
    if (!read_ok) {
        if (err) *err = path + ": short read";
        return DBD_ERR_IO;
    }
    text[size] = '\0';

    // Header, as make_CSR reads it: the first line (symmetric or not), then
    // comment lines, then the size line.
    int64_t pos = 0, p0, p1;
    bool symmetric = false;
    if (strstr(path.c_str(), ".dat") == nullptr && host_piece(text, size, pos, p0, p1)) {
        std::string first(text + p0, (size_t)(p1 - p0));
        symmetric = strstr(first.c_str(), "symmetric") != nullptr;
    }
    int64_t nr = -1, nc = -1, ne = -1;
    while (host_piece(text, size, pos, p0, p1)) {
        std::string line(text + p0, (size_t)(p1 - p0));
        if (line[0] == '%' || line[0] == '#') continue;
        std::vector<std::string> tok;
        const char *s = line.c_str();
        while (tok.size() < 3) {
            while (*s && strchr("\t, ", *s)) ++s;
            if (!*s) break;
            const char *t0 = s;
            while (*s && !strchr("\t, ", *s)) ++s;
            tok.emplace_back(t0, (size_t)(s - t0));
        }
        if (tok.size() < 3) {
            if (err) *err = path + ": wrong format";
            return DBD_ERR_IO;
        }
        nr = atoi(tok[0].c_str()) + 1;
        nc = atoi(tok[1].c_str()) + 1;
        ne = atoi(tok[2].c_str());
        break;
    }
    if (nr < 1 || nc < 1 || ne < 0) {
        if (err) *err = path + ": missing size line";
        return DBD_ERR_IO;
    }
    (void)ne;  // the entry count comes from the lines themselves, as in the reference's loop

    // Body on the device.
    const int64_t n = size - pos;
    cudaStream_t st;
    MTX_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    struct StreamFree {
        cudaStream_t s;
        ~StreamFree() { cudaStreamDestroy(s); }
    } sf{st};
    Dev dText, dTileCnt, dTileOff, dPart, dStarts, dEdgeCnt, dEdgeOff, dFlags;
    MTX_CK(cudaMalloc(&dText.p, (size_t)n + 16), "text");
    MTX_CK(cudaMemcpyAsync(dText.p, text + pos, (size_t)n, cudaMemcpyHostToDevice, st), "text copy");
    const int64_t ntiles = std::max<int64_t>((n + kTextTile - 1) / kTextTile, 1);
    MTX_CK(cudaMalloc(&dTileCnt.p, sizeof(int32_t) * (size_t)ntiles), "tiles");
    MTX_CK(cudaMalloc(&dTileOff.p, sizeof(int64_t) * (size_t)(ntiles + 1)), "tiles");
    MTX_CK(cudaMalloc(&dPart.p, sizeof(int64_t) * (size_t)(std::max<int64_t>(ntiles, 256) + 2)), "scan");
    MTX_CK(cudaMalloc(&dFlags.p, 4 * sizeof(unsigned long long)), "flags");
    MTX_CK(cudaMemsetAsync(dFlags.p, 0, 4 * sizeof(unsigned long long), st), "flags");
    k_nl_count<<<(unsigned)ntiles, 256, 0, st>>>(dText.as<char>(), n, dTileCnt.as<int32_t>());
    launch_row_scan(ntiles, dTileCnt.as<int32_t>(), dPart.as<int64_t>(), dTileOff.as<int64_t>(), st);
    int64_t nl = 0;
    MTX_CK(cudaMemcpyAsync(&nl, dTileOff.as<int64_t>() + ntiles, sizeof(int64_t), cudaMemcpyDeviceToHost, st),
           "newline count");
    MTX_CK(cudaStreamSynchronize(st), "newline count");
    const int64_t nlines = nl + 1;
    MTX_CK(cudaMalloc(&dStarts.p, sizeof(int64_t) * (size_t)(nlines + 1)), "lines");
    k_line_starts<<<(unsigned)ntiles, 256, 0, st>>>(dText.as<char>(), n, dTileOff.as<int64_t>(),
                                                    dStarts.as<int64_t>());

    // Entries per line, their positions, then the entries.
    MTX_CK(cudaMalloc(&dEdgeCnt.p, sizeof(int32_t) * (size_t)nlines), "line counts");
    MTX_CK(cudaMalloc(&dEdgeOff.p, sizeof(int64_t) * (size_t)(nlines + 1)), "line offsets");
    LineArgs la{};
    la.t = dText.as<char>();
    la.n = n;
    la.starts = dStarts.as<int64_t>();
    la.nlines = nlines;
    la.symmetric = symmetric ? 1 : 0;
    la.edgeCnt = dEdgeCnt.as<int32_t>();
    la.slowN = dFlags.as<unsigned long long>();
    la.badLine = dFlags.as<unsigned long long>() + 1;
    const unsigned lgrid = (unsigned)((nlines + 255) / 256);
    k_lines<false><<<lgrid, 256, 0, st>>>(la);
    Dev dPart2;
    const int64_t nparts = (nlines + kScanTile - 1) / kScanTile;
    MTX_CK(cudaMalloc(&dPart2.p, sizeof(int64_t) * (size_t)(nparts + 2)), "scan");
    launch_row_scan(nlines, dEdgeCnt.as<int32_t>(), dPart2.as<int64_t>(), dEdgeOff.as<int64_t>(), st);
    int64_t hv[2] = {0, 0};
    unsigned long long hf2[2] = {0, 0};
    MTX_CK(cudaMemcpyAsync(&hv[0], dEdgeOff.as<int64_t>() + nlines, sizeof(int64_t), cudaMemcpyDeviceToHost, st),
           "entry count");
    MTX_CK(cudaMemcpyAsync(hf2, dFlags.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "flags");
    MTX_CK(cudaStreamSynchronize(st), "line pass");
    if (hf2[1]) {
        if (err) *err = path + ": entry line without a column";
        return DBD_ERR_IO;
    }
    const int64_t E = hv[0];
    const int64_t nslow = (int64_t)hf2[0];
    if (E > INT32_MAX || nr > INT32_MAX) {
        if (err) *err = path + ": more entries or rows than the .csr layout holds";
        return DBD_ERR_IO;
    }
    const size_t e1 = (size_t)std::max<int64_t>(E, 1);
    Dev dFrom, dTo, dVal, dSlowE, dSlowT, dK0, dK1, dV0, dV1, dPtr, dCol, dV32;
    MTX_CK(cudaMalloc(&dFrom.p, 4 * e1), "entries");
    MTX_CK(cudaMalloc(&dTo.p, 4 * e1), "entries");
    MTX_CK(cudaMalloc(&dVal.p, 4 * e1), "entries");
    MTX_CK(cudaMalloc(&dSlowE.p, 8 * (size_t)std::max<int64_t>(nslow, 1)), "slow values");
    MTX_CK(cudaMalloc(&dSlowT.p, 8 * (size_t)std::max<int64_t>(nslow, 1)), "slow values");
    MTX_CK(cudaMemsetAsync(dFlags.p, 0, sizeof(unsigned long long), st), "flags");
    la.edgeOff = dEdgeOff.as<int64_t>();
    la.from = dFrom.as<int32_t>();
    la.to = dTo.as<int32_t>();
    la.val = dVal.as<float>();
    la.slowEdge = dSlowE.as<int64_t>();
    la.slowTok = dSlowT.as<int64_t>();
    k_lines<true><<<lgrid, 256, 0, st>>>(la);
    if (nslow > 0)
        k_slow_values<<<(unsigned)((nslow + 63) / 64), 64, 0, st>>>(dText.as<char>(), dSlowE.as<int64_t>(),
                                                                    dSlowT.as<int64_t>(), nslow, dVal.as<float>());

    // Stable sort by row.
    MTX_CK(cudaMalloc(&dK0.p, 4 * e1), "sort");
    MTX_CK(cudaMalloc(&dK1.p, 4 * e1), "sort");
    MTX_CK(cudaMalloc(&dV0.p, 4 * e1), "sort");
    MTX_CK(cudaMalloc(&dV1.p, 4 * e1), "sort");
    int *dBad = reinterpret_cast<int *>(dFlags.as<unsigned long long>() + 2);
    MTX_CK(cudaMemsetAsync(dBad, 0, sizeof(int), st), "flags");
    if (E > 0)
        k_check_edges<<<(unsigned)std::min<int64_t>((E + 255) / 256, 65535), 256, 0, st>>>(
            dFrom.as<int32_t>(), dTo.as<int32_t>(), E, nr, nc, dK0.as<uint32_t>(), dV0.as<uint32_t>(), dBad);
    int bad = 0;
    MTX_CK(cudaMemcpyAsync(&bad, dBad, sizeof(int), cudaMemcpyDeviceToHost, st), "flags");
    MTX_CK(cudaStreamSynchronize(st), "entry pass");
    if (bad) {
        if (err) *err = path + ": entry outside the declared size";
        return DBD_ERR_IO;
    }
    const int64_t stiles = std::max<int64_t>((E + kSortTile - 1) / kSortTile, 1);
    Dev dHist, dHistOff, dPart3;
    MTX_CK(cudaMalloc(&dHist.p, sizeof(int32_t) * 256 * (size_t)stiles), "sort");
    MTX_CK(cudaMalloc(&dHistOff.p, sizeof(int64_t) * (256 * (size_t)stiles + 1)), "sort");
    MTX_CK(cudaMalloc(&dPart3.p, sizeof(int64_t) * (size_t)((256 * stiles + kScanTile - 1) / kScanTile + 2)), "sort");
    int bits = 0;
    while (bits < 32 && ((uint64_t)(nr - 1) >> bits) != 0) ++bits;
    uint32_t *kin = dK0.as<uint32_t>(), *kout = dK1.as<uint32_t>();
    uint32_t *vin = dV0.as<uint32_t>(), *vout = dV1.as<uint32_t>();
    for (int shift = 0; shift < bits && E > 0; shift += 8) {
        k_sort_hist<<<(unsigned)stiles, 32, 0, st>>>(kin, E, shift, dHist.as<int32_t>(), stiles);
        launch_row_scan(256 * stiles, dHist.as<int32_t>(), dPart3.as<int64_t>(), dHistOff.as<int64_t>(), st);
        k_sort_scatter<<<(unsigned)stiles, 32, 0, st>>>(kin, vin, kout, vout, E, shift, dHistOff.as<int64_t>(),
                                                        stiles);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    MTX_CK(cudaMalloc(&dPtr.p, sizeof(int32_t) * (size_t)(nr + 1)), "csr");
    MTX_CK(cudaMalloc(&dCol.p, 4 * e1), "csr");
    MTX_CK(cudaMalloc(&dV32.p, 4 * e1), "csr");
    k_build_csr<<<(unsigned)std::min<int64_t>((E + 256) / 256, 65535), 256, 0, st>>>(
        kin, vin, dTo.as<int32_t>(), dVal.as<float>(), E, nr, dPtr.as<int32_t>(), dCol.as<int32_t>(),
        dV32.as<float>());
    MTX_CK(cudaGetLastError(), "launch");

    m->n_rows = nr;
    m->n_cols = nc;
    m->nnz = E;
    m->src_fp32 = 1;
    m->row_ptr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nr + 1));
    m->col_idx = (int32_t *)malloc(4 * e1);
    m->val = (double *)malloc(8 * e1);
    std::vector<float> v32(e1);
    if (!m->row_ptr || !m->col_idx || !m->val) {
        dbd_csr_host_free(m);
        if (err) *err = "out of host memory converting " + path;
        return DBD_ERR_OOM_HOST;
    }
    ce = cudaMemcpyAsync(m->row_ptr, dPtr.p, sizeof(int32_t) * (size_t)(nr + 1), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(m->col_idx, dCol.p, 4 * (size_t)E, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(v32.data(), dV32.p, 4 * (size_t)E, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) {
        dbd_csr_host_free(m);
        return cuda_err(err, ce, "result copy");
    }
    for (int64_t i = 0; i < E; ++i) m->val[i] = (double)v32[(size_t)i];
    // Cache as <path>.csr in the reference layout, as the host conversion does.
    const std::string cache = path + ".csr";
    FILE *o = fopen(cache.c_str(), "wb");
    if (o) {
        const int32_t hdr[3] = {(int32_t)nr, (int32_t)nc, (int32_t)E};
        bool ok = fwrite(hdr, sizeof(hdr), 1, o) == 1 &&
                  fwrite(m->row_ptr, sizeof(int32_t), (size_t)(nr + 1), o) == (size_t)(nr + 1) &&
                  (E == 0 || (fwrite(m->col_idx, 4, (size_t)E, o) == (size_t)E &&
                              fwrite(v32.data(), 4, (size_t)E, o) == (size_t)E));
        ok = (fclose(o) == 0) && ok;
        if (!ok) {
            dbd_csr_host_free(m);
            if (err) *err = "cannot write " + cache;
            return DBD_ERR_IO;
        }
    }
    return DBD_OK;
}

}  // namespace dbd
