// csr_io.cpp -- CSR files: the reference's .csr layout, this library's FP64
// .dcsr layout, and the reference's Matrix Market / .dat conversion.
//
// .csr  (ZIP:dbd/src/readInput.cpp:26-42, written at :166-175):
//        int32 nr, nc, ne; int32 ptr[nr+1]; int32 idx[ne]; float32 val[ne]
// .dcsr (this library): "DBDCSR64" magic; int64 nr, nc, ne;
//        int32 ptr[nr+1]; int32 idx[ne]; float64 val[ne]
//
// The conversion reproduces make_CSR (readInput.cpp:48-176) byte for byte on
// well-formed input, including its quirks: the header's row and column counts
// are taken +1 so the 1-based indices of the file are kept as they are (row 0
// and column 0 stay empty, :68,75); a missing value reads as 1.0 (:113-114);
// "symmetric" in the first line mirrors every off-diagonal entry (:116-122);
// entries are stably ordered by row (the base-10 LSD radix sort of :192-215 is
// a stable sort on the row).  Values pass through float32 as in the reference.
// Deviation: row_ptr entries after the last non-empty row are filled (the
// reference leaves them uninitialised unless that row is the last one).
#include "dbd_io.h"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

namespace dbd {

namespace {

const char kMagic[8] = {'D', 'B', 'D', 'C', 'S', 'R', '6', '4'};

bool file_exists(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

bool read_exact(FILE *f, void *dst, size_t bytes) {
    return bytes == 0 || fread(dst, 1, bytes, f) == bytes;
}

bool write_exact(FILE *f, const void *src, size_t bytes) {
    return bytes == 0 || fwrite(src, 1, bytes, f) == bytes;
}

int fail(std::string *err, const std::string &msg) {
    if (err) *err = msg;
    return DBD_ERR_IO;
}

int alloc_host(dbd_csr_host *m, std::string *err) {
    m->row_ptr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m->n_rows + 1));
    m->col_idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m->nnz > 0 ? m->nnz : 1));
    m->val = (double *)malloc(sizeof(double) * (size_t)(m->nnz > 0 ? m->nnz : 1));
    if (!m->row_ptr || !m->col_idx || !m->val) {
        free(m->row_ptr);
        free(m->col_idx);
        free(m->val);
        m->row_ptr = nullptr;
        m->col_idx = nullptr;
        m->val = nullptr;
        if (err) *err = "out of host memory reading CSR";
        return DBD_ERR_OOM_HOST;
    }
    return DBD_OK;
}

int read_dcsr(const std::string &p, dbd_csr_host *m, std::string *err) {
    FILE *f = fopen(p.c_str(), "rb");
    if (!f) return fail(err, "cannot open " + p + ": " + strerror(errno));
    char magic[8];
    int64_t hdr[3];
    if (!read_exact(f, magic, 8) || memcmp(magic, kMagic, 8) != 0 || !read_exact(f, hdr, sizeof(hdr))) {
        fclose(f);
        return fail(err, p + ": not a .dcsr file");
    }
    m->n_rows = hdr[0];
    m->n_cols = hdr[1];
    m->nnz = hdr[2];
    m->src_fp32 = 0;
    if (m->n_rows < 0 || m->n_cols < 0 || m->nnz < 0 || m->nnz > INT32_MAX || m->n_rows >= INT32_MAX) {
        fclose(f);
        return fail(err, p + ": header out of range");
    }
    int rc = alloc_host(m, err);
    if (rc) {
        fclose(f);
        return rc;
    }
    bool ok = read_exact(f, m->row_ptr, sizeof(int32_t) * (size_t)(m->n_rows + 1)) &&
              read_exact(f, m->col_idx, sizeof(int32_t) * (size_t)m->nnz) &&
              read_exact(f, m->val, sizeof(double) * (size_t)m->nnz);
    fclose(f);
    if (!ok) {
        dbd_csr_host_free(m);
        return fail(err, p + ": truncated");
    }
    return DBD_OK;
}

int read_ref_csr(const std::string &p, dbd_csr_host *m, std::string *err) {
    FILE *f = fopen(p.c_str(), "rb");
    if (!f) return fail(err, "cannot open " + p + ": " + strerror(errno));
    int32_t hdr[3];
    if (!read_exact(f, hdr, sizeof(hdr))) {
        fclose(f);
        return fail(err, p + ": truncated header");
    }
    m->n_rows = hdr[0];
    m->n_cols = hdr[1];
    m->nnz = hdr[2];
    m->src_fp32 = 1;
    if (m->n_rows < 0 || m->n_cols < 0 || m->nnz < 0) {
        fclose(f);
        return fail(err, p + ": negative header");
    }
    int rc = alloc_host(m, err);
    if (rc) {
        fclose(f);
        return rc;
    }
    std::vector<float> v((size_t)m->nnz);
    bool ok = read_exact(f, m->row_ptr, sizeof(int32_t) * (size_t)(m->n_rows + 1)) &&
              read_exact(f, m->col_idx, sizeof(int32_t) * (size_t)m->nnz) &&
              read_exact(f, v.data(), sizeof(float) * (size_t)m->nnz);
    fclose(f);
    if (!ok) {
        dbd_csr_host_free(m);
        return fail(err, p + ": truncated");
    }
    for (int64_t i = 0; i < m->nnz; ++i) m->val[i] = (double)v[(size_t)i];
    return DBD_OK;
}

// One token of the reference's strtok(line, "\t, ") split.
const char *next_token(char *&s) {
    static const char *delims = "\t, ";
    while (*s && strchr(delims, *s)) ++s;
    if (!*s) return nullptr;
    const char *tok = s;
    while (*s && !strchr(delims, *s)) ++s;
    if (*s) *s++ = '\0';
    return tok;
}

struct Edge {
    int32_t from, to;
    float val;
};

int convert_matrix_file(const std::string &path, dbd_csr_host *m, std::string *err) {
    FILE *f = fopen(path.c_str(), "rt");
    if (!f) return fail(err, "cannot open " + path + ": " + strerror(errno));
    char line[200];
    bool symmetric = false;
    if (strstr(path.c_str(), ".dat") == nullptr) {
        if (fgets(line, sizeof(line), f) && strstr(line, "symmetric")) symmetric = true;
    }
    int64_t nr = -1, nc = -1, ne = -1;
    while (fgets(line, sizeof(line), f)) {
        if (line[0] == '%' || line[0] == '#') continue;
        char *s = line;
        const char *t1 = next_token(s), *t2 = t1 ? next_token(s) : nullptr,
                   *t3 = t2 ? next_token(s) : nullptr;
        if (!t1 || !t2 || !t3) {
            fclose(f);
            return fail(err, path + ": wrong format");
        }
        nr = atoi(t1) + 1;
        nc = atoi(t2) + 1;
        ne = atoi(t3);
        if (symmetric) ne *= 2;
        break;
    }
    if (nr < 1 || nc < 1 || ne < 0) {
        fclose(f);
        return fail(err, path + ": missing size line");
    }
    std::vector<Edge> edges;
    edges.reserve((size_t)ne);
    while (fgets(line, sizeof(line), f)) {
        char *s = line;
        const char *t1 = next_token(s);
        if (!t1) continue;
        const char *t2 = next_token(s);
        if (!t2) {
            fclose(f);
            return fail(err, path + ": entry line without a column");
        }
        const char *t3 = next_token(s);
        Edge e;
        e.from = atoi(t1);
        e.to = atoi(t2);
        e.val = t3 ? (float)atof(t3) : 1.0f;
        edges.push_back(e);
        if (symmetric && e.from != e.to) edges.push_back(Edge{e.to, e.from, e.val});
    }
    fclose(f);
    for (const Edge &e : edges) {
        if (e.from < 0 || e.from >= nr || e.to < 0 || e.to >= nc) {
            return fail(err, path + ": entry outside the declared size");
        }
    }
    m->n_rows = nr;
    m->n_cols = nc;
    m->nnz = (int64_t)edges.size();
    m->src_fp32 = 1;
    int rc = alloc_host(m, err);
    if (rc) return rc;
    // Stable counting sort by row.
    std::vector<int64_t> cnt((size_t)nr + 1, 0);
    for (const Edge &e : edges) ++cnt[(size_t)e.from + 1];
    for (int64_t r = 0; r < nr; ++r) cnt[(size_t)r + 1] += cnt[(size_t)r];
    for (int64_t r = 0; r <= nr; ++r) m->row_ptr[r] = (int32_t)cnt[(size_t)r];
    std::vector<float> v32((size_t)m->nnz);
    for (const Edge &e : edges) {
        const int64_t pos = cnt[(size_t)e.from]++;
        m->col_idx[pos] = e.to;
        v32[(size_t)pos] = e.val;
    }
    for (int64_t i = 0; i < m->nnz; ++i) m->val[i] = (double)v32[(size_t)i];
    // Cache as <path>.csr in the reference layout.
    const std::string cache = path + ".csr";
    FILE *o = fopen(cache.c_str(), "wb");
    if (o) {
        int32_t hdr[3] = {(int32_t)nr, (int32_t)nc, (int32_t)m->nnz};
        bool ok = write_exact(o, hdr, sizeof(hdr)) &&
                  write_exact(o, m->row_ptr, sizeof(int32_t) * (size_t)(nr + 1)) &&
                  write_exact(o, m->col_idx, sizeof(int32_t) * (size_t)m->nnz) &&
                  write_exact(o, v32.data(), sizeof(float) * (size_t)m->nnz);
        ok = (fclose(o) == 0) && ok;
        if (!ok) {
            dbd_csr_host_free(m);
            return fail(err, "cannot write " + cache);
        }
    }
    return DBD_OK;
}

}  // namespace

int read_csr_file(const std::string &path, dbd_csr_host *out, std::string *err) {
    memset(out, 0, sizeof(*out));
    if (file_exists(path + ".dcsr")) return read_dcsr(path + ".dcsr", out, err);
    if (file_exists(path + ".csr")) return read_ref_csr(path + ".csr", out, err);
    if (file_exists(path)) return convert_matrix_file(path, out, err);
    return fail(err, "no " + path + ".dcsr, " + path + ".csr or " + path);
}

int read_csr_file_gpu(const std::string &path, int device, dbd_csr_host *out, std::string *err) {
    memset(out, 0, sizeof(*out));
    if (file_exists(path + ".dcsr")) return read_dcsr(path + ".dcsr", out, err);
    if (file_exists(path + ".csr")) return read_ref_csr(path + ".csr", out, err);
    if (file_exists(path)) return convert_matrix_file_gpu(path, device, out, err);
    return fail(err, "no " + path + ".dcsr, " + path + ".csr or " + path);
}

int write_csr_file(const std::string &path, const dbd_csr_view *m, int fp64, std::string *err) {
    if (m->on_device) {
        if (err) *err = "dbd_write_csr takes host arrays";
        return DBD_ERR_INVALID;
    }
    if (m->n_rows < 0 || m->nnz < 0 || m->nnz > INT32_MAX) {
        if (err) *err = "CSR size out of range";
        return DBD_ERR_INVALID;
    }
    FILE *o = fopen(path.c_str(), "wb");
    if (!o) return fail(err, "cannot create " + path + ": " + strerror(errno));
    bool ok = true;
    const size_t ne = (size_t)m->nnz;
    if (fp64) {
        int64_t hdr[3] = {m->n_rows, m->n_cols, m->nnz};
        ok = write_exact(o, kMagic, 8) && write_exact(o, hdr, sizeof(hdr));
    } else {
        int32_t hdr[3] = {(int32_t)m->n_rows, (int32_t)m->n_cols, (int32_t)m->nnz};
        ok = write_exact(o, hdr, sizeof(hdr));
    }
    ok = ok && write_exact(o, m->row_ptr, sizeof(int32_t) * (size_t)(m->n_rows + 1)) &&
         write_exact(o, m->col_idx, sizeof(int32_t) * ne);
    if (ok) {
        if (fp64) {
            if (m->val_fp32) {
                std::vector<double> v(ne);
                for (size_t i = 0; i < ne; ++i) v[i] = ((const float *)m->val)[i];
                ok = write_exact(o, v.data(), sizeof(double) * ne);
            } else {
                ok = write_exact(o, m->val, sizeof(double) * ne);
            }
        } else {
            if (m->val_fp32) {
                ok = write_exact(o, m->val, sizeof(float) * ne);
            } else {
                std::vector<float> v(ne);
                for (size_t i = 0; i < ne; ++i) v[i] = (float)((const double *)m->val)[i];
                ok = write_exact(o, v.data(), sizeof(float) * ne);
            }
        }
    }
    ok = (fclose(o) == 0) && ok;
    return ok ? DBD_OK : fail(err, "short write to " + path);
}

}  // namespace dbd

extern "C" void dbd_csr_host_free(dbd_csr_host *m) {
    if (!m) return;
    free(m->row_ptr);
    free(m->col_idx);
    free(m->val);
    m->row_ptr = nullptr;
    m->col_idx = nullptr;
    m->val = nullptr;
}
