// writer.cpp -- the +I/O output writer (see writer.h).
#include "writer.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include <errno.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/dbd.h"

namespace dbd {
namespace {

using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

enum FaultKind { FAULT_NONE = 0, FAULT_ENOSPC, FAULT_SHORT, FAULT_STALL };

struct Fault {
    int kind = FAULT_NONE;
    int64_t after = 0;  // bytes written before the fault applies (stall: milliseconds per write)
};

// DBD_IO_FAULT=enospc@N | short@N | stall@MS (host-side fault injection for tests).
Fault parse_fault() {
    Fault f;
    const char *e = getenv("DBD_IO_FAULT");
    if (!e || !*e) return f;
    const char *at = strchr(e, '@');
    const long long v = at ? atoll(at + 1) : 0;
    if (!strncmp(e, "enospc", 6)) f.kind = FAULT_ENOSPC;
    else if (!strncmp(e, "short", 5)) f.kind = FAULT_SHORT;
    else if (!strncmp(e, "stall", 5)) f.kind = FAULT_STALL;
    f.after = v;
    return f;
}

struct Stream {
    const char *name = "";
    int fd = -1;
    int64_t off = 0;        // logical bytes written (file position of the next byte before wrapping)
    int64_t wrap = 0;       // > 0: positions wrap at this many bytes (a multiple of kIoAlign)
    char *carry = nullptr;  // the partial block [off & ~(A-1), off) (direct writes only)
};

constexpr char kMagic[8] = {'D', 'B', 'D', 'P', 'R', 'O', 'G', '1'};

// Progress manifest of a resumable +I/O run.
struct Manifest {
    char magic[8];
    int64_t m, nnz;
    uint64_t fingerprint;
    int32_t flags, pad;
    int64_t row_done, idx_bytes, val_bytes;
    uint64_t check;
};

uint64_t manifest_check(const Manifest &g) {
    uint64_t h = 0x243F6A8885A308D3ull;
    const int64_t f[] = {g.m, g.nnz, (int64_t)g.fingerprint, g.flags, g.row_done, g.idx_bytes, g.val_bytes};
    for (int64_t x : f) h = (h ^ (uint64_t)x) * 0x100000001B3ull + 0x9E3779B97F4A7C15ull;
    return h;
}

}  // namespace

char *aligned_bytes(int64_t bytes) {
    void *p = nullptr;
    if (posix_memalign(&p, (size_t)kIoAlign, (size_t)std::max<int64_t>(bytes, kIoAlign)) != 0) return nullptr;
    memset(p, 0, (size_t)std::max<int64_t>(bytes, kIoAlign));
    return static_cast<char *>(p);
}

struct ChunkWriter {
    std::string dir;
    WriterOpts o;
    bool direct = false;
    Stream idx, val;
    Fault fault;
    int64_t total = 0;   // bytes written to the data files
    double busy = 0.0;   // seconds inside writes
    char *f32 = nullptr; // aligned staging of float32 values
    int64_t f32cap = 0;

    std::string path(const char *name) const {
        std::string d = dir.empty() ? "." : dir;
        if (d.back() != '/') d += '/';
        return d + name;
    }
    int64_t val_elem() const { return o.val_fp32 ? 4 : 8; }
    int flag_bits() const { return (o.val_fp32 ? 1 : 0) | (o.ptr32 ? 2 : 0); }

    int write_at(Stream &s, const char *p, int64_t len, int64_t pos, std::string *err) {
        while (len > 0) {
            int64_t at = pos, lim = len;
            if (s.wrap > 0) {
                at = pos % s.wrap;
                lim = std::min<int64_t>(len, s.wrap - at);
            }
            size_t step = (size_t)std::min<int64_t>(lim, (int64_t)1 << 30);
            ssize_t r;
            if (fault.kind == FAULT_STALL) std::this_thread::sleep_for(std::chrono::milliseconds(fault.after));
            if (fault.kind == FAULT_ENOSPC && total >= fault.after) {
                errno = ENOSPC;
                r = -1;
            } else {
                if (fault.kind == FAULT_SHORT && total >= fault.after && (int64_t)step > kIoAlign)
                    step = direct ? (size_t)((int64_t)step / 2 / kIoAlign * kIoAlign) : step / 2;
                r = ::pwrite(s.fd, p, step, (off_t)at);
            }
            if (r < 0) {
                if (errno == EINTR) continue;
                *err = std::string("pwrite ") + s.name + ": " + strerror(errno);
                return DBD_ERR_IO;
            }
            if (r == 0 || (direct && r % kIoAlign != 0)) {
                *err = std::string("pwrite ") + s.name + ": short write of " + std::to_string((long long)r) +
                       " of " + std::to_string((long long)step) + " bytes";
                return DBD_ERR_IO;
            }
            p += r;
            len -= r;
            pos += r;
            total += r;
        }
        return DBD_OK;
    }

    // Appends len bytes found at base + lead; with O_DIRECT, lead equals
    // s.off mod kIoAlign and base[0, lead) is headroom.
    int put(Stream &s, char *base, int64_t lead, int64_t len, std::string *err) {
        if (len <= 0) return DBD_OK;
        if (!direct) {
            int rc = write_at(s, base + lead, len, s.off, err);
            if (!rc) s.off += len;
            return rc;
        }
        if (lead != s.off % kIoAlign) {
            *err = std::string(s.name) + ": chunk not laid out at its file offset modulo 4 KiB";
            return DBD_ERR_INVALID;
        }
        memcpy(base, s.carry, (size_t)lead);
        const int64_t tot = lead + len, full = tot / kIoAlign * kIoAlign;
        if (full > 0) {
            int rc = write_at(s, base, full, s.off - lead, err);
            if (rc) return rc;
        }
        memcpy(s.carry, base + full, (size_t)(tot - full));
        s.off += len;
        return DBD_OK;
    }

    // Writes the partial last block padded with zeros (direct writes), so
    // that every logical byte is on the device; a later chunk rewrites it.
    int flush_partial(Stream &s, std::string *err) {
        const int64_t rem = s.off % kIoAlign;
        if (!direct || rem == 0) return DBD_OK;
        char *blk = aligned_bytes(kIoAlign);
        if (!blk) return DBD_ERR_OOM_HOST;
        memcpy(blk, s.carry, (size_t)rem);
        const int64_t t = total;
        int rc = write_at(s, blk, kIoAlign, s.off - rem, err);
        total = t + rem;  // count logical bytes only
        free(blk);
        return rc;
    }

    int checkpoint(int64_t row_done, std::string *err) {
        int rc = flush_partial(idx, err);
        if (!rc) rc = flush_partial(val, err);
        if (rc) return rc;
        if (fdatasync(idx.fd) != 0 || fdatasync(val.fd) != 0) {
            *err = std::string("fdatasync: ") + strerror(errno);
            return DBD_ERR_IO;
        }
        Manifest g;
        memset(&g, 0, sizeof(g));
        memcpy(g.magic, kMagic, sizeof(kMagic));
        g.m = o.m;
        g.nnz = o.nnz;
        g.fingerprint = o.fingerprint;
        g.flags = flag_bits();
        g.row_done = row_done;
        g.idx_bytes = idx.off;
        g.val_bytes = val.off;
        g.check = manifest_check(g);
        const std::string tmp = path("DBD.progress.tmp");
        const int fd = ::open(tmp.c_str(), O_CREAT | O_TRUNC | O_WRONLY, 0644);
        if (fd < 0) {
            *err = "cannot write " + tmp + ": " + strerror(errno);
            return DBD_ERR_IO;
        }
        const bool ok = ::write(fd, &g, sizeof(g)) == (ssize_t)sizeof(g) && fsync(fd) == 0;
        ::close(fd);
        if (!ok || rename(tmp.c_str(), path("DBD.progress").c_str()) != 0) {
            *err = "cannot record progress in " + path("DBD.progress");
            return DBD_ERR_IO;
        }
        return DBD_OK;
    }

    // A manifest of this product whose recorded bytes the files still hold.
    bool read_manifest(Manifest *g) {
        const int fd = ::open(path("DBD.progress").c_str(), O_RDONLY);
        if (fd < 0) return false;
        const bool ok = ::read(fd, g, sizeof(*g)) == (ssize_t)sizeof(*g);
        ::close(fd);
        if (!ok || memcmp(g->magic, kMagic, sizeof(kMagic)) != 0 || g->check != manifest_check(*g)) return false;
        if (g->m != o.m || g->nnz != o.nnz || g->fingerprint != o.fingerprint || g->flags != flag_bits()) return false;
        if (g->row_done < 0 || g->row_done > o.m) return false;
        struct stat st;
        if (stat(path("Idx.output").c_str(), &st) != 0 || st.st_size < g->idx_bytes) return false;
        if (stat(path("Val.output").c_str(), &st) != 0 || st.st_size < g->val_bytes) return false;
        return true;
    }

    int open_stream(Stream &s, const char *name, bool truncate, std::string *err) {
        s.name = name;
        const std::string p = path(name);
        const int base = O_CREAT | O_RDWR | (truncate ? O_TRUNC : 0);
        s.fd = -1;
        if (direct) {
            s.fd = ::open(p.c_str(), base | O_DIRECT, 0644);
            if (s.fd < 0 && errno != EINVAL) {
                *err = "cannot open " + p + ": " + strerror(errno);
                return DBD_ERR_IO;
            }
            if (s.fd < 0) direct = false;  // the filesystem refuses O_DIRECT: page-cache writes
        }
        if (s.fd < 0) s.fd = ::open(p.c_str(), base, 0644);
        if (s.fd < 0) {
            *err = "cannot open " + p + ": " + strerror(errno);
            return DBD_ERR_IO;
        }
        return DBD_OK;
    }

    void close_all() {
        if (idx.fd >= 0) ::close(idx.fd);
        if (val.fd >= 0) ::close(val.fd);
        idx.fd = val.fd = -1;
    }
};

int writer_open(const std::string &dir, const WriterOpts &o, ChunkWriter **out, int64_t *resume_row,
                std::string *err) {
    *out = nullptr;
    if (resume_row) *resume_row = 0;
    if (o.resume && o.rotate_bytes > 0) {
        *err = "a resumable output cannot wrap (io_rotate_gib)";
        return DBD_ERR_INVALID;
    }
    ChunkWriter *w = new (std::nothrow) ChunkWriter();
    if (!w) return DBD_ERR_OOM_HOST;
    w->dir = dir;
    w->o = o;
    w->direct = o.direct;
    w->fault = parse_fault();
    w->idx.carry = aligned_bytes(kIoAlign);
    w->val.carry = aligned_bytes(kIoAlign);
    if (!w->idx.carry || !w->val.carry) {
        writer_close(w);
        return DBD_ERR_OOM_HOST;
    }
    Manifest g;
    const bool resume = o.resume && w->read_manifest(&g);
    // Both files are opened the same way; if the second refuses O_DIRECT the
    // first is reopened without it.
    int rc = w->open_stream(w->idx, "Idx.output", !resume, err);
    if (!rc) {
        const bool d0 = w->direct;
        rc = w->open_stream(w->val, "Val.output", !resume, err);
        if (!rc && d0 && !w->direct) {
            ::close(w->idx.fd);
            w->idx.fd = -1;
            rc = w->open_stream(w->idx, "Idx.output", !resume, err);
        }
    }
    if (rc) {
        writer_close(w);
        return rc;
    }
    ::unlink(w->path("Ptr.output").c_str());
    if (o.rotate_bytes > 0) {
        const int64_t vb = w->val_elem();
        w->idx.wrap = std::max<int64_t>(kIoAlign, (o.rotate_bytes * 4 / (4 + vb)) / kIoAlign * kIoAlign);
        w->val.wrap = std::max<int64_t>(kIoAlign, (o.rotate_bytes * vb / (4 + vb)) / kIoAlign * kIoAlign);
    }
    if (resume) {
        w->idx.off = g.idx_bytes;
        w->val.off = g.val_bytes;
        for (Stream *s : {&w->idx, &w->val}) {
            const int64_t rem = s->off % kIoAlign;
            if (w->direct && rem && ::pread(s->fd, s->carry, (size_t)kIoAlign, (off_t)(s->off - rem)) < rem) {
                *err = std::string("cannot reread the last block of ") + s->name;
                writer_close(w);
                return DBD_ERR_IO;
            }
        }
        if (resume_row) *resume_row = g.row_done;
    } else if (o.resume) {
        ::unlink(w->path("DBD.progress").c_str());
    }
    *out = w;
    return DBD_OK;
}

int64_t writer_idx_lead(const ChunkWriter *w) { return w->direct ? w->idx.off % kIoAlign : 0; }

// Values are written straight from the caller's buffer when they arrive in
// the file's type (FP64, or float32 from a float32 source); FP64 values for
// a float32 file go through the writer's own staging instead (lead 0).
static bool val_direct(const ChunkWriter *w) { return !w->o.val_fp32 || w->o.src_fp32; }

int64_t writer_val_lead(const ChunkWriter *w) {
    return (w->direct && val_direct(w)) ? w->val.off % kIoAlign : 0;
}

int64_t writer_lead_for(const ChunkWriter *w, int64_t entry, int val) {
    if (!w->direct || (val && !val_direct(w))) return 0;
    return (entry * (val ? w->val_elem() : 4)) % kIoAlign;
}

int writer_append(ChunkWriter *w, char *idx_base, char *val_base, int64_t n, int64_t row_end, std::string *err) {
    const auto t0 = Clock::now();
    int rc = w->put(w->idx, idx_base, writer_idx_lead(w), 4 * n, err);
    if (!rc) {
        if (w->o.val_fp32 && !w->o.src_fp32) {
            // Convert into aligned staging laid out at the file offset modulo 4 KiB.
            const int64_t lead = w->direct ? w->val.off % kIoAlign : 0;
            const int64_t need = lead + 4 * n + kIoAlign;
            if (need > w->f32cap) {
                free(w->f32);
                w->f32 = aligned_bytes(need);
                w->f32cap = w->f32 ? need : 0;
                if (!w->f32) rc = DBD_ERR_OOM_HOST;
            }
            if (!rc) {
                const double *src = reinterpret_cast<const double *>(val_base);
                float *dst = reinterpret_cast<float *>(w->f32 + lead);
                for (int64_t i = 0; i < n; ++i) dst[i] = (float)src[i];
                rc = w->put(w->val, w->f32, lead, 4 * n, err);
            }
        } else {
            rc = w->put(w->val, val_base, writer_val_lead(w), w->val_elem() * n, err);
        }
    }
    if (!rc && w->o.resume) rc = w->checkpoint(row_end, err);
    w->busy += seconds_since(t0);
    return rc;
}

int writer_finish(ChunkWriter *w, const int64_t *row_ptr, double *t_fsync, std::string *err) {
    const auto t0 = Clock::now();
    int rc = w->flush_partial(w->idx, err);
    if (!rc) rc = w->flush_partial(w->val, err);
    // Drop the zero padding of the last block (files that did not wrap).
    for (Stream *s : {&w->idx, &w->val})
        if (!rc && w->direct && (s->wrap == 0 || s->off <= s->wrap) && ftruncate(s->fd, (off_t)s->off) != 0) {
            *err = std::string("ftruncate ") + s->name + ": " + strerror(errno);
            rc = DBD_ERR_IO;
        }
    if (rc) return rc;
    // Ptr.output (write_Ptr, ZIP:dbd/src/writeFile.cpp:177-196).
    const std::string pp = w->path("Ptr.output");
    const int fd = ::open(pp.c_str(), O_CREAT | O_TRUNC | O_WRONLY, 0644);
    if (fd < 0) {
        *err = "cannot create " + pp + ": " + strerror(errno);
        return DBD_ERR_IO;
    }
    Stream ps;
    ps.name = "Ptr.output";
    ps.fd = fd;
    const bool d = w->direct;
    w->direct = false;  // the small row-pointer file goes through the page cache
    const int64_t m = w->o.m;
    if (w->o.ptr32) {
        if (w->o.nnz > INT32_MAX) {
            rc = DBD_ERR_OVERFLOW;
            *err = "nnz(C) does not fit a 32-bit Ptr.output";
        } else {
            std::vector<int32_t> p32((size_t)m + 1);
            for (int64_t r = 0; r <= m; ++r) p32[(size_t)r] = (int32_t)row_ptr[r];
            rc = w->put(ps, reinterpret_cast<char *>(p32.data()), 0, 4 * (m + 1), err);
        }
    } else {
        rc = w->put(ps, reinterpret_cast<char *>(const_cast<int64_t *>(row_ptr)), 0, 8 * (m + 1), err);
    }
    w->direct = d;
    w->busy += seconds_since(t0);
    const auto tf = Clock::now();
    if (!rc && (fsync(fd) != 0 || fsync(w->idx.fd) != 0 || fsync(w->val.fd) != 0)) {
        rc = DBD_ERR_IO;
        *err = std::string("fsync: ") + strerror(errno);
    }
    if (t_fsync) *t_fsync = seconds_since(tf);
    if (::close(fd) != 0 && !rc) {
        rc = DBD_ERR_IO;
        *err = "close Ptr.output";
    }
    if (!rc && w->o.resume) ::unlink(w->path("DBD.progress").c_str());
    return rc;
}

void writer_close(ChunkWriter *w) {
    if (!w) return;
    w->close_all();
    free(w->idx.carry);
    free(w->val.carry);
    free(w->f32);
    delete w;
}

double writer_busy(const ChunkWriter *w) { return w->busy; }
int64_t writer_bytes(const ChunkWriter *w) { return w->total; }
bool writer_is_direct(const ChunkWriter *w) { return w->direct; }

}  // namespace dbd

// ---- C ABI: the writer on caller buffers -----------------------------------

struct dbd_writer {
    dbd::ChunkWriter *w = nullptr;
    std::string err;
    char *ib = nullptr, *vb = nullptr;  // aligned staging
    int64_t icap = 0, vcap = 0;
};

extern "C" {

int dbd_writer_open(const char *out_dir, int64_t n_rows, int64_t nnz, uint64_t fingerprint, int flags,
                    double rotate_gib, dbd_writer **out, int64_t *resume_row) {
    if (!out || n_rows < 0 || nnz < 0 || rotate_gib < 0) return DBD_ERR_INVALID;
    *out = nullptr;
    dbd_writer *h = new (std::nothrow) dbd_writer();
    if (!h) return DBD_ERR_OOM_HOST;
    dbd::WriterOpts o;
    o.direct = !(flags & DBD_WRITER_BUFFERED);
    o.val_fp32 = (flags & DBD_WRITER_VAL_FP32) != 0;
    o.ptr32 = (flags & DBD_WRITER_PTR32) != 0;
    o.resume = (flags & DBD_WRITER_RESUME) != 0;
    o.rotate_bytes = (int64_t)(rotate_gib * 1024.0 * 1024.0 * 1024.0);
    o.m = n_rows;
    o.nnz = nnz;
    o.fingerprint = fingerprint;
    int rc = dbd::writer_open(out_dir ? out_dir : ".", o, &h->w, resume_row, &h->err);
    if (rc) {
        fprintf(stderr, "dbd_writer_open: %s\n", h->err.c_str());
        delete h;
        return rc;
    }
    *out = h;
    return DBD_OK;
}

int dbd_writer_append(dbd_writer *h, int64_t row_end, const int32_t *col_idx, const double *val, int64_t n) {
    if (!h || n < 0 || (n > 0 && (!col_idx || !val))) return DBD_ERR_INVALID;
    const int64_t li = dbd::writer_idx_lead(h->w), lv = dbd::writer_val_lead(h->w);
    const int64_t ni = dbd::writer_slot_bytes(n, 4), nv = dbd::writer_slot_bytes(n, 8);
    if (ni > h->icap) {
        free(h->ib);
        h->ib = dbd::aligned_bytes(ni);
        h->icap = h->ib ? ni : 0;
    }
    if (nv > h->vcap) {
        free(h->vb);
        h->vb = dbd::aligned_bytes(nv);
        h->vcap = h->vb ? nv : 0;
    }
    if (!h->ib || !h->vb) return DBD_ERR_OOM_HOST;
    if (n) {
        memcpy(h->ib + li, col_idx, sizeof(int32_t) * (size_t)n);
        memcpy(h->vb + lv, val, sizeof(double) * (size_t)n);
    }
    return dbd::writer_append(h->w, h->ib, h->vb, n, row_end, &h->err);
}

int dbd_writer_finish(dbd_writer *h, const int64_t *row_ptr, double *t_fsync) {
    if (!h || !row_ptr) return DBD_ERR_INVALID;
    return dbd::writer_finish(h->w, row_ptr, t_fsync, &h->err);
}

const char *dbd_writer_error(const dbd_writer *h) { return h ? h->err.c_str() : ""; }

int dbd_writer_is_direct(const dbd_writer *h) { return h && dbd::writer_is_direct(h->w) ? 1 : 0; }

void dbd_writer_close(dbd_writer *h) {
    if (!h) return;
    dbd::writer_close(h->w);
    free(h->ib);
    free(h->vb);
    delete h;
}

}  // extern "C"
