// writer.h -- the +I/O output writer of libdbd (internal).
//
// Appends C's entries to Idx.output / Val.output in row order, chunk after
// chunk, then writes Ptr.output.  The reference fwrites each finished block
// through stdio from its writer pthread (ZIP:dbd/src/writeFile.cpp:13-154;
// the binding variant writeFile_binding.cpp:60-160 joins consecutive blocks
// into one fwrite); here:
//
//  * O_DIRECT by default: every write is 4 KiB-aligned in the file and in
//    memory and bypasses the page cache, so the bytes go to the device at its
//    rate instead of piling up as dirty pages for a long fsync.  The caller
//    lays each chunk out so that its first byte sits at the same offset
//    modulo 4 KiB in memory as in the file, with 4 KiB of headroom before it;
//    the writer completes the partial block left by the previous chunk in
//    that headroom, writes the aligned whole blocks straight from the pinned
//    slot (no copy), and keeps the new partial block for the next chunk.
//    Filesystems that refuse O_DIRECT get page-cache writes instead.
//  * A chunk is one write per file (the reference's coalescing, done at the
//    size of a chunk of row blocks instead of a few blocks).
//  * Resumable: with a progress manifest (DBD.progress), every chunk is made
//    durable (fdatasync) before the manifest records the rows written; a
//    later run on the same product continues after the last recorded row.
//  * Host-side fault injection for tests: DBD_IO_FAULT=enospc@N | short@N |
//    stall@MS fails with ENOSPC, writes half of each request, or sleeps MS
//    before each write, once N bytes have been written.
#pragma once

#include <cstdint>
#include <string>

namespace dbd {

constexpr int64_t kIoAlign = 4096;

struct WriterOpts {
    bool direct = true;        // O_DIRECT (falls back to page-cache writes)
    bool val_fp32 = false;     // Val.output as float32
    bool src_fp32 = false;     // the value buffers handed to writer_append hold float32 (val_fp32 too)
    bool ptr32 = false;        // Ptr.output as int32
    int64_t rotate_bytes = 0;  // > 0: Idx+Val wrap after this many bytes in total
    bool resume = false;       // progress manifest + continue after the last durable row
    int64_t m = 0, nnz = 0;    // rows and entries of the whole product
    uint64_t fingerprint = 0;  // identity of the product (resume)
};

struct ChunkWriter;

// Opens (or, with resume and a matching manifest, reopens) the output files
// in dir.  *resume_row receives the first row still to be written.
int writer_open(const std::string &dir, const WriterOpts &o, ChunkWriter **w, int64_t *resume_row,
                std::string *err);
// Appends the next chunk: n entries ending at row row_end.  idx_base / val_base
// are 4 KiB-aligned buffers holding the column indices at idx_base +
// writer_idx_lead(w) and the values (FP64, or float32 with src_fp32) at
// val_base + writer_val_lead(w),
// each with the lead bytes before them free for the writer's use (without
// O_DIRECT the leads are 0).
int writer_append(ChunkWriter *w, char *idx_base, char *val_base, int64_t n, int64_t row_end, std::string *err);
// Byte offsets of the next chunk's first index / value inside its buffers.
int64_t writer_idx_lead(const ChunkWriter *w);
int64_t writer_val_lead(const ChunkWriter *w);
// Lead (in bytes) that a chunk starting at entry e will get, known before
// the earlier chunks are written.
int64_t writer_lead_for(const ChunkWriter *w, int64_t entry, int val);
// Writes Ptr.output from the product's m + 1 row pointers, makes everything
// durable and removes the manifest.
int writer_finish(ChunkWriter *w, const int64_t *row_ptr, double *t_fsync, std::string *err);
void writer_close(ChunkWriter *w);
double writer_busy(const ChunkWriter *w);
int64_t writer_bytes(const ChunkWriter *w);
bool writer_is_direct(const ChunkWriter *w);

// 4 KiB-aligned, zeroed host allocation (free with free()).
char *aligned_bytes(int64_t bytes);

// Bytes a buffer needs to hold n entries of `elem` bytes after any lead.
inline int64_t writer_slot_bytes(int64_t n, int64_t elem) {
    return ((n * elem + 2 * kIoAlign) + kIoAlign - 1) / kIoAlign * kIoAlign;
}

}  // namespace dbd
