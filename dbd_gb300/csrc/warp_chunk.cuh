// Device helpers shared by the multiply and adjoint kernels: the error word
// and the warp-level enumeration of the products of up to 32 consecutive A
// entries (product t, 0 <= t < total, comes from the lane whose inclusive
// length prefix first exceeds t).
#pragma once

#include "dbd_internal.h"

namespace dbd {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// First error wins: a device check records its code once and never traps.
__device__ __forceinline__ void raise(int *err, int code) { atomicCAS(err, 0, code); }

struct Chunk {
    int32_t bs;    // first position of B_k in B.idx
    int32_t len;   // |B_k|
    int32_t incl;  // inclusive prefix of len over lanes
    double a;      // A value of this lane's entry
    int32_t total; // products of the chunk
};

__device__ __forceinline__ Chunk load_chunk(const CsrDev &A, const CsrDev &B, int32_t e, int32_t eEnd,
                                            int lane) {
    Chunk c;
    c.bs = 0;
    c.len = 0;
    c.a = 0.0;
    if (e + lane < eEnd) {
        const int32_t k = A.idx[e + lane];
        c.bs = B.ptr[k];
        c.len = B.ptr[k + 1] - c.bs;
        c.a = A.val[e + lane];
    }
    int32_t x = c.len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    c.incl = x;
    c.total = __shfl_sync(FULL, x, 31);
    return c;
}

// Owner lane of product t (all 32 lanes must call; t may be out of range).
__device__ __forceinline__ int chunk_owner(const Chunk &c, int32_t t) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int32_t v = __shfl_sync(FULL, c.incl, lo + step - 1);
        if (v <= t) lo += step;
    }
    return lo;
}

}  // namespace
}  // namespace dbd
