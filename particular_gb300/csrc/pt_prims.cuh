// Device-wide primitives used by the Barnes-Hut build: exclusive scan of u32 and a
// stable LSD radix sort of (u64 key, u32 value) pairs.
#pragma once

#include "pt_common.cuh"

namespace pt {

// Scratch for the primitives; grow-only, owned by a subsystem.
struct PrimScratch {
    DevBuf scan;   // block sums of every recursion level
    DevBuf hist;   // radix histograms / offsets
    DevBuf keys2;  // ping-pong keys
    DevBuf vals2;  // ping-pong values
};

// out[0..n] = exclusive prefix sums of in[0..n), out[n] = total. in may equal out
// only if n == 0. All enqueued on ctx->stream.
int scan_u32(pt_ctx *ctx, PrimScratch &s, const uint32_t *in, uint32_t *out, int n);

// Sorts keys (and their values) ascending by the low `bits` bits, stably. The
// result ends in keys/vals.
int radix_sort_u64(pt_ctx *ctx, PrimScratch &s, uint64_t *keys, uint32_t *vals, int n, int bits);

void prim_free(pt_ctx *ctx, PrimScratch &s);

}  // namespace pt
