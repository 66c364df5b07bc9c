// Internal helpers shared by the translation units of libparticular_cuda.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "particular_cuda.h"

namespace pt {

// Thread-local last-error message (pt_last_error()).
int set_error(int code, const char *fmt, ...);
void clear_error();

// Grow-only device buffer owned by a context. Never shrinks; freed with the context.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
};

enum BufSlot : int {
    BUF_AFF = 0,   // targets, float4
    BUF_SRC,       // sources, float4
    BUF_OUT,       // accelerations, float3
    BUF_PART,      // split-j partial sums
    BUF_OUT64,     // f64 outputs
    BUF_SOA,       // sources as padded x[], y[], z[], mu[] arrays
    BUF_LF_BODY,   // leapfrog state for the host entry point
    BUF_LF_VEL,
    BUF_LF_ACC,
    BUF_COUNT
};

}  // namespace pt

struct pt_ctx {
    int device = 0;
    int sm_count = 0;
    int max_smem_optin = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    size_t capacity_limit = 0;  // 0 = unlimited
    size_t bytes_held = 0;
    unsigned long long launches = 0;
    // Bumped whenever a context buffer is allocated, reallocated or freed: CUDA graphs
    // that captured buffer addresses are captured again when it has moved.
    unsigned long long buf_epoch = 0;
    pt::DevBuf bufs[pt::BUF_COUNT];
    // Extra subsystems hang off the context lazily.
    void *bh = nullptr;
    void *lf = nullptr;
    void *ens = nullptr;
    void *mlp = nullptr;
    // True while a CUDA graph is being captured on `stream`: buffers must not grow.
    bool capturing = false;
    // True while a leapfrog step sequence runs: Barnes-Hut walks keep the error word
    // of earlier steps instead of clearing it, so the sequence's caller sees them all.
    bool keep_errors = false;
    // Optional phase timing: events recorded at phase boundaries of the last call.
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
};

namespace pt {

// Ensures ctx->bufs[slot] holds at least `bytes`; returns PT_OK or an error code.
int ensure(pt_ctx *ctx, int slot, size_t bytes);
// Generic grow-only buffer (for subsystems that keep their own DevBufs).
int ensure_buf(pt_ctx *ctx, DevBuf &b, size_t bytes);
void free_buf(pt_ctx *ctx, DevBuf &b);

// Checks the launch just made; counts it.
int check_launch(pt_ctx *ctx, const char *what);
int check_cuda(cudaError_t e, const char *what);

// Records phase boundary k (0 = start, 1 = build done, 2 = walk done) when enabled.
inline void mark(pt_ctx *ctx, int k) {
    if (ctx->timing) cudaEventRecord(ctx->ev[k], ctx->stream);
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Barnes-Hut settings held by the context that its launches take as parameters
// (pt_bh.cu): graphs that captured them compare these before a replay.
struct BhTuning {
    float local_ratio = 0.f, rel_alpha = 0.f, rel_mono = 0.f, theta_inner = 0.f;
    int stack_cap = 0, learned_cap = 0;
    const void *mlp = nullptr;
    bool operator==(const BhTuning &o) const {
        return local_ratio == o.local_ratio && rel_alpha == o.rel_alpha && rel_mono == o.rel_mono &&
               theta_inner == o.theta_inner && stack_cap == o.stack_cap && learned_cap == o.learned_cap &&
               mlp == o.mlp;
    }
};
BhTuning bh_tuning(pt_ctx *ctx);
// The Barnes-Hut error word of the context (device int, bit 2 = learned records
// overflowed), or nullptr before the first Barnes-Hut call.
int *bh_error_word(pt_ctx *ctx);
// After a step sequence with PT_BH_LEARNED: synchronises, reads the error word and,
// when records overflowed, grows the automatic record capacity for the next call and
// returns PT_ERR_CAPACITY.
int bh_learned_overflow(pt_ctx *ctx, const char *fn);
// The brute-force launch plan forced on this thread by pt_bf_set_plan (0 = automatic):
// part of the shape a captured leapfrog graph was recorded for.
void bf_forced_plan(int *targets_per_thread, int *slices);

}  // namespace pt

#define PT_TRY(expr)                    \
    do {                                \
        int _pt_rc = (expr);            \
        if (_pt_rc != PT_OK) return _pt_rc; \
    } while (0)

#define PT_CUDA(expr) PT_TRY(::pt::check_cuda((expr), #expr))
