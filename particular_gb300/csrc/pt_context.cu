// Context lifetime, error reporting and grow-only device buffers.
//
// The context is this library's GpuResources (particular/src/gpu/mod.rs:84-143):
// the reference creates its wgpu pipeline and buffers lazily and reallocates a
// buffer whenever the requested size differs (gpu/resources.rs:26-40); here the
// buffers only grow, so a steady-state loop allocates nothing.
#include "pt_common.cuh"

#include <new>

namespace pt {

static thread_local char g_err[1024] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_err[0] = '\0'; }

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PT_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(PT_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return set_error(PT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(pt_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(PT_ERR_CUDA, "launch of %s: %s", what, cudaGetErrorString(e));
    return PT_OK;
}

int ensure_buf(pt_ctx *ctx, DevBuf &b, size_t bytes) {
    if (bytes <= b.cap) return PT_OK;
    if (ctx->capturing)
        return set_error(PT_ERR_INVALID, "a buffer would grow during CUDA graph capture (%zu bytes)", bytes);
    // Grow by 1/8 extra so slowly growing sizes do not reallocate every call.
    size_t want = bytes + bytes / 8;
    want = (want + 255) & ~size_t(255);
    size_t after = ctx->bytes_held - b.cap + want;
    if (ctx->capacity_limit && after > ctx->capacity_limit) {
        want = bytes;
        after = ctx->bytes_held - b.cap + want;
        if (after > ctx->capacity_limit)
            return set_error(PT_ERR_CAPACITY,
                             "context capacity limit %zu bytes exceeded (need %zu held)",
                             ctx->capacity_limit, after);
    }
    ++ctx->buf_epoch;  // the buffer's address changes
    if (b.ptr) {
        // Work already enqueued may still read the old buffer.
        cudaStreamSynchronize(ctx->stream);
        cudaFree(b.ptr);
        ctx->bytes_held -= b.cap;
        b.ptr = nullptr;
        b.cap = 0;
    }
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        cudaGetLastError();
        return set_error(PT_ERR_OOM, "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
    }
    b.cap = want;
    ctx->bytes_held += want;
    return PT_OK;
}

void free_buf(pt_ctx *ctx, DevBuf &b) {
    if (b.ptr) {
        ++ctx->buf_epoch;
        cudaFree(b.ptr);
        ctx->bytes_held -= b.cap;
    }
    b.ptr = nullptr;
    b.cap = 0;
}

int ensure(pt_ctx *ctx, int slot, size_t bytes) { return ensure_buf(ctx, ctx->bufs[slot], bytes); }

}  // namespace pt

// Defined by the Barnes-Hut, leapfrog and ensemble translation units.
void pt_bh_state_free(pt_ctx *ctx);
void pt_lf_state_free(pt_ctx *ctx);
void pt_ens_state_free(pt_ctx *ctx);
void pt_mlp_state_free(pt_ctx *ctx);

extern "C" {

const char *pt_last_error(void) { return pt::g_err; }

int pt_ctx_create(pt_ctx **out, int device) {
    pt::clear_error();
    if (!out) return pt::set_error(PT_ERR_INVALID, "pt_ctx_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    PT_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
        return pt::set_error(PT_ERR_INVALID, "pt_ctx_create: device %d out of range (%d devices)",
                             device, ndev);
    PT_CUDA(cudaSetDevice(device));
    pt_ctx *c = new (std::nothrow) pt_ctx();
    if (!c) return pt::set_error(PT_ERR_OOM, "pt_ctx_create: host allocation failed");
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return pt::check_cuda(e, "pt_ctx_create");
    }
    c->stream = c->own_stream;
    *out = c;
    return PT_OK;
}

void pt_ctx_destroy(pt_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    pt_lf_state_free(ctx);
    pt_ens_state_free(ctx);
    pt_bh_state_free(ctx);
    pt_mlp_state_free(ctx);
    for (auto &b : ctx->bufs) pt::free_buf(ctx, b);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int pt_ctx_set_stream(pt_ctx *ctx, void *stream) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_ctx_set_stream: ctx is NULL");
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return PT_OK;
}

int pt_ctx_set_capacity_limit(pt_ctx *ctx, size_t bytes) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_ctx_set_capacity_limit: ctx is NULL");
    ctx->capacity_limit = bytes;
    return PT_OK;
}

size_t pt_ctx_device_bytes(const pt_ctx *ctx) { return ctx ? ctx->bytes_held : 0; }

uint64_t pt_ctx_launch_count(const pt_ctx *ctx) { return ctx ? ctx->launches : 0; }

int pt_ctx_sm_count(const pt_ctx *ctx) { return ctx ? ctx->sm_count : 0; }

int pt_ctx_set_timing(pt_ctx *ctx, int enable) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_ctx_set_timing: ctx is NULL");
    PT_CUDA(cudaSetDevice(ctx->device));
    if (enable)
        for (auto &e : ctx->ev)
            if (!e) PT_CUDA(cudaEventCreate(&e));
    ctx->timing = enable != 0;
    return PT_OK;
}

int pt_last_timing(pt_ctx *ctx, pt_timing *out) {
    pt::clear_error();
    if (!ctx || !out) return pt::set_error(PT_ERR_INVALID, "pt_last_timing: NULL argument");
    if (!ctx->timing) return pt::set_error(PT_ERR_INVALID, "pt_last_timing: timing is not enabled");
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_CUDA(cudaEventSynchronize(ctx->ev[2]));
    PT_CUDA(cudaEventElapsedTime(&out->build_ms, ctx->ev[0], ctx->ev[1]));
    PT_CUDA(cudaEventElapsedTime(&out->walk_ms, ctx->ev[1], ctx->ev[2]));
    return PT_OK;
}

int pt_ctx_synchronize(pt_ctx *ctx) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_ctx_synchronize: ctx is NULL");
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

}  // extern "C"

// ---- FP32 FMA-pipe peak probe --------------------------------------------
// Measured FP32 pipe throughput at the current clock: every thread runs 8
// independent FFMA chains; the grid fills every SM. flops = 2 * chains * iters * threads.
namespace pt {
__global__ void __launch_bounds__(256) fp32_peak_kernel(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
          x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
        x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1.2345f) out[0] = s;  // keeps the chains alive
}
}  // namespace pt

extern "C" int pt_measure_fp32_peak(pt_ctx *ctx, double *tflops) {
    pt::clear_error();
    if (!ctx || !tflops) return pt::set_error(PT_ERR_INVALID, "pt_measure_fp32_peak: NULL argument");
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_TRY(pt::ensure(ctx, pt::BUF_OUT64, 256));
    float *out = static_cast<float *>(ctx->bufs[pt::BUF_OUT64].ptr);
    const int iters = 1 << 16;
    const int blocks = ctx->sm_count * 8;
    cudaEvent_t e0, e1;
    PT_CUDA(cudaEventCreate(&e0));
    PT_CUDA(cudaEventCreate(&e1));
    pt::fp32_peak_kernel<<<blocks, 256, 0, ctx->stream>>>(out, iters, 0.9999f, 1e-4f);
    int rc = pt::check_launch(ctx, "fp32_peak_kernel");
    float best = 1e30f;
    for (int rep = 0; rep < 3 && rc == PT_OK; ++rep) {
        cudaEventRecord(e0, ctx->stream);
        pt::fp32_peak_kernel<<<blocks, 256, 0, ctx->stream>>>(out, iters, 0.9999f, 1e-4f);
        rc = pt::check_launch(ctx, "fp32_peak_kernel");
        cudaEventRecord(e1, ctx->stream);
        if (rc == PT_OK) rc = pt::check_cuda(cudaEventSynchronize(e1), "fp32 peak sync");
        float ms = 0.f;
        if (rc == PT_OK) cudaEventElapsedTime(&ms, e0, e1);
        if (ms > 0.f && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != PT_OK) return rc;
    const double flops = 2.0 * 8.0 * double(iters) * double(blocks) * 256.0;
    *tflops = flops / (double(best) * 1e-3) / 1e12;
    return PT_OK;
}
