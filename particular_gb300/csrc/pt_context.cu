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
        cudaFree(b.ptr);
        ctx->bytes_held -= b.cap;
    }
    b.ptr = nullptr;
    b.cap = 0;
}

int ensure(pt_ctx *ctx, int slot, size_t bytes) { return ensure_buf(ctx, ctx->bufs[slot], bytes); }

}  // namespace pt

// Defined by the Barnes-Hut translation unit.
void pt_bh_state_free(pt_ctx *ctx);

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
    pt_bh_state_free(ctx);
    for (auto &b : ctx->bufs) pt::free_buf(ctx, b);
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

int pt_ctx_synchronize(pt_ctx *ctx) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_ctx_synchronize: ctx is NULL");
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

}  // extern "C"
