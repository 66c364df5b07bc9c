// Kick-drift-kick leapfrog around the acceleration methods, optionally replayed
// from a CUDA graph.
//
// The reference computes accelerations only (particular/src/lib.rs:9-16); its own
// benchmark and tests integrate with a semi-implicit Euler loop around them
// (particular/benches/benchmark.rs:81, gravity/newtonian/mod.rs:318-330). This
// driver keeps positions, masses and velocities resident and runs
//     v += a dt/2;  x += v dt;  a = accel(x);  v += a dt/2
// per step, fusing the closing half kick of one step with the opening half kick of
// the next (one full kick + drift kernel per step), so a call of `steps` steps costs
// `steps` acceleration evaluations. The accelerations of the final positions are left
// in `acc` so the next call continues without recomputing them.
#include "pt_common.cuh"

#include <climits>
#include <new>

int pt_bf_accel_f32_device(pt_ctx *, const float *, size_t, const float *, size_t, float, int, uint32_t, float *);
int pt_bh_accel_f32_device(pt_ctx *, const float *, size_t, const float *, size_t, float, float, uint32_t, float *);

namespace pt {
namespace lf {

// v += a * kick; x += v * dt   (kick = dt/2 for the first step, dt afterwards)
__global__ void kick_drift(float4 *__restrict__ body, float4 *__restrict__ vel, const float *__restrict__ acc,
                           int n, float kick, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = vel[i];
    float4 x = body[i];
    v.x = fmaf(acc[3 * size_t(i)], kick, v.x);
    v.y = fmaf(acc[3 * size_t(i) + 1], kick, v.y);
    v.z = fmaf(acc[3 * size_t(i) + 2], kick, v.z);
    x.x = fmaf(v.x, dt, x.x);
    x.y = fmaf(v.y, dt, x.y);
    x.z = fmaf(v.z, dt, x.z);
    vel[i] = v;
    body[i] = x;
}

__global__ void kick(float4 *__restrict__ vel, const float *__restrict__ acc, int n, float k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = vel[i];
    v.x = fmaf(acc[3 * size_t(i)], k, v.x);
    v.y = fmaf(acc[3 * size_t(i) + 1], k, v.y);
    v.z = fmaf(acc[3 * size_t(i) + 2], k, v.z);
    vel[i] = v;
}

struct Graph {
    cudaGraphExec_t exec = nullptr;
    // the shape the graph was captured for
    const void *body = nullptr, *vel = nullptr, *acc = nullptr;
    size_t n = 0;
    int steps = 0, method = 0;
    float dt = 0.f, theta = 0.f, softening = 0.f;
    uint32_t flags = 0;
    cudaStream_t stream = nullptr;
    BhTuning tune;                 // Barnes-Hut settings baked into the captured launches
    int plan_k = 0, plan_s = 0;    // the brute-force plan forced by pt_bf_set_plan at capture
    unsigned long long epoch = 0;  // the context's buffer addresses it captured
    uint64_t kernels = 0;
    bool same(const void *b, const void *v, const void *a, size_t n_, int s, int m, float d, float t, float e,
              uint32_t f, cudaStream_t st, const BhTuning &tu, int pk, int ps, unsigned long long ep) const {
        return exec && body == b && vel == v && acc == a && n == n_ && steps == s && method == m && dt == d &&
               theta == t && softening == e && flags == f && stream == st && epoch == ep &&
               (method != PT_METHOD_BARNES_HUT || tune == tu) &&
               (method != PT_METHOD_BRUTE_FORCE || (plan_k == pk && plan_s == ps));
    }
};

// Keeps the Barnes-Hut error word across the steps of one call (restored on return).
struct KeepErrors {
    pt_ctx *ctx;
    bool prev;
    explicit KeepErrors(pt_ctx *c) : ctx(c), prev(c->keep_errors) { c->keep_errors = true; }
    ~KeepErrors() { ctx->keep_errors = prev; }
};

// Clears the Barnes-Hut error word before a step sequence (nothing to clear before
// the first Barnes-Hut call: the walk then clears it itself).
static int clear_bh_errors(pt_ctx *ctx) {
    if (int *e = bh_error_word(ctx)) PT_CUDA(cudaMemsetAsync(e, 0, sizeof(int), ctx->stream));
    return PT_OK;
}

struct State {
    Graph graph;
};

static State *state(pt_ctx *ctx) {
    if (!ctx->lf) ctx->lf = new (std::nothrow) State();
    return static_cast<State *>(ctx->lf);
}

static int accel(pt_ctx *ctx, const float *body, float *acc, size_t n, int method, float theta, float softening,
                 uint32_t flags) {
    if (method == PT_METHOD_BRUTE_FORCE)
        return pt_bf_accel_f32_device(ctx, body, n, body, n, softening, 1, flags, acc);
    return pt_bh_accel_f32_device(ctx, body, n, body, n, theta, softening, flags, acc);
}

// The step sequence (no allocation happens inside when buffers are already grown).
static int enqueue_steps(pt_ctx *ctx, float4 *body, float4 *vel, float *acc, size_t n, float dt, int steps,
                         int method, float theta, float softening, uint32_t flags) {
    const int blocks = int((n + 255) / 256);
    for (int s = 0; s < steps; ++s) {
        kick_drift<<<blocks, 256, 0, ctx->stream>>>(body, vel, acc, int(n), s == 0 ? 0.5f * dt : dt, dt);
        PT_TRY(check_launch(ctx, "kick_drift"));
        PT_TRY(accel(ctx, reinterpret_cast<float *>(body), acc, n, method, theta, softening, flags));
    }
    kick<<<blocks, 256, 0, ctx->stream>>>(vel, acc, int(n), 0.5f * dt);
    return check_launch(ctx, "kick");
}

}  // namespace lf
}  // namespace pt

void pt_lf_state_free(pt_ctx *ctx) {
    auto *S = static_cast<pt::lf::State *>(ctx->lf);
    if (!S) return;
    if (S->graph.exec) cudaGraphExecDestroy(S->graph.exec);
    delete S;
    ctx->lf = nullptr;
}

extern "C" int pt_leapfrog_device(pt_ctx *ctx, float *d_body, float *d_vel, float *d_acc, size_t n, float dt,
                                  int steps, int method, float theta, float softening, uint32_t flags,
                                  int use_graph) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_leapfrog_device: ctx is NULL");
    if (n == 0 || steps <= 0) return PT_OK;
    if (!d_body || !d_vel || !d_acc) return set_error(PT_ERR_INVALID, "pt_leapfrog_device: NULL buffer");
    if (!aligned16(d_body) || !aligned16(d_vel))
        return set_error(PT_ERR_INVALID, "pt_leapfrog_device: bodies and velocities must be 16-byte aligned");
    if (method != PT_METHOD_BRUTE_FORCE && method != PT_METHOD_BARNES_HUT)
        return set_error(PT_ERR_INVALID, "pt_leapfrog_device: unknown method %d", method);
    if (n > size_t(INT_MAX) / 8) return set_error(PT_ERR_INVALID, "pt_leapfrog_device: n=%zu too large", n);
    PT_CUDA(cudaSetDevice(ctx->device));
    lf::State *S = lf::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "leapfrog state allocation failed");
    float4 *body = reinterpret_cast<float4 *>(d_body);
    float4 *vel = reinterpret_cast<float4 *>(d_vel);
    // With the learned correction, record overflows of any step are reported after the
    // sequence (synchronously) as PT_ERR_CAPACITY.
    const bool learned = method == PT_METHOD_BARNES_HUT && (flags & PT_BH_LEARNED);
    lf::KeepErrors keep(ctx);
    if (!use_graph) {
        PT_TRY(lf::clear_bh_errors(ctx));
        PT_TRY(lf::enqueue_steps(ctx, body, vel, d_acc, n, dt, steps, method, theta, softening, flags));
        return learned ? bh_learned_overflow(ctx, "pt_leapfrog_device") : PT_OK;
    }
    lf::Graph &G = S->graph;
    int plan_k = 0, plan_s = 0;
    bf_forced_plan(&plan_k, &plan_s);
    if (!G.same(d_body, d_vel, d_acc, n, steps, method, dt, theta, softening, flags, ctx->stream,
                bh_tuning(ctx), plan_k, plan_s, ctx->buf_epoch)) {
        if (G.exec) {
            cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
        }
        // Grow every buffer the sequence needs before capturing: evaluate the
        // accelerations of the current positions eagerly (the value `acc` must hold
        // on entry anyway), so nothing allocates inside the capture.
        PT_TRY(lf::accel(ctx, d_body, d_acc, n, method, theta, softening, flags));
        PT_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaGraph_t g = nullptr;
        PT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        const uint64_t before = ctx->launches;
        const int rc = lf::enqueue_steps(ctx, body, vel, d_acc, n, dt, steps, method, theta, softening, flags);
        G.kernels = ctx->launches - before;
        ctx->launches = before;  // captured, not run: counted per replay below
        ctx->capturing = false;
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (rc != PT_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        PT_CUDA(ce);
        const cudaError_t ie = cudaGraphInstantiate(&G.exec, g, 0);
        cudaGraphDestroy(g);
        PT_CUDA(ie);
        G.body = d_body;
        G.vel = d_vel;
        G.acc = d_acc;
        G.n = n;
        G.steps = steps;
        G.method = method;
        G.dt = dt;
        G.theta = theta;
        G.softening = softening;
        G.flags = flags;
        G.stream = ctx->stream;
        G.tune = bh_tuning(ctx);
        G.plan_k = plan_k;
        G.plan_s = plan_s;
        G.epoch = ctx->buf_epoch;  // no buffer grows during the capture
    }
    PT_TRY(lf::clear_bh_errors(ctx));
    PT_CUDA(cudaGraphLaunch(G.exec, ctx->stream));
    ctx->launches += G.kernels;  // the kernels the replayed graph runs
    if (learned) {
        const int rc = bh_learned_overflow(ctx, "pt_leapfrog_device");
        if (rc != PT_OK) {
            // captured with too little room for the records: capture again next call
            cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
        }
        return rc;
    }
    return PT_OK;
}

extern "C" int pt_leapfrog(pt_ctx *ctx, float *body, float *vel, size_t n, float dt, int steps, int method,
                           float theta, float softening, uint32_t flags) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_leapfrog: ctx is NULL");
    if (n == 0 || steps <= 0) return PT_OK;
    if (!body || !vel) return set_error(PT_ERR_INVALID, "pt_leapfrog: NULL buffer");
    if (n > size_t(INT_MAX) / 8) return set_error(PT_ERR_INVALID, "pt_leapfrog: n=%zu too large", n);
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_TRY(ensure(ctx, BUF_LF_BODY, 16 * n));
    PT_TRY(ensure(ctx, BUF_LF_VEL, 16 * n));
    PT_TRY(ensure(ctx, BUF_LF_ACC, 12 * n));
    float *d_body = static_cast<float *>(ctx->bufs[BUF_LF_BODY].ptr);
    float *d_vel = static_cast<float *>(ctx->bufs[BUF_LF_VEL].ptr);
    float *d_acc = static_cast<float *>(ctx->bufs[BUF_LF_ACC].ptr);
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(d_body, body, 16 * n, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemcpyAsync(d_vel, vel, 16 * n, cudaMemcpyHostToDevice, st));
    PT_TRY(lf::accel(ctx, d_body, d_acc, n, method, theta, softening, flags));
    PT_TRY(pt_leapfrog_device(ctx, d_body, d_vel, d_acc, n, dt, steps, method, theta, softening, flags, 0));
    PT_CUDA(cudaMemcpyAsync(body, d_body, 16 * n, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaMemcpyAsync(vel, d_vel, 16 * n, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}
