// Training and evaluation of the learned far-field correction (pt_mlp.cuh).
//
// Data: snapshots' trees are walked with the reference opening rule at theta_outer;
// every accepted cell that theta_inner would have opened (a "marginal" cell) yields a
// sample: its features and the residual between the exact sum over the cell's bodies
// (the brute-force pair kernel, compensated) and the cell's monopole + quadrupole
// value, divided by M / |r|^2. The reference has no learned part; the FP64 brute force
// judges what the network gains.
// Training: one fused kernel runs forward and backward for 64 samples per CTA
// (activations in shared memory, BF16-rounded weights, FP32 accumulation) and adds
// its weight gradients to a global buffer; an Adam kernel updates FP32 master
// weights and rewrites their BF16-rounded copies.
#include "pt_common.cuh"
#include "pt_f32x2.cuh"
#include "pt_mlp.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <new>
#include <random>
#include <vector>

namespace pt {
namespace mlp {

constexpr int TB = 64;      // samples per training CTA
constexpr int HP = H + 1;   // padded row stride of activations
constexpr int XP = IN + 1;
constexpr int SMEM_FLOATS = NPARAM + 3 + TB * XP + 4 * TB * HP + TB * 4;

__device__ __forceinline__ uint32_t hash32(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return uint32_t(x);
}

// ---- samples ---------------------------------------------------------------
__global__ void mlp_samples(TreeView tv, int stride, int n_targets, float th_out2, float th_in2, float eps2,
                            float *__restrict__ feat, float *__restrict__ targ, unsigned *__restrict__ count,
                            unsigned cap) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_targets) return;
    const int T = tv.counters[1];
    const float4 p = tv.sbody[size_t(t) * stride];
    int node = 0;
    while (node < T) {
        const float4 A = tv.nodeA[node];
        const int4 B = tv.nodeB[node];
        const float dx = A.x - p.x, dy = A.y - p.y, dz = A.z - p.z;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (d2 == 0.0f) {
            node = B.y;
            continue;
        }
        const float w = __int_as_float(B.x);
        if (B.z < 0 && th_out2 * d2 < w * w) {
            ++node;
            continue;
        }
        if (B.z < 0 && th_in2 * d2 < w * w && A.w > 0.0f) {
            const float4 q0 = tv.nodeQ[2 * node], q1 = tv.nodeQ[2 * node + 1];
            const float q[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
            float f[IN];
            const float r2 = features(p.x, p.y, p.z, A, q, tv.nodeG[node], f);
            // exact: the brute-force pair kernel over the cell's bodies, compensated
            const int2 R = tv.nodeR[node];
            float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
            for (int b = R.x; b < R.y; ++b) {
                const float4 s = tv.sbody[b];
                float ax = 0.f, ay = 0.f, az = 0.f;
                const float ex = s.x - p.x, ey = s.y - p.y, ez = s.z - p.z;
                if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) == 0.0f) continue;
                interact1<false>(s.x, s.y, s.z, s.w, p.x, p.y, p.z, ax, ay, az, eps2);
                two_sum_acc(sx, cx, ax);
                two_sum_acc(sy, cy, ay);
                two_sum_acc(sz, cz, az);
            }
            // monopole + quadrupole, as the walk evaluates them
            const float inv = rsqrt_ftz(d2 + eps2);
            const float inv2 = inv * inv;
            const float sc = (A.w * inv) * inv2;
            const float qx = fmaf(q[0], dx, fmaf(q[1], dy, q[2] * dz));
            const float qy = fmaf(q[1], dx, fmaf(q[3], dy, q[4] * dz));
            const float qz = fmaf(q[2], dx, fmaf(q[4], dy, q[5] * dz));
            const float dqd = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
            const float inv5 = inv2 * inv2 * inv;
            const float c7 = 2.5f * dqd * inv5 * inv2;
            const float apx = fmaf(dx, sc, fmaf(c7, dx, -qx * inv5));
            const float apy = fmaf(dy, sc, fmaf(c7, dy, -qy * inv5));
            const float apz = fmaf(dz, sc, fmaf(c7, dz, -qz * inv5));
            const float norm = r2 / A.w;  // 1 / (M / |r|^2)
            const unsigned slot = atomicAdd(count, 1u);
            if (slot < cap) {
#pragma unroll
                for (int i = 0; i < IN; ++i) feat[size_t(slot) * IN + i] = f[i];
                targ[size_t(slot) * 3 + 0] = ((sx + cx) - apx) * norm;
                targ[size_t(slot) * 3 + 1] = ((sy + cy) - apy) * norm;
                targ[size_t(slot) * 3 + 2] = ((sz + cz) - apz) * norm;
            }
        }
        node = B.y;
    }
}

__global__ void target_power(const float *__restrict__ targ, unsigned n, double *__restrict__ out) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < size_t(n) * 3; i += gridDim.x * size_t(blockDim.x))
        acc += double(targ[i]) * targ[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// ---- training ----------------------------------------------------------------
// P: BF16-rounded parameters (FP32 values). Samples: index[g] if index, else a hash
// of (seed, g) modulo count. grad += d loss / d params; loss += batch loss.
__global__ void __launch_bounds__(TB)
    mlp_fwd_bwd(const float *__restrict__ P, const float *__restrict__ feat, const float *__restrict__ targ,
                const uint32_t *__restrict__ index, unsigned count, int batch, unsigned long long seed,
                float inv_scale, float *__restrict__ grad, double *__restrict__ loss) {
    extern __shared__ float sm[];
    float *sP = sm;
    float *X = sP + NPARAM + 3;
    float *H1 = X + TB * XP;
    float *D1 = H1 + TB * HP;
    float *H2 = D1 + TB * HP;
    float *D2 = H2 + TB * HP;
    float *DY = D2 + TB * HP;
    const int s = threadIdx.x;
    for (int k = s; k < NPARAM; k += TB) sP[k] = P[k];
    const int g = blockIdx.x * TB + s;
    const bool valid = g < batch;
    uint32_t id = 0;
    if (valid) id = index ? index[g] : hash32(seed * 0x9E3779B97F4A7C15ull + uint64_t(g)) % count;
    float t[OUT] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < IN; ++i) X[s * XP + i] = valid ? feat[size_t(id) * IN + i] : 0.f;
#pragma unroll
    for (int c = 0; c < OUT; ++c) t[c] = valid ? targ[size_t(id) * 3 + c] * inv_scale : 0.f;
    __syncthreads();
    // forward (own sample)
    for (int j = 0; j < H; ++j) {
        float z = sP[B1 + j];
#pragma unroll
        for (int i = 0; i < IN; ++i) z = fmaf(sP[W1 + j * IN + i], X[s * XP + i], z);
        float d;
        H1[s * HP + j] = gelu_d(z, d);
        D1[s * HP + j] = d;
    }
    float y[OUT] = {sP[B3], sP[B3 + 1], sP[B3 + 2]};
    for (int j = 0; j < H; ++j) {
        float z = sP[B2 + j];
#pragma unroll 16
        for (int i = 0; i < H; ++i) z = fmaf(sP[W2 + j * H + i], H1[s * HP + i], z);
        float d;
        const float h = gelu_d(z, d);
        H2[s * HP + j] = h;
        D2[s * HP + j] = d;
#pragma unroll
        for (int c = 0; c < OUT; ++c) y[c] = fmaf(sP[W3 + c * H + j], h, y[c]);
    }
    float l = 0.f;
    float dy[OUT];
#pragma unroll
    for (int c = 0; c < OUT; ++c) {
        const float e = y[c] - t[c];
        dy[c] = valid ? 2.0f * e / float(batch) : 0.f;
        l += valid ? e * e / float(batch) : 0.f;
        DY[s * 4 + c] = dy[c];
    }
    // G2 = (W3^T dy) o gelu'(z2), stored over D2
    for (int j = 0; j < H; ++j) {
        const float a = fmaf(sP[W3 + j], dy[0], fmaf(sP[W3 + H + j], dy[1], sP[W3 + 2 * H + j] * dy[2]));
        D2[s * HP + j] *= a;
    }
    // G1 = (W2^T G2) o gelu'(z1), stored over D1
    for (int i = 0; i < H; ++i) {
        float a = 0.f;
#pragma unroll 16
        for (int j = 0; j < H; ++j) a = fmaf(sP[W2 + j * H + i], D2[s * HP + j], a);
        D1[s * HP + i] *= a;
    }
    __syncthreads();
    // weight gradients: thread j owns row j of W1 and W2 and column j of W3
    const int j = s;
    float gb1 = 0.f, gb2 = 0.f;
    float gw1[IN];
#pragma unroll
    for (int i = 0; i < IN; ++i) gw1[i] = 0.f;
    float gw3[OUT] = {0.f, 0.f, 0.f};
    for (int r = 0; r < TB; ++r) {
        const float g1 = D1[r * HP + j];
        gb1 += g1;
#pragma unroll
        for (int i = 0; i < IN; ++i) gw1[i] = fmaf(g1, X[r * XP + i], gw1[i]);
        const float h2 = H2[r * HP + j];
#pragma unroll
        for (int c = 0; c < OUT; ++c) gw3[c] = fmaf(DY[r * 4 + c], h2, gw3[c]);
        gb2 += D2[r * HP + j];
    }
#pragma unroll
    for (int i = 0; i < IN; ++i) atomicAdd(grad + W1 + j * IN + i, gw1[i]);
    atomicAdd(grad + B1 + j, gb1);
    atomicAdd(grad + B2 + j, gb2);
#pragma unroll
    for (int c = 0; c < OUT; ++c) atomicAdd(grad + W3 + c * H + j, gw3[c]);
    for (int i = 0; i < H; ++i) {
        float a = 0.f;
        for (int r = 0; r < TB; ++r) a = fmaf(D2[r * HP + j], H1[r * HP + i], a);
        atomicAdd(grad + W2 + j * H + i, a);
    }
    if (s < OUT) {
        float a = 0.f;
        for (int r = 0; r < TB; ++r) a += DY[r * 4 + s];
        atomicAdd(grad + B3 + s, a);
    }
    // batch loss
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((s & 31) == 0) atomicAdd(loss, double(l));
}

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Adam on the FP32 master weights; P receives their BF16-rounded copies. The output
// scale is not trained.
__global__ void mlp_adam(float *__restrict__ master, float *__restrict__ P, float *__restrict__ grad,
                         float *__restrict__ m1, float *__restrict__ m2, float lr, float b1, float b2, float eps,
                         float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= SCALE) return;
    const float gk = grad[k];
    grad[k] = 0.f;
    const float a = b1 * m1[k] + (1.f - b1) * gk;
    const float v = b2 * m2[k] + (1.f - b2) * gk * gk;
    m1[k] = a;
    m2[k] = v;
    const float w = master[k] - lr * (a / c1) / (sqrtf(v / c2) + eps);
    master[k] = w;
    P[k] = bf16_round(w);
}

__global__ void mlp_predict(const float *__restrict__ P, const float *__restrict__ feat, int n,
                            float *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float f[IN];
#pragma unroll
    for (int i = 0; i < IN; ++i) f[i] = feat[size_t(s) * IN + i];
    float o[OUT];
    forward<false>(P, f, o);
#pragma unroll
    for (int c = 0; c < OUT; ++c) out[size_t(s) * 3 + c] = o[c];
}

// FP32 parameters (BF16 values) -> BF16 pairs in B-fragment order + bias block.
__global__ void mlp_pack_tc(const float *__restrict__ P, uint32_t *__restrict__ W, float *__restrict__ bias) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < TC_WORDS) {
        int layer, n, p;
        tc_word_source(k, layer, n, p);
        float lo = 0.f, hi = 0.f;
        if (layer == 1) {
            lo = 2 * p < IN ? P[W1 + n * IN + 2 * p] : 0.f;
            hi = 2 * p + 1 < IN ? P[W1 + n * IN + 2 * p + 1] : 0.f;
        } else if (layer == 2) {
            lo = P[W2 + n * H + 2 * p];
            hi = P[W2 + n * H + 2 * p + 1];
        } else if (n < OUT) {
            lo = P[W3 + n * H + 2 * p];
            hi = P[W3 + n * H + 2 * p + 1];
        }
        W[k] = pack_bf16(lo, hi);
    }
    if (k < 64) {
        bias[k] = P[B1 + k];
        bias[64 + k] = P[B2 + k];
    }
    if (k < 8) bias[128 + k] = k < OUT ? P[B3 + k] : 0.f;
    if (k == 0) bias[TC_SCALE] = P[SCALE];
}

// Tensor-core predictions per cell (the walk's inference path), 32 rows per warp.
__global__ void mlp_predict_tc(const uint32_t *__restrict__ W, const float *__restrict__ bias,
                               const float *__restrict__ feat, int n, float *__restrict__ out) {
    __shared__ float X[4][32 * TC_XS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = (blockIdx.x * 4 + warp) * 32;
    if (row0 >= n) return;
    const int r = row0 + lane;
    for (int i = 0; i < 16; ++i) X[warp][lane * TC_XS + i] = (r < n && i < IN) ? feat[size_t(r) * IN + i] : 0.f;
    __syncwarp();
    float y[2][4];
    tc_batch(X[warp], W, bias, y);
    const int g = lane >> 2, t = lane & 3;
    const float sc = bias[TC_SCALE];
    for (int mt = 0; mt < 2; ++mt)
        for (int h = 0; h < 2; ++h) {
            const int row = row0 + 16 * mt + g + 8 * h;
            for (int c = 0; c < 2; ++c) {
                const int col = 2 * t + c;
                if (row < n && col < OUT) out[size_t(row) * 3 + col] = y[mt][2 * h + c] * sc;
            }
        }
}

struct State;
static int install(pt_ctx *ctx, State &S);

struct State {
    DevBuf master, params, grad, m1, m2, loss, feat, targ, count, power, scratch, tcw, tcb;
    unsigned cap = 0;
    long long adam_t = 0;
    float theta_inner = 0.5f;
    bool initialised = false;
};

static State *state(pt_ctx *ctx) {
    if (!ctx->mlp) ctx->mlp = new (std::nothrow) State();
    return static_cast<State *>(ctx->mlp);
}

static int ensure_params(pt_ctx *ctx, State &S) {
    const size_t b = sizeof(float) * NPARAM;
    PT_TRY(ensure_buf(ctx, S.master, b));
    PT_TRY(ensure_buf(ctx, S.params, b));
    PT_TRY(ensure_buf(ctx, S.grad, b));
    PT_TRY(ensure_buf(ctx, S.m1, b));
    PT_TRY(ensure_buf(ctx, S.m2, b));
    PT_TRY(ensure_buf(ctx, S.loss, sizeof(double) * 2));
    return PT_OK;
}

static int upload(pt_ctx *ctx, State &S, const std::vector<float> &host) {
    PT_TRY(ensure_params(ctx, S));
    std::vector<float> rounded(host);
    for (int k = 0; k < SCALE; ++k) rounded[k] = __bfloat162float(__float2bfloat16_rn(host[k]));
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(S.master.ptr, host.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemcpyAsync(S.params.ptr, rounded.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemsetAsync(S.grad.ptr, 0, sizeof(float) * NPARAM, st));
    PT_CUDA(cudaMemsetAsync(S.m1.ptr, 0, sizeof(float) * NPARAM, st));
    PT_CUDA(cudaMemsetAsync(S.m2.ptr, 0, sizeof(float) * NPARAM, st));
    PT_CUDA(cudaStreamSynchronize(st));
    S.adam_t = 0;
    S.initialised = true;
    return install(ctx, S);
}

// Packs the current parameters for the tensor-core path and hands them to the walk.
static int install(pt_ctx *ctx, State &S) {
    PT_TRY(ensure_buf(ctx, S.tcw, sizeof(uint32_t) * TC_WORDS));
    PT_TRY(ensure_buf(ctx, S.tcb, sizeof(float) * TC_BIAS));
    mlp_pack_tc<<<(TC_WORDS + 255) / 256, 256, 0, ctx->stream>>>(static_cast<const float *>(S.params.ptr),
                                                                 static_cast<uint32_t *>(S.tcw.ptr),
                                                                 static_cast<float *>(S.tcb.ptr));
    PT_TRY(check_launch(ctx, "mlp_pack_tc"));
    return bh_set_mlp(ctx, static_cast<const uint32_t *>(S.tcw.ptr), static_cast<const float *>(S.tcb.ptr),
                      S.theta_inner);
}

}  // namespace mlp

// Builds the Barnes-Hut tree of d_src (defined with the Barnes-Hut build).
int bh_build_only(pt_ctx *ctx, const float4 *d_src, int n);

}  // namespace pt

void pt_mlp_state_free(pt_ctx *ctx) {
    auto *S = static_cast<pt::mlp::State *>(ctx->mlp);
    if (!S) return;
    pt::DevBuf *all[] = {&S->master, &S->params, &S->grad, &S->m1, &S->m2, &S->loss,
                         &S->feat, &S->targ, &S->count, &S->power, &S->scratch, &S->tcw, &S->tcb};
    for (auto *b : all) pt::free_buf(ctx, *b);
    delete S;
    ctx->mlp = nullptr;
}

extern "C" {

int pt_mlp_init(pt_ctx *ctx, uint64_t seed) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_mlp_init: ctx is NULL");
    PT_CUDA(cudaSetDevice(ctx->device));
    mlp::State *S = mlp::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "mlp state allocation failed");
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> h(mlp::NPARAM, 0.f);
    // He initialisation for the hidden layers; the output layer starts at zero, so
    // an untrained model predicts no correction.
    const float s1 = std::sqrt(2.f / mlp::IN), s2 = std::sqrt(2.f / mlp::H);
    for (int k = 0; k < mlp::H * mlp::IN; ++k) h[mlp::W1 + k] = s1 * nd(rng);
    for (int k = 0; k < mlp::H * mlp::H; ++k) h[mlp::W2 + k] = s2 * nd(rng);
    h[mlp::SCALE] = 1.f;
    return mlp::upload(ctx, *S, h);
}

int pt_mlp_set_params(pt_ctx *ctx, const float *params, size_t n, float theta_inner) {
    using namespace pt;
    clear_error();
    if (!ctx || !params) return set_error(PT_ERR_INVALID, "pt_mlp_set_params: NULL argument");
    if (n != size_t(mlp::NPARAM))
        return set_error(PT_ERR_INVALID, "pt_mlp_set_params: expected %d parameters, got %zu", mlp::NPARAM, n);
    PT_CUDA(cudaSetDevice(ctx->device));
    mlp::State *S = mlp::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "mlp state allocation failed");
    S->theta_inner = theta_inner;
    return mlp::upload(ctx, *S, std::vector<float>(params, params + n));
}

int pt_mlp_get_params(pt_ctx *ctx, float *params, size_t n) {
    using namespace pt;
    clear_error();
    if (!ctx || !params || n != size_t(mlp::NPARAM))
        return set_error(PT_ERR_INVALID, "pt_mlp_get_params: bad arguments");
    auto *S = static_cast<mlp::State *>(ctx->mlp);
    if (!S || !S->initialised) return set_error(PT_ERR_INVALID, "pt_mlp_get_params: no model");
    PT_CUDA(cudaSetDevice(ctx->device));
    PT_CUDA(cudaMemcpyAsync(params, S->params.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

// Appends the samples of one snapshot (bodies on the device) to the dataset.
int pt_mlp_generate(pt_ctx *ctx, const float *d_bodies, size_t n, int n_targets, float theta_outer,
                    float theta_inner, float softening, size_t capacity, size_t *total) {
    using namespace pt;
    clear_error();
    if (!ctx || !d_bodies || !total) return set_error(PT_ERR_INVALID, "pt_mlp_generate: NULL argument");
    if (n < 2 || n > size_t(INT_MAX / 8) || n_targets <= 0 || capacity == 0 || capacity > (size_t(1) << 31))
        return set_error(PT_ERR_INVALID, "pt_mlp_generate: bad sizes");
    if (!aligned16(d_bodies)) return set_error(PT_ERR_INVALID, "pt_mlp_generate: bodies must be 16-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    mlp::State *S = mlp::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "mlp state allocation failed");
    if (!S->feat.ptr || S->cap != unsigned(capacity)) {
        PT_TRY(ensure_buf(ctx, S->feat, sizeof(float) * mlp::IN * capacity));
        PT_TRY(ensure_buf(ctx, S->targ, sizeof(float) * 3 * capacity));
        PT_TRY(ensure_buf(ctx, S->count, sizeof(unsigned)));
        PT_CUDA(cudaMemsetAsync(S->count.ptr, 0, sizeof(unsigned), ctx->stream));
        S->cap = unsigned(capacity);
    }
    S->theta_inner = theta_inner;
    PT_TRY(bh_build_only(ctx, reinterpret_cast<const float4 *>(d_bodies), int(n)));
    TreeView tv;
    PT_TRY(bh_tree_view(ctx, &tv));
    const int nt = std::min<int>(n_targets, int(n));
    const int stride = int(n / size_t(nt));
    mlp::mlp_samples<<<(nt + 127) / 128, 128, 0, ctx->stream>>>(
        tv, stride, nt, theta_outer * theta_outer, theta_inner * theta_inner, softening * softening,
        static_cast<float *>(S->feat.ptr), static_cast<float *>(S->targ.ptr), static_cast<unsigned *>(S->count.ptr),
        S->cap);
    PT_TRY(check_launch(ctx, "mlp_samples"));
    unsigned c = 0;
    PT_CUDA(cudaMemcpyAsync(&c, S->count.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    *total = std::min(c, S->cap);
    return PT_OK;
}

int pt_mlp_reset_dataset(pt_ctx *ctx) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_mlp_reset_dataset: ctx is NULL");
    auto *S = static_cast<mlp::State *>(ctx->mlp);
    if (S && S->count.ptr) PT_CUDA(cudaMemsetAsync(S->count.ptr, 0, sizeof(unsigned), ctx->stream));
    return PT_OK;
}

// Copies the first n samples out (features n x 12, targets n x 3).
int pt_mlp_export_dataset(pt_ctx *ctx, float *features, float *targets, size_t n) {
    using namespace pt;
    clear_error();
    auto *S = ctx ? static_cast<mlp::State *>(ctx->mlp) : nullptr;
    if (!S || !S->feat.ptr || n > S->cap) return set_error(PT_ERR_INVALID, "pt_mlp_export_dataset: no such data");
    if (features)
        PT_CUDA(cudaMemcpyAsync(features, S->feat.ptr, sizeof(float) * mlp::IN * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (targets)
        PT_CUDA(cudaMemcpyAsync(targets, S->targ.ptr, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

// Trains on the dataset for `steps` Adam steps of `batch` random samples. The first
// call after initialisation sets the output scale to the targets' RMS. loss_out
// receives the mean loss of the last 10% of steps (in scaled units).
int pt_mlp_train(pt_ctx *ctx, int steps, int batch, float lr, uint64_t seed, float *loss_out) {
    using namespace pt;
    clear_error();
    auto *S = ctx ? static_cast<mlp::State *>(ctx->mlp) : nullptr;
    if (!S || !S->initialised) return set_error(PT_ERR_INVALID, "pt_mlp_train: initialise the model first");
    if (!S->feat.ptr) return set_error(PT_ERR_INVALID, "pt_mlp_train: no dataset");
    if (steps <= 0 || batch <= 0 || batch > (1 << 22)) return set_error(PT_ERR_INVALID, "pt_mlp_train: bad sizes");
    PT_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    unsigned count = 0;
    PT_CUDA(cudaMemcpyAsync(&count, S->count.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    count = std::min(count, S->cap);
    if (count == 0) return set_error(PT_ERR_INVALID, "pt_mlp_train: empty dataset");
    // output scale = RMS of the targets (fixed once per model)
    float scale = 1.f;
    PT_CUDA(cudaMemcpyAsync(&scale, static_cast<float *>(S->params.ptr) + mlp::SCALE, sizeof(float),
                            cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (S->adam_t == 0) {
        PT_TRY(ensure_buf(ctx, S->power, sizeof(double)));
        PT_CUDA(cudaMemsetAsync(S->power.ptr, 0, sizeof(double), st));
        mlp::target_power<<<256, 256, 0, st>>>(static_cast<float *>(S->targ.ptr), count,
                                               static_cast<double *>(S->power.ptr));
        PT_TRY(check_launch(ctx, "target_power"));
        double pw = 0.0;
        PT_CUDA(cudaMemcpyAsync(&pw, S->power.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
        PT_CUDA(cudaStreamSynchronize(st));
        scale = float(std::sqrt(pw / (3.0 * count)));
        if (!(scale > 0.f)) scale = 1.f;
        PT_CUDA(cudaMemcpyAsync(static_cast<float *>(S->params.ptr) + mlp::SCALE, &scale, sizeof(float),
                                cudaMemcpyHostToDevice, st));
        PT_CUDA(cudaMemcpyAsync(static_cast<float *>(S->master.ptr) + mlp::SCALE, &scale, sizeof(float),
                                cudaMemcpyHostToDevice, st));
    }
    const size_t smem = sizeof(float) * mlp::SMEM_FLOATS;
    PT_CUDA(cudaFuncSetAttribute(mlp::mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int blocks = (batch + mlp::TB - 1) / mlp::TB;
    double *loss = static_cast<double *>(S->loss.ptr);
    double loss_sum = 0.0;
    int loss_n = 0;
    const int tail = std::max(1, steps / 10);
    for (int k = 0; k < steps; ++k) {
        PT_CUDA(cudaMemsetAsync(loss, 0, sizeof(double), st));
        mlp::mlp_fwd_bwd<<<blocks, mlp::TB, smem, st>>>(
            static_cast<const float *>(S->params.ptr), static_cast<const float *>(S->feat.ptr),
            static_cast<const float *>(S->targ.ptr), nullptr, count, batch, seed + uint64_t(k) * 7919u,
            1.f / scale, static_cast<float *>(S->grad.ptr), loss);
        PT_TRY(check_launch(ctx, "mlp_fwd_bwd"));
        ++S->adam_t;
        const float c1 = 1.f - std::pow(0.9f, float(S->adam_t)), c2 = 1.f - std::pow(0.999f, float(S->adam_t));
        mlp::mlp_adam<<<(mlp::SCALE + 255) / 256, 256, 0, st>>>(
            static_cast<float *>(S->master.ptr), static_cast<float *>(S->params.ptr),
            static_cast<float *>(S->grad.ptr), static_cast<float *>(S->m1.ptr), static_cast<float *>(S->m2.ptr), lr,
            0.9f, 0.999f, 1e-8f, c1, c2);
        PT_TRY(check_launch(ctx, "mlp_adam"));
        if (k >= steps - tail) {
            double l = 0.0;
            PT_CUDA(cudaMemcpyAsync(&l, loss, sizeof(double), cudaMemcpyDeviceToHost, st));
            PT_CUDA(cudaStreamSynchronize(st));
            loss_sum += l;
            ++loss_n;
        }
    }
    PT_CUDA(cudaStreamSynchronize(st));
    if (loss_out) *loss_out = float(loss_sum / std::max(1, loss_n));
    return mlp::install(ctx, *S);
}

// Loss and its gradient for host samples (features b x 12, targets b x 3) at the
// current parameters: the check of the training kernel. grad has NPARAM floats
// (the scale entry is 0); targets are divided by the model's output scale.
int pt_mlp_loss_grad(pt_ctx *ctx, const float *features, const float *targets, int batch, float *grad,
                     double *loss_out) {
    using namespace pt;
    clear_error();
    auto *S = ctx ? static_cast<mlp::State *>(ctx->mlp) : nullptr;
    if (!S || !S->initialised || !features || !targets || !grad || batch <= 0)
        return set_error(PT_ERR_INVALID, "pt_mlp_loss_grad: bad arguments");
    PT_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t need = sizeof(float) * size_t(batch) * (mlp::IN + 3) + sizeof(uint32_t) * size_t(batch);
    PT_TRY(ensure_buf(ctx, S->scratch, need));
    float *f = static_cast<float *>(S->scratch.ptr);
    float *t = f + size_t(batch) * mlp::IN;
    uint32_t *idx = reinterpret_cast<uint32_t *>(t + size_t(batch) * 3);
    std::vector<uint32_t> iota(batch);
    for (int i = 0; i < batch; ++i) iota[i] = uint32_t(i);
    PT_CUDA(cudaMemcpyAsync(f, features, sizeof(float) * batch * mlp::IN, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemcpyAsync(t, targets, sizeof(float) * batch * 3, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemcpyAsync(idx, iota.data(), sizeof(uint32_t) * batch, cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemsetAsync(S->grad.ptr, 0, sizeof(float) * mlp::NPARAM, st));
    PT_CUDA(cudaMemsetAsync(S->loss.ptr, 0, sizeof(double), st));
    float scale = 1.f;
    PT_CUDA(cudaMemcpyAsync(&scale, static_cast<float *>(S->params.ptr) + mlp::SCALE, sizeof(float),
                            cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    const size_t smem = sizeof(float) * mlp::SMEM_FLOATS;
    PT_CUDA(cudaFuncSetAttribute(mlp::mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    mlp::mlp_fwd_bwd<<<(batch + mlp::TB - 1) / mlp::TB, mlp::TB, smem, st>>>(
        static_cast<const float *>(S->params.ptr), f, t, idx, unsigned(batch), batch, 0ull, 1.f / scale,
        static_cast<float *>(S->grad.ptr), static_cast<double *>(S->loss.ptr));
    PT_TRY(check_launch(ctx, "mlp_fwd_bwd"));
    PT_CUDA(cudaMemcpyAsync(grad, S->grad.ptr, sizeof(float) * mlp::NPARAM, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaMemcpyAsync(loss_out, S->loss.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaMemsetAsync(S->grad.ptr, 0, sizeof(float) * mlp::NPARAM, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}

// The same predictions through the walk's tensor-core path (BF16 activations).
int pt_mlp_predict_tc(pt_ctx *ctx, const float *features, int n, float *out) {
    using namespace pt;
    clear_error();
    auto *S = ctx ? static_cast<mlp::State *>(ctx->mlp) : nullptr;
    if (!S || !S->initialised || !S->tcw.ptr || !features || !out || n <= 0)
        return set_error(PT_ERR_INVALID, "pt_mlp_predict_tc: bad arguments");
    PT_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    PT_TRY(ensure_buf(ctx, S->scratch, sizeof(float) * size_t(n) * (mlp::IN + 3)));
    float *f = static_cast<float *>(S->scratch.ptr);
    float *o = f + size_t(n) * mlp::IN;
    PT_CUDA(cudaMemcpyAsync(f, features, sizeof(float) * size_t(n) * mlp::IN, cudaMemcpyHostToDevice, st));
    mlp::mlp_predict_tc<<<(n + 127) / 128, 128, 0, st>>>(static_cast<const uint32_t *>(S->tcw.ptr),
                                                         static_cast<const float *>(S->tcb.ptr), f, n, o);
    PT_TRY(check_launch(ctx, "mlp_predict_tc"));
    PT_CUDA(cudaMemcpyAsync(out, o, sizeof(float) * size_t(n) * 3, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}

// Predictions (n x 3, residual / (M / |r|^2)) for host features (n x 12).
int pt_mlp_predict(pt_ctx *ctx, const float *features, int n, float *out) {
    using namespace pt;
    clear_error();
    auto *S = ctx ? static_cast<mlp::State *>(ctx->mlp) : nullptr;
    if (!S || !S->initialised || !features || !out || n <= 0)
        return set_error(PT_ERR_INVALID, "pt_mlp_predict: bad arguments");
    PT_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    PT_TRY(ensure_buf(ctx, S->scratch, sizeof(float) * size_t(n) * (mlp::IN + 3)));
    float *f = static_cast<float *>(S->scratch.ptr);
    float *o = f + size_t(n) * mlp::IN;
    PT_CUDA(cudaMemcpyAsync(f, features, sizeof(float) * size_t(n) * mlp::IN, cudaMemcpyHostToDevice, st));
    mlp::mlp_predict<<<(n + 127) / 128, 128, 0, st>>>(static_cast<const float *>(S->params.ptr), f, n, o);
    PT_TRY(check_launch(ctx, "mlp_predict"));
    PT_CUDA(cudaMemcpyAsync(out, o, sizeof(float) * size_t(n) * 3, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}

}  // extern "C"
