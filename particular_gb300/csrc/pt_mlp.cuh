// The learned far-field correction: a 12 -> 64 -> 64 -> 3 MLP with GELU (tanh
// form) that predicts, for a Barnes-Hut cell accepted at a loose opening angle, the
// residual between the exact sum over the cell's bodies and the cell's monopole +
// quadrupole value, from features in the cell's frame:
//   f[0..2]  unit offset r / |r|, r = target - centre of mass
//   f[3]     size / distance ratio w / |r|
//   f[4..8]  traceless quadrupole / (M w^2): Qxx, Qxy, Qxz, Qyy, Qyz (Qzz = -Qxx-Qyy)
//   f[9..11] (centre of mass - geometric centre of the cell) / w
// output    residual / (M / |r|^2), global axes.
// Parameters are FP32 copies of BF16 values (the model's weights are BF16; all
// arithmetic accumulates in FP32). Layout of the flat parameter vector:
#pragma once

#include "pt_common.cuh"

namespace pt {
namespace mlp {

constexpr int IN = 12, H = 64, OUT = 3;
constexpr int W1 = 0;                // [H][IN]
constexpr int B1 = W1 + H * IN;      // [H]
constexpr int W2 = B1 + H;           // [H][H]
constexpr int B2 = W2 + H * H;       // [H]
constexpr int W3 = B2 + H;           // [OUT][H]
constexpr int B3 = W3 + OUT * H;     // [OUT]
constexpr int SCALE = B3 + OUT;      // output scale (targets were divided by it)
constexpr int NPARAM = SCALE + 1;    // 5188 (PT_MLP_NPARAM)
static_assert(NPARAM == PT_MLP_NPARAM, "parameter count");

constexpr float GELU_C = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float GELU_A = 0.044715f;

__device__ __forceinline__ float tanh_fast(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// gelu(x) = x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
template <bool FAST>
__device__ __forceinline__ float gelu(float x) {
    const float u = GELU_C * fmaf(GELU_A * x, x * x, x);
    const float t = FAST ? tanh_fast(u) : tanhf(u);
    return 0.5f * x * (1.0f + t);
}

// gelu and its derivative
__device__ __forceinline__ float gelu_d(float x, float &d) {
    const float x2 = x * x;
    const float u = GELU_C * fmaf(GELU_A * x, x2, x);
    const float t = tanhf(u);
    d = 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_C * fmaf(3.0f * GELU_A, x2, 1.0f);
    return 0.5f * x * (1.0f + t);
}

// Features of target p for a cell (com, mass m, quadrupole q[6] = Qxx Qxy Qxz Qyy Qyz
// Qzz, geometric centre g, width w). Returns |r|^2.
__device__ __forceinline__ float features(float px, float py, float pz, float4 com, const float *q, float4 g,
                                          float *f) {
    const float rx = px - com.x, ry = py - com.y, rz = pz - com.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float ir = rsqrtf(r2);
    const float w = g.w;
    f[0] = rx * ir;
    f[1] = ry * ir;
    f[2] = rz * ir;
    f[3] = w * ir;
    const float qs = 1.0f / (com.w * w * w);
    f[4] = q[0] * qs;
    f[5] = q[1] * qs;
    f[6] = q[2] * qs;
    f[7] = q[3] * qs;
    f[8] = q[4] * qs;
    const float iw = 1.0f / w;
    f[9] = (com.x - g.x) * iw;
    f[10] = (com.y - g.y) * iw;
    f[11] = (com.z - g.z) * iw;
    return r2;
}

// Forward pass with parameters P (any address space the caller chooses). out[3] is
// the predicted residual / (M / |r|^2).
template <bool FAST, class Params>
__device__ __forceinline__ void forward(const Params &P, const float *f, float *out) {
    float h1[H];
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
        float z = P[B1 + j];
#pragma unroll
        for (int i = 0; i < IN; ++i) z = fmaf(P[W1 + j * IN + i], f[i], z);
        h1[j] = gelu<FAST>(z);
    }
    float y0 = P[B3 + 0], y1 = P[B3 + 1], y2 = P[B3 + 2];
#pragma unroll 2
    for (int j = 0; j < H; ++j) {
        float z = P[B2 + j];
#pragma unroll 16
        for (int i = 0; i < H; ++i) z = fmaf(P[W2 + j * H + i], h1[i], z);
        const float h2 = gelu<FAST>(z);
        y0 = fmaf(P[W3 + 0 * H + j], h2, y0);
        y1 = fmaf(P[W3 + 1 * H + j], h2, y1);
        y2 = fmaf(P[W3 + 2 * H + j], h2, y2);
    }
    const float sc = P[SCALE];
    out[0] = y0 * sc;
    out[1] = y1 * sc;
    out[2] = y2 * sc;
}

}  // namespace mlp

// Raw device pointers to the last Barnes-Hut tree of a context (preorder).
struct TreeView {
    const float4 *nodeA;  // centre of mass, mass
    const int4 *nodeB;    // width bits, skip, first body (-1 = cell), body count
    const float4 *nodeQ;  // 2 per node: Qxx Qxy Qxz Qyy | Qyz Qzz
    const float4 *nodeG;  // cell centre, width
    const int2 *nodeR;    // bodies [x, y) in key order
    const float4 *sbody;  // bodies in key order
    const int *counters;  // [0] leaves, [1] nodes
    int n_src;
};
int bh_tree_view(pt_ctx *ctx, TreeView *out);
// Installs the packed tensor-core weights and bias block for PT_BH_LEARNED.
int bh_set_mlp(pt_ctx *ctx, const uint32_t *d_tc_weights, const float *d_tc_bias, float theta_inner);

}  // namespace pt

// ---- tensor-core inference (mma.sync m16n8k16, BF16 x BF16 -> FP32) -----------
// A warp evaluates 32 cells at once: rows = cells (two m16 tiles), the layers are
// [32 x 16] x [16 x 64], [32 x 64] x [64 x 64], [32 x 64] x [64 x 8]. The FP32
// accumulator fragment of one layer is, register for register, the BF16 A fragment
// of the next after GELU, so activations never leave registers. Weights are stored
// pre-swizzled in B-fragment order, so a lane fetches its fragments with 64- and
// 128-bit loads (g = lane / 4, t = lane % 4, pair p = BF16 weights of k = 2p, 2p+1
// for output n):
//   W1f [8 n-tiles][32 lanes] uint2  {p = t, p = 4 + t} of n = 8 nt + g (k >= 12 zero)
//   W2f [8 n-tiles][32 lanes] 2 uint4 {8 kt + t, 8 kt + 4 + t} for kt = 0..3
//   W3f [32 lanes] 2 uint4, n = g (n >= 3 zero)
// bias block: b1[64], b2[64], b3[8], scale.
namespace pt {
namespace mlp {

constexpr int TC_W1 = 0, TC_W2 = 8 * 32 * 2, TC_W3 = TC_W2 + 8 * 32 * 8;
constexpr int TC_WORDS = TC_W3 + 32 * 8;  // uint32 words of packed weights (2816)
constexpr int TC_BIAS = 64 + 64 + 8 + 1;
constexpr int TC_SCALE = 136;  // output scale within the bias block
constexpr int TC_XS = 17;      // row stride (floats) of a batch's features in shared memory

// Packed word k of the fragment layout above, from the flat FP32 parameters.
__host__ __device__ inline void tc_word_source(int k, int &layer, int &n, int &p) {
    int lane, pr;
    if (k < TC_W2) {
        const int nt = k / 64;
        lane = (k / 2) % 32;
        pr = (k % 2) * 4;
        layer = 1;
        n = 8 * nt + lane / 4;
    } else if (k < TC_W3) {
        const int q = k - TC_W2, w = q % 8;
        lane = (q / 8) % 32;
        pr = 8 * (w / 2) + (w % 2) * 4;
        layer = 2;
        n = 8 * (q / 256) + lane / 4;
    } else {
        const int q = k - TC_W3, w = q % 8;
        lane = q / 8;
        pr = 8 * (w / 2) + (w % 2) * 4;
        layer = 3;
        n = lane / 4;
    }
    p = pr + lane % 4;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Fragment loads the compiler may not hoist out of a caller's loop (the walk calls
// tc_batch inside its traversal loop; hoisted, the 88 weight words would stay live
// in registers across the whole walk).
__device__ __forceinline__ uint4 ld4(const uint4 *p) {
    uint4 v;
    asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld2(const uint2 *p) {
    uint2 v;
    asm volatile("ld.global.nc.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ float2 ld2f(const float2 *p) {
    float2 v;
    asm volatile("ld.global.nc.v2.f32 {%0,%1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}

// X: this warp's [32][TC_XS] features in shared memory (16 used: 12 features, then
// zeros; rows without a cell all zero).
// y[mt][4]: outputs of rows (16 mt + g, 16 mt + g + 8), columns (2t, 2t + 1), before
// the output scale.
__device__ __forceinline__ void tc_batch(const float *__restrict__ X, const uint32_t *__restrict__ W,
                                         const float *__restrict__ bias, float (&y)[2][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint2 *W1f = reinterpret_cast<const uint2 *>(W + TC_W1) + lane;
    const uint4 *W2f = reinterpret_cast<const uint4 *>(W + TC_W2) + 2 * lane;
    const uint4 *W3f = reinterpret_cast<const uint4 *>(W + TC_W3) + 2 * lane;
    const float2 *b1 = reinterpret_cast<const float2 *>(bias) + t;
    const float2 *b2 = reinterpret_cast<const float2 *>(bias + 64) + t;
    const float2 b3 = ld2f(reinterpret_cast<const float2 *>(bias + 128) + t);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const float *r0 = X + (16 * mt + g) * TC_XS, *r1 = r0 + 8 * TC_XS;
        const uint32_t a[4] = {pack_bf16(r0[2 * t], r0[2 * t + 1]), pack_bf16(r1[2 * t], r1[2 * t + 1]),
                               pack_bf16(r0[8 + 2 * t], r0[9 + 2 * t]), pack_bf16(r1[8 + 2 * t], r1[9 + 2 * t])};
        // layer 1 -> A fragments of layer 2 (k tile kt = hidden units 16 kt .. 16 kt + 15)
        uint32_t h1[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float2 bb = ld2f(b1 + 4 * nt);
            float c[4] = {bb.x, bb.y, bb.x, bb.y};
            const uint2 w = ld2(W1f + 32 * nt);
            mma_bf16(c, a, w.x, w.y);
            const int kt = nt >> 1, hi = (nt & 1) * 2;
            h1[kt][hi] = pack_bf16(gelu<true>(c[0]), gelu<true>(c[1]));
            h1[kt][hi + 1] = pack_bf16(gelu<true>(c[2]), gelu<true>(c[3]));
        }
        // layer 2 -> A fragments of layer 3
        uint32_t h2[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float2 bb = ld2f(b2 + 4 * nt);
            float c[4] = {bb.x, bb.y, bb.x, bb.y};
            const uint4 u0 = ld4(W2f + 64 * nt), u1 = ld4(W2f + 64 * nt + 1);
            mma_bf16(c, h1[0], u0.x, u0.y);
            mma_bf16(c, h1[1], u0.z, u0.w);
            mma_bf16(c, h1[2], u1.x, u1.y);
            mma_bf16(c, h1[3], u1.z, u1.w);
            const int kt = nt >> 1, hi = (nt & 1) * 2;
            h2[kt][hi] = pack_bf16(gelu<true>(c[0]), gelu<true>(c[1]));
            h2[kt][hi + 1] = pack_bf16(gelu<true>(c[2]), gelu<true>(c[3]));
        }
        // layer 3 (columns 0..2 used)
        float c[4] = {b3.x, b3.y, b3.x, b3.y};
        const uint4 u0 = ld4(W3f), u1 = ld4(W3f + 1);
        mma_bf16(c, h2[0], u0.x, u0.y);
        mma_bf16(c, h2[1], u0.z, u0.w);
        mma_bf16(c, h2[2], u1.x, u1.y);
        mma_bf16(c, h2[3], u1.z, u1.w);
#pragma unroll
        for (int k = 0; k < 4; ++k) y[mt][k] = c[k];
    }
}

}  // namespace mlp
}  // namespace pt
