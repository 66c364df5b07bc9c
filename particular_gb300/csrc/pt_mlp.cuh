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
// Installs FP32 parameters (device pointer, mlp::NPARAM floats) for PT_BH_LEARNED.
int bh_set_mlp(pt_ctx *ctx, const float *d_params, float theta_inner);

}  // namespace pt
