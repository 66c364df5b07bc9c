// Packed FP32 helpers for sm_100+: one f32x2 instruction does two lanes of work,
// halving the issue slots the FMA pipe needs. A value of type f2 holds two f32 in
// one 64-bit register pair (lo, hi).
#pragma once

#include <cuda_runtime.h>

namespace pt {

typedef unsigned long long f2;

__device__ __forceinline__ f2 pk2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// One MUFU.RSQ, no denormal fix-up (the softened n_s is a normal number).
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Knuth two-sum: s + c tracks the running sum with the rounding error of each add.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float t) {
    const float sn = s + t;
    const float bp = sn - s;
    const float err = (s - (sn - bp)) + (t - bp);
    s = sn;
    c += err;
}

// Two pairs (one target; sources in the lo and hi lanes) of the per-pair kernel
// a = d * mu / n_s^1.5 with n_s = |d|^2 + eps^2 (particular/src/gravity/impls/mod.rs:
// 156-165): 12 FMA-pipe lane-ops as 6 f32x2 instructions + 2 MUFU. GUARD zeroes
// the contribution of n_s == 0 (checked with eps == 0: the body itself).
template <bool GUARD>
__device__ __forceinline__ void interact2(f2 xj, f2 yj, f2 zj, f2 mj, f2 xi, f2 yi, f2 zi, f2 &ax, f2 &ay,
                                          f2 &az, f2 e2) {
    const f2 dx = sub2(xj, xi);
    const f2 dy = sub2(yj, yi);
    const f2 dz = sub2(zj, zi);
    const f2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
    float r0, r1;
    upk2(r2, r0, r1);
    float i0 = rsqrt_ftz(r0), i1 = rsqrt_ftz(r1);
    if (GUARD) {
        i0 = (r0 > 0.0f) ? i0 : 0.0f;
        i1 = (r1 > 0.0f) ? i1 : 0.0f;
    }
    const f2 inv = pk2(i0, i1);
    const f2 s = mul2(mul2(mj, inv), mul2(inv, inv));
    ax = fma2(dx, s, ax);
    ay = fma2(dy, s, ay);
    az = fma2(dz, s, az);
}

template <bool GUARD>
__device__ __forceinline__ void interact1(float xj, float yj, float zj, float mj, float xi, float yi, float zi,
                                          float &ax, float &ay, float &az, float eps2) {
    const float dx = xj - xi, dy = yj - yi, dz = zj - zi;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    float inv = rsqrt_ftz(r2);
    if (GUARD) inv = (r2 > 0.0f) ? inv : 0.0f;
    const float s = (mj * inv) * (inv * inv);
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

}  // namespace pt
