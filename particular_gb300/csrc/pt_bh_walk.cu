// cuda::BarnesHut walks over the tree of pt_bh_build.cu (sequential.rs:466-505):
//  * bh_walk_masked: the default method, the reference's per-body rule with one
//    shared traversal per warp (accept/open masks on stack ranges and list entries);
//  * bh_walk_group (PT_BH_GROUP): a cell opened for all 64 bodies of a warp when any
//    of them opens it, lists evaluated densely, optional quadrupoles, local
//    expansions of far nodes (PT_BH_LOCAL), the error-bound opening radius
//    (PT_BH_RELATIVE, with its per-group estimate bh_group_scale) and the learned
//    correction's records;
//  * bh_walk64: the reference rule over DVec3 bodies in double;
//  * lane_walk: the per-body cursor walk the others fall back to when a stack runs out.
#include "pt_bh.cuh"

#include <type_traits>

namespace pt {
namespace bh {

// ---- walk ------------------------------------------------------------------

// PT_BH_RELATIVE: a cell of mass m and width w is also opened within squared distance
// r2, where its truncation bound m w^p / d^(p+2) (p = 3 with quadrupoles, 2 without)
// reaches alpha |a|; ginv = 1 / (alpha |a|) of the target's group, 0 when off.
template <bool QUAD>
__device__ __forceinline__ float rel_r2(float m, float w, float ginv) {
    if (!(ginv > 0.f && m > 0.f)) return 0.f;
    return QUAD ? __powf(m * w * w * w * ginv, 0.4f) : sqrtf(m * w * w * ginv);
}

// The reference's per-body walk (sequential.rs) for this lane's target p, the cursor
// being the warp minimum of the lanes' next nodes: all 32 lanes take part. Adds the
// accepted nodes' accelerations to (ax, ay, az) and counts them.
template <bool QUAD>
__device__ __forceinline__ void lane_walk(float4 p, bool valid, int T, const float4 *__restrict__ nodeA,
                                          const int4 *__restrict__ nodeB, const float4 *__restrict__ nodeQ,
                                          const float4 *__restrict__ sbody, float th2, float eps2, float &ax,
                                          float &ay, float &az, unsigned &nacc, unsigned &nvisit,
                                          unsigned &ncell, float ginv = 0.f) {
    int resume = valid ? 0 : T;
    int node = 0;
    while (node < T) {
        const float4 A = __ldg(nodeA + node);
        const int4 B = __ldg(nodeB + node);
        const bool active = node >= resume;
        float dx = 0.f, dy = 0.f, dz = 0.f, d2 = 0.f;
        bool open = false, zero = false;
        if (active) {
            dx = A.x - p.x;
            dy = A.y - p.y;
            dz = A.z - p.z;
            d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            zero = (d2 == 0.0f);
            const float w = __int_as_float(B.x);
            open = !zero && B.z < 0 && (th2 * d2 < w * w || d2 < rel_r2<QUAD>(A.w, w, ginv));
        }
        int next = resume;
        if (active) {
            ++nvisit;
            if (zero) {
                next = resume = B.y;  // the whole node is skipped (sequential.rs:485-487)
            } else if (open) {
                next = node + 1;
            } else {
                if (B.z >= 0 && B.w > 1) {  // a bucket leaf: its bodies one by one
                    for (int b = B.z; b < B.z + B.w; ++b) {
                        const float4 q = __ldg(sbody + b);
                        const float ex = q.x - p.x, ey = q.y - p.y, ez = q.z - p.z;
                        const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                        if (e2 == 0.0f) continue;
                        const float inv = rsqrt_ftz(e2 + eps2);
                        const float s = (q.w * inv) * (inv * inv);
                        ax = fmaf(ex, s, ax);
                        ay = fmaf(ey, s, ay);
                        az = fmaf(ez, s, az);
                    }
                } else {
                    const float inv = rsqrt_ftz(d2 + eps2);
                    const float inv2 = inv * inv;
                    const float s = (A.w * inv) * inv2;
                    ax = fmaf(dx, s, ax);
                    ay = fmaf(dy, s, ay);
                    az = fmaf(dz, s, az);
                    if (QUAD && B.z < 0) {  // traceless quadrupole of the cell
                        const float4 q0 = __ldg(nodeQ + 2 * node);
                        const float4 q1 = __ldg(nodeQ + 2 * node + 1);
                        // q0 = (Qxx, Qxy, Qxz, Qyy), q1 = (Qyz, Qzz)
                        const float qx = fmaf(q0.x, dx, fmaf(q0.y, dy, q0.z * dz));
                        const float qy = fmaf(q0.y, dx, fmaf(q0.w, dy, q1.x * dz));
                        const float qz = fmaf(q0.z, dx, fmaf(q1.x, dy, q1.y * dz));
                        const float dqd = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
                        const float inv5 = inv2 * inv2 * inv;
                        const float c7 = 2.5f * dqd * inv5 * inv2;
                        ax += fmaf(c7, dx, -qx * inv5);
                        ay += fmaf(c7, dy, -qy * inv5);
                        az += fmaf(c7, dz, -qz * inv5);
                    }
                }
                ++nacc;
                ncell += B.z < 0;
                next = resume = B.y;
            }
        }
        node = __reduce_min_sync(0xffffffffu, next);
    }
}

// ---- group walk (PT_BH_GROUP) ----------------------------------------------
// One warp walks for 32 x GW_TPL (64) key-adjacent targets. Each step pops up to 32
// nodes from a shared-memory stack of sibling ranges (independent loads, one per
// lane), opens a cell when the reference's per-body rule opens it for at least one of
// the targets (so never less accurate than that rule), and appends accepted nodes to
// shared-memory interaction lists. A full list is evaluated densely: every lane runs
// its targets against all entries, two entries per packed f32x2 instruction.
// Warps (groups) per CTA of the group walk. A CTA's slot is held until its slowest
// warp ends, so with one warp per CTA no warp slot idles behind a neighbouring group's
// longer walk; the local-expansion lists are sized (64 cells, 88 bodies) so that 20
// one-warp CTAs fit an SM's shared memory. Measured at N = 4M (walk ms): headline
// configuration 5.40 with 2 warps per CTA (72 / 96 entries) -> 5.25 with 1 (64 / 88);
// quadrupole + group + local at theta 0.52 12.19 -> 11.74; quadrupole + group at theta
// 0.52 16.30 -> 15.19 (4 warps per CTA: 5.47, 12.43, 16.40). Persistent warps taking
// groups from a counter instead spilled (96 -> 116 bytes) and were slower (5.85 ms).
#ifndef PT_GW_WARPS
#define PT_GW_WARPS 1
#endif
constexpr int GW_WARPS = PT_GW_WARPS;


// Interaction lists in structure-of-arrays form. Cells carry their quadrupole
// when QUAD; single bodies never need one.
template <int NF, int CAP_>
struct IList {
    static constexpr int CAP = CAP_;
    float f[NF][CAP + 2];
};

// A body's acceleration as a compensated FP32 sum (running sum s, rounding errors c).
// Each evaluated list chunk (up to 128 entries) is summed in plain FP32 in two packed
// partials and enters the running sum through TwoSum, so the rounding error of the
// total does not grow with the number of chunks: it is that of one chunk's sum.
struct CSum {
    float sx, sy, sz, cx, cy, cz;
};

__device__ __forceinline__ void csum_zero(CSum &a) { a.sx = a.sy = a.sz = a.cx = a.cy = a.cz = 0.f; }

__device__ __forceinline__ void csum_fold(CSum &a, f2 tx, f2 ty, f2 tz) {
    float l, h;
    upk2(tx, l, h);
    two_sum_acc(a.sx, a.cx, l + h);
    upk2(ty, l, h);
    two_sum_acc(a.sy, a.cy, l + h);
    upk2(tz, l, h);
    two_sum_acc(a.sz, a.cz, l + h);
}

// Where a warp keeps its bodies' compensated sums: in registers, or, in the kernel
// whose registers the traversal state fills (the quadrupole group walk with local
// expansions, 96 registers for 20 warps per SM: 56 bytes spilled, walk +15 %), in shared
// memory as [value][lane] (conflict-free; touched once per evaluated chunk; walk +2.5 %
// over plain FP32 sums). Measured at N = 4M: the other group walks +1.2 % in registers
// (+2.7 % in shared memory), the masked walk +1.6 %.
template <int TPL>
struct RegSums {
    CSum c[TPL];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < TPL; ++i) csum_zero(c[i]);
    }
    __device__ __forceinline__ void fold(int i, f2 tx, f2 ty, f2 tz) { csum_fold(c[i], tx, ty, tz); }
    __device__ __forceinline__ void total(int i, float &x, float &y, float &z) const {
        x = c[i].sx + c[i].cx;
        y = c[i].sy + c[i].cy;
        z = c[i].sz + c[i].cz;
    }
};

template <int TPL>
struct SmemSums {
    float (*v)[32];  // [6 * TPL][32]: per body sx, sy, sz, cx, cy, cz
    int lane;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 6 * TPL; ++k) v[k][lane] = 0.f;
    }
    __device__ __forceinline__ void fold(int i, f2 tx, f2 ty, f2 tz) {
        CSum a;
        a.sx = v[6 * i][lane], a.sy = v[6 * i + 1][lane], a.sz = v[6 * i + 2][lane];
        a.cx = v[6 * i + 3][lane], a.cy = v[6 * i + 4][lane], a.cz = v[6 * i + 5][lane];
        csum_fold(a, tx, ty, tz);
        v[6 * i][lane] = a.sx, v[6 * i + 1][lane] = a.sy, v[6 * i + 2][lane] = a.sz;
        v[6 * i + 3][lane] = a.cx, v[6 * i + 4][lane] = a.cy, v[6 * i + 5][lane] = a.cz;
    }
    __device__ __forceinline__ void total(int i, float &x, float &y, float &z) const {
        x = v[6 * i][lane] + v[6 * i + 3][lane];
        y = v[6 * i + 1][lane] + v[6 * i + 4][lane];
        z = v[6 * i + 2][lane] + v[6 * i + 5][lane];
    }
};

// Two list entries (packed lo/hi: monopole x, y, z, m and, for NF = 10, the negated
// traceless quadrupole N = -Q as Nxx Nxy Nxz Nyy Nyz Nzz) for one target. With
// u = N d and c = d.u:
//   a += d (m / r^3 + 2.5 (d.Q.d) / r^7) - (Q d) / r^5 = d (sc - 2.5 c / r^7) + u / r^5
template <int NF, bool GUARD>
__device__ __forceinline__ void eval_pair(const f2 (&q)[NF], f2 px, f2 py, f2 pz, f2 e2, f2 &ax, f2 &ay, f2 &az) {
    const f2 dx = sub2(q[0], px);
    const f2 dy = sub2(q[1], py);
    const f2 dz = sub2(q[2], pz);
    const f2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
    float r0, r1;
    upk2(r2, r0, r1);
    float i0 = rsqrt_ftz(r0), i1 = rsqrt_ftz(r1);
    if (GUARD) {
        i0 = (r0 > 0.0f) ? i0 : 0.0f;
        i1 = (r1 > 0.0f) ? i1 : 0.0f;
    }
    const f2 inv = pk2(i0, i1);
    const f2 inv2 = mul2(inv, inv);
    const f2 sc = mul2(mul2(q[3], inv), inv2);
    if constexpr (NF == 10) {
        const f2 ux = fma2(q[4], dx, fma2(q[5], dy, mul2(q[6], dz)));
        const f2 uy = fma2(q[5], dx, fma2(q[7], dy, mul2(q[8], dz)));
        const f2 uz = fma2(q[6], dx, fma2(q[8], dy, mul2(q[9], dz)));
        const f2 c = fma2(dx, ux, fma2(dy, uy, mul2(dz, uz)));
        const f2 inv5 = mul2(mul2(inv2, inv2), inv);
        const f2 k = mul2(c, mul2(inv2, pk2(-2.5f, -2.5f)));
        const f2 s2 = fma2(inv5, k, sc);
        ax = fma2(dx, s2, fma2(inv5, ux, ax));
        ay = fma2(dy, s2, fma2(inv5, uy, ay));
        az = fma2(dz, s2, fma2(inv5, uz, az));
    } else {
        ax = fma2(dx, sc, ax);
        ay = fma2(dy, sc, ay);
        az = fma2(dz, sc, az);
    }
}

// Evaluates entries [0, cnt) of a list for this lane's TPL targets, two entries per
// packed instruction; each pair of entries is read from shared memory once for all
// of the lane's targets.
template <int NF, int CAP, bool GUARD, int TPL, class Sums>
__device__ __forceinline__ void eval_list(IList<NF, CAP> &Lst, int cnt, const f2 (&px)[TPL], const f2 (&py)[TPL],
                                          const f2 (&pz)[TPL], f2 e2, Sums &acc) {
    const int lane = threadIdx.x & 31;
    f2 ax[TPL], ay[TPL], az[TPL];
#pragma unroll
    for (int i = 0; i < TPL; ++i) ax[i] = ay[i] = az[i] = pk2(0.f, 0.f);
    __syncwarp();
    if (cnt & 1) {  // pad with a massless entry far away: contributes exactly 0
        if (lane < NF) Lst.f[lane][cnt] = (lane < 3) ? 1e30f : 0.0f;
        __syncwarp();
        ++cnt;
    }
#pragma unroll 2
    for (int e = 0; e < cnt; e += 2) {
        f2 q[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) q[k] = *reinterpret_cast<const f2 *>(&Lst.f[k][e]);
#pragma unroll
        for (int i = 0; i < TPL; ++i) eval_pair<NF, GUARD>(q, px[i], py[i], pz[i], e2, ax[i], ay[i], az[i]);
    }
#pragma unroll
    for (int i = 0; i < TPL; ++i) acc.fold(i, ax[i], ay[i], az[i]);
    __syncwarp();
}

// ---- learned correction: records of marginal cells ---------------------------
// The walk (PT_BH_LEARNED) does not evaluate the network itself: it records the
// node index of every marginal cell (accepted at theta, opened at theta_inner) in
// chunks of LCHUNK entries that each belong to one warp (one group of 64 targets),
// chained per group in walk order, and the group's centre. A tensor-core kernel then
// evaluates all records (bh_learned_eval) and bh_learned_apply adds each group's
// sum, chunk by chunk in chain order, so results do not depend on scheduling.
constexpr int LCHUNK = 128;

struct LearnedRecords {
    int *rec;        // [cap][LCHUNK] node indices, -1 = padding
    int *chunk_group;  // [cap]
    int *next;       // [cap] next chunk of the same group, -1 = last
    int *head;       // [groups] first chunk of the group, -1 = none
    float4 *centre;  // [groups] mean position of the group's targets
    float4 *part;    // [cap] the chunk's summed correction
    int *used;       // chunks handed out (may exceed cap: then nothing past cap is written)
    int cap;
};

// One warp per chunk (grid-stride): features of the 128 recorded cells at the group
// centre, four 32-row tensor-core batches, the chunk's sum into part[chunk]. (It holds
// 2 CTAs per SM at ~242 registers; capped at 168 for 3 CTAs it spills 128 bytes and
// the learned step at N = 4M went from 9.95 to 10.69 ms.)
// Cells whose size/distance ratio at the group centre lies outside the range the
// model was trained on ([lo, hi]) get no correction.
__global__ void __launch_bounds__(128) bh_learned_eval(LearnedRecords L, const float4 *__restrict__ nodeA,
                                                      const float4 *__restrict__ nodeQ,
                                                      const float4 *__restrict__ nodeG,
                                                      const uint32_t *__restrict__ W, const float *__restrict__ bias,
                                                      float lo, float hi) {
    __shared__ float X[4][32 * mlp::TC_XS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int used = min(*L.used, L.cap);
    const float sc = __ldg(bias + mlp::TC_SCALE);
    float *Xw = X[warp];
    for (int c = blockIdx.x * 4 + warp; c < used; c += gridDim.x * 4) {
        const float4 gc = L.centre[L.chunk_group[c]];
        float rx = 0.f, ry = 0.f, rz = 0.f;
        for (int b = 0; b < LCHUNK / 32; ++b) {
            const int node = L.rec[size_t(c) * LCHUNK + b * 32 + lane];
            if (__ballot_sync(0xffffffffu, node >= 0) == 0u) break;  // padding fills the chunk's tail
            float f[mlp::IN];
            float a = 0.f;  // M / |r|^2 of this row's cell, 0 = no correction
            if (node >= 0) {
                const float4 A = __ldg(nodeA + node);
                const float4 q0 = __ldg(nodeQ + 2 * node), q1 = __ldg(nodeQ + 2 * node + 1);
                const float q[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
                const float r2 = mlp::features(gc.x, gc.y, gc.z, A, q, __ldg(nodeG + node), f);
                if (f[3] >= lo && f[3] <= hi) a = A.w / r2;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) Xw[lane * mlp::TC_XS + i] = (i < mlp::IN && a != 0.f) ? f[i] : 0.f;
            __syncwarp();
            float y[2][4];
            mlp::tc_batch(Xw, W, bias, y);
            __syncwarp();
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float s = __shfl_sync(0xffffffffu, a, 16 * mt + 8 * h + g);
                    if (t == 0) {
                        rx = fmaf(y[mt][2 * h], s, rx);
                        ry = fmaf(y[mt][2 * h + 1], s, ry);
                    } else if (t == 1) {
                        rz = fmaf(y[mt][2 * h], s, rz);
                    }
                }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rx += __shfl_xor_sync(0xffffffffu, rx, off);
            ry += __shfl_xor_sync(0xffffffffu, ry, off);
            rz += __shfl_xor_sync(0xffffffffu, rz, off);
        }
        if (lane == 0) L.part[c] = make_float4(rx * sc, ry * sc, rz * sc, 0.f);
    }
}

// out[target] += the sum of its group's chunk corrections, in chain order.
__global__ void bh_learned_apply(LearnedRecords L, const uint32_t *__restrict__ tidx, int n_aff, int group_shift,
                                 float *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_aff) return;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    // chunk indices grow along a chain (each is taken after its predecessor)
    for (int c = L.head[t >> group_shift], prev = -1; c > prev && c < L.cap; prev = c, c = L.next[c]) {
        const float4 v = L.part[c];
        cx += v.x;
        cy += v.y;
        cz += v.z;
    }
    const uint32_t o = tidx[t];
    out[3 * size_t(o) + 0] += cx;
    out[3 * size_t(o) + 1] += cy;
    out[3 * size_t(o) + 2] += cz;
}

// ---- local (Taylor) expansion of far nodes about the group centre -------------
// PT_BH_LOCAL: an accepted node far from the group (group radius R < ratio * d, d
// from the group's box centre g to the node's centre of mass) is not added to the
// interaction lists. The lane that popped it adds the node's softened monopole (+
// quadrupole) field to a second-order expansion of the acceleration about g:
// a(g + r) = a0 + T r + 1/2 H : r r, with
//   a0 = m d s^-3/2,  T_ij = 3m d_i d_j s^-5/2 - m delta_ij s^-3/2,
//   H_ijk = 15m d_i d_j d_k s^-7/2 - 3m s^-5/2 (delta_ij d_k + delta_ik d_j + delta_jk d_i)
// (s = |d|^2 + eps^2: the exact derivatives of the softened kernel), plus the
// quadrupole's a0 and T. The expansion costs one lane ~150 flops per far node
// instead of every target's list entry; its truncation error is ~(R/d)^3.
struct LocalExp {
    float ax, ay, az;                                      // a(g)
    float txx, txy, txz, tyy, tyz, tzz;                    // d a_i / d x_j
    float hxxx, hxxy, hxxz, hxyy, hxyz, hxzz, hyyy, hyyz, hyzz, hzzz;  // d2 a_i / dx_j dx_k
};

// Adds the softened monopole (+ traceless quadrupole q, when given) field of a node
// at offset d = com - g, mass m, to the expansion about g.
__device__ __forceinline__ void local_add(LocalExp &L, float dx, float dy, float dz, float m, float eps2,
                                          const float4 *q0p, const float4 *q1p) {
    const float s = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float inv = rsqrt_ftz(s);
    const float inv2 = inv * inv;
    const float i3 = m * inv * inv2;      // m s^-3/2
    const float i5 = 3.0f * i3 * inv2;    // 3 m s^-5/2
    const float i7 = 5.0f * i5 * inv2;    // 15 m s^-7/2
    L.ax = fmaf(i3, dx, L.ax);
    L.ay = fmaf(i3, dy, L.ay);
    L.az = fmaf(i3, dz, L.az);
    const float xx = dx * dx, yy = dy * dy, zz = dz * dz, xy = dx * dy, xz = dx * dz, yz = dy * dz;
    L.txx += fmaf(i5, xx, -i3);
    L.txy = fmaf(i5, xy, L.txy);
    L.txz = fmaf(i5, xz, L.txz);
    L.tyy += fmaf(i5, yy, -i3);
    L.tyz = fmaf(i5, yz, L.tyz);
    L.tzz += fmaf(i5, zz, -i3);
    const float ax7 = i7 * dx, ay7 = i7 * dy, az7 = i7 * dz;
    L.hxxx += fmaf(ax7, xx, -3.0f * i5 * dx);
    L.hxxy += fmaf(ax7, xy, -i5 * dy);
    L.hxxz += fmaf(ax7, xz, -i5 * dz);
    L.hxyy += fmaf(ax7, yy, -i5 * dx);
    L.hxyz = fmaf(ax7, yz, L.hxyz);
    L.hxzz += fmaf(ax7, zz, -i5 * dx);
    L.hyyy += fmaf(ay7, yy, -3.0f * i5 * dy);
    L.hyyz += fmaf(ay7, yz, -i5 * dz);
    L.hyzz += fmaf(ay7, zz, -i5 * dy);
    L.hzzz += fmaf(az7, zz, -3.0f * i5 * dz);
    if (q0p) {
        const float4 q0 = __ldg(q0p), q1 = __ldg(q1p);  // Qxx Qxy Qxz Qyy | Qyz Qzz
        const float ux = fmaf(q0.x, dx, fmaf(q0.y, dy, q0.z * dz));
        const float uy = fmaf(q0.y, dx, fmaf(q0.w, dy, q1.x * dz));
        const float uz = fmaf(q0.z, dx, fmaf(q1.x, dy, q1.y * dz));
        const float c = fmaf(dx, ux, fmaf(dy, uy, dz * uz));
        const float j5 = inv2 * inv2 * inv, j7 = j5 * inv2, j9 = j7 * inv2;
        const float c7 = 2.5f * c * j7;
        L.ax += fmaf(c7, dx, -ux * j5);
        L.ay += fmaf(c7, dy, -uy * j5);
        L.az += fmaf(c7, dz, -uz * j5);
        const float f5 = 5.0f * j7, g9 = 17.5f * c * j9;
        L.txx += fmaf(q0.x, j5, fmaf(g9, xx, -fmaf(2.0f * f5, ux * dx, c7)));
        L.tyy += fmaf(q0.w, j5, fmaf(g9, yy, -fmaf(2.0f * f5, uy * dy, c7)));
        L.tzz += fmaf(q1.y, j5, fmaf(g9, zz, -fmaf(2.0f * f5, uz * dz, c7)));
        L.txy += fmaf(q0.y, j5, fmaf(g9, xy, -f5 * fmaf(ux, dy, uy * dx)));
        L.txz += fmaf(q0.z, j5, fmaf(g9, xz, -f5 * fmaf(ux, dz, uz * dx)));
        L.tyz += fmaf(q1.x, j5, fmaf(g9, yz, -f5 * fmaf(uy, dz, uz * dy)));
    }
}

__device__ __forceinline__ void local_reduce(LocalExp &L) {
    float *f = &L.ax;
#pragma unroll
    for (int k = 0; k < 19; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o);
}

// a(g + d) from the expansion
__device__ __forceinline__ void local_eval(const LocalExp &L, float dx, float dy, float dz, float &ax, float &ay,
                                           float &az) {
    const float xx = dx * dx, yy = dy * dy, zz = dz * dz, xy2 = 2.0f * dx * dy, xz2 = 2.0f * dx * dz,
                yz2 = 2.0f * dy * dz;
    ax = L.ax + fmaf(L.txx, dx, fmaf(L.txy, dy, L.txz * dz)) +
         0.5f * fmaf(L.hxxx, xx, fmaf(L.hxyy, yy, fmaf(L.hxzz, zz, fmaf(L.hxxy, xy2, fmaf(L.hxxz, xz2, L.hxyz * yz2)))));
    ay = L.ay + fmaf(L.txy, dx, fmaf(L.tyy, dy, L.tyz * dz)) +
         0.5f * fmaf(L.hxxy, xx, fmaf(L.hyyy, yy, fmaf(L.hyzz, zz, fmaf(L.hxyy, xy2, fmaf(L.hxyz, xz2, L.hyyz * yz2)))));
    az = L.az + fmaf(L.txz, dx, fmaf(L.tyz, dy, L.tzz * dz)) +
         0.5f * fmaf(L.hxxz, xx, fmaf(L.hyyz, yy, fmaf(L.hzzz, zz, fmaf(L.hxyz, xy2, fmaf(L.hxzz, xz2, L.hyzz * yz2)))));
}

// PT_BH_LOCAL: adds queued far node e (2 x node index + 1 for a cell) to this lane's
// expansion coefficients, kept in shared memory as [coefficient][lane].
template <bool QUAD>
__device__ __forceinline__ void local_add_node(float (*lx)[32], int lane, int e, const float4 *__restrict__ nodeA,
                                               const float4 *__restrict__ nodeQ, float gx, float gy, float gz,
                                               float eps2) {
    const int node = e >> 1;
    const bool q = QUAD && (e & 1);
    const float4 A = __ldg(nodeA + node);
    LocalExp t;
    float *tf = &t.ax;
#pragma unroll
    for (int k = 0; k < 19; ++k) tf[k] = lx[k][lane];
    local_add(t, A.x - gx, A.y - gy, A.z - gz, A.w, eps2, q ? nodeQ + 2 * node : nullptr,
              q ? nodeQ + 2 * node + 1 : nullptr);
#pragma unroll
    for (int k = 0; k < 19; ++k) lx[k][lane] = tf[k];
}

// Targets per lane of the group walk: a warp walks for 32 * GW_TPL key-adjacent
// targets, and each list entry read from shared memory serves all of a lane's
// targets. Measured at N = 4M bulge+disk, theta 0.5, quadrupole: 1 -> 18.3 ms
// (p95 8.2e-4), 2 -> 16.6 ms (7.7e-4), 4 -> 17.7 ms (7.5e-4); the larger box opens
// more cells (13.5e9 -> 15.2e9 -> 17.6e9 pairs) but traversal is shared by more
// targets.
#ifndef PT_GW_TPL
#define PT_GW_TPL 2
#endif
constexpr int GW_TPL = PT_GW_TPL;
constexpr int GW_GROUP = 32 * GW_TPL;
constexpr int GW_SHIFT = GW_TPL == 1 ? 5 : GW_TPL == 2 ? 6 : 7;
static_assert(GW_GROUP == (1 << GW_SHIFT), "targets per lane: 1, 2 or 4");
// PT_BH_LOCAL walk: occupancy (counted in CTAs of 4 warps per SM, so 5 = 20 warps)
// and list capacities. Both registers (96) and shared memory (11 KB per warp) hold it
// at 20 warps per SM; 24 warps with lists of 64 cells and 96 bodies (80 registers, 84
// bytes spilled) measured 6.9 ms against 6.1 ms at N = 4M.
#ifndef PT_GW_LMINB
#define PT_GW_LMINB 5
#endif
#ifndef PT_GW_LCELLS
#define PT_GW_LCELLS 64
#endif
#ifndef PT_GW_LBODIES
#define PT_GW_LBODIES 88
#endif
// Stack ranges per warp of the PT_BH_LOCAL walk. (21 warps per SM, with lists of 56
// cells / 80 bodies and 272 ranges, measured the same as 20: 5.21 against 5.20 ms.)
#ifndef PT_GW_LSTACK
#define PT_GW_LSTACK 288
#endif
// Opened cells with at most this many nodes below them are summed body by body at
// once instead of being walked level by level (loaded 32 nodes per round; 0 = off).
// The calibrated headline at N = 4M (fastest configuration within the error margin)
// for limits 7 / 15 / 31 / 47 / 63 / 95 / 127: 5.26 / 5.65 / 6.07 / 6.10 / 6.05 /
// 5.92 / 5.77 e8 bodies/s.
#ifndef PT_GW_FLAT
#define PT_GW_FLAT 31
#endif
constexpr int GW_FLAT = PT_GW_FLAT;
static_assert(GW_FLAT >= 0 && GW_FLAT <= 1023, "flattened subtree size");
#ifndef PT_GW_MINB
#define PT_GW_MINB (GW_TPL == 1 ? 6 : 5)  // 4-warp CTAs per SM the register budget is set for
#endif
template <bool QUAD, bool GUARD, bool LEARNED, bool LOCAL, bool REL>
__global__ void __launch_bounds__(32 * GW_WARPS, (LOCAL ? PT_GW_LMINB : PT_GW_MINB) * 4 / GW_WARPS)
    bh_walk_group(const float4 *__restrict__ tbody, const uint32_t *__restrict__ tidx, int n_aff,
                  const float4 *__restrict__ nodeA, const int4 *__restrict__ nodeB, const float4 *__restrict__ nodeQ,
                  const float4 *__restrict__ nodeG, const float4 *__restrict__ sbody, const int *__restrict__ counters,
                  float th2, float th_in2, LearnedRecords LR, float eps2, float *__restrict__ out,
                  unsigned long long *__restrict__ stats, int *__restrict__ err, int stack_cap,
                  float local_ratio, const float *__restrict__ gscale, float mono_beta) {
    static_assert(!(LEARNED && LOCAL), "PT_BH_LEARNED and PT_BH_LOCAL are exclusive");
    static_assert(!(LEARNED && REL), "PT_BH_LEARNED and PT_BH_RELATIVE are exclusive");
    constexpr int NFC = QUAD ? 10 : 4;
    constexpr int TPL = GW_TPL;
    using CellList = IList<NFC, LOCAL ? PT_GW_LCELLS : 96>;
    using BodyList = IList<4, LOCAL ? PT_GW_LBODIES : 128>;
    // PT_BH_LOCAL keeps its 19 expansion coefficients per lane in shared memory
    // ([coefficient][lane]: no bank conflicts) and queues far nodes (up to 63) so that
    // they are expanded 32 at a time, one per lane, instead of by the few lanes that
    // popped them; the stack is trimmed to 288 ranges so that 20 warps stay resident per SM.
    constexpr int STK = LOCAL ? PT_GW_LSTACK : GW_STACK;
    stack_cap = min(stack_cap, STK);
    __shared__ int2 s_stack[GW_WARPS][STK];
    __shared__ __align__(16) CellList s_cells[GW_WARPS];
    __shared__ __align__(16) BodyList s_bodies[GW_WARPS];
    __shared__ float s_lx[GW_WARPS][LOCAL ? 19 : 1][32];
    __shared__ int s_far[GW_WARPS][LOCAL ? 64 : 1];
    __shared__ float s_sums[GW_WARPS][QUAD && LOCAL ? 6 * GW_TPL : 1][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int group = blockIdx.x * GW_WARPS + warp;
    const int g0 = group * GW_GROUP;
    if (g0 >= n_aff) return;
    // this lane's targets: g0 + lane, g0 + 32 + lane, ...
    float4 p[TPL];
    bool valid[TPL];
#pragma unroll
    for (int i = 0; i < TPL; ++i) {
        const int t = g0 + 32 * i + lane;
        valid[i] = t < n_aff;
        p[i] = tbody[valid[i] ? t : g0];
    }
    const int nvalid = min(GW_GROUP, n_aff - g0);
    const unsigned lt = (1u << lane) - 1u;
    // PT_BH_RELATIVE: 1 / (alpha |a|) of this group (warp-uniform), and its 2/5 power,
    // the factor of a cell's (M w^3)^(2/5) kept in its nodeB.w
    const float ginv = (REL && !QUAD) ? gscale[group] : 0.f;
    const float gq = (REL && QUAD) ? __powf(gscale[group], 0.4f) : 0.f;
    // PT_BH_RELATIVE with quadrupoles: an accepted cell whose monopole truncation bound
    // M w^2 / d^4 (the quadrupole term it would drop) stays within mono_beta alpha |a|
    // from every body of the group enters the body list, without its quadrupole.
    const float gmono = (REL && QUAD && mono_beta > 0.f) ? gscale[group] / mono_beta : 0.f;
    int2 *stack = s_stack[warp];
    const int T = counters[1];
    CellList &Lc = s_cells[warp];
    BodyList &Lb = s_bodies[warp];

    // the bounding box of the group's targets: it settles most opening decisions
    // without the per-target vote
    float mn0 = p[0].x, mn1 = p[0].y, mn2 = p[0].z, mx0 = p[0].x, mx1 = p[0].y, mx2 = p[0].z;
#pragma unroll
    for (int i = 1; i < TPL; ++i) {
        mn0 = fminf(mn0, p[i].x), mn1 = fminf(mn1, p[i].y), mn2 = fminf(mn2, p[i].z);
        mx0 = fmaxf(mx0, p[i].x), mx1 = fmaxf(mx1, p[i].y), mx2 = fmaxf(mx2, p[i].z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn0 = fminf(mn0, __shfl_xor_sync(0xffffffffu, mn0, o));
        mn1 = fminf(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mn2 = fminf(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
    }
    // the group centre, where learned corrections are evaluated
    float gcx = 0.f, gcy = 0.f, gcz = 0.f;
    if (LEARNED) {
#pragma unroll
        for (int i = 0; i < TPL; ++i)
            if (valid[i]) gcx += p[i].x, gcy += p[i].y, gcz += p[i].z;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gcx += __shfl_xor_sync(0xffffffffu, gcx, o);
            gcy += __shfl_xor_sync(0xffffffffu, gcy, o);
            gcz += __shfl_xor_sync(0xffffffffu, gcz, o);
        }
        const float nv = float(nvalid);
        gcx /= nv;
        gcy /= nv;
        gcz /= nv;
    }
    // PT_BH_LOCAL: the expansion centre g (box centre) and the far radius^2
    const float lgx = 0.5f * (mn0 + mx0), lgy = 0.5f * (mn1 + mx1), lgz = 0.5f * (mn2 + mx2);
    const float rg2 = 0.25f * fmaf(mx0 - mn0, mx0 - mn0, fmaf(mx1 - mn1, mx1 - mn1, (mx2 - mn2) * (mx2 - mn2)));
    const float far2 = LOCAL ? rg2 / (local_ratio * local_ratio) : 0.f;
    if (LOCAL)
        for (int k = 0; k < 19; ++k) s_lx[warp][k][lane] = 0.f;
    unsigned nlocal = 0, nlocalq = 0;  // warp-uniform: far nodes, those with a quadrupole
    int Nf = 0;                     // queued far nodes
    // learned: the warp's current record chunk and its fill; the previous chunk links to
    // the next one (head of the group's chain first)
    int chunk = -1, fill = LCHUNK;
    unsigned long long learned = 0;

    const f2 e2 = pk2(eps2, eps2);
    // the lane's two targets packed, for the opening vote
    const f2 vx01 = pk2(p[0].x, p[TPL - 1].x), vy01 = pk2(p[0].y, p[TPL - 1].y), vz01 = pk2(p[0].z, p[TPL - 1].z);
    f2 px[TPL], py[TPL], pz[TPL];
    // the bodies' compensated sums over the evaluated lists
    using Sums = typename std::conditional<QUAD && LOCAL, SmemSums<TPL>, RegSums<TPL>>::type;
    Sums bsum;
    if constexpr (QUAD && LOCAL) bsum = Sums{s_sums[warp], lane};
    bsum.zero();
#pragma unroll
    for (int i = 0; i < TPL; ++i) {
        px[i] = pk2(p[i].x, p[i].x);
        py[i] = pk2(p[i].y, p[i].y);
        pz[i] = pk2(p[i].z, p[i].z);
    }
    // Stack entries are sibling ranges (first, end): `first` is the next node to
    // visit, its later siblings follow by skip pointers up to `end`. A pop visits one
    // node of a range (two when lanes are idle) and pushes back its remaining
    // siblings and, for each opened cell, its children (pre+1, skip). The stack
    // therefore stays within about 32 ranges per tree level.
    if (lane == 0) stack[0] = make_int2(0, T);
    __syncwarp();
    int S = 1, Nc = 0, Nb = 0, maxS = 1;
    unsigned entries = 0, visits = 0, centries = 0;
    bool failed = false;
    while (S > 0) {
        // each pop pushes at most two ranges: never more than the room left
        const int k = min(min(32, S), max(1, (stack_cap - S) / 2));
        const bool first = lane < k;
        int2 range = first ? stack[S - 1 - lane] : make_int2(0, 0);
        __syncwarp();
        S -= k;
        int node = range.x;
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 B = make_int4(0, 0, 0, 0);
        bool open = false;
        if (first) {
            A = __ldg(nodeA + node);
            B = __ldg(nodeB + node);
        }
        // A pop of fewer than 32 ranges leaves lanes idle: lane k + i then also takes
        // the second node of range i (its first node's skip pointer), and the rest of
        // the range passes to it. Each range still pushes at most three ranges, within
        // the room k was sized for (2 per popped range).
        bool second = false;
        if (k < 32) {
            const int src = lane >= k ? lane - k : lane;
            const int nxt = __shfl_sync(0xffffffffu, B.y, src);
            const int end = __shfl_sync(0xffffffffu, range.y, src);
            if (lane >= k && src < k && nxt < end) {
                second = true;
                node = nxt;
                range = make_int2(nxt, end);
                A = __ldg(nodeA + node);
                B = __ldg(nodeB + node);
            }
        }
        const unsigned msecond = __ballot_sync(0xffffffffu, second);
        // its rest went to lane + k
        const bool handed = first && lane + k < 32 && ((msecond >> (lane + k)) & 1u);
        const bool have = first || second;
        visits += k + __popc(msecond);
        // Open iff the per-body rule opens for at least one target: some target with
        // nonzero d^2 (targets with d^2 == 0 skip the cell under that rule and do not
        // vote) and theta^2 d^2 < w^2. Settled without a vote: cells accepted even from
        // the nearest point of the targets' box (maybe false) and cells opened even
        // from its farthest corner (sure). Rounding is monotone, so these box bounds
        // never contradict the per-target values. The remaining cells are voted on one
        // at a time: each lane tests its own target, a ballot collects the votes.
        // PT_BH_RELATIVE adds a second opening radius per cell (rr2), tested the same way.
        bool maybe = false, sure = false, monoq = false;
        float w = 0.f, rr2 = 0.f;
        if (have && B.z < 0) {
            w = __int_as_float(B.x);
            if (REL) rr2 = QUAD ? __int_as_float(B.w) * gq : rel_r2<false>(A.w, w, ginv);
            const float e0 = fmaxf(fmaxf(mn0 - A.x, A.x - mx0), 0.f);
            const float e1 = fmaxf(fmaxf(mn1 - A.y, A.y - mx1), 0.f);
            const float e2b = fmaxf(fmaxf(mn2 - A.z, A.z - mx2), 0.f);
            const float emin2 = fmaf(e0, e0, fmaf(e1, e1, e2b * e2b));
            maybe = (LEARNED ? th_in2 : th2) * emin2 < w * w || (REL && emin2 < rr2);
            if (REL && QUAD) monoq = emin2 * emin2 >= A.w * w * w * gmono && gmono > 0.f;
            const float f0 = fmaxf(A.x - mn0, mx0 - A.x);
            const float f1 = fmaxf(A.y - mn1, mx1 - A.y);
            const float f2b = fmaxf(A.z - mn2, mx2 - A.z);
            const float dmax2 = fmaf(f0, f0, fmaf(f1, f1, f2b * f2b));
            // dmax2 > 0: some target is off the centre of mass
            sure = dmax2 > 0.0f && (th2 * dmax2 < w * w || (REL && dmax2 < rr2));
        }
        open = sure;
        bool marginal = false;
        unsigned amb = __ballot_sync(0xffffffffu, maybe && !sure);
        while (amb) {
            const int j = __ffs(amb) - 1;
            amb &= amb - 1;
            const float cx = __shfl_sync(0xffffffffu, A.x, j);
            const float cy = __shfl_sync(0xffffffffu, A.y, j);
            const float cz = __shfl_sync(0xffffffffu, A.z, j);
            const float cw = __shfl_sync(0xffffffffu, w, j);
            const float crr = REL ? __shfl_sync(0xffffffffu, rr2, j) : 0.f;
            bool o1 = false, i1 = false;
            const float cw2 = cw * cw;
            if constexpr (TPL == 2) {  // both targets in one packed pass (same IEEE ops)
                const f2 dx = sub2(pk2(cx, cx), vx01), dy = sub2(pk2(cy, cy), vy01), dz = sub2(pk2(cz, cz), vz01);
                float d0, d1;
                upk2(fma2(dx, dx, fma2(dy, dy, mul2(dz, dz))), d0, d1);
                o1 = (d0 > 0.0f && (th2 * d0 < cw2 || (REL && d0 < crr))) ||
                     (d1 > 0.0f && (th2 * d1 < cw2 || (REL && d1 < crr)));
                if (LEARNED) i1 = (d0 > 0.0f && th_in2 * d0 < cw2) || (d1 > 0.0f && th_in2 * d1 < cw2);
            } else {
#pragma unroll
                for (int i = 0; i < TPL; ++i) {
                    const float dx = cx - p[i].x, dy = cy - p[i].y, dz = cz - p[i].z;
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    o1 |= d2 > 0.0f && (th2 * d2 < cw2 || (REL && d2 < crr));
                    if (LEARNED) i1 |= d2 > 0.0f && th_in2 * d2 < cw2;
                }
            }
            const unsigned vo = __ballot_sync(0xffffffffu, o1);
            if (lane == j) open = vo != 0u;
            if (LEARNED) {
                // accepted by every target, but opened by one at theta_inner
                const unsigned vi = __ballot_sync(0xffffffffu, i1);
                if (lane == j) marginal = vo == 0u && vi != 0u && A.w > 0.0f;
            }
        }
        if (LEARNED) {
            const unsigned mm = __ballot_sync(0xffffffffu, marginal);
            const int nm = __popc(mm);
            if (nm && fill + nm > LCHUNK) {
                // pad the current chunk's tail, take the next chunk and link it
                if (chunk >= 0 && chunk < LR.cap)
                    for (int i = fill + lane; i < LCHUNK; i += 32) LR.rec[size_t(chunk) * LCHUNK + i] = -1;
                int nc = 0;
                if (lane == 0) nc = atomicAdd(LR.used, 1);
                nc = __shfl_sync(0xffffffffu, nc, 0);
                if (lane == 0) {
                    if (nc < LR.cap) {
                        LR.chunk_group[nc] = group;
                        LR.next[nc] = -1;
                    } else {
                        atomicOr(err, 2);
                    }
                    if (chunk < 0) LR.head[group] = nc;
                    else if (chunk < LR.cap) LR.next[chunk] = nc;
                }
                chunk = nc;
                fill = 0;
            }
            if (marginal && chunk < LR.cap) LR.rec[size_t(chunk) * LCHUNK + fill + __popc(mm & lt)] = node;
            fill += nm;
            learned += nm;
        }
        const bool rest = have && !handed && B.y < range.y;  // later siblings remain
        // An opened cell with at most GW_FLAT nodes below it is not pushed: the bodies
        // of its leaves go straight to the body list (below). Exact sums instead of its
        // descendants' multipoles, so never less accurate; it saves the pops and votes
        // of the tree's last levels.
        const bool flat = GW_FLAT > 0 && open && B.y - node - 1 <= GW_FLAT;
        const bool kids = open && !flat;
        const int np = int(rest) + int(kids);
        // each lane's pushes follow those of the lanes below it
        const unsigned mrest = __ballot_sync(0xffffffffu, rest), mopen = __ballot_sync(0xffffffffu, kids);
        const int total = __popc(mrest) + __popc(mopen);
        int slot = S + __popc(mrest & lt) + __popc(mopen & lt);
        if (slot + np > stack_cap) {
            failed = true;  // never written out of bounds
        } else {
            if (rest) stack[slot++] = make_int2(B.y, range.y);
            if (kids) stack[slot++] = make_int2(node + 1, B.y);  // children on top: popped first
        }
        if (__any_sync(0xffffffffu, failed)) {
            failed = true;
            break;
        }
        S += total;
        maxS = max(maxS, S);
        const bool acc = have && !open;
        bool farc = false;
        if (LOCAL && acc && (B.z < 0 || B.w == 1) && A.w != 0.0f) {  // cells and single bodies
            const float dx = A.x - lgx, dy = A.y - lgy, dz = A.z - lgz;
            farc = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > far2;
        }
        if (LOCAL) {
            const unsigned mf = __ballot_sync(0xffffffffu, farc);
            if (mf) {
                // the low bit asks for the cell's quadrupole (not for monopole-only cells)
                const bool farq = farc && B.z < 0 && !monoq;
                if (farc) s_far[warp][Nf + __popc(mf & lt)] = 2 * node + (farq ? 1 : 0);
                if (QUAD) nlocalq += __popc(__ballot_sync(0xffffffffu, farq));
                Nf += __popc(mf);
                nlocal += __popc(mf);
                __syncwarp();
                if (Nf >= 32) {  // the newest 32: one per lane
                    Nf -= 32;
                    local_add_node<QUAD>(s_lx[warp], lane, s_far[warp][Nf + lane], nodeA, nodeQ, lgx, lgy, lgz,
                                         eps2);
                    __syncwarp();
                }
            }
        }
        const bool bucket = acc && B.z >= 0 && B.w > 1;
        const bool cellacc = acc && B.z < 0 && !farc && !monoq;
        // single bodies, and cells whose quadrupole term is negligible (monoq): monopoles
        const bool bodyacc = acc && (B.z >= 0 ? B.w == 1 : monoq) && !farc;
        // accepted cells -> the cell list (with their quadrupoles)
        const unsigned mc = __ballot_sync(0xffffffffu, cellacc);
        const int nc1 = __popc(mc);
        if (Nc + nc1 > CellList::CAP) {
            eval_list<NFC, CellList::CAP, GUARD, TPL>(Lc, Nc, px, py, pz, e2, bsum);
            entries += Nc;
            centries += Nc;
            Nc = 0;
        }
        if (cellacc) {
            const int e = Nc + __popc(mc & lt);
            Lc.f[0][e] = A.x;
            Lc.f[1][e] = A.y;
            Lc.f[2][e] = A.z;
            Lc.f[3][e] = A.w;
            if constexpr (QUAD) {  // negated: the list evaluation's form
                const float4 q0 = __ldg(nodeQ + 2 * node);
                const float4 q1 = __ldg(nodeQ + 2 * node + 1);
                Lc.f[4][e] = -q0.x;
                Lc.f[5][e] = -q0.y;
                Lc.f[6][e] = -q0.z;
                Lc.f[7][e] = -q0.w;
                Lc.f[8][e] = -q1.x;
                Lc.f[9][e] = -q1.y;
            }
        }
        Nc += nc1;
        // accepted single-body leaves -> the body list (monopole only)
        const unsigned mb1 = __ballot_sync(0xffffffffu, bodyacc);
        const int nb1 = __popc(mb1);
        if (Nb + nb1 > BodyList::CAP) {
            eval_list<4, BodyList::CAP, GUARD, TPL>(Lb, Nb, px, py, pz, e2, bsum);
            entries += Nb;
            Nb = 0;
        }
        if (bodyacc) {
            const int e = Nb + __popc(mb1 & lt);
            Lb.f[0][e] = A.x;
            Lb.f[1][e] = A.y;
            Lb.f[2][e] = A.z;
            Lb.f[3][e] = A.w;
        }
        Nb += nb1;
        // bodies [f, f + c) of the key-ordered array -> the body list (warp-uniform f, c)
        auto append_bodies = [&](int f, int c) {
            for (int base = 0; base < c; base += 32) {
                const int n = min(32, c - base);
                if (Nb + n > BodyList::CAP) {
                    eval_list<4, BodyList::CAP, GUARD, TPL>(Lb, Nb, px, py, pz, e2, bsum);
                    entries += Nb;
                    Nb = 0;
                }
                if (lane < n) {
                    const float4 q = __ldg(sbody + f + base + lane);
                    Lb.f[0][Nb + lane] = q.x;
                    Lb.f[1][Nb + lane] = q.y;
                    Lb.f[2][Nb + lane] = q.z;
                    Lb.f[3][Nb + lane] = q.w;
                }
                Nb += n;
            }
        };
        unsigned mb = __ballot_sync(0xffffffffu, bucket);
        while (mb) {  // leaves holding several bodies: one entry per body
            const int src = __ffs(mb) - 1;
            mb &= mb - 1;
            append_bodies(__shfl_sync(0xffffffffu, B.z, src), __shfl_sync(0xffffffffu, B.w, src));
        }
        // Small opened subtrees, all of this pop's at once: their nodes are numbered
        // across the warp (a prefix sum of the subtrees' sizes) and loaded 32 at a
        // time, one per lane; the leaves' bodies go to the body list.
        if constexpr (GW_FLAT > 0) {
            const int fcnt = flat ? B.y - node - 1 : 0;
            int fincl = fcnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, fincl, o);
                if (lane >= o) fincl += t;
            }
            const int ftot = __shfl_sync(0xffffffffu, fincl, 31);
            visits += ftot;
            for (int fb = 0; fb < ftot; fb += 32) {
                const int j = fb + lane;
                // the subtree holding node j: the number of lanes whose prefix ends at or before j
                int o = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, fincl, o + step - 1);
                    if (v <= j) o += step;
                }
                o = min(o, 31);
                const int first = __shfl_sync(0xffffffffu, node, o) + 1;
                const int before = __shfl_sync(0xffffffffu, fincl, o) - __shfl_sync(0xffffffffu, fcnt, o);
                const int nd = first + j - before;
                int4 lb = make_int4(0, 0, -1, 0);
                float4 la = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j < ftot) lb = __ldg(nodeB + nd);
                const bool one = lb.z >= 0 && lb.w == 1;  // a single-body leaf: its record is the body
                if (one) la = __ldg(nodeA + nd);
                const unsigned m1 = __ballot_sync(0xffffffffu, one);
                const int n1 = __popc(m1);
                if (Nb + n1 > BodyList::CAP) {
                    eval_list<4, BodyList::CAP, GUARD, TPL>(Lb, Nb, px, py, pz, e2, bsum);
                    entries += Nb;
                    Nb = 0;
                }
                if (one) {
                    const int e = Nb + __popc(m1 & lt);
                    Lb.f[0][e] = la.x;
                    Lb.f[1][e] = la.y;
                    Lb.f[2][e] = la.z;
                    Lb.f[3][e] = la.w;
                }
                Nb += n1;
                unsigned mm = __ballot_sync(0xffffffffu, lb.z >= 0 && lb.w > 1);
                while (mm) {
                    const int s2 = __ffs(mm) - 1;
                    mm &= mm - 1;
                    append_bodies(__shfl_sync(0xffffffffu, lb.z, s2), __shfl_sync(0xffffffffu, lb.w, s2));
                }
            }
        }
        __syncwarp();
    }
    eval_list<NFC, CellList::CAP, GUARD, TPL>(Lc, Nc, px, py, pz, e2, bsum);
    eval_list<4, BodyList::CAP, GUARD, TPL>(Lb, Nb, px, py, pz, e2, bsum);
    entries += Nc + Nb;
    centries += Nc;
    float rx[TPL], ry[TPL], rz[TPL];
#pragma unroll
    for (int i = 0; i < TPL; ++i) bsum.total(i, rx[i], ry[i], rz[i]);
    if (LOCAL) {
        if (lane < Nf) local_add_node<QUAD>(s_lx[warp], lane, s_far[warp][lane], nodeA, nodeQ, lgx, lgy, lgz, eps2);
        __syncwarp();
        LocalExp LX;
        float *lf = &LX.ax;
#pragma unroll
        for (int k = 0; k < 19; ++k) lf[k] = s_lx[warp][k][lane];
        local_reduce(LX);
#pragma unroll
        for (int i = 0; i < TPL; ++i) {
            float lx, ly, lz;
            local_eval(LX, p[i].x - lgx, p[i].y - lgy, p[i].z - lgz, lx, ly, lz);
            rx[i] += lx;
            ry[i] += ly;
            rz[i] += lz;
        }
    }
    const unsigned long long nv = unsigned(nvalid);
    unsigned long long s_acc = entries * nv, s_vis = visits * nv, s_cell = centries * nv;
    if (failed) {
        // The stack ran out (failed is warp-uniform): this warp's targets take the
        // reference's per-body walk instead, which needs no stack.
        unsigned na = 0, nvis = 0, nc = 0;
#pragma unroll
        for (int i = 0; i < TPL; ++i) {
            rx[i] = ry[i] = rz[i] = 0.f;
            lane_walk<QUAD>(p[i], valid[i], T, nodeA, nodeB, nodeQ, sbody, th2, eps2, rx[i], ry[i], rz[i], na, nvis,
                            nc, REL ? gscale[group] : 0.f);
        }
        unsigned long long a = na, v = nvis, c = nc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            v += __shfl_xor_sync(0xffffffffu, v, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        s_acc = a;
        s_vis = v;
        s_cell = c;
    }
    if (LEARNED) {
        if (chunk >= 0 && chunk < LR.cap)
            for (int i = fill + lane; i < LCHUNK; i += 32) LR.rec[size_t(chunk) * LCHUNK + i] = -1;
        if (lane == 0) {
            if (chunk < 0 || failed) LR.head[group] = -1;  // a fallback warp keeps the plain result
            LR.centre[group] = make_float4(gcx, gcy, gcz, 0.f);
        }
    }
#pragma unroll
    for (int i = 0; i < TPL; ++i)
        if (valid[i]) {
            const uint32_t o = tidx[g0 + 32 * i + lane];
            out[3 * size_t(o) + 0] = rx[i];
            out[3 * size_t(o) + 1] = ry[i];
            out[3 * size_t(o) + 2] = rz[i];
        }
    if (stats && lane == 0) {
        atomicAdd(stats + 0, s_acc);
        atomicAdd(stats + 1, s_vis);
        if (LEARNED) atomicAdd(stats + 4, learned);
        if (LOCAL && !failed) {
            atomicAdd(stats + 7, nlocal);
            if (QUAD) atomicAdd(stats + 8, nlocalq);
        }
        atomicAdd(stats + 5, s_cell);
        atomicAdd(stats + 2, 1ull);
        atomicMax(stats + 3, (unsigned long long)maxS);
        if (failed) atomicAdd(stats + 6, 1ull);
    }
}

// PT_BH_RELATIVE: |a| estimated at the centre of each group's box by a walk at theta
// = 1.5 with monopoles; gscale[g] = 1 / (alpha |a|), the factor of the group walk's
// error bound. (At N = 4M bulge+disk, estimates from theta 1.0 and 1.5 walks select
// the same cells up to 0.2 %; 1.5 visits about half the nodes.)
// The per-point cursor walk: the node index only grows, so the loop ends.
__device__ __forceinline__ void scale_cursor_walk(float cx, float cy, float cz, const float4 *__restrict__ nodeA,
                                                  const int4 *__restrict__ nodeB, int T, float eps2, float &ax,
                                                  float &ay, float &az) {
    for (int node = 0; node < T;) {
        const float4 A = __ldg(nodeA + node);
        const int4 B = __ldg(nodeB + node);
        const float dx = A.x - cx, dy = A.y - cy, dz = A.z - cz;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (B.z < 0) {
            const float w = __int_as_float(B.x);
            if (2.25f * d2 < w * w) {  // theta = 1.5: open
                ++node;
                continue;
            }
        }
        if (d2 > 0.f) {
            const float inv = rsqrt_ftz(d2 + eps2);
            const float s = (A.w * inv) * (inv * inv);
            ax = fmaf(dx, s, ax);
            ay = fmaf(dy, s, ay);
            az = fmaf(dz, s, az);
        }
        node = B.y;
    }
}

// One thread per group: the group's box, then the cursor walk from its centre. (One
// warp per group walking with a range stack, one node per lane and pop, was slower at
// N = 4M: the walk phase, which includes this kernel, went from 5.68 to 5.85 ms. Its
// 65536 warps take several waves, each pop a round trip to L2, while the threads'
// cursor walks mostly hit L1 in the tree's upper levels. Eight threads per group, each
// walking one of the root's children's subtrees, took the same 0.124 ms: the group's
// own octant holds most of the visits. Four lanes per group popping up to four ranges
// of a shared-memory stack per step took 0.18 ms: a walk from one point keeps few
// ranges open, so the steps stayed nearly as many and each cost more.)
__global__ void __launch_bounds__(128)
    bh_group_scale(const float4 *__restrict__ tbody, int n_aff, const float4 *__restrict__ nodeA,
                   const int4 *__restrict__ nodeB, const int *__restrict__ counters, float eps2, float alpha,
                   float *__restrict__ gscale) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int g0 = g * GW_GROUP;
    if (g0 >= n_aff) return;
    const int g1 = min(n_aff, g0 + GW_GROUP);
    float4 p = tbody[g0];
    float mn0 = p.x, mn1 = p.y, mn2 = p.z, mx0 = p.x, mx1 = p.y, mx2 = p.z;
    for (int t = g0 + 1; t < g1; ++t) {
        p = tbody[t];
        mn0 = fminf(mn0, p.x), mn1 = fminf(mn1, p.y), mn2 = fminf(mn2, p.z);
        mx0 = fmaxf(mx0, p.x), mx1 = fmaxf(mx1, p.y), mx2 = fmaxf(mx2, p.z);
    }
    float ax = 0.f, ay = 0.f, az = 0.f;
    scale_cursor_walk(0.5f * (mn0 + mx0), 0.5f * (mn1 + mx1), 0.5f * (mn2 + mx2), nodeA, nodeB, counters[1], eps2,
                      ax, ay, az);
    const float a = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
    gscale[g] = 1.f / (alpha * fmaxf(a, 1e-30f));
}

// ---- masked group walk: the reference's rule, per body, with shared traversal ----
// The default method (no PT_BH_GROUP). One warp walks for MW_TPL x 32 key-adjacent
// bodies (MW_TPL per lane) like bh_walk_group, but every stack range carries the
// masks of the bodies that still descend into it, and every list entry the masks of
// the bodies that accept it: each body's accepted set is exactly the reference's
// (sequential.rs:470-505: skip a node at d^2 == 0, open a cell when theta^2 d^2 <
// w^2, else accept). A list entry is evaluated for every body and weighted by the
// body's mask bit. Sums run in list order instead of the reference's visit order
// (rounding-level differences).
// Warps (groups) per CTA of the masked walk: one, so that a finished group's slot is
// refilled at once (walk at N = 4M, 4 / 2 / 1 warps per CTA: theta 0.5 14.57 / 14.46 /
// 14.26 ms, with quadrupoles 22.79 / 22.60 / 22.64, theta 0.3 40.06 / 40.36 / 39.87).
#ifndef PT_MW_WARPS
#define PT_MW_WARPS 1
#endif
constexpr int MW_WARPS = PT_MW_WARPS;
// Stack ranges per warp of the masked walk: 320 fit 20 one-warp CTAs per SM in shared
// memory (384: 18). Walk at N = 4M, 384 -> 320: theta 0.5 13.96 -> 13.81 ms, with
// quadrupoles 22.51 -> 22.38, theta 0.3 39.40 -> 39.03 (12 of 65536 warps then run out
// of stack and take the per-body cursor walk: the same accepted sets).
#ifndef PT_MW_STACK
#define PT_MW_STACK 320
#endif
constexpr int MW_STACK = PT_MW_STACK;
// List capacities of the masked walk (88 cells / 112 bodies, for 21 warps per SM, and
// 17 with quadrupoles, measured 0.3-0.6 % slower).
#ifndef PT_MW_CELLS
#define PT_MW_CELLS 96
#endif
#ifndef PT_MW_BODIES
#define PT_MW_BODIES 128
#endif
constexpr int MW_TPL = 2;  // bodies per lane; mask word i covers bodies g0 + 32 i + lane

// Entry pair (packed lo/hi) for one body, weighted by the body's bits of the two
// entries' masks (qm = the pair's mask words for this body's word).
template <int NF, bool GUARD>
__device__ __forceinline__ void eval_pair_masked(const f2 *q, f2 qm, f2 px, f2 py, f2 pz, f2 e2, f2 &ax, f2 &ay,
                                                 f2 &az) {
    const int lane = threadIdx.x & 31;
    float m0, m1;
    upk2(qm, m0, m1);
    const f2 bit = pk2(float((__float_as_uint(m0) >> lane) & 1u), float((__float_as_uint(m1) >> lane) & 1u));
    const f2 dx = sub2(q[0], px);
    const f2 dy = sub2(q[1], py);
    const f2 dz = sub2(q[2], pz);
    const f2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
    float r0, r1;
    upk2(r2, r0, r1);
    float i0 = rsqrt_ftz(r0), i1 = rsqrt_ftz(r1);
    if (GUARD) {
        i0 = (r0 > 0.0f) ? i0 : 0.0f;
        i1 = (r1 > 0.0f) ? i1 : 0.0f;
    }
    const f2 inv = mul2(pk2(i0, i1), bit);  // a body outside the entry's mask adds exactly 0
    const f2 inv2 = mul2(inv, inv);
    const f2 sc = mul2(mul2(q[3], inv), inv2);
    if constexpr (NF == 10) {
        const f2 ux = fma2(q[4], dx, fma2(q[5], dy, mul2(q[6], dz)));
        const f2 uy = fma2(q[5], dx, fma2(q[7], dy, mul2(q[8], dz)));
        const f2 uz = fma2(q[6], dx, fma2(q[8], dy, mul2(q[9], dz)));
        const f2 c = fma2(dx, ux, fma2(dy, uy, mul2(dz, uz)));
        const f2 inv5 = mul2(mul2(inv2, inv2), inv);
        const f2 k = mul2(c, mul2(inv2, pk2(-2.5f, -2.5f)));
        const f2 s2 = fma2(inv5, k, sc);
        ax = fma2(dx, s2, fma2(inv5, ux, ax));
        ay = fma2(dy, s2, fma2(inv5, uy, ay));
        az = fma2(dz, s2, fma2(inv5, uz, az));
    } else {
        ax = fma2(dx, sc, ax);
        ay = fma2(dy, sc, ay);
        az = fma2(dz, sc, az);
    }
}

// Lists hold NF fields then MW_TPL mask words per entry.
template <int NF, int CAP, bool GUARD>
__device__ __forceinline__ void eval_list_masked(IList<NF + MW_TPL, CAP> &Lst, int cnt, const f2 (&px)[MW_TPL],
                                                 const f2 (&py)[MW_TPL], const f2 (&pz)[MW_TPL], f2 e2,
                                                 RegSums<MW_TPL> &acc) {
    const int lane = threadIdx.x & 31;
    f2 ax[MW_TPL], ay[MW_TPL], az[MW_TPL];
#pragma unroll
    for (int i = 0; i < MW_TPL; ++i) ax[i] = ay[i] = az[i] = pk2(0.f, 0.f);
    __syncwarp();
    if (cnt & 1) {  // pad: far away, massless, empty masks
        if (lane < NF + MW_TPL) Lst.f[lane][cnt] = (lane < 3) ? 1e30f : 0.0f;
        __syncwarp();
        ++cnt;
    }
#pragma unroll 2
    for (int e = 0; e < cnt; e += 2) {
        f2 q[NF + MW_TPL];
#pragma unroll
        for (int k = 0; k < NF + MW_TPL; ++k) q[k] = *reinterpret_cast<const f2 *>(&Lst.f[k][e]);
#pragma unroll
        for (int i = 0; i < MW_TPL; ++i)
            eval_pair_masked<NF, GUARD>(q, q[NF + i], px[i], py[i], pz[i], e2, ax[i], ay[i], az[i]);
    }
#pragma unroll
    for (int i = 0; i < MW_TPL; ++i) acc.fold(i, ax[i], ay[i], az[i]);
    __syncwarp();
}

template <bool QUAD, bool GUARD>
__global__ void __launch_bounds__(32 * MW_WARPS)
    bh_walk_masked(const float4 *__restrict__ tbody, const uint32_t *__restrict__ tidx, int n_aff,
                   const float4 *__restrict__ nodeA, const int4 *__restrict__ nodeB,
                   const float4 *__restrict__ nodeQ, const float4 *__restrict__ sbody,
                   const int *__restrict__ counters, float th2, float eps2, float *__restrict__ out,
                   unsigned long long *__restrict__ stats) {
    constexpr int NFC = QUAD ? 10 : 4;
    constexpr int TPL = MW_TPL;
    static_assert(TPL == 2, "stack entries hold two mask words");
    using CellList = IList<NFC + TPL, PT_MW_CELLS>;  // + the masks of the accepting bodies
    using BodyList = IList<4 + TPL, PT_MW_BODIES>;
    __shared__ int4 s_stack[MW_WARPS][MW_STACK];  // (first, end, mask word 0, mask word 1)
    __shared__ __align__(16) CellList s_cells[MW_WARPS];
    __shared__ __align__(16) BodyList s_bodies[MW_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g0 = (blockIdx.x * MW_WARPS + warp) * 32 * TPL;
    if (g0 >= n_aff) return;
    float4 p[TPL];
    bool valid[TPL];
    unsigned vmask[TPL];
#pragma unroll
    for (int i = 0; i < TPL; ++i) {
        const int t = g0 + 32 * i + lane;
        valid[i] = t < n_aff;
        p[i] = tbody[valid[i] ? t : g0];
        vmask[i] = __ballot_sync(0xffffffffu, valid[i]);
    }
    const unsigned lt = (1u << lane) - 1u;
    int4 *stack = s_stack[warp];
    const int T = counters[1];
    CellList &Lc = s_cells[warp];
    BodyList &Lb = s_bodies[warp];
    float mn0 = fminf(p[0].x, p[1].x), mn1 = fminf(p[0].y, p[1].y), mn2 = fminf(p[0].z, p[1].z);
    float mx0 = fmaxf(p[0].x, p[1].x), mx1 = fmaxf(p[0].y, p[1].y), mx2 = fmaxf(p[0].z, p[1].z);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn0 = fminf(mn0, __shfl_xor_sync(0xffffffffu, mn0, o));
        mn1 = fminf(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mn2 = fminf(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
    }
    const f2 e2 = pk2(eps2, eps2);
    f2 px[TPL], py[TPL], pz[TPL];
    RegSums<TPL> bsum;  // the bodies' compensated sums over the evaluated lists
    bsum.zero();
#pragma unroll
    for (int i = 0; i < TPL; ++i) {
        px[i] = pk2(p[i].x, p[i].x);
        py[i] = pk2(p[i].y, p[i].y);
        pz[i] = pk2(p[i].z, p[i].z);
    }
    if (lane == 0) stack[0] = make_int4(0, T, int(vmask[0]), int(vmask[1]));
    __syncwarp();
    int S = 1, Nc = 0, Nb = 0;
    unsigned long long acc_pairs = 0, cell_pairs = 0, visit_pairs = 0;
    bool failed = false;
    while (S > 0) {
        const int k = min(min(32, S), max(1, (MW_STACK - S) / 2));
        const bool first = lane < k;
        int4 r = first ? stack[S - 1 - lane] : make_int4(0, 0, 0, 0);
        __syncwarp();
        S -= k;
        int node = r.x;
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 B = make_int4(0, 0, 0, 0);
        if (first) {
            A = __ldg(nodeA + node);
            B = __ldg(nodeB + node);
        }
        // A pop of fewer than 32 ranges leaves lanes idle: lane k + i then also takes
        // the second node of range i (its first node's skip pointer) with the range's
        // masks, and the rest of the range passes to it. Each range still pushes at
        // most three ranges, within the room k was sized for (2 per popped range).
        bool second = false;
        if (k < 32) {
            const int src = lane >= k ? lane - k : lane;
            const int nxt = __shfl_sync(0xffffffffu, B.y, src);
            const int end = __shfl_sync(0xffffffffu, r.y, src);
            const int m0 = __shfl_sync(0xffffffffu, r.z, src), m1 = __shfl_sync(0xffffffffu, r.w, src);
            if (lane >= k && src < k && nxt < end) {
                second = true;
                node = nxt;
                r = make_int4(nxt, end, m0, m1);
                A = __ldg(nodeA + node);
                B = __ldg(nodeB + node);
            }
        }
        const unsigned msecond = __ballot_sync(0xffffffffu, second);
        // its rest went to lane + k
        const bool handed = first && lane + k < 32 && ((msecond >> (lane + k)) & 1u);
        const bool have = first || second;
        const unsigned mk0 = unsigned(r.z), mk1 = unsigned(r.w);
        visit_pairs += __popc(mk0) + __popc(mk1);
        // Per node: which of its bodies open it and which accept it. The bodies' box
        // settles most nodes; a node whose centre of mass lies inside the box (a body
        // may coincide with it: skipped) or whose rule differs across the box is
        // voted on, each lane testing its own bodies.
        const bool cell = B.z < 0;
        const float w = cell ? __int_as_float(B.x) : 0.f;
        unsigned op0 = 0, op1 = 0, ac0 = 0, ac1 = 0;
        bool need = false;
        if (have && (mk0 | mk1)) {
            const float e0 = fmaxf(fmaxf(mn0 - A.x, A.x - mx0), 0.f);
            const float e1 = fmaxf(fmaxf(mn1 - A.y, A.y - mx1), 0.f);
            const float e2b = fmaxf(fmaxf(mn2 - A.z, A.z - mx2), 0.f);
            const float db2 = fmaf(e0, e0, fmaf(e1, e1, e2b * e2b));
            const bool inside = !(db2 > 0.0f);
            if (inside) {
                need = true;
            } else if (!cell || !(th2 * db2 < w * w)) {  // every body accepts
                ac0 = mk0;
                ac1 = mk1;
            } else {
                const float f0 = fmaxf(A.x - mn0, mx0 - A.x);
                const float f1 = fmaxf(A.y - mn1, mx1 - A.y);
                const float f2b = fmaxf(A.z - mn2, mx2 - A.z);
                if (th2 * fmaf(f0, f0, fmaf(f1, f1, f2b * f2b)) < w * w) {  // every body opens
                    op0 = mk0;
                    op1 = mk1;
                } else {
                    need = true;
                }
            }
        }
        unsigned vm = __ballot_sync(0xffffffffu, need);
        while (vm) {
            const int j = __ffs(vm) - 1;
            vm &= vm - 1;
            const float cx = __shfl_sync(0xffffffffu, A.x, j);
            const float cy = __shfl_sync(0xffffffffu, A.y, j);
            const float cz = __shfl_sync(0xffffffffu, A.z, j);
            const float cw = __shfl_sync(0xffffffffu, w, j);
            const unsigned mj0 = __shfl_sync(0xffffffffu, mk0, j), mj1 = __shfl_sync(0xffffffffu, mk1, j);
            const bool cj = __shfl_sync(0xffffffffu, cell, j);
            const f2 dx = sub2(pk2(cx, cx), pk2(p[0].x, p[1].x));
            const f2 dy = sub2(pk2(cy, cy), pk2(p[0].y, p[1].y));
            const f2 dz = sub2(pk2(cz, cz), pk2(p[0].z, p[1].z));
            float d0, d1;
            upk2(fma2(dx, dx, fma2(dy, dy, mul2(dz, dz))), d0, d1);
            const bool in0 = (mj0 >> lane) & 1u, in1 = (mj1 >> lane) & 1u;
            const bool o0 = in0 && cj && d0 > 0.0f && th2 * d0 < cw * cw;
            const bool o1 = in1 && cj && d1 > 0.0f && th2 * d1 < cw * cw;
            const unsigned om0 = __ballot_sync(0xffffffffu, o0), om1 = __ballot_sync(0xffffffffu, o1);
            const unsigned am0 = __ballot_sync(0xffffffffu, in0 && !o0 && d0 > 0.0f);
            const unsigned am1 = __ballot_sync(0xffffffffu, in1 && !o1 && d1 > 0.0f);
            if (lane == j) {
                op0 = om0;
                op1 = om1;
                ac0 = am0;
                ac1 = am1;
            }
        }
        // push: later siblings share the parent's masks; children get the opening bodies
        const bool rest = have && !handed && (mk0 | mk1) && B.y < r.y;
        const bool opn = (op0 | op1) != 0u;
        const unsigned mrest = __ballot_sync(0xffffffffu, rest), mopen = __ballot_sync(0xffffffffu, opn);
        const int total = __popc(mrest) + __popc(mopen);
        int slot = S + __popc(mrest & lt) + __popc(mopen & lt);
        if (slot + int(rest) + int(opn) > MW_STACK) {
            failed = true;
        } else {
            if (rest) stack[slot++] = make_int4(B.y, r.y, int(mk0), int(mk1));
            if (opn) stack[slot++] = make_int4(node + 1, B.y, int(op0), int(op1));
        }
        if (__any_sync(0xffffffffu, failed)) {
            failed = true;
            break;
        }
        S += total;
        const int na = __popc(ac0) + __popc(ac1);
        acc_pairs += na;
        const bool accd = na != 0;
        const bool bucket = accd && !cell && B.w > 1;
        const bool cellacc = accd && cell;
        const bool bodyacc = accd && !cell && B.w == 1;
        if (cellacc) cell_pairs += na;
        const unsigned mc = __ballot_sync(0xffffffffu, cellacc);
        const int nc1 = __popc(mc);
        if (Nc + nc1 > CellList::CAP) {
            eval_list_masked<NFC, CellList::CAP, GUARD>(Lc, Nc, px, py, pz, e2, bsum);
            Nc = 0;
        }
        if (cellacc) {
            const int e = Nc + __popc(mc & lt);
            Lc.f[0][e] = A.x;
            Lc.f[1][e] = A.y;
            Lc.f[2][e] = A.z;
            Lc.f[3][e] = A.w;
            if constexpr (QUAD) {  // negated: the list evaluation's form
                const float4 q0 = __ldg(nodeQ + 2 * node);
                const float4 q1 = __ldg(nodeQ + 2 * node + 1);
                Lc.f[4][e] = -q0.x;
                Lc.f[5][e] = -q0.y;
                Lc.f[6][e] = -q0.z;
                Lc.f[7][e] = -q0.w;
                Lc.f[8][e] = -q1.x;
                Lc.f[9][e] = -q1.y;
            }
            Lc.f[NFC][e] = __uint_as_float(ac0);
            Lc.f[NFC + 1][e] = __uint_as_float(ac1);
        }
        Nc += nc1;
        const unsigned mb1 = __ballot_sync(0xffffffffu, bodyacc);
        const int nb1 = __popc(mb1);
        if (Nb + nb1 > BodyList::CAP) {
            eval_list_masked<4, BodyList::CAP, GUARD>(Lb, Nb, px, py, pz, e2, bsum);
            Nb = 0;
        }
        if (bodyacc) {
            const int e = Nb + __popc(mb1 & lt);
            Lb.f[0][e] = A.x;
            Lb.f[1][e] = A.y;
            Lb.f[2][e] = A.z;
            Lb.f[3][e] = A.w;
            Lb.f[4][e] = __uint_as_float(ac0);
            Lb.f[5][e] = __uint_as_float(ac1);
        }
        Nb += nb1;
        unsigned mbk = __ballot_sync(0xffffffffu, bucket);
        while (mbk) {  // leaves holding several bodies: one entry per body, the leaf's masks
            const int src = __ffs(mbk) - 1;
            mbk &= mbk - 1;
            const int f = __shfl_sync(0xffffffffu, B.z, src);
            const int c = __shfl_sync(0xffffffffu, B.w, src);
            const unsigned b0 = __shfl_sync(0xffffffffu, ac0, src), b1 = __shfl_sync(0xffffffffu, ac1, src);
            for (int base = 0; base < c; base += 32) {
                const int n = min(32, c - base);
                if (Nb + n > BodyList::CAP) {
                    eval_list_masked<4, BodyList::CAP, GUARD>(Lb, Nb, px, py, pz, e2, bsum);
                    Nb = 0;
                }
                if (lane < n) {
                    const float4 q = __ldg(sbody + f + base + lane);
                    Lb.f[0][Nb + lane] = q.x;
                    Lb.f[1][Nb + lane] = q.y;
                    Lb.f[2][Nb + lane] = q.z;
                    Lb.f[3][Nb + lane] = q.w;
                    Lb.f[4][Nb + lane] = __uint_as_float(b0);
                    Lb.f[5][Nb + lane] = __uint_as_float(b1);
                }
                Nb += n;
            }
        }
        __syncwarp();
    }
    eval_list_masked<NFC, CellList::CAP, GUARD>(Lc, Nc, px, py, pz, e2, bsum);
    eval_list_masked<4, BodyList::CAP, GUARD>(Lb, Nb, px, py, pz, e2, bsum);
    float rx[TPL], ry[TPL], rz[TPL];
#pragma unroll
    for (int i = 0; i < TPL; ++i) bsum.total(i, rx[i], ry[i], rz[i]);
    if (failed) {  // the stack ran out: the per-body cursor walk instead (warp-uniform)
        unsigned na = 0, nv = 0, nc = 0;
#pragma unroll
        for (int i = 0; i < TPL; ++i) {
            rx[i] = ry[i] = rz[i] = 0.f;
            lane_walk<QUAD>(p[i], valid[i], T, nodeA, nodeB, nodeQ, sbody, th2, eps2, rx[i], ry[i], rz[i], na, nv,
                            nc);
        }
        acc_pairs = na;
        cell_pairs = nc;
        visit_pairs = nv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {  // per-lane counts -> the warp's
        acc_pairs += __shfl_xor_sync(0xffffffffu, acc_pairs, o);
        cell_pairs += __shfl_xor_sync(0xffffffffu, cell_pairs, o);
        visit_pairs += __shfl_xor_sync(0xffffffffu, visit_pairs, o);
    }
#pragma unroll
    for (int i = 0; i < TPL; ++i)
        if (valid[i]) {
            const uint32_t o = tidx[g0 + 32 * i + lane];
            out[3 * size_t(o) + 0] = rx[i];
            out[3 * size_t(o) + 1] = ry[i];
            out[3 * size_t(o) + 2] = rz[i];
        }
    if (stats && lane == 0) {
        atomicAdd(stats + 0, acc_pairs);
        atomicAdd(stats + 1, visit_pairs);
        atomicAdd(stats + 2, 1ull);
        atomicAdd(stats + 5, cell_pairs);
        if (failed) atomicAdd(stats + 6, 1ull);
    }
}

// ---- the reference rule over DVec3 bodies (f64 method) -------------------------
// As bh_walk_masked with one body per lane, in double: node data, widths and the
// per-pair kernel (impl_acceleration_cpu_scalar!(DVec3, f64): d * (m / (n_s sqrt
// n_s)), IEEE-rounded in the reference's order) are f64; accepted sets per body
// are the reference's. Monopole only, as the reference.
constexpr int W64_WARPS = 4;
constexpr int W64_STACK = 384;

__device__ __forceinline__ void pair64(double px, double py, double pz, double cx, double cy, double cz, double m,
                                       double eps2, double &ax, double &ay, double &az) {
    const double dx = __dsub_rn(cx, px), dy = __dsub_rn(cy, py), dz = __dsub_rn(cz, pz);
    const double n = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (n == 0.0) return;  // checked: d itself, which is zero
    const double ns = __dadd_rn(n, eps2);
    const double s = __ddiv_rn(m, __dmul_rn(ns, __dsqrt_rn(ns)));
    ax = __dadd_rn(ax, __dmul_rn(dx, s));
    ay = __dadd_rn(ay, __dmul_rn(dy, s));
    az = __dadd_rn(az, __dmul_rn(dz, s));
}

struct List64 {
    static constexpr int CAP = 128;
    double f[4][CAP];
    unsigned mask[CAP];
};

__device__ __forceinline__ void eval_list64(const List64 &Lst, int cnt, double px, double py, double pz, double eps2,
                                            double &ax, double &ay, double &az) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int e = 0; e < cnt; ++e)
        if ((Lst.mask[e] >> lane) & 1u) pair64(px, py, pz, Lst.f[0][e], Lst.f[1][e], Lst.f[2][e], Lst.f[3][e], eps2, ax, ay, az);
    __syncwarp();
}

__global__ void __launch_bounds__(32 * W64_WARPS)
    bh_walk64(const double4_32a *__restrict__ tbody, const uint32_t *__restrict__ tidx, int n_aff,
              const double4_32a *__restrict__ nodeA, const int4 *__restrict__ nodeB,
              const double4_32a *__restrict__ nodeG, const double4_32a *__restrict__ sbody,
              const int *__restrict__ counters, double th2, double eps2, double *__restrict__ out,
              unsigned long long *__restrict__ stats, int *__restrict__ err) {
    __shared__ int4 s_stack[W64_WARPS][W64_STACK];
    __shared__ List64 s_list[W64_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int group = blockIdx.x * W64_WARPS + warp;
    if (group * 32 >= n_aff) return;
    const int t = group * 32 + lane;
    const bool valid = t < n_aff;
    const double4_32a p = tbody[valid ? t : group * 32];
    const unsigned lt = (1u << lane) - 1u;
    const unsigned valid_mask = __ballot_sync(0xffffffffu, valid);
    int4 *stack = s_stack[warp];
    List64 &Lst = s_list[warp];
    const int T = counters[1];
    double mn0 = p.x, mn1 = p.y, mn2 = p.z, mx0 = p.x, mx1 = p.y, mx2 = p.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn0 = fmin(mn0, __shfl_xor_sync(0xffffffffu, mn0, o));
        mn1 = fmin(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mn2 = fmin(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx0 = fmax(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmax(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmax(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
    }
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (lane == 0) stack[0] = make_int4(0, T, int(valid_mask), 0);
    __syncwarp();
    int S = 1, Nl = 0;
    unsigned long long acc_pairs = 0, visit_pairs = 0;
    bool failed = false;
    while (S > 0) {
        const int k = min(min(32, S), max(1, (W64_STACK - S) / 2));
        const bool have = lane < k;
        const int4 r = have ? stack[S - 1 - lane] : make_int4(0, 0, 0, 0);
        __syncwarp();
        S -= k;
        const int node = r.x;
        const unsigned mask = unsigned(r.z);
        double4_32a A;
        A.x = A.y = A.z = A.w = 0.0;
        int4 B = make_int4(0, 0, 0, 0);
        double w = 0.0;
        if (have) {
            A = nodeA[node];
            B = __ldg(nodeB + node);
            if (B.z < 0) w = nodeG[node].w;
        }
        visit_pairs += __popc(mask);
        const bool cell = B.z < 0;
        unsigned open_m = 0, acc_m = 0;
        bool need = false;
        if (have && mask) {
            const double e0 = fmax(fmax(mn0 - A.x, A.x - mx0), 0.0);
            const double e1 = fmax(fmax(mn1 - A.y, A.y - mx1), 0.0);
            const double e2b = fmax(fmax(mn2 - A.z, A.z - mx2), 0.0);
            const double db2 = __dadd_rn(__dadd_rn(__dmul_rn(e0, e0), __dmul_rn(e1, e1)), __dmul_rn(e2b, e2b));
            if (!(db2 > 0.0)) {
                need = true;
            } else if (!cell || !(__dmul_rn(th2, db2) < __dmul_rn(w, w))) {
                acc_m = mask;
            } else {
                const double f0 = fmax(A.x - mn0, mx0 - A.x), f1 = fmax(A.y - mn1, mx1 - A.y);
                const double f2b = fmax(A.z - mn2, mx2 - A.z);
                const double dm2 = __dadd_rn(__dadd_rn(__dmul_rn(f0, f0), __dmul_rn(f1, f1)), __dmul_rn(f2b, f2b));
                if (__dmul_rn(th2, dm2) < __dmul_rn(w, w)) open_m = mask;
                else need = true;
            }
        }
        unsigned vm = __ballot_sync(0xffffffffu, need);
        while (vm) {
            const int j = __ffs(vm) - 1;
            vm &= vm - 1;
            const double cx = __shfl_sync(0xffffffffu, A.x, j), cy = __shfl_sync(0xffffffffu, A.y, j);
            const double cz = __shfl_sync(0xffffffffu, A.z, j), cw = __shfl_sync(0xffffffffu, w, j);
            const unsigned mj = __shfl_sync(0xffffffffu, mask, j);
            const bool cj = __shfl_sync(0xffffffffu, cell, j);
            // the reference's d^2: (com - body) squared, x, y, z in order
            const double dx = __dsub_rn(cx, p.x), dy = __dsub_rn(cy, p.y), dz = __dsub_rn(cz, p.z);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            const bool mine = (mj >> lane) & 1u;
            const bool o = mine && cj && d2 > 0.0 && __dmul_rn(th2, d2) < __dmul_rn(cw, cw);
            const bool a = mine && !o && d2 > 0.0;
            const unsigned om = __ballot_sync(0xffffffffu, o), am = __ballot_sync(0xffffffffu, a);
            if (lane == j) {
                open_m = om;
                acc_m = am;
            }
        }
        const bool rest = have && mask && B.y < r.y;
        const bool opn = open_m != 0u;
        const unsigned mrest = __ballot_sync(0xffffffffu, rest), mopen = __ballot_sync(0xffffffffu, opn);
        const int total = __popc(mrest) + __popc(mopen);
        int slot = S + __popc(mrest & lt) + __popc(mopen & lt);
        if (slot + int(rest) + int(opn) > W64_STACK) {
            failed = true;
        } else {
            if (rest) stack[slot++] = make_int4(B.y, r.y, int(mask), 0);
            if (opn) stack[slot++] = make_int4(node + 1, B.y, int(open_m), 0);
        }
        if (__any_sync(0xffffffffu, failed)) {
            failed = true;
            break;
        }
        S += total;
        acc_pairs += __popc(acc_m);
        // accepted cells and single bodies: one list entry with the accepting mask;
        // several-body leaves: one entry per body
        const bool single = acc_m != 0u && (cell || B.w == 1);
        const unsigned ms = __ballot_sync(0xffffffffu, single);
        const int ns = __popc(ms);
        if (Nl + ns > List64::CAP) {
            eval_list64(Lst, Nl, p.x, p.y, p.z, eps2, ax, ay, az);
            Nl = 0;
        }
        if (single) {
            const int e = Nl + __popc(ms & lt);
            Lst.f[0][e] = A.x;
            Lst.f[1][e] = A.y;
            Lst.f[2][e] = A.z;
            Lst.f[3][e] = A.w;
            Lst.mask[e] = acc_m;
        }
        Nl += ns;
        unsigned mbk = __ballot_sync(0xffffffffu, acc_m != 0u && !cell && B.w > 1);
        while (mbk) {
            const int src = __ffs(mbk) - 1;
            mbk &= mbk - 1;
            const int f = __shfl_sync(0xffffffffu, B.z, src), c = __shfl_sync(0xffffffffu, B.w, src);
            const unsigned bm = __shfl_sync(0xffffffffu, acc_m, src);
            for (int base = 0; base < c; base += 32) {
                const int n = min(32, c - base);
                if (Nl + n > List64::CAP) {
                    eval_list64(Lst, Nl, p.x, p.y, p.z, eps2, ax, ay, az);
                    Nl = 0;
                }
                if (lane < n) {
                    const double4_32a q = sbody[f + base + lane];
                    Lst.f[0][Nl + lane] = q.x;
                    Lst.f[1][Nl + lane] = q.y;
                    Lst.f[2][Nl + lane] = q.z;
                    Lst.f[3][Nl + lane] = q.w;
                    Lst.mask[Nl + lane] = bm;
                }
                Nl += n;
            }
        }
        __syncwarp();
    }
    eval_list64(Lst, Nl, p.x, p.y, p.z, eps2, ax, ay, az);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc_pairs += __shfl_xor_sync(0xffffffffu, acc_pairs, o);
        visit_pairs += __shfl_xor_sync(0xffffffffu, visit_pairs, o);
    }
    if (failed) {  // no stackless fallback in f64: the bodies are NaN and the call fails
        ax = ay = az = __longlong_as_double(0x7ff8000000000000ll);
        if (lane == 0) atomicOr(err, 1);
    }
    if (valid) {
        const uint32_t o = tidx[t];
        out[3 * size_t(o) + 0] = ax;
        out[3 * size_t(o) + 1] = ay;
        out[3 * size_t(o) + 2] = az;
    }
    if (stats && lane == 0) {
        atomicAdd(stats + 0, acc_pairs);
        atomicAdd(stats + 1, visit_pairs);
        atomicAdd(stats + 2, 1ull);
    }
}


using WalkKernel = void (*)(const float4 *, const uint32_t *, int, const float4 *, const int4 *, const float4 *,
                            const float4 *, const int *, float, float, float *, unsigned long long *);
using GroupKernel = void (*)(const float4 *, const uint32_t *, int, const float4 *, const int4 *, const float4 *,
                             const float4 *, const float4 *, const int *, float, float, LearnedRecords, float,
                             float *, unsigned long long *, int *, int, float, const float *, float);

static WalkKernel masked_kernel(bool quad, bool guard) {
    if (quad) return guard ? bh_walk_masked<true, true> : bh_walk_masked<true, false>;
    return guard ? bh_walk_masked<false, true> : bh_walk_masked<false, false>;
}

template <bool LEARNED, bool LOCAL, bool REL>
static GroupKernel group_kernel_q(bool quad, bool guard) {
    if (quad)
        return guard ? bh_walk_group<true, true, LEARNED, LOCAL, REL> : bh_walk_group<true, false, LEARNED, LOCAL, REL>;
    return guard ? bh_walk_group<false, true, LEARNED, LOCAL, REL> : bh_walk_group<false, false, LEARNED, LOCAL, REL>;
}

static GroupKernel group_kernel(bool quad, bool guard, bool learned, bool local, bool rel) {
    if (learned) return group_kernel_q<true, false, false>(quad, guard);
    if (local) return rel ? group_kernel_q<false, true, true>(quad, guard) : group_kernel_q<false, true, false>(quad, guard);
    return rel ? group_kernel_q<false, false, true>(quad, guard) : group_kernel_q<false, false, false>(quad, guard);
}



int run(pt_ctx *ctx, const float4 *d_aff, int n_aff, const float4 *d_src, int n_src, float theta,
               float softening, uint32_t flags, float *d_out) {
    cudaStream_t st = ctx->stream;
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * size_t(n_aff), st));
        return PT_OK;
    }
    State *Sp = state(ctx);
    if (!Sp) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    State &S = *Sp;
    mark(ctx, 0);
    PT_TRY(build(ctx, S, d_src, n_src));
    const bool same = (d_aff == d_src) && (n_aff == n_src);
    const float4 *tbody;
    const uint32_t *tidx;
    if (same) {
        tbody = as<float4>(S.sbody);
        tidx = as<uint32_t>(S.idx);
    } else {
        PT_TRY(sort_targets(ctx, S, d_aff, n_aff));
        tbody = as<float4>(S.tbody);
        tidx = as<uint32_t>(S.tidx);
    }
    return walk(ctx, S, tbody, tidx, n_aff, theta, softening, flags, d_out);
}

// The f64 method: build over DVec3 bodies, walk with the reference rule in double.
int run64(pt_ctx *ctx, const double4_32a *d_aff, int n_aff, const double4_32a *d_src, int n_src,
                 double theta, double softening, double *d_out) {
    cudaStream_t st = ctx->stream;
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * 3 * size_t(n_aff), st));
        return PT_OK;
    }
    State *Sp = state(ctx);
    if (!Sp) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    State &S = *Sp;
    mark(ctx, 0);
    PT_TRY(build_t<double>(ctx, S, d_src, n_src));
    const bool same = (d_aff == d_src) && (n_aff == n_src);
    if (!same) PT_TRY(sort_targets_t<double>(ctx, S, d_aff, n_aff));
    const double4_32a *tbody = same ? as<double4_32a>(S.sbody64) : as<double4_32a>(S.tbody64);
    const uint32_t *tidx = same ? as<uint32_t>(S.idx) : as<uint32_t>(S.tidx);
    unsigned long long *stats = reinterpret_cast<unsigned long long *>(S.counters.ptr) + 2;
    int *err = as<int>(S.counters) + 3;
    PT_CUDA(cudaMemsetAsync(stats, 0, 9 * sizeof(unsigned long long), st));
    PT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    mark(ctx, 1);
    bh_walk64<<<(n_aff + 32 * W64_WARPS - 1) / (32 * W64_WARPS), 32 * W64_WARPS, 0, st>>>(
        tbody, tidx, n_aff, as<double4_32a>(S.nodeA64), as<int4>(S.nodeB), as<double4_32a>(S.nodeG64),
        as<double4_32a>(S.sbody64), as<int>(S.counters), theta * theta, softening * softening, d_out, stats, err);
    PT_TRY(check_launch(ctx, "bh_walk64"));
    mark(ctx, 2);
    return PT_OK;
}

// Walks the context's current tree for targets tbody (key-sorted; tidx maps them back
// to the caller's order) and writes accelerations to d_out.
int walk(pt_ctx *ctx, State &S, const float4 *tbody, const uint32_t *tidx, int n_aff, float theta,
                float softening, uint32_t flags, float *d_out) {
    cudaStream_t st = ctx->stream;
    if (S.f64) return set_error(PT_ERR_INVALID, "the context's tree holds DVec3 bodies: walk it with the f64 method");
    // counters: int[4] = {leaves, nodes, cells, error} then u64[8] = {interactions,
    // visits, warps, max group stack, learned records, cell interactions, warps that
    // fell back to the per-body walk, far nodes taken by the local expansion}
    unsigned long long *stats = reinterpret_cast<unsigned long long *>(S.counters.ptr) + 2;
    int *err = as<int>(S.counters) + 3;
    PT_CUDA(cudaMemsetAsync(stats, 0, 9 * sizeof(unsigned long long), st));
    // within a leapfrog sequence the error word collects every step's errors
    if (!ctx->keep_errors) PT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    const float th2 = theta * theta;
    const float eps2 = softening * softening;
    const bool quad = flags & PT_BH_QUADRUPOLE;
    mark(ctx, 1);
    if (flags & PT_BH_GROUP) {
        const int groups = (n_aff + GW_GROUP - 1) / GW_GROUP;
        const bool learned = flags & PT_BH_LEARNED;
        if (learned && !S.mlp_w) return set_error(PT_ERR_INVALID, "PT_BH_LEARNED needs a model (pt_mlp_*)");
        LearnedRecords LR{};
        if (learned) {
            PT_TRY(ensure_buf(ctx, S.lhead, sizeof(int) * size_t(groups)));
            PT_TRY(ensure_buf(ctx, S.lcentre, sizeof(float4) * size_t(groups)));
            PT_TRY(ensure_buf(ctx, S.lused, sizeof(int)));
            if (S.lcap_fixed > 0) S.lcap = S.lcap_fixed;
            else if (S.lcap == 0) S.lcap = std::max(1024, 2 * groups);
        }
        const float *gscale = nullptr;
        if (flags & PT_BH_RELATIVE) {
            PT_TRY(ensure_buf(ctx, S.gscale, sizeof(float) * size_t(groups)));
            bh_group_scale<<<blocks(groups, 128), 128, 0, st>>>(tbody, n_aff, as<float4>(S.nodeA), as<int4>(S.nodeB),
                                                                as<int>(S.counters), eps2, S.rel_alpha,
                                                                as<float>(S.gscale));
            PT_TRY(check_launch(ctx, "bh_group_scale"));
            gscale = as<float>(S.gscale);
        }
        for (int attempt = 0;; ++attempt) {
            if (learned) {
                PT_TRY(ensure_buf(ctx, S.lrec, sizeof(int) * size_t(S.lcap) * LCHUNK));
                PT_TRY(ensure_buf(ctx, S.lgroup, sizeof(int) * size_t(S.lcap)));
                PT_TRY(ensure_buf(ctx, S.lnext, sizeof(int) * size_t(S.lcap)));
                PT_TRY(ensure_buf(ctx, S.lpart, sizeof(float4) * size_t(S.lcap)));
                LR = LearnedRecords{as<int>(S.lrec),   as<int>(S.lgroup),   as<int>(S.lnext), as<int>(S.lhead),
                                    as<float4>(S.lcentre), as<float4>(S.lpart), as<int>(S.lused), S.lcap};
                PT_CUDA(cudaMemsetAsync(LR.used, 0, sizeof(int), st));
            }
            group_kernel(quad, eps2 == 0.0f, learned, flags & PT_BH_LOCAL, gscale != nullptr)<<<(groups + GW_WARPS - 1) / GW_WARPS,
                                                                          32 * GW_WARPS, 0, st>>>(
                tbody, tidx, n_aff, as<float4>(S.nodeA), as<int4>(S.nodeB), as<float4>(S.nodeQ), as<float4>(S.nodeG),
                as<float4>(S.sbody), as<int>(S.counters), th2, S.theta_inner * S.theta_inner, LR, eps2, d_out, stats,
                err, S.stack_cap > 0 ? S.stack_cap : GW_STACK, S.local_ratio, gscale, S.rel_mono);
            PT_TRY(check_launch(ctx, "bh_walk_group"));
            // Outside stream capture (and with the automatic capacity) the record count
            // is checked and the walk rerun with room for all records; otherwise an
            // overflow sets error bit 2, which the callers report as PT_ERR_CAPACITY.
            if (!learned || ctx->capturing || attempt > 0 || S.lcap_fixed > 0) break;
            int used = 0;
            PT_CUDA(cudaMemcpyAsync(&used, LR.used, sizeof(int), cudaMemcpyDeviceToHost, st));
            PT_CUDA(cudaStreamSynchronize(st));
            if (used <= S.lcap) break;
            S.lcap = used + used / 4;
            PT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
            PT_CUDA(cudaMemsetAsync(stats, 0, 9 * sizeof(unsigned long long), st));
        }
        if (learned) {
            bh_learned_eval<<<ctx->sm_count * 4, 128, 0, st>>>(LR, as<float4>(S.nodeA), as<float4>(S.nodeQ),
                                                               as<float4>(S.nodeG), S.mlp_w, S.mlp_b,
                                                               S.theta_inner, theta);
            PT_TRY(check_launch(ctx, "bh_learned_eval"));
            bh_learned_apply<<<blocks(n_aff), 256, 0, st>>>(LR, tidx, n_aff, GW_SHIFT, d_out);
            PT_TRY(check_launch(ctx, "bh_learned_apply"));
        }
        PT_TRY(check_launch(ctx, "bh_walk_group"));
        mark(ctx, 2);
        return PT_OK;
    }
    masked_kernel(quad, eps2 == 0.0f)<<<(n_aff + 32 * MW_TPL * MW_WARPS - 1) / (32 * MW_TPL * MW_WARPS),
                                        32 * MW_WARPS, 0, st>>>(
        tbody, tidx, n_aff, as<float4>(S.nodeA), as<int4>(S.nodeB), as<float4>(S.nodeQ), as<float4>(S.sbody),
        as<int>(S.counters), th2, eps2, d_out, stats);
    PT_TRY(check_launch(ctx, "bh_walk_masked"));
    mark(ctx, 2);
    return PT_OK;
}


}  // namespace bh
}  // namespace pt
