// Barnes-Hut internals shared by the build (pt_bh_build.cu), the walks
// (pt_bh_walk.cu) and the C ABI (pt_bh.cu): the per-context state, the FP64 moment
// record, the scalar-type traits and the functions the units call each other by.
#pragma once

#include "pt_common.cuh"
#include "pt_prims.cuh"
#include "pt_f32x2.cuh"
#include "pt_mlp.cuh"

#include <algorithm>
#include <climits>
#include <new>


namespace pt {
namespace bh {

constexpr int LEVELS = 21;   // 63-bit keys

struct Moments {  // FP64 cell data used while combining children (DVec3 trees, bucket leaves)
    double m, cx, cy, cz;
    double sxx, sxy, sxz, syy, syz, szz;  // second moment about the centre of mass
    double count;
    double pad;
};

// Scalar type of the bodies: float (glam Vec3) or double (glam DVec3). The build
// replays the reference's subdivision in that type, with explicitly rounded ops.
template <class T>
struct Prec;
template <>
struct Prec<float> {
    using V4 = float4;
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float min(float a, float b) { return fminf(a, b); }
    static __device__ __forceinline__ float max(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ V4 make(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
};
template <>
struct Prec<double> {
    using V4 = double4_32a;
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double min(double a, double b) { return fmin(a, b); }
    static __device__ __forceinline__ double max(double a, double b) { return fmax(a, b); }
    static __device__ __forceinline__ V4 make(double x, double y, double z, double w) {
        V4 r;
        r.x = x, r.y = y, r.z = z, r.w = w;
        return r;
    }
};


struct State {
    PrimScratch prims;
    DevBuf box_part, box;
    DevBuf keys, idx, sbody;
    DevBuf flags, uscan, ukey, ufirst;
    DevBuf bfirst, blast, bdelta, bparent, lparent, top, oparent, loparent;
    DevBuf cnt, pscan, pre, nkid, kid, cslot, lslot, levels, by_level;
    DevBuf nodeA, nodeB, nodeQ, nodeG, nodeR, mom;
    DevBuf sbody64, nodeA64, nodeG64, tbody64;  // the f64 (DVec3) method's bodies and nodes
    DevBuf tkeys, tidx, tbody;
    DevBuf counters;
    DevBuf out;
    DevBuf aff_h, src_h;  // staging for the host-pointer entry point
    DevBuf lrec, lgroup, lnext, lpart, lhead, lcentre, lused;  // learned-correction records
    DevBuf gscale;                    // PT_BH_RELATIVE: 1 / (alpha |a|) per group
    int lcap = 0;                     // record chunks allocated
    int lcap_fixed = 0;               // > 0: record chunks fixed by pt_bh_set_learned_capacity
    int stack_cap = 0;                // group-walk stack ranges per warp in use (0 = all)
    uint64_t generation = 0;          // trees built so far (0 = none)
    bool f64 = false;                 // the current tree was built over DVec3 bodies
    bool user_tree = false;           // the current tree came from pt_bh_load_tree (monopoles only)
    float local_ratio = 0.1f;         // PT_BH_LOCAL: far when group radius < ratio * distance
    float rel_alpha = 2.5e-3f;        // PT_BH_RELATIVE: opened where the bound exceeds alpha |a|
    float rel_mono = 0.1f;            // PT_BH_RELATIVE + quadrupole: monopole-only cells below rel_mono alpha |a|
    const uint32_t *mlp_w = nullptr;  // learned correction: packed BF16 weights (owned by the MLP state)
    const float *mlp_b = nullptr;     // and its bias block
    float theta_inner = 0.5f;
    int cap_n = 0;
    int last_n_src = 0;
    // a second stream for build work that does not depend on the tree chain (the
    // sorted bodies' gather), joined back before the layout
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

inline State *state(pt_ctx *ctx) {
    if (!ctx->bh) ctx->bh = new (std::nothrow) State();
    return static_cast<State *>(ctx->bh);
}

template <class T>
inline T *as(DevBuf &b) {
    return static_cast<T *>(b.ptr);
}

inline int blocks(int n, int t = 256) { return (n + t - 1) / t; }

// Sibling ranges per warp. A pop takes fewer nodes when the stack is nearly full, and
// a warp that still runs out takes the per-body walk (counted, not an error). At
// N = 4M bulge+disk the deepest stack seen is 239 ranges at theta 0.5 and 379 at 0.3.
// 384 ranges keep a CTA at 36 KB of shared memory (5-6 CTAs per SM).
#ifndef PT_GW_STACK
#define PT_GW_STACK 384
#endif
constexpr int GW_STACK = PT_GW_STACK;

// tree build over the affecting bodies (pt_bh_build.cu); float = Vec3, double = DVec3
template <class T>
int build_t(pt_ctx *ctx, State &S, const typename Prec<T>::V4 *d_src, int n);
int build(pt_ctx *ctx, State &S, const float4 *d_src, int n);
// separate targets sorted along the tree's keys into S.tbody / S.tbody64
template <class T>
int sort_targets_t(pt_ctx *ctx, State &S, const typename Prec<T>::V4 *d_aff, int n);
int sort_targets(pt_ctx *ctx, State &S, const float4 *d_aff, int n);
// walks (pt_bh_walk.cu)
int walk(pt_ctx *ctx, State &S, const float4 *tbody, const uint32_t *tidx, int n_aff, float theta,
         float softening, uint32_t flags, float *d_out);
int run(pt_ctx *ctx, const float4 *d_aff, int n_aff, const float4 *d_src, int n_src, float theta, float softening,
        uint32_t flags, float *d_out);
int run64(pt_ctx *ctx, const double4_32a *d_aff, int n_aff, const double4_32a *d_src, int n_src, double theta,
          double softening, double *d_out);
int validate(const char *fn, size_t n_aff, size_t n_src, uint32_t flags);

}  // namespace bh
}  // namespace pt
