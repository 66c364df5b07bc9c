// cuda::BarnesHut { theta }: on-device octree build and a warp-synchronous walk.
//
// The tree is the reference's orthtree (particular/src/tree/mod.rs:91-138) built in
// parallel instead of recursively:
//  1. bbox_*   : the square root box of BoundingBox::square_with
//                (particular/src/tree/partition.rs:274-292), in the same f32 ops.
//  2. make_keys: each body replays the reference's subdivision for 21 levels
//                (centre = (min+max)/2, child bit = pos < centre, tree/mod.rs:116-124,
//                partition.rs:332-359), giving a 63-bit key whose prefixes are exactly
//                the reference's cells. The digit stored is 7 - orthant, so ascending
//                keys follow the reference's LIFO visiting order (children pushed 0..7,
//                popped 7..0, sequential.rs:489-495).
//  3. radix sort of (key, body) pairs; bodies gathered into key order.
//  4. equal keys collapse into one leaf unit (coincident bodies, or bodies closer
//     than 2^-21 of the root box: deeper than the key resolves).
//  5. Karras (2012) binary radix tree over the unique keys; a binary node is an
//     octree cell where its common-prefix level changes. Single-child chains of the
//     reference tree disappear: accepting a chain cell or its only child adds the
//     same (COM, M), so the result is unchanged.
//  6. cells are laid out in depth-first preorder with skip pointers (index after
//     the subtree), leaves interleaved; every cell gets a list of its children and
//     the cells are bucketed by octree level.
//  7. moments (mass, centre of mass, second moment -> traceless quadrupole): the
//     leaves, then one launch per octree level, deepest first, a thread per cell
//     combining its children (parallel-axis theorem), in compensated FP32 for f32
//     trees and FP64 for DVec3 trees.
#include "pt_bh.cuh"

#include <type_traits>

namespace pt {
namespace bh {

// ---- 1. root box -----------------------------------------------------------
template <class T>
__global__ void bbox_partial(const typename Prec<T>::V4 *__restrict__ src, int n, T *__restrict__ part) {
    using P = Prec<T>;
    T mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const typename P::V4 p = src[i];
        mn[0] = P::min(mn[0], p.x);
        mn[1] = P::min(mn[1], p.y);
        mn[2] = P::min(mn[2], p.z);
        mx[0] = P::max(mx[0], p.x);
        mx[1] = P::max(mx[1], p.y);
        mx[2] = P::max(mx[2], p.z);
    }
    __shared__ T s[6][256];
    for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = mn[a];
        s[3 + a][threadIdx.x] = mx[a];
    }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int a = 0; a < 3; ++a) {
                s[a][threadIdx.x] = P::min(s[a][threadIdx.x], s[a][threadIdx.x + w]);
                s[3 + a][threadIdx.x] = P::max(s[3 + a][threadIdx.x], s[3 + a][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

// box = {min x,y,z, max x,y,z} of BoundingBox::square_with: centre = midpoint of the
// AABB, half = (max extent + 0) / 2 (MidPoint::half), min/max = centre -/+ half.
// One block of 256 threads folds the per-block extents (min/max: exact in any
// order), then thread 0 forms the reference's square root box.
template <class T>
__global__ void bbox_final(const T *__restrict__ part, int nb, T *__restrict__ box) {
    using P = Prec<T>;
    T mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int a = 0; a < 3; ++a) {
            mn[a] = P::min(mn[a], part[b * 6 + a]);
            mx[a] = P::max(mx[a], part[b * 6 + 3 + a]);
        }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; ++a) {
            mn[a] = P::min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = P::max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    __shared__ T s[6][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            s[a][warp] = mn[a];
            s[3 + a][warp] = mx[a];
        }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < int(blockDim.x >> 5); ++w)
        for (int a = 0; a < 3; ++a) {
            mn[a] = P::min(mn[a], s[a][w]);
            mx[a] = P::max(mx[a], s[3 + a][w]);
        }
    T half = 0;
    T c[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = P::mul(P::add(mn[a], mx[a]), T(0.5));
        half = P::max(half, P::sub(mx[a], mn[a]));
    }
    half = P::mul(P::add(half, T(0)), T(0.5));
    for (int a = 0; a < 3; ++a) {
        box[a] = P::sub(c[a], half);
        box[3 + a] = P::add(c[a], half);
    }
}

// ---- 2. keys ---------------------------------------------------------------
template <class T>
__device__ __forceinline__ uint64_t key_of(T px, T py, T pz, const T *box) {
    using P = Prec<T>;
    T mn0 = box[0], mn1 = box[1], mn2 = box[2], mx0 = box[3], mx1 = box[4], mx2 = box[5];
    uint64_t key = 0;
#pragma unroll 3
    for (int l = 0; l < LEVELS; ++l) {
        const T c0 = P::mul(P::add(mn0, mx0), T(0.5));
        const T c1 = P::mul(P::add(mn1, mx1), T(0.5));
        const T c2 = P::mul(P::add(mn2, mx2), T(0.5));
        const int b0 = px < c0, b1 = py < c1, b2 = pz < c2;
        if (b0) mx0 = c0; else mn0 = c0;
        if (b1) mx1 = c1; else mn1 = c1;
        if (b2) mx2 = c2; else mn2 = c2;
        const int o = b0 | (b1 << 1) | (b2 << 2);
        key = (key << 3) | uint64_t(7 - o);
    }
    return key;
}

template <class T>
__global__ void make_keys(const typename Prec<T>::V4 *__restrict__ bodies, int n, const T *__restrict__ box_g,
                          uint64_t *__restrict__ keys, uint32_t *__restrict__ idx) {
    __shared__ T box[6];
    if (threadIdx.x < 6) box[threadIdx.x] = box_g[threadIdx.x];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const typename Prec<T>::V4 p = bodies[i];
    keys[i] = key_of<T>(p.x, p.y, p.z, box);
    idx[i] = uint32_t(i);
}

template <class V4>
__global__ void gather_bodies(const V4 *__restrict__ src, const uint32_t *__restrict__ idx, int n,
                              V4 *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = src[idx[k]];
}

// ---- 4. unique keys -> leaf units ------------------------------------------
__global__ void unit_flags(const uint64_t *__restrict__ keys, int n, uint32_t *__restrict__ flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) flags[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1u : 0u;
}

// counters[0] = M (units)
__global__ void unit_fill(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ flags,
                          const uint32_t *__restrict__ uscan, int n, uint64_t *__restrict__ ukey,
                          uint32_t *__restrict__ ufirst, int *__restrict__ counters) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (flags[k]) {
        const uint32_t u = uscan[k];
        ukey[u] = keys[k];
        ufirst[u] = uint32_t(k);
    }
    if (k == 0) {
        const uint32_t M = uscan[n];
        ufirst[M] = uint32_t(n);
        counters[0] = int(M);
    }
}

// ---- 5. Karras binary radix tree ---------------------------------------------
__device__ __forceinline__ int kdelta(const uint64_t *__restrict__ k, int M, int i, int j) {
    if (j < 0 || j >= M) return -1;
    return __clzll(k[i] ^ k[j]) - 1;  // bit 63 is always 0: prefix length of the 63-bit keys
}

__global__ void karras(const uint64_t *__restrict__ ukey, const int *__restrict__ counters, int *__restrict__ bfirst,
                       int *__restrict__ blast, int *__restrict__ bdelta, int *__restrict__ bparent,
                       int *__restrict__ lparent) {
    const int M = counters[0];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M - 1) return;
    const int d = (kdelta(ukey, M, i, i + 1) - kdelta(ukey, M, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(ukey, M, i, i - d);
    int lmax = 2;
    while (kdelta(ukey, M, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(ukey, M, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = kdelta(ukey, M, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(ukey, M, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    bfirst[i] = first;
    blast[i] = last;
    bdelta[i] = dnode;
    if (first == gamma) lparent[gamma] = i; else bparent[gamma] = i;
    if (last == gamma + 1) lparent[gamma + 1] = i; else bparent[gamma + 1] = i;
    if (i == 0) bparent[0] = -1;
}

// A binary node is an octree cell iff it is the root or its common-prefix level
// (delta / 3) exceeds its parent's.
__global__ void octree_top(const int *__restrict__ counters, const int *__restrict__ bdelta,
                           const int *__restrict__ bparent, uint8_t *__restrict__ top) {
    const int M = counters[0];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M - 1) return;
    top[i] = (i == 0 || bdelta[bparent[i]] / 3 < bdelta[i] / 3) ? 1 : 0;
}

__device__ __forceinline__ int climb(int p, const uint8_t *__restrict__ top, const int *__restrict__ bparent) {
    while (!top[p]) p = bparent[p];
    return p;
}

// Octree parents, child counts (nkid, zeroed before) with each child's slot in its
// parent's child list, the count of cells starting at each unit, and the count of
// cells per octree level (levels[L], zeroed before).
__global__ void octree_links(const int *__restrict__ counters, const int *__restrict__ bfirst,
                             const int *__restrict__ bparent, const int *__restrict__ lparent,
                             const uint8_t *__restrict__ top, const int *__restrict__ bdelta,
                             int *__restrict__ oparent, int *__restrict__ loparent, uint32_t *__restrict__ cnt,
                             int *__restrict__ nkid, uint8_t *__restrict__ cslot, uint8_t *__restrict__ lslot,
                             int *__restrict__ levels) {
    __shared__ int h[LEVELS];
    if (threadIdx.x < LEVELS) h[threadIdx.x] = 0;
    __syncthreads();
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < M - 1 && top[k]) {
        const int op = (k == 0) ? -1 : climb(bparent[k], top, bparent);
        oparent[k] = op;
        if (op >= 0) cslot[k] = uint8_t(atomicAdd(&nkid[op], 1));  // < 8: one child per octant
        atomicAdd(&cnt[bfirst[k]], 1u);
        atomicAdd(&h[bdelta[k] / 3], 1);
    }
    if (k < M) {
        const int op = (M == 1) ? -1 : climb(lparent[k], top, bparent);
        loparent[k] = op;
        if (op >= 0) lslot[k] = uint8_t(atomicAdd(&nkid[op], 1));
    }
    __syncthreads();
    if (threadIdx.x < LEVELS && h[threadIdx.x]) atomicAdd(&levels[threadIdx.x], h[threadIdx.x]);
}

// levels[0 .. LEVELS) = cells per level, levels[LEVELS + 1 + L] = offset of level L in
// by_level, levels[2 LEVELS + 2 + L] = its fill cursor.
__global__ void level_offsets(int *__restrict__ levels) {
    if (threadIdx.x != 0) return;
    int acc = 0;
    for (int L = 0; L < LEVELS; ++L) {
        levels[LEVELS + 1 + L] = acc;
        levels[2 * LEVELS + 2 + L] = acc;
        acc += levels[L];
    }
    levels[2 * LEVELS + 1] = acc;
}

// ---- 7. moments ------------------------------------------------------------
// Leaves first (in the layout pass, one thread per leaf unit), then the cells one
// octree level per launch, deepest first, one thread per cell: every cell's children are complete
// when it is combined, and it reads them from its child list, all loads at once.
// The order of every sum is fixed by the tree. (A single bottom-up launch in which
// the last child to arrive combined its parent was slower, 2.04 against 1.81 ms of
// build at N = 4M: its climbing lanes wait on L2 with 4 of 32 lanes active.)
// Children's records are read once, through L2 (ld.global.cg).
__device__ __forceinline__ float4 ld_cg(const float4 *p) { return __ldcg(p); }
__device__ __forceinline__ double4_32a ld_cg(const double4_32a *p) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    double4_32a r;
    r.x = a.x, r.y = a.y, r.z = b.x, r.w = b.y;
    return r;
}
__device__ __forceinline__ Moments ld_cg(const Moments *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    double2 v[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) v[i] = __ldcg(q + i);
    Moments r;
    r.m = v[0].x, r.cx = v[0].y, r.cy = v[1].x, r.cz = v[1].y;
    r.sxx = v[2].x, r.sxy = v[2].y, r.sxz = v[3].x, r.syy = v[3].y, r.syz = v[4].x, r.szz = v[4].y;
    r.count = v[5].x, r.pad = v[5].y;
    return r;
}

// Cell record of f32 trees, in FP32. The centre of mass and the mass are unevaluated
// sums hi + lo with hi = nodeA, and a child's offset from its parent's geometric
// centre G is formed as (hi - G) + lo: hi and G lie within a cell width of each
// other, so every sum below is relative to the cell width, not to the position.
struct Rec32 {
    float4 lo;  // centre of mass - nodeA.xyz, mass - nodeA.w
    float4 s0;  // second moment about the centre of mass: xx xy xz yy
    float4 s1;  // yz zz, body count (int bits), 0
};

// Knuth's TwoSum: returns s = fl(a + b) and sets e with s + e == a + b exactly.
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ void store_quad(float4 *nodeQ, int pk, float sxx, float sxy, float sxz, float syy,
                                           float syz, float szz) {
    const float tr = sxx + syy + szz;
    nodeQ[2 * pk] = make_float4(3.f * sxx - tr, 3.f * sxy, 3.f * sxz, 3.f * syy - tr);
    nodeQ[2 * pk + 1] = make_float4(3.f * syz, 3.f * szz - tr, 0.f, 0.f);
}

__device__ __forceinline__ void store_cell(const Moments &m, int pk, Moments *mom, double4_32a *nodeA, float4 *) {
    mom[pk] = m;
    nodeA[pk] = Prec<double>::make(m.cx, m.cy, m.cz, m.m);  // the f64 method is monopole only
}

__device__ __forceinline__ void store_cell(const Moments &m, int pk, Rec32 *rec, float4 *nodeA, float4 *nodeQ) {
    const float hx = float(m.cx), hy = float(m.cy), hz = float(m.cz), hm = float(m.m);
    nodeA[pk] = make_float4(hx, hy, hz, hm);
    rec[pk].lo = make_float4(float(m.cx - hx), float(m.cy - hy), float(m.cz - hz), float(m.m - hm));
    rec[pk].s0 = make_float4(float(m.sxx), float(m.sxy), float(m.sxz), float(m.syy));
    rec[pk].s1 = make_float4(float(m.syz), float(m.szz), __int_as_float(int(m.count)), 0.f);
    if (nodeQ)
        store_quad(nodeQ, pk, float(m.sxx), float(m.sxy), float(m.sxz), float(m.syy), float(m.syz), float(m.szz));
}

// Leaves: a single body is its own cell data (no record: parents read nodeA; no
// quadrupole: the walks read it for cells only); several (coincident, or closer
// than the key resolution) get FP64 moments.
template <class V4, class R>
__device__ void leaf(int pk, int f, int e, const V4 *__restrict__ sbody, R *rec, V4 *nodeA, float4 *nodeQ) {
    if (e - f == 1) {
        nodeA[pk] = sbody[f];
        return;
    }
    Moments m{};
    double sx = 0, sy = 0, sz = 0;
    for (int b = f; b < e; ++b) {
        const V4 p = sbody[b];
        m.m += p.w;
        sx += double(p.w) * p.x;
        sy += double(p.w) * p.y;
        sz += double(p.w) * p.z;
    }
    m.count = e - f;
    if (m.m != 0.0) {
        m.cx = sx / m.m;
        m.cy = sy / m.m;
        m.cz = sz / m.m;
    } else {  // massless: plain mean (gravity/impls/mod.rs:127-129)
        for (int b = f; b < e; ++b) {
            const V4 p = sbody[b];
            m.cx += p.x;
            m.cy += p.y;
            m.cz += p.z;
        }
        m.cx /= m.count;
        m.cy /= m.count;
        m.cz /= m.count;
    }
    for (int b = f; b < e; ++b) {
        const V4 p = sbody[b];
        const double dx = p.x - m.cx, dy = p.y - m.cy, dz = p.z - m.cz;
        m.sxx += p.w * dx * dx;
        m.sxy += p.w * dx * dy;
        m.sxz += p.w * dx * dz;
        m.syy += p.w * dy * dy;
        m.syz += p.w * dy * dz;
        m.szz += p.w * dz * dz;
    }
    store_cell(m, pk, rec, nodeA, nodeQ);
}

// Children of binary cell p: kid[8p .. 8p + nkid[p]) hold 2 x preorder index + 1 for
// a single body (it has no record: its nodeA is its data). Filled in octree_links'
// slot order, they are sorted back into preorder, the reference's child order, so
// every sum runs in a fixed order; their loads are independent of each other.
struct Kids {
    int e[8];
    int n;
};

__device__ __forceinline__ void cswap(int &a, int &b) {
    const int lo = min(a, b), hi = max(a, b);
    a = lo, b = hi;
}

__device__ __forceinline__ Kids load_kids(int p, const int *__restrict__ kid, const int *__restrict__ nkid) {
    Kids K;
    K.n = nkid[p];
    const int4 a = reinterpret_cast<const int4 *>(kid)[2 * p];
    const int4 b = reinterpret_cast<const int4 *>(kid)[2 * p + 1];
    K.e[0] = a.x, K.e[1] = a.y, K.e[2] = a.z, K.e[3] = a.w, K.e[4] = b.x, K.e[5] = b.y, K.e[6] = b.z, K.e[7] = b.w;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (i >= K.n) K.e[i] = INT_MAX;
    // Batcher's odd-even merge sort of 8 keys (19 compare-exchanges)
    cswap(K.e[0], K.e[1]), cswap(K.e[2], K.e[3]), cswap(K.e[4], K.e[5]), cswap(K.e[6], K.e[7]);
    cswap(K.e[0], K.e[2]), cswap(K.e[1], K.e[3]), cswap(K.e[4], K.e[6]), cswap(K.e[5], K.e[7]);
    cswap(K.e[1], K.e[2]), cswap(K.e[5], K.e[6]);
    cswap(K.e[0], K.e[4]), cswap(K.e[1], K.e[5]), cswap(K.e[2], K.e[6]), cswap(K.e[3], K.e[7]);
    cswap(K.e[2], K.e[4]), cswap(K.e[3], K.e[5]);
    cswap(K.e[1], K.e[2]), cswap(K.e[3], K.e[4]), cswap(K.e[5], K.e[6]);
    return K;
}

// f32 trees: one pass over the children in FP32, sums about the cell's geometric
// centre G, then moved to the centre of mass C by the parallel-axis rule
// S_C = S_G - P P^T / M with P = sum m (c - G) = M (C - G).
__device__ void cell(int pv, const Kids &K, const float4 *__restrict__ nodeG, Rec32 *rec, float4 *nodeA,
                     float4 *nodeQ, int4 *nodeB) {
    const float4 g = nodeG[pv];
    float mh = 0.f, ml = 0.f, px = 0.f, py = 0.f, pz = 0.f;
    float sxx = 0.f, sxy = 0.f, sxz = 0.f, syy = 0.f, syz = 0.f, szz = 0.f;
    int count = 0;
    // Straight-line over the 8 slots (no early exit): every slot's address is valid (an
    // empty slot names the first child), so all the children's loads can be in flight at
    // once; the sums still run slot by slot.
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const bool v = i < K.n;
        const int ke = v ? K.e[i] : K.e[0];
        const int c = ke >> 1;
        const bool has_rec = v && !(ke & 1);
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 a = v ? ld_cg(nodeA + c) : zero;
        float4 lo = zero, s0 = zero, s1 = zero;
        int cn = 1;
        if (has_rec) {
            lo = ld_cg(&rec[c].lo);
            s0 = ld_cg(&rec[c].s0);
            s1 = ld_cg(&rec[c].s1);
            cn = __float_as_int(s1.z);
        }
        if (!v) continue;
        const float dx = __fsub_rn(a.x, g.x) + lo.x, dy = __fsub_rn(a.y, g.y) + lo.y, dz = __fsub_rn(a.z, g.z) + lo.z;
        float e;
        mh = two_sum(mh, a.w, e);
        ml += e + lo.w;
        const float mx = a.w * dx, my = a.w * dy, mz = a.w * dz;
        px += mx;
        py += my;
        pz += mz;
        sxx += s0.x + mx * dx;
        sxy += s0.y + mx * dy;
        sxz += s0.z + mx * dz;
        syy += s0.w + my * dy;
        syz += s1.x + my * dz;
        szz += s1.y + mz * dz;
        count += cn;
    }
    float e;
    const float M = two_sum(mh, ml, e);
    const float Ml = e;
    float ox, oy, oz;
    if (M != 0.f) {
        const float inv = 1.f / M;
        ox = px * inv, oy = py * inv, oz = pz * inv;  // C - G
        sxx -= px * ox;
        sxy -= px * oy;
        sxz -= px * oz;
        syy -= py * oy;
        syz -= py * oz;
        szz -= pz * oz;
    } else {  // massless: plain mean of the bodies (gravity/impls/mod.rs:127-129), a rare second pass
        float ux = 0.f, uy = 0.f, uz = 0.f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (i >= K.n) break;
            const int c = K.e[i] >> 1;
            const float4 a = ld_cg(nodeA + c);
            float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
            float cn = 1.f;
            if (!(K.e[i] & 1)) {
                lo = ld_cg(&rec[c].lo);
                cn = float(__float_as_int(ld_cg(&rec[c].s1).z));
            }
            ux += cn * (__fsub_rn(a.x, g.x) + lo.x);
            uy += cn * (__fsub_rn(a.y, g.y) + lo.y);
            uz += cn * (__fsub_rn(a.z, g.z) + lo.z);
        }
        ox = ux / float(count), oy = uy / float(count), oz = uz / float(count);
    }
    float ex, ey, ez;
    const float hx = two_sum(g.x, ox, ex), hy = two_sum(g.y, oy, ey), hz = two_sum(g.z, oz, ez);
    nodeA[pv] = make_float4(hx, hy, hz, M);
    // a cell's nodeB.w (a leaf's body count) holds (M w^3)^(2/5): the error-bound
    // opening radius^2 is this times (alpha |a|)^(-2/5) of the walking group
    nodeB[pv].w = __float_as_int(M > 0.f ? __powf(M * g.w * g.w * g.w, 0.4f) : 0.f);
    rec[pv].lo = make_float4(ex, ey, ez, Ml);
    rec[pv].s0 = make_float4(sxx, sxy, sxz, syy);
    rec[pv].s1 = make_float4(syz, szz, __int_as_float(count), 0.f);
    if (nodeQ) store_quad(nodeQ, pv, sxx, sxy, sxz, syy, syz, szz);
}

// f64 trees (DVec3 bodies): the same combination in FP64.
__device__ void cell(int pv, const Kids &K, const double4_32a *__restrict__ nodeG, Moments *mom,
                     double4_32a *nodeA, float4 *, int4 *) {
    const double4_32a g = nodeG[pv];
    const double gx = g.x, gy = g.y, gz = g.z;
    Moments m{};
    double px = 0, py = 0, pz = 0;
    for (int i = 0; i < K.n; ++i) {
        const int c = K.e[i] >> 1;
        double cx, cy, cz, cmm, cn, sxx = 0, sxy = 0, sxz = 0, syy = 0, syz = 0, szz = 0;
        if (K.e[i] & 1) {
            const double4_32a a = ld_cg(nodeA + c);
            cx = a.x, cy = a.y, cz = a.z, cmm = a.w, cn = 1.0;
        } else {
            const Moments cm = ld_cg(mom + c);
            cx = cm.cx, cy = cm.cy, cz = cm.cz, cmm = cm.m, cn = cm.count;
            sxx = cm.sxx, sxy = cm.sxy, sxz = cm.sxz, syy = cm.syy, syz = cm.syz, szz = cm.szz;
        }
        const double dx = cx - gx, dy = cy - gy, dz = cz - gz;
        m.m += cmm;
        m.count += cn;
        const double mx = cmm * dx, my = cmm * dy, mz = cmm * dz;
        px += mx;
        py += my;
        pz += mz;
        m.sxx += sxx + mx * dx;
        m.sxy += sxy + mx * dy;
        m.sxz += sxz + mx * dz;
        m.syy += syy + my * dy;
        m.syz += syz + my * dz;
        m.szz += szz + mz * dz;
    }
    if (m.m != 0.0) {
        const double inv = 1.0 / m.m;
        const double ox = px * inv, oy = py * inv, oz = pz * inv;  // C - G
        m.cx = gx + ox;
        m.cy = gy + oy;
        m.cz = gz + oz;
        m.sxx -= px * ox;
        m.sxy -= px * oy;
        m.sxz -= px * oz;
        m.syy -= py * oy;
        m.syz -= py * oz;
        m.szz -= pz * oz;
    } else {  // massless: plain mean of the bodies (gravity/impls/mod.rs:127-129), a rare second pass
        double ux = 0, uy = 0, uz = 0;
        for (int i = 0; i < K.n; ++i) {
            const int c = K.e[i] >> 1;
            double cx, cy, cz, cn;
            if (K.e[i] & 1) {
                const double4_32a a = ld_cg(nodeA + c);
                cx = a.x, cy = a.y, cz = a.z, cn = 1.0;
            } else {
                const Moments cm = ld_cg(mom + c);
                cx = cm.cx, cy = cm.cy, cz = cm.cz, cn = cm.count;
            }
            ux += cn * (cx - gx);
            uy += cn * (cy - gy);
            uz += cn * (cz - gz);
        }
        m.cx = gx + ux / m.count;
        m.cy = gy + uy / m.count;
        m.cz = gz + uz / m.count;
    }
    store_cell(m, pv, mom, nodeA, nullptr);
}

template <class T>
using Record = typename std::conditional<sizeof(T) == 4, Rec32, Moments>::type;

// ---- 6. preorder layout (and the leaves' records) ---------------------------
// nodeB = {width bits, skip, first body (-1: internal cell), body count}.
// counters[1] = T (cells + leaves), counters[2] = internal cells.
template <class T>
__global__ void layout(int *counters, const int *__restrict__ bfirst,
                       const int *__restrict__ blast, const int *__restrict__ bdelta,
                       const uint8_t *__restrict__ top, const int *__restrict__ oparent,
                       const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ pscan,
                       const uint64_t *__restrict__ ukey, const uint32_t *__restrict__ ufirst,
                       const T *__restrict__ box, int *__restrict__ pre, int4 *__restrict__ nodeB,
                       typename Prec<T>::V4 *__restrict__ nodeG, int2 *__restrict__ nodeR,
                       const int *__restrict__ loparent, const uint8_t *__restrict__ cslot,
                       const uint8_t *__restrict__ lslot, int *__restrict__ kid, int *__restrict__ levels,
                       int *__restrict__ by_level, const typename Prec<T>::V4 *__restrict__ sbody, Record<T> *rec,
                       typename Prec<T>::V4 *nodeA, float4 *nodeQ) {
    using P = Prec<T>;
    __shared__ int h[LEVELS], base[LEVELS];
    if (threadIdx.x < LEVELS) h[threadIdx.x] = 0;
    __syncthreads();
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int lvl = -1, lrank = 0;  // this cell's octree level and rank among the block's
    if (k == 0) {
        counters[1] = M + int(pscan[M]);
        counters[2] = int(pscan[M]);
    }
    if (k < M - 1 && top[k]) {
        const int b = bfirst[k];
        int r = 0;
        for (int p = oparent[k]; p >= 0 && bfirst[p] == b; p = oparent[p]) ++r;
        const int pk = b + int(pscan[b]) + r;
        pre[k] = pk;
        const int after = blast[k] + 1;
        const int skip = after + int(pscan[after]);
        // Cell box at level L along the key's path: BoundingBox::width() of the
        // reference cell (partition.rs:322-327) and its centre, replayed in the same
        // f32 ops.
        const int L = bdelta[k] / 3;
        const uint64_t key = ukey[b];
        T mn0 = box[0], mn1 = box[1], mn2 = box[2], mx0 = box[3], mx1 = box[4], mx2 = box[5];
        for (int l = 0; l < L; ++l) {
            const int o = 7 - int((key >> (3 * (LEVELS - 1 - l))) & 7u);
            const T c0 = P::mul(P::add(mn0, mx0), T(0.5));
            const T c1 = P::mul(P::add(mn1, mx1), T(0.5));
            const T c2 = P::mul(P::add(mn2, mx2), T(0.5));
            if (o & 1) mx0 = c0; else mn0 = c0;
            if (o & 2) mx1 = c1; else mn1 = c1;
            if (o & 4) mx2 = c2; else mn2 = c2;
        }
        const T w = P::sub(mx0, mn0);
        // the f32 walk reads the width from nodeB.x; the f64 walk from nodeG.w
        nodeB[pk] = make_int4(sizeof(T) == 4 ? __float_as_int(float(w)) : 0, skip, -1, 0);
        nodeG[pk] = P::make(T(0.5) * (mn0 + mx0), T(0.5) * (mn1 + mx1), T(0.5) * (mn2 + mx2), w);
        nodeR[pk] = make_int2(int(ufirst[b]), int(ufirst[blast[k] + 1]));
        // the cell's entry in its parent's child list
        if (k != 0) kid[8 * oparent[k] + cslot[k]] = 2 * pk;
        lvl = L;
        lrank = atomicAdd(&h[L], 1);
    }
    if (k < M) {
        const int pk = k + int(pscan[k]) + int(cnt[k]);
        const int f = int(ufirst[k]);
        const int nb = int(ufirst[k + 1]) - f;
        nodeB[pk] = make_int4(0, pk + 1, f, nb);
        // (no nodeG / nodeR for leaves: the cell centre and body range are read for
        // cells only, by the f64 walk's widths and the learned features and samples)
        const int op = loparent[k];
        if (op >= 0) kid[8 * op + lslot[k]] = 2 * pk + (nb == 1 ? 1 : 0);
        leaf(pk, f, f + nb, sbody, rec, nodeA, nodeQ);  // the leaf's moment record
    }
    // cells bucketed by octree level (one range per level and block)
    __syncthreads();
    if (threadIdx.x < LEVELS && h[threadIdx.x])
        base[threadIdx.x] = atomicAdd(&levels[2 * LEVELS + 2 + threadIdx.x], h[threadIdx.x]);
    __syncthreads();
    if (lvl >= 0) by_level[base[lvl] + lrank] = k;
}

// The cells of octree level L (levels below: done), one thread each.
template <class T>
__global__ void __launch_bounds__(256)
    cells_level(int L, const int *__restrict__ levels, const int *__restrict__ by_level,
                const int *__restrict__ pre, const int *__restrict__ kid, const int *__restrict__ nkid,
                const typename Prec<T>::V4 *__restrict__ nodeG, Record<T> *rec, typename Prec<T>::V4 *nodeA,
                float4 *nodeQ, int4 *nodeB) {
    const int begin = levels[LEVELS + 1 + L], end = begin + levels[L];
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        const int k = by_level[i];
        cell(pre[k], load_kids(k, kid, nkid), nodeG, rec, nodeA, nodeQ, nodeB);
    }
}

// Levels TOP_LEVELS - 1 .. 0 (at most 8^L cells each, 585 in all) in one block, a
// barrier between levels: these levels hold few cells, and one launch each cost
// ~17 us of latency at N = 4M. (Level 4 too, up to 4096 cells at several cells per
// thread, made the block take 66 us.)
constexpr int TOP_LEVELS = 4;

template <class T>
__global__ void __launch_bounds__(512)
    cells_top(const int *__restrict__ levels, const int *__restrict__ by_level, const int *__restrict__ pre,
              const int *__restrict__ kid, const int *__restrict__ nkid, const typename Prec<T>::V4 *__restrict__ nodeG,
              Record<T> *rec, typename Prec<T>::V4 *nodeA, float4 *nodeQ, int4 *nodeB) {
    for (int L = TOP_LEVELS - 1; L >= 0; --L) {
        const int begin = levels[LEVELS + 1 + L], end = begin + levels[L];
        for (int i = begin + threadIdx.x; i < end; i += blockDim.x) {
            const int k = by_level[i];
            cell(pre[k], load_kids(k, kid, nkid), nodeG, rec, nodeA, nodeQ, nodeB);
        }
        __syncthreads();  // the level's records (global, read through L2) before its parents
    }
}

template <class T>
int build_t(pt_ctx *ctx, State &S, const typename Prec<T>::V4 *d_src, int n) {
    using V4 = typename Prec<T>::V4;
    constexpr bool F64 = sizeof(T) == 8;
    // the f64 method keeps its own body, node and box arrays (the rest is shared)
    DevBuf &sb = F64 ? S.sbody64 : S.sbody;
    DevBuf &nA = F64 ? S.nodeA64 : S.nodeA;
    DevBuf &nG = F64 ? S.nodeG64 : S.nodeG;
    cudaStream_t st = ctx->stream;
    const size_t N = size_t(n);
    PT_TRY(ensure_buf(ctx, S.box_part, sizeof(T) * 6 * 1024));
    PT_TRY(ensure_buf(ctx, S.box, sizeof(T) * 8));
    PT_TRY(ensure_buf(ctx, S.keys, sizeof(uint64_t) * N));
    PT_TRY(ensure_buf(ctx, S.idx, sizeof(uint32_t) * N));
    PT_TRY(ensure_buf(ctx, sb, sizeof(V4) * N));
    PT_TRY(ensure_buf(ctx, S.flags, sizeof(uint32_t) * N));
    PT_TRY(ensure_buf(ctx, S.uscan, sizeof(uint32_t) * (N + 1)));
    PT_TRY(ensure_buf(ctx, S.ukey, sizeof(uint64_t) * N));
    PT_TRY(ensure_buf(ctx, S.ufirst, sizeof(uint32_t) * (N + 1)));
    PT_TRY(ensure_buf(ctx, S.bfirst, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.blast, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.bdelta, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.bparent, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.lparent, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.top, N));
    PT_TRY(ensure_buf(ctx, S.oparent, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.loparent, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.cnt, sizeof(uint32_t) * (N + 1)));
    PT_TRY(ensure_buf(ctx, S.pscan, sizeof(uint32_t) * (N + 2)));
    PT_TRY(ensure_buf(ctx, S.pre, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.nkid, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.levels, sizeof(int) * (3 * LEVELS + 8)));
    PT_TRY(ensure_buf(ctx, S.by_level, sizeof(int) * N));
    PT_TRY(ensure_buf(ctx, S.kid, sizeof(int) * 8 * N));
    PT_TRY(ensure_buf(ctx, S.cslot, N));
    PT_TRY(ensure_buf(ctx, S.lslot, N));
    PT_TRY(ensure_buf(ctx, nA, sizeof(V4) * 2 * N));
    PT_TRY(ensure_buf(ctx, S.nodeB, sizeof(int4) * 2 * N));
    if (!F64) PT_TRY(ensure_buf(ctx, S.nodeQ, sizeof(float4) * 4 * N));
    PT_TRY(ensure_buf(ctx, nG, sizeof(V4) * 2 * N));
    float4 *nodeQ = F64 ? nullptr : as<float4>(S.nodeQ);
    PT_TRY(ensure_buf(ctx, S.nodeR, sizeof(int2) * 2 * N));
    PT_TRY(ensure_buf(ctx, S.mom, sizeof(Moments) * 2 * N));
    PT_TRY(ensure_buf(ctx, S.counters, sizeof(unsigned long long) * 16));

    const int nb = std::min(1024, blocks(n));
    bbox_partial<T><<<nb, 256, 0, st>>>(d_src, n, as<T>(S.box_part));
    PT_TRY(check_launch(ctx, "bbox_partial"));
    bbox_final<T><<<1, 256, 0, st>>>(as<T>(S.box_part), nb, as<T>(S.box));
    PT_TRY(check_launch(ctx, "bbox_final"));
    make_keys<T><<<blocks(n), 256, 0, st>>>(d_src, n, as<T>(S.box), as<uint64_t>(S.keys), as<uint32_t>(S.idx));
    PT_TRY(check_launch(ctx, "make_keys"));
    PT_TRY(radix_sort_u64(ctx, S.prims, as<uint64_t>(S.keys), as<uint32_t>(S.idx), n, 3 * LEVELS));
    // The bodies' gather into key order runs on a second stream beside the tree chain
    // (unit flags .. octree links) and joins before the layout, its first reader.
    if (!S.aux) {
        PT_CUDA(cudaStreamCreateWithFlags(&S.aux, cudaStreamNonBlocking));
        PT_CUDA(cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming));
        PT_CUDA(cudaEventCreateWithFlags(&S.join, cudaEventDisableTiming));
    }
    PT_CUDA(cudaEventRecord(S.fork, st));
    PT_CUDA(cudaStreamWaitEvent(S.aux, S.fork, 0));
    gather_bodies<V4><<<blocks(n), 256, 0, S.aux>>>(d_src, as<uint32_t>(S.idx), n, as<V4>(sb));
    PT_TRY(check_launch(ctx, "gather_bodies"));
    PT_CUDA(cudaEventRecord(S.join, S.aux));
    unit_flags<<<blocks(n), 256, 0, st>>>(as<uint64_t>(S.keys), n, as<uint32_t>(S.flags));
    PT_TRY(check_launch(ctx, "unit_flags"));
    PT_TRY(scan_u32(ctx, S.prims, as<uint32_t>(S.flags), as<uint32_t>(S.uscan), n));
    int *counters = as<int>(S.counters);
    unit_fill<<<blocks(n), 256, 0, st>>>(as<uint64_t>(S.keys), as<uint32_t>(S.flags), as<uint32_t>(S.uscan), n,
                                        as<uint64_t>(S.ukey), as<uint32_t>(S.ufirst), counters);
    PT_TRY(check_launch(ctx, "unit_fill"));
    karras<<<blocks(n), 256, 0, st>>>(as<uint64_t>(S.ukey), counters, as<int>(S.bfirst), as<int>(S.blast),
                                     as<int>(S.bdelta), as<int>(S.bparent), as<int>(S.lparent));
    PT_TRY(check_launch(ctx, "karras"));
    octree_top<<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bdelta), as<int>(S.bparent), as<uint8_t>(S.top));
    PT_TRY(check_launch(ctx, "octree_top"));
    PT_CUDA(cudaMemsetAsync(S.cnt.ptr, 0, sizeof(uint32_t) * (N + 1), st));
    PT_CUDA(cudaMemsetAsync(S.nkid.ptr, 0, sizeof(int) * N, st));
    PT_CUDA(cudaMemsetAsync(S.levels.ptr, 0, sizeof(int) * (3 * LEVELS + 8), st));
    int *levels = as<int>(S.levels);
    octree_links<<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bfirst), as<int>(S.bparent), as<int>(S.lparent),
                                           as<uint8_t>(S.top), as<int>(S.bdelta), as<int>(S.oparent),
                                           as<int>(S.loparent), as<uint32_t>(S.cnt), as<int>(S.nkid),
                                           as<uint8_t>(S.cslot), as<uint8_t>(S.lslot), levels);
    PT_TRY(check_launch(ctx, "octree_links"));
    level_offsets<<<1, 32, 0, st>>>(levels);
    PT_TRY(check_launch(ctx, "level_offsets"));
    PT_TRY(scan_u32(ctx, S.prims, as<uint32_t>(S.cnt), as<uint32_t>(S.pscan), n + 1));
    PT_CUDA(cudaStreamWaitEvent(st, S.join, 0));  // the gathered bodies
    layout<T><<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bfirst), as<int>(S.blast), as<int>(S.bdelta),
                                     as<uint8_t>(S.top), as<int>(S.oparent), as<uint32_t>(S.cnt),
                                     as<uint32_t>(S.pscan), as<uint64_t>(S.ukey), as<uint32_t>(S.ufirst),
                                     as<T>(S.box), as<int>(S.pre), as<int4>(S.nodeB), as<V4>(nG),
                                     as<int2>(S.nodeR), as<int>(S.loparent), as<uint8_t>(S.cslot),
                                     as<uint8_t>(S.lslot), as<int>(S.kid), levels, as<int>(S.by_level), as<V4>(sb),
                                     as<Record<T>>(S.mom), as<V4>(nA), nodeQ);
    PT_TRY(check_launch(ctx, "layout"));

    const int lvl_grid = std::max(1, std::min(blocks(n), 8 * ctx->sm_count));
    for (int L = LEVELS - 1; L >= TOP_LEVELS; --L) {
        // level L holds at most 8^L cells: shallow levels get a grid of their size
        const long long cap = L < 10 ? (1ll << (3 * L)) : (long long)n;
        const int grid = int(std::max(1ll, std::min<long long>(lvl_grid, (std::min<long long>(cap, n) + 255) / 256)));
        cells_level<T><<<grid, 256, 0, st>>>(L, levels, as<int>(S.by_level), as<int>(S.pre), as<int>(S.kid),
                                                as<int>(S.nkid), as<V4>(nG), as<Record<T>>(S.mom), as<V4>(nA),
                                                nodeQ, as<int4>(S.nodeB));
        PT_TRY(check_launch(ctx, "cells_level"));
    }
    cells_top<T><<<1, 512, 0, st>>>(levels, as<int>(S.by_level), as<int>(S.pre), as<int>(S.kid), as<int>(S.nkid),
                                    as<V4>(nG), as<Record<T>>(S.mom), as<V4>(nA), nodeQ, as<int4>(S.nodeB));
    PT_TRY(check_launch(ctx, "cells_top"));
    S.last_n_src = n;
    S.f64 = F64;
    S.user_tree = false;
    ++S.generation;
    return PT_OK;
}

int build(pt_ctx *ctx, State &S, const float4 *d_src, int n) { return build_t<float>(ctx, S, d_src, n); }

// Sorts separate targets along the same keys (same root box) for coherent warps.
template <class T>
int sort_targets_t(pt_ctx *ctx, State &S, const typename Prec<T>::V4 *d_aff, int n) {
    using V4 = typename Prec<T>::V4;
    DevBuf &tb = sizeof(T) == 8 ? S.tbody64 : S.tbody;
    cudaStream_t st = ctx->stream;
    PT_TRY(ensure_buf(ctx, S.tkeys, sizeof(uint64_t) * size_t(n)));
    PT_TRY(ensure_buf(ctx, S.tidx, sizeof(uint32_t) * size_t(n)));
    PT_TRY(ensure_buf(ctx, tb, sizeof(V4) * size_t(n)));
    make_keys<T><<<blocks(n), 256, 0, st>>>(d_aff, n, as<T>(S.box), as<uint64_t>(S.tkeys), as<uint32_t>(S.tidx));
    PT_TRY(check_launch(ctx, "make_keys(targets)"));
    PT_TRY(radix_sort_u64(ctx, S.prims, as<uint64_t>(S.tkeys), as<uint32_t>(S.tidx), n, 3 * LEVELS));
    gather_bodies<V4><<<blocks(n), 256, 0, st>>>(d_aff, as<uint32_t>(S.tidx), n, as<V4>(tb));
    return check_launch(ctx, "gather_bodies(targets)");
}

int sort_targets(pt_ctx *ctx, State &S, const float4 *d_aff, int n) {
    return sort_targets_t<float>(ctx, S, d_aff, n);
}


template int build_t<double>(pt_ctx *, State &, const Prec<double>::V4 *, int);
template int sort_targets_t<double>(pt_ctx *, State &, const Prec<double>::V4 *, int);

}  // namespace bh
}  // namespace pt
