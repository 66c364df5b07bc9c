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
//     the subtree), leaves interleaved: the walk needs no stack.
//  7. moments bottom-up in FP64 (mass, centre of mass, second moment -> traceless
//     quadrupole): cells are bucketed by octree level and combined level by level,
//     deepest first, one thread per cell (parallel-axis theorem). No thread ever
//     waits on another.
#include "pt_bh.cuh"

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

// Octree parents, child counts and the count of cells starting at each unit.
__global__ void octree_links(const int *__restrict__ counters, const int *__restrict__ bfirst,
                             const int *__restrict__ bparent, const int *__restrict__ lparent,
                             const uint8_t *__restrict__ top, int *__restrict__ oparent, int *__restrict__ loparent,
                             uint32_t *__restrict__ cnt) {
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < M - 1 && top[k]) {
        const int op = (k == 0) ? -1 : climb(bparent[k], top, bparent);
        oparent[k] = op;
        atomicAdd(&cnt[bfirst[k]], 1u);
    }
    if (k < M) {
        const int op = (M == 1) ? -1 : climb(lparent[k], top, bparent);
        loparent[k] = op;
    }
}

// ---- 6. preorder layout ------------------------------------------------------
// nodeB = {width bits, skip, first body (-1: internal cell), body count}.
// counters[1] = T (cells + leaves), counters[2] = internal cells.
template <class T>
__global__ void layout(int *counters, const int *__restrict__ bfirst,
                       const int *__restrict__ blast, const int *__restrict__ bdelta,
                       const uint8_t *__restrict__ top, const int *__restrict__ oparent,
                       const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ pscan,
                       const uint64_t *__restrict__ ukey, const uint32_t *__restrict__ ufirst,
                       const T *__restrict__ box, int *__restrict__ pre, int4 *__restrict__ nodeB,
                       typename Prec<T>::V4 *__restrict__ nodeG, int2 *__restrict__ nodeR) {
    using P = Prec<T>;
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
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
    }
    if (k < M) {
        const int pk = k + int(pscan[k]) + int(cnt[k]);
        const int f = int(ufirst[k]);
        nodeB[pk] = make_int4(0, pk + 1, f, int(ufirst[k + 1]) - f);
        nodeG[pk] = P::make(T(0), T(0), T(0), T(0));
        nodeR[pk] = make_int2(f, int(ufirst[k + 1]));
    }
}

// ---- 7. moments ------------------------------------------------------------
template <class T>
__device__ void store_cell(const Moments &m, int pk, Moments *__restrict__ mom, typename Prec<T>::V4 *__restrict__ nodeA,
                           float4 *__restrict__ nodeQ) {
    mom[pk] = m;
    nodeA[pk] = Prec<T>::make(T(m.cx), T(m.cy), T(m.cz), T(m.m));
    if (!nodeQ) return;  // the f64 method is monopole only
    const double tr = m.sxx + m.syy + m.szz;
    nodeQ[2 * pk] = make_float4(float(3 * m.sxx - tr), float(3 * m.sxy), float(3 * m.sxz), float(3 * m.syy - tr));
    nodeQ[2 * pk + 1] = make_float4(float(3 * m.syz), float(3 * m.szz - tr), 0.f, 0.f);
}

// Leaves: a single body is its own cell data; several (coincident, or closer than
// the key resolution) get FP64 moments.
template <class T>
__global__ void leaf_moments(const int *__restrict__ counters, const uint32_t *__restrict__ ufirst,
                             const typename Prec<T>::V4 *__restrict__ sbody, const uint32_t *__restrict__ pscan,
                             const uint32_t *__restrict__ cnt, Moments *__restrict__ mom,
                             typename Prec<T>::V4 *__restrict__ nodeA, float4 *__restrict__ nodeQ) {
    using V4 = typename Prec<T>::V4;
    const int M = counters[0];
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= M) return;
    const int f = int(ufirst[u]), e = int(ufirst[u + 1]);
    const int pk = u + int(pscan[u]) + int(cnt[u]);
    if (e - f == 1) {
        nodeA[pk] = sbody[f];
        if (nodeQ) {
            nodeQ[2 * pk] = make_float4(0.f, 0.f, 0.f, 0.f);
            nodeQ[2 * pk + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
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
    store_cell<T>(m, pk, mom, nodeA, nodeQ);
}

// Cells per octree level: lcount[L], then by_level sorted by level (counting sort).
// levels[0..LEVELS] = counts, levels[LEVELS+1 ..] = offsets, then cursors.
__global__ void cell_level_count(const int *__restrict__ counters, const int *__restrict__ bdelta,
                                 const uint8_t *__restrict__ top, int *__restrict__ levels) {
    __shared__ int h[LEVELS];
    if (threadIdx.x < LEVELS) h[threadIdx.x] = 0;
    __syncthreads();
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < M - 1 && top[k]) atomicAdd(&h[bdelta[k] / 3], 1);
    __syncthreads();
    if (threadIdx.x < LEVELS && h[threadIdx.x]) atomicAdd(&levels[threadIdx.x], h[threadIdx.x]);
}

__global__ void cell_level_offsets(int *__restrict__ levels) {
    if (threadIdx.x != 0) return;
    int acc = 0;
    for (int L = 0; L < LEVELS; ++L) {
        levels[LEVELS + 1 + L] = acc;      // offset
        levels[2 * LEVELS + 2 + L] = acc;  // cursor
        acc += levels[L];
    }
    levels[2 * LEVELS + 1] = acc;
}

// Each block reserves one range per level with a single global atomic.
__global__ void cell_level_scatter(const int *__restrict__ counters, const int *__restrict__ bdelta,
                                   const uint8_t *__restrict__ top, int *__restrict__ levels,
                                   int *__restrict__ by_level) {
    __shared__ int h[LEVELS], base[LEVELS];
    if (threadIdx.x < LEVELS) h[threadIdx.x] = 0;
    __syncthreads();
    const int M = counters[0];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool cell = k < M - 1 && top[k];
    const int L = cell ? bdelta[k] / 3 : 0;
    const int local = cell ? atomicAdd(&h[L], 1) : 0;
    __syncthreads();
    if (threadIdx.x < LEVELS && h[threadIdx.x])
        base[threadIdx.x] = atomicAdd(&levels[2 * LEVELS + 2 + threadIdx.x], h[threadIdx.x]);
    __syncthreads();
    if (cell) by_level[base[L] + local] = k;
}

// Combines every cell of octree level L from its children (levels > L: done), in one
// pass over the children: sums about the cell's geometric centre G (offsets within
// a cell width, no cancellation), then moved to the centre of mass C by the
// parallel-axis rule S_C = S_G - P P^T / M with P = sum m (c - G) = M (C - G).
template <class T>
__global__ void cell_moments_level(int L, const int *__restrict__ levels, const int *__restrict__ by_level,
                                   const int *__restrict__ pre, const int4 *__restrict__ nodeB,
                                   const typename Prec<T>::V4 *__restrict__ nodeG, Moments *__restrict__ mom,
                                   typename Prec<T>::V4 *__restrict__ nodeA, float4 *__restrict__ nodeQ) {
    using V4 = typename Prec<T>::V4;
    const int begin = levels[LEVELS + 1 + L], end_l = begin + levels[L];
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end_l; i += gridDim.x * blockDim.x) {
        const int pv = pre[by_level[i]];
        const int end = nodeB[pv].y;
        const V4 g = nodeG[pv];
        const double gx = g.x, gy = g.y, gz = g.z;
        Moments m{};
        double px = 0, py = 0, pz = 0;
        for (int c = pv + 1; c < end;) {
            const int4 cb = nodeB[c];
            double cx, cy, cz, cmm, cn, sxx = 0, sxy = 0, sxz = 0, syy = 0, syz = 0, szz = 0;
            if (cb.z >= 0 && cb.w == 1) {  // a single body, read from nodeA
                const V4 a = nodeA[c];
                cx = a.x, cy = a.y, cz = a.z, cmm = a.w, cn = 1.0;
            } else {
                const Moments &cm = mom[c];
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
            c = cb.y;
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
            for (int c = pv + 1; c < end;) {
                const int4 cb = nodeB[c];
                double cx, cy, cz, cn;
                if (cb.z >= 0 && cb.w == 1) {
                    const V4 a = nodeA[c];
                    cx = a.x, cy = a.y, cz = a.z, cn = 1.0;
                } else {
                    cx = mom[c].cx, cy = mom[c].cy, cz = mom[c].cz, cn = mom[c].count;
                }
                ux += cn * (cx - gx);
                uy += cn * (cy - gy);
                uz += cn * (cz - gz);
                c = cb.y;
            }
            m.cx = gx + ux / m.count;
            m.cy = gy + uy / m.count;
            m.cz = gz + uz / m.count;
        }
        store_cell<T>(m, pv, mom, nodeA, nodeQ);
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
    PT_TRY(ensure_buf(ctx, S.levels, sizeof(int) * (3 * LEVELS + 8)));
    PT_TRY(ensure_buf(ctx, S.by_level, sizeof(int) * N));
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
    gather_bodies<V4><<<blocks(n), 256, 0, st>>>(d_src, as<uint32_t>(S.idx), n, as<V4>(sb));
    PT_TRY(check_launch(ctx, "gather_bodies"));
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
    PT_CUDA(cudaMemsetAsync(S.levels.ptr, 0, sizeof(int) * (3 * LEVELS + 8), st));
    octree_links<<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bfirst), as<int>(S.bparent), as<int>(S.lparent),
                                           as<uint8_t>(S.top), as<int>(S.oparent), as<int>(S.loparent),
                                           as<uint32_t>(S.cnt));
    PT_TRY(check_launch(ctx, "octree_links"));
    PT_TRY(scan_u32(ctx, S.prims, as<uint32_t>(S.cnt), as<uint32_t>(S.pscan), n + 1));
    layout<T><<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bfirst), as<int>(S.blast), as<int>(S.bdelta),
                                     as<uint8_t>(S.top), as<int>(S.oparent), as<uint32_t>(S.cnt),
                                     as<uint32_t>(S.pscan), as<uint64_t>(S.ukey), as<uint32_t>(S.ufirst),
                                     as<T>(S.box), as<int>(S.pre), as<int4>(S.nodeB), as<V4>(nG),
                                     as<int2>(S.nodeR));
    PT_TRY(check_launch(ctx, "layout"));

    int *levels = as<int>(S.levels);
    cell_level_count<<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bdelta), as<uint8_t>(S.top), levels);
    PT_TRY(check_launch(ctx, "cell_level_count"));
    cell_level_offsets<<<1, 32, 0, st>>>(levels);
    PT_TRY(check_launch(ctx, "cell_level_offsets"));
    cell_level_scatter<<<blocks(n), 256, 0, st>>>(counters, as<int>(S.bdelta), as<uint8_t>(S.top), levels,
                                                 as<int>(S.by_level));
    PT_TRY(check_launch(ctx, "cell_level_scatter"));
    leaf_moments<T><<<blocks(n), 256, 0, st>>>(counters, as<uint32_t>(S.ufirst), as<V4>(sb),
                                              as<uint32_t>(S.pscan), as<uint32_t>(S.cnt), as<Moments>(S.mom),
                                              as<V4>(nA), nodeQ);
    PT_TRY(check_launch(ctx, "leaf_moments"));
    const int lvl_grid = std::max(1, std::min(blocks(n), 8 * ctx->sm_count));
    for (int L = LEVELS - 1; L >= 0; --L) {
        cell_moments_level<T><<<lvl_grid, 256, 0, st>>>(L, levels, as<int>(S.by_level), as<int>(S.pre),
                                                        as<int4>(S.nodeB), as<V4>(nG), as<Moments>(S.mom),
                                                        as<V4>(nA), nodeQ);
        PT_TRY(check_launch(ctx, "cell_moments_level"));
    }
    S.last_n_src = n;
    S.f64 = F64;
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
