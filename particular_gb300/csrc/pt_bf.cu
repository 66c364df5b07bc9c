// cuda::BruteForce: all-pairs gravitational acceleration on sm_103a.
//
// Computes, for every affected body i, out_i = sum_j a(x_i, s_j) with the
// per-pair kernel of particular/src/gravity/impls/mod.rs:150-166:
//     d = x_j - x_i;  n = |d|^2;  checked && n == 0 -> d;
//     else a = d * (mu_j / (n_s * sqrt(n_s))),  n_s = n + eps^2
// (the sum that sequential::BruteForce folds, particular/src/sequential.rs:189-193,
// and that the wgpu shader tiles, particular/src/gpu/bruteforce_shared.wgsl:16-28).
//
// Three kernels:
//  * bf_fast  : the throughput path. CTAs own an i-block of THREADS*K targets (K
//               targets per thread) and a j-slice; source tiles of TILE bodies, in
//               structure-of-arrays form (bf_to_soa), are staged in shared memory by
//               cp.async through a STAGES-deep ring; every thread reads them as warp
//               broadcasts and evaluates two pairs per packed f32x2 instruction
//               (12 FMA-pipe lanes-ops and one MUFU rsqrt per pair). Sums are plain
//               FP32 inside a tile and compensated (two-sum) across tiles. j-slices
//               (grid.y) keep all SMs busy at small N; their partials are combined by
//               bf_fixup in a fixed order, so the result is deterministic.
//  * bf_exact : one thread per target, sequential j order, IEEE sqrt/div and no
//               contraction: bit-identical to sequential::BruteForce.
//  * bf_f64   : the same formula in double, the error judge.
#include "pt_common.cuh"
#include "pt_f32x2.cuh"

#include <algorithm>
#include <climits>
#include <cmath>

namespace pt {
namespace bf {

constexpr int THREADS = 128;
constexpr int TILE = 256;  // sources per stage: 4 KiB
constexpr int STAGES = 4;
constexpr int COPIES = TILE / THREADS;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Stages sources [j0 + t*TILE, min(j_end, j0 + (t+1)*TILE)) into `stage`.
__device__ __forceinline__ void load_tile(float4 *stage, const float4 *__restrict__ src, int j0,
                                          int j_end, int t) {
    const int base = j0 + t * TILE;
#pragma unroll
    for (int r = 0; r < COPIES; ++r) {
        const int e = threadIdx.x + r * THREADS;
        if (base + e < j_end) cp_async16(stage + e, src + base + e);
    }
}

// Runs f(tile_ptr, count) over the sources [j0, j_end) through the cp.async ring.
// Every thread of the CTA must call it (it synchronises the CTA).
template <class F>
__device__ __forceinline__ void for_each_tile(float4 (*tiles)[TILE], const float4 *__restrict__ src,
                                              int j0, int j_end, F &&f) {
    const int ntiles = (j_end - j0 + TILE - 1) / TILE;
#pragma unroll
    for (int st = 0; st < STAGES - 1; ++st) {
        if (st < ntiles) load_tile(tiles[st], src, j0, j_end, st);
        cp_async_commit();
    }
    for (int t = 0; t < ntiles; ++t) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();  // tile t visible to all; tile t-1 fully consumed
        const int nt = t + STAGES - 1;
        if (nt < ntiles) load_tile(tiles[nt % STAGES], src, j0, j_end, nt);
        cp_async_commit();
        f(static_cast<const float4 *>(tiles[t % STAGES]), min(TILE, j_end - (j0 + t * TILE)));
    }
    cp_async_wait<0>();
}

// Sources in structure-of-arrays form (x[], y[], z[], mu[], each padded to a
// multiple of TILE) so that one LDS.128 yields two packed source pairs.
struct SoaTile {
    float c[4][TILE];
};

__device__ __forceinline__ void load_tile_soa(SoaTile &stage, const float *__restrict__ soa, int n_pad, int j0,
                                              int j_end, int t) {
    const int base = j0 + t * TILE;
    constexpr int QUADS = TILE / 4;
#pragma unroll
    for (int r = 0; r < (4 * QUADS) / THREADS; ++r) {
        const int c = threadIdx.x + r * THREADS;
        const int a = c / QUADS, q = c % QUADS;
        if (base + 4 * q < j_end) cp_async16(&stage.c[a][4 * q], soa + size_t(a) * n_pad + base + 4 * q);
    }
}

// part (when non-null): [gridDim.y][2][n_aff] float4 = per-slice (sum, compensation).
template <int K, bool GUARD>
__global__ void __launch_bounds__(THREADS)
    bf_fast(const float4 *__restrict__ aff, int n_aff, const float *__restrict__ soa, int n_src, int n_pad,
            float eps2, int slice_len, float4 *__restrict__ part, float *__restrict__ out) {
    __shared__ __align__(16) SoaTile tiles[STAGES];
    const int i0 = blockIdx.x * (THREADS * K);
    const int j0 = blockIdx.y * slice_len;
    const int j_end = min(n_src, j0 + slice_len);
    const int ntiles = (j_end - j0 + TILE - 1) / TILE;

    float xi[K], yi[K], zi[K], sx[K], sy[K], sz[K], cx[K], cy[K], cz[K];
    f2 xi2[K], yi2[K], zi2[K], ax[K], ay[K], az[K];
    const f2 e2 = pk2(eps2, eps2);
    const f2 zero2 = pk2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = i0 + k * THREADS + threadIdx.x;
        const float4 p = (i < n_aff) ? aff[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        xi[k] = p.x;
        yi[k] = p.y;
        zi[k] = p.z;
        xi2[k] = pk2(p.x, p.x);
        yi2[k] = pk2(p.y, p.y);
        zi2[k] = pk2(p.z, p.z);
        ax[k] = ay[k] = az[k] = zero2;
        sx[k] = sy[k] = sz[k] = 0.f;
        cx[k] = cy[k] = cz[k] = 0.f;
    }

#pragma unroll
    for (int st = 0; st < STAGES - 1; ++st) {
        if (st < ntiles) load_tile_soa(tiles[st], soa, n_pad, j0, j_end, st);
        cp_async_commit();
    }
    for (int t = 0; t < ntiles; ++t) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        const int nt = t + STAGES - 1;
        if (nt < ntiles) load_tile_soa(tiles[nt % STAGES], soa, n_pad, j0, j_end, nt);
        cp_async_commit();
        const SoaTile &T = tiles[t % STAGES];
        const int cnt = min(TILE, j_end - (j0 + t * TILE));
        if (cnt == TILE) {
            const float4 *X = reinterpret_cast<const float4 *>(T.c[0]);
            const float4 *Y = reinterpret_cast<const float4 *>(T.c[1]);
            const float4 *Z = reinterpret_cast<const float4 *>(T.c[2]);
            const float4 *M = reinterpret_cast<const float4 *>(T.c[3]);
#pragma unroll 2
            for (int q = 0; q < TILE / 4; ++q) {
                const float4 x = X[q], y = Y[q], z = Z[q], m = M[q];
                const f2 xa = pk2(x.x, x.y), xb = pk2(x.z, x.w);
                const f2 ya = pk2(y.x, y.y), yb = pk2(y.z, y.w);
                const f2 za = pk2(z.x, z.y), zb = pk2(z.z, z.w);
                const f2 ma = pk2(m.x, m.y), mb = pk2(m.z, m.w);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    interact2<GUARD>(xa, ya, za, ma, xi2[k], yi2[k], zi2[k], ax[k], ay[k], az[k], e2);
                    interact2<GUARD>(xb, yb, zb, mb, xi2[k], yi2[k], zi2[k], ax[k], ay[k], az[k], e2);
                }
            }
#pragma unroll
            for (int k = 0; k < K; ++k) {
                float l, h;
                upk2(ax[k], l, h);
                two_sum_acc(sx[k], cx[k], l + h);
                upk2(ay[k], l, h);
                two_sum_acc(sy[k], cy[k], l + h);
                upk2(az[k], l, h);
                two_sum_acc(sz[k], cz[k], l + h);
                ax[k] = ay[k] = az[k] = zero2;
            }
        } else {
#pragma unroll 1
            for (int jj = 0; jj < cnt; ++jj) {
                const float xj = T.c[0][jj], yj = T.c[1][jj], zj = T.c[2][jj], mj = T.c[3][jj];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
                    interact1<GUARD>(xj, yj, zj, mj, xi[k], yi[k], zi[k], a0, a1, a2, eps2);
                    two_sum_acc(sx[k], cx[k], a0);
                    two_sum_acc(sy[k], cy[k], a1);
                    two_sum_acc(sz[k], cz[k], a2);
                }
            }
        }
    }
    cp_async_wait<0>();

#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = i0 + k * THREADS + threadIdx.x;
        if (i >= n_aff) continue;
        if (part) {
            float4 *ps = part + size_t(blockIdx.y) * 2 * size_t(n_aff);
            ps[i] = make_float4(sx[k], sy[k], sz[k], 0.f);
            ps[size_t(n_aff) + i] = make_float4(cx[k], cy[k], cz[k], 0.f);
        } else {
            out[3 * size_t(i) + 0] = sx[k] + cx[k];
            out[3 * size_t(i) + 1] = sy[k] + cy[k];
            out[3 * size_t(i) + 2] = sz[k] + cz[k];
        }
    }
}

// Sources (x, y, z, mu) rows -> four padded arrays (tail zero-filled, never read
// as sources because every loop is bounded by n_src).
__global__ void bf_to_soa(const float4 *__restrict__ src, int n, int n_pad, float *__restrict__ soa) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    const float4 p = (i < n) ? src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    soa[i] = p.x;
    soa[size_t(n_pad) + i] = p.y;
    soa[2 * size_t(n_pad) + i] = p.z;
    soa[3 * size_t(n_pad) + i] = p.w;
}

// Combines the slices' (sum, compensation) pairs in slice order, in double.
__global__ void bf_fixup(const float4 *__restrict__ part, int n_aff, int slices, float *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_aff) return;
    double x = 0.0, y = 0.0, z = 0.0;
    for (int s = 0; s < slices; ++s) {
        const float4 a = part[size_t(s) * 2 * size_t(n_aff) + i];
        const float4 c = part[size_t(s) * 2 * size_t(n_aff) + size_t(n_aff) + i];
        x += double(a.x) + double(c.x);
        y += double(a.y) + double(c.y);
        z += double(a.z) + double(c.z);
    }
    out[3 * size_t(i) + 0] = float(x);
    out[3 * size_t(i) + 1] = float(y);
    out[3 * size_t(i) + 2] = float(z);
}

// Bit-identical restatement of sequential::BruteForce (sequential.rs:189-193 over
// gravity/impls/mod.rs:156-165): every operation is an explicitly rounded IEEE op.
// VEC3A: glam Vec3A / Vec4's own kernel, a = (d * m) / (n_s sqrt(n_s)) per component
// (particular/src/gravity/impls/glam.rs:260-275), instead of d * (m / ...).
template <bool VEC3A>
__global__ void __launch_bounds__(THREADS)
    bf_exact(const float4 *__restrict__ aff, int n_aff, const float4 *__restrict__ src, int n_src,
             float soft2, int checked, float *__restrict__ out) {
    __shared__ __align__(16) float4 tiles[STAGES][TILE];
    const int i = blockIdx.x * THREADS + threadIdx.x;
    const float4 pi = (i < n_aff) ? aff[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for_each_tile(tiles, src, 0, n_src, [&](const float4 *T, int cnt) {
#pragma unroll 1
        for (int jj = 0; jj < cnt; ++jj) {
            const float4 p = T[jj];
            const float dx = __fsub_rn(p.x, pi.x);
            const float dy = __fsub_rn(p.y, pi.y);
            const float dz = __fsub_rn(p.z, pi.z);
            const float n = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            float ax, ay, az;
            if (checked && n == 0.0f) {
                ax = dx;
                ay = dy;
                az = dz;
            } else {
                const float ns = __fadd_rn(n, soft2);
                const float den = __fmul_rn(ns, __fsqrt_rn(ns));
                if (VEC3A) {
                    ax = __fdiv_rn(__fmul_rn(dx, p.w), den);
                    ay = __fdiv_rn(__fmul_rn(dy, p.w), den);
                    az = __fdiv_rn(__fmul_rn(dz, p.w), den);
                } else {
                    const float s = __fdiv_rn(p.w, den);
                    ax = __fmul_rn(dx, s);
                    ay = __fmul_rn(dy, s);
                    az = __fmul_rn(dz, s);
                }
            }
            sx = __fadd_rn(sx, ax);
            sy = __fadd_rn(sy, ay);
            sz = __fadd_rn(sz, az);
        }
    });
    if (i < n_aff) {
        out[3 * size_t(i) + 0] = sx;
        out[3 * size_t(i) + 1] = sy;
        out[3 * size_t(i) + 2] = sz;
    }
}

// FP64 judge: f32 inputs widened, double arithmetic and accumulation. grid.y splits
// the sources into slices whose partial sums (part, [slices][3 * n_aff]) are added
// in slice order by bf_f64_fixup; with one slice the kernel writes out directly.
__global__ void __launch_bounds__(THREADS)
    bf_f64(const float4 *__restrict__ aff, int n_aff, const float4 *__restrict__ src, int n_src,
           double soft2, int checked, int slice_len, double *__restrict__ part, double *__restrict__ out) {
    __shared__ __align__(16) float4 tiles[STAGES][TILE];
    const int i = blockIdx.x * THREADS + threadIdx.x;
    const int j0 = blockIdx.y * slice_len;
    const int j_end = min(n_src, j0 + slice_len);
    const float4 pi = (i < n_aff) ? aff[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const double xi = pi.x, yi = pi.y, zi = pi.z;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for_each_tile(tiles, src, j0, j_end, [&](const float4 *T, int cnt) {
#pragma unroll 2
        for (int jj = 0; jj < cnt; ++jj) {
            const float4 p = T[jj];
            const double dx = double(p.x) - xi, dy = double(p.y) - yi, dz = double(p.z) - zi;
            const double n = dx * dx + dy * dy + dz * dz;
            if (checked && n == 0.0) continue;
            const double ns = n + soft2;
            const double s = double(p.w) / (ns * sqrt(ns));
            sx += dx * s;
            sy += dy * s;
            sz += dz * s;
        }
    });
    if (i < n_aff) {
        double *o = part ? part + size_t(blockIdx.y) * 3 * size_t(n_aff) : out;
        o[3 * size_t(i) + 0] = sx;
        o[3 * size_t(i) + 1] = sy;
        o[3 * size_t(i) + 2] = sz;
    }
}

__global__ void bf_f64_fixup(const double *__restrict__ part, int n_aff, int slices, double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 3 * n_aff) return;
    double acc = 0.0;
    for (int s = 0; s < slices; ++s) acc += part[size_t(s) * 3 * size_t(n_aff) + k];
    out[k] = acc;
}

// glam DVec3 bodies (impl_acceleration_cpu_scalar!(DVec3, f64) at
// particular/src/gravity/impls/glam.rs:234 over gravity/impls/mod.rs:150-166, folded
// as sequential.rs:189-193): the exact kernel in double. Every operation is an
// explicitly rounded IEEE op and j runs in order, so the result is the reference's
// bit for bit. Bodies are double[4] (x, y, z, mu); a tile of 256 sources is staged
// in shared memory per step.
__global__ void __launch_bounds__(THREADS)
    bf_dvec3(const double *__restrict__ aff, int n_aff, const double *__restrict__ src, int n_src, double soft2,
             int checked, double *__restrict__ out) {
    __shared__ __align__(16) double tile[TILE][4];
    const int i = blockIdx.x * THREADS + threadIdx.x;
    double xi = 0.0, yi = 0.0, zi = 0.0;
    if (i < n_aff) {
        xi = aff[4 * size_t(i) + 0];
        yi = aff[4 * size_t(i) + 1];
        zi = aff[4 * size_t(i) + 2];
    }
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int j0 = 0; j0 < n_src; j0 += TILE) {
        const int cnt = min(TILE, n_src - j0);
        __syncthreads();
        for (int k = threadIdx.x; k < 4 * cnt; k += THREADS) (&tile[0][0])[k] = src[4 * size_t(j0) + k];
        __syncthreads();
#pragma unroll 1
        for (int jj = 0; jj < cnt; ++jj) {
            const double dx = __dsub_rn(tile[jj][0], xi);
            const double dy = __dsub_rn(tile[jj][1], yi);
            const double dz = __dsub_rn(tile[jj][2], zi);
            const double n = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            double ax, ay, az;
            if (checked && n == 0.0) {
                ax = dx;
                ay = dy;
                az = dz;
            } else {
                const double ns = __dadd_rn(n, soft2);
                const double s = __ddiv_rn(tile[jj][3], __dmul_rn(ns, __dsqrt_rn(ns)));
                ax = __dmul_rn(dx, s);
                ay = __dmul_rn(dy, s);
                az = __dmul_rn(dz, s);
            }
            sx = __dadd_rn(sx, ax);
            sy = __dadd_rn(sy, ay);
            sz = __dadd_rn(sz, az);
        }
    }
    if (i < n_aff) {
        out[3 * size_t(i) + 0] = sx;
        out[3 * size_t(i) + 1] = sy;
        out[3 * size_t(i) + 2] = sz;
    }
}

using FastKernel = void (*)(const float4 *, int, const float *, int, int, float, int, float4 *, float *);

template <int K>
FastKernel pick(bool guard) {
    return guard ? bf_fast<K, true> : bf_fast<K, false>;
}

FastKernel fast_kernel(int K, bool guard) {
    switch (K) {
        case 1: return pick<1>(guard);
        case 2: return pick<2>(guard);
        default: return pick<4>(guard);
    }
}

struct Plan {
    int K = 4;
    int slices = 1;
    int slice_len = 0;
    int n_ib = 0;
};

// Occupancy of the fast kernels, cached per (K, guard).
static int occupancy(int K, bool guard) {
    static int cache[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    const int kk = K == 1 ? 0 : (K == 2 ? 1 : 2);
    int &o = cache[kk][guard ? 1 : 0];
    if (o == 0) {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, fast_kernel(K, guard), THREADS, 0) != cudaSuccess || v < 1)
            v = 1;
        o = v;
    }
    return o;
}

// Picks K and the number of j-slices by a wave model: CTAs of equal cost run in
// ceil(ctas / slots) waves; minimise waves * per-CTA work, plus the fixup pass.
static Plan plan(const pt_ctx *ctx, int n_aff, int n_src, bool guard, int force_k, int force_s) {
    Plan p;
    // K=1 wins below ~2^18 targets: its 56 registers leave room for 9 CTAs per SM,
    // which hides the MUFU and shared-memory latency better than K=4's ILP.
    p.K = force_k ? force_k : (n_aff >= (1 << 18) ? 2 : 1);
    p.n_ib = (n_aff + THREADS * p.K - 1) / (THREADS * p.K);
    const int tiles = (n_src + TILE - 1) / TILE;
    const long long slots = (long long)std::max(1, ctx->sm_count) * occupancy(p.K, guard);
    int best_s = 1;
    double best_cost = 1e300;
    const int max_s = std::max(1, std::min(tiles, 256));
    for (int s = 1; s <= max_s; ++s) {
        const int len_tiles = (tiles + s - 1) / s;
        const int s_eff = (tiles + len_tiles - 1) / len_tiles;
        if (s_eff != s) continue;
        const long long ctas = (long long)p.n_ib * s;
        const long long waves = (ctas + slots - 1) / slots;
        // per-CTA cost ~ tiles it streams (plus a fixed tile of start-up);
        // fixup reads 32 B per target per slice.
        double cost = double(waves) * (len_tiles + 1) * p.K;
        if (s > 1) cost += 0.02 * s * (double(n_aff) / double(slots * THREADS)) + 1.0;
        if (cost < best_cost * 0.999) {
            best_cost = cost;
            best_s = s;
        }
    }
    if (force_s) best_s = std::max(1, std::min(force_s, std::max(1, tiles)));
    const int len_tiles = (tiles + best_s - 1) / best_s;
    p.slice_len = len_tiles * TILE;
    p.slices = (n_src + p.slice_len - 1) / p.slice_len;
    return p;
}

struct Forced {
    int k = 0, s = 0;
};
static thread_local Forced g_forced;

}  // namespace bf

void bf_forced_plan(int *targets_per_thread, int *slices) {
    *targets_per_thread = bf::g_forced.k;
    *slices = bf::g_forced.s;
}

// Launches the fast or exact f32 brute force on device buffers (ctx->stream).
int bf_launch_f32(pt_ctx *ctx, const float4 *aff, int n_aff, const float4 *src, int n_src,
                  float softening, int checked, uint32_t flags, float *out) {
    using namespace bf;
    cudaStream_t st = ctx->stream;
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * 3 * size_t(n_aff), st));
        return PT_OK;
    }
    const float soft2 = softening * softening;
    if (flags & PT_BF_EXACT) {
        dim3 grid((n_aff + THREADS - 1) / THREADS);
        if (flags & PT_BF_VEC3A) bf_exact<true><<<grid, THREADS, 0, st>>>(aff, n_aff, src, n_src, soft2, checked, out);
        else bf_exact<false><<<grid, THREADS, 0, st>>>(aff, n_aff, src, n_src, soft2, checked, out);
        return check_launch(ctx, "bf_exact");
    }
    const bool guard = checked && soft2 == 0.0f;
    Plan p = plan(ctx, n_aff, n_src, guard, g_forced.k, g_forced.s);
    float4 *part = nullptr;
    if (p.slices > 1) {
        PT_TRY(ensure(ctx, BUF_PART, sizeof(float4) * 2 * size_t(n_aff) * size_t(p.slices)));
        part = static_cast<float4 *>(ctx->bufs[BUF_PART].ptr);
    }
    const int n_pad = (n_src + TILE - 1) / TILE * TILE;
    PT_TRY(ensure(ctx, BUF_SOA, sizeof(float) * 4 * size_t(n_pad)));
    float *soa = static_cast<float *>(ctx->bufs[BUF_SOA].ptr);
    mark(ctx, 0);
    bf_to_soa<<<(n_pad + 255) / 256, 256, 0, st>>>(src, n_src, n_pad, soa);
    PT_TRY(check_launch(ctx, "bf_to_soa"));
    mark(ctx, 1);
    dim3 grid(p.n_ib, p.slices);
    fast_kernel(p.K, guard)<<<grid, THREADS, 0, st>>>(aff, n_aff, soa, n_src, n_pad, soft2, p.slice_len, part, out);
    PT_TRY(check_launch(ctx, "bf_fast"));
    if (part) {
        bf_fixup<<<(n_aff + 255) / 256, 256, 0, st>>>(part, n_aff, p.slices, out);
        PT_TRY(check_launch(ctx, "bf_fixup"));
    }
    mark(ctx, 2);
    return PT_OK;
}

int bf_launch_f64(pt_ctx *ctx, const float4 *aff, int n_aff, const float4 *src, int n_src,
                  double softening, int checked, double *out) {
    using namespace bf;
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 3 * size_t(n_aff), ctx->stream));
        return PT_OK;
    }
    const int n_ib = (n_aff + THREADS - 1) / THREADS;
    const int tiles = (n_src + TILE - 1) / TILE;
    int slices = std::max(1, std::min(tiles, (4 * ctx->sm_count + n_ib - 1) / n_ib));
    const int slice_len = (tiles + slices - 1) / slices * TILE;
    slices = (n_src + slice_len - 1) / slice_len;
    double *part = nullptr;
    if (slices > 1) {
        PT_TRY(ensure(ctx, BUF_PART, sizeof(double) * 3 * size_t(n_aff) * size_t(slices)));
        part = static_cast<double *>(ctx->bufs[BUF_PART].ptr);
    }
    dim3 grid(n_ib, slices);
    bf_f64<<<grid, THREADS, 0, ctx->stream>>>(aff, n_aff, src, n_src, softening * softening, checked, slice_len,
                                             part, out);
    PT_TRY(check_launch(ctx, "bf_f64"));
    if (part) {
        bf_f64_fixup<<<(3 * n_aff + 255) / 256, 256, 0, ctx->stream>>>(part, n_aff, slices, out);
        PT_TRY(check_launch(ctx, "bf_f64_fixup"));
    }
    return PT_OK;
}

int bf_launch_dvec3(pt_ctx *ctx, const double *aff, int n_aff, const double *src, int n_src, double softening,
                    int checked, double *out) {
    using namespace bf;
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 3 * size_t(n_aff), ctx->stream));
        return PT_OK;
    }
    mark(ctx, 1);
    bf_dvec3<<<(n_aff + THREADS - 1) / THREADS, THREADS, 0, ctx->stream>>>(aff, n_aff, src, n_src,
                                                                          softening * softening, checked, out);
    PT_TRY(check_launch(ctx, "bf_dvec3"));
    mark(ctx, 2);
    return PT_OK;
}

static int validate_sizes(const char *fn, size_t n_aff, size_t n_src) {
    const size_t lim = size_t(INT_MAX) / 8;
    if (n_aff > lim || n_src > lim)
        return set_error(PT_ERR_INVALID, "%s: n_aff=%zu n_src=%zu exceed the limit %zu", fn, n_aff, n_src, lim);
    return PT_OK;
}

}  // namespace pt

extern "C" {

int pt_bf_set_plan(pt_ctx *ctx, int targets_per_thread, int slices) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_bf_set_plan: ctx is NULL");
    if (!(targets_per_thread == 0 || targets_per_thread == 1 || targets_per_thread == 2 ||
          targets_per_thread == 4) || slices < 0)
        return pt::set_error(PT_ERR_INVALID, "pt_bf_set_plan: targets_per_thread must be 0, 1, 2 or 4 and slices >= 0");
    pt::bf::g_forced.k = targets_per_thread;
    pt::bf::g_forced.s = slices;
    return PT_OK;
}

int pt_bf_accel_f32_device(pt_ctx *ctx, const float *d_aff, size_t n_aff, const float *d_src, size_t n_src,
                           float softening, int checked, uint32_t flags, float *d_out) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f32_device: ctx is NULL");
    if (flags & ~(PT_BF_EXACT | PT_BF_VEC3A)) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f32_device: unknown flags 0x%x", flags);
    PT_TRY(pt::validate_sizes("pt_bf_accel_f32_device", n_aff, n_src));
    if (n_aff && (!d_aff || !d_out)) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f32_device: NULL buffer");
    if (n_src && !d_src) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f32_device: NULL affecting buffer");
    if ((n_aff && !pt::aligned16(d_aff)) || (n_src && !pt::aligned16(d_src)))
        return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f32_device: body buffers must be 16-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    return pt::bf_launch_f32(ctx, reinterpret_cast<const float4 *>(d_aff), int(n_aff),
                             reinterpret_cast<const float4 *>(d_src), int(n_src), softening, checked, flags, d_out);
}

int pt_bf_accel_f64_device(pt_ctx *ctx, const float *d_aff, size_t n_aff, const float *d_src, size_t n_src,
                           double softening, int checked, double *d_out) {
    pt::clear_error();
    if (!ctx) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f64_device: ctx is NULL");
    PT_TRY(pt::validate_sizes("pt_bf_accel_f64_device", n_aff, n_src));
    if (n_aff && (!d_aff || !d_out)) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f64_device: NULL buffer");
    if (n_src && !d_src) return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f64_device: NULL affecting buffer");
    if ((n_aff && !pt::aligned16(d_aff)) || (n_src && !pt::aligned16(d_src)))
        return pt::set_error(PT_ERR_INVALID, "pt_bf_accel_f64_device: body buffers must be 16-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    return pt::bf_launch_f64(ctx, reinterpret_cast<const float4 *>(d_aff), int(n_aff),
                             reinterpret_cast<const float4 *>(d_src), int(n_src), softening, checked, d_out);
}

int pt_bf_accel_f32(pt_ctx *ctx, const float *aff, size_t n_aff, const float *src, size_t n_src, float softening,
                    int checked, uint32_t flags, float *out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32: ctx is NULL");
    if (flags & ~(PT_BF_EXACT | PT_BF_VEC3A)) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32: unknown flags 0x%x", flags);
    PT_TRY(validate_sizes("pt_bf_accel_f32", n_aff, n_src));
    if (n_aff && (!aff || !out)) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32: NULL buffer");
    if (n_src && !src) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32: NULL affecting buffer");
    if (n_aff == 0) return PT_OK;
    PT_CUDA(cudaSetDevice(ctx->device));
    const bool same = (aff == src) && (n_aff == n_src);
    PT_TRY(ensure(ctx, BUF_AFF, 16 * n_aff));
    if (!same && n_src) PT_TRY(ensure(ctx, BUF_SRC, 16 * n_src));
    PT_TRY(ensure(ctx, BUF_OUT, 12 * n_aff));
    float *d_aff = static_cast<float *>(ctx->bufs[BUF_AFF].ptr);
    float *d_src = same ? d_aff : static_cast<float *>(ctx->bufs[BUF_SRC].ptr);
    float *d_out = static_cast<float *>(ctx->bufs[BUF_OUT].ptr);
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(d_aff, aff, 16 * n_aff, cudaMemcpyHostToDevice, st));
    if (!same && n_src) PT_CUDA(cudaMemcpyAsync(d_src, src, 16 * n_src, cudaMemcpyHostToDevice, st));
    PT_TRY(bf_launch_f32(ctx, reinterpret_cast<const float4 *>(d_aff), int(n_aff),
                         reinterpret_cast<const float4 *>(d_src), int(n_src), softening, checked, flags, d_out));
    PT_CUDA(cudaMemcpyAsync(out, d_out, 12 * n_aff, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}

int pt_bf_accel_dvec3_device(pt_ctx *ctx, const double *d_aff, size_t n_aff, const double *d_src, size_t n_src,
                             double softening, int checked, double *d_out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3_device: ctx is NULL");
    PT_TRY(validate_sizes("pt_bf_accel_dvec3_device", n_aff, n_src));
    if (n_aff && (!d_aff || !d_out)) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3_device: NULL buffer");
    if (n_src && !d_src) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3_device: NULL affecting buffer");
    PT_CUDA(cudaSetDevice(ctx->device));
    mark(ctx, 0);
    return bf_launch_dvec3(ctx, d_aff, int(n_aff), d_src, int(n_src), softening, checked, d_out);
}

int pt_bf_accel_dvec3(pt_ctx *ctx, const double *aff, size_t n_aff, const double *src, size_t n_src,
                      double softening, int checked, double *out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3: ctx is NULL");
    PT_TRY(validate_sizes("pt_bf_accel_dvec3", n_aff, n_src));
    if (n_aff && (!aff || !out)) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3: NULL buffer");
    if (n_src && !src) return set_error(PT_ERR_INVALID, "pt_bf_accel_dvec3: NULL affecting buffer");
    if (n_aff == 0) return PT_OK;
    PT_CUDA(cudaSetDevice(ctx->device));
    const bool same = (aff == src) && (n_aff == n_src);
    PT_TRY(ensure(ctx, BUF_AFF, 32 * n_aff));
    if (!same && n_src) PT_TRY(ensure(ctx, BUF_SRC, 32 * n_src));
    PT_TRY(ensure(ctx, BUF_OUT64, 24 * n_aff));
    double *d_aff = static_cast<double *>(ctx->bufs[BUF_AFF].ptr);
    double *d_src = same ? d_aff : static_cast<double *>(ctx->bufs[BUF_SRC].ptr);
    double *d_out = static_cast<double *>(ctx->bufs[BUF_OUT64].ptr);
    cudaStream_t st = ctx->stream;
    mark(ctx, 0);
    PT_CUDA(cudaMemcpyAsync(d_aff, aff, 32 * n_aff, cudaMemcpyHostToDevice, st));
    if (!same && n_src) PT_CUDA(cudaMemcpyAsync(d_src, src, 32 * n_src, cudaMemcpyHostToDevice, st));
    PT_TRY(bf_launch_dvec3(ctx, d_aff, int(n_aff), d_src, int(n_src), softening, checked, d_out));
    PT_CUDA(cudaMemcpyAsync(out, d_out, 24 * n_aff, cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    return PT_OK;
}

}  // extern "C"

// ---- allocation-free brute force ------------------------------------------
// pt_bf_accel_f32_noalloc runs the same kernels as pt_bf_accel_f32_device
// (bf_to_soa -> bf_fast -> bf_fixup) but takes its scratch from one file-scope
// device array instead of context buffers, so a call never allocates device
// memory. It serves callers that cannot call cudaMalloc: host programs that own
// every byte of device memory through their own pool or fixed budget, and
// time-critical loops where cudaMalloc/cudaFree's implicit device-wide
// synchronisation is not acceptable.
#include <mutex>

namespace pt {
namespace bf {

// Sources as x[], y[], z[], mu[] (16 B per padded source) and the j-slice
// partials (32 B per target per slice): 16 MiB in total, held by every device
// that loads this module until the process exits.
constexpr size_t NOALLOC_SOA_BYTES = size_t(8) << 20;
constexpr size_t NOALLOC_PART_BYTES = size_t(8) << 20;
static_assert(size_t(PT_NOALLOC_MAX_SOURCES) * 16 <= NOALLOC_SOA_BYTES, "scratch too small");
static_assert(PT_NOALLOC_MAX_SOURCES % TILE == 0, "padded sources must fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SOA_BYTES + NOALLOC_PART_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 128;
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static int g_noalloc_sms[NOALLOC_MAX_DEVICES];

// Once per device, with that device current: the device address of the scratch
// array (in host code its name is only a host-side stand-in) and the SM count.
static int noalloc_setup(int dev, unsigned char **ptr, int *sms) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return set_error(PT_ERR_INVALID, "pt_bf_accel_f32_noalloc: device %d unsupported", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        PT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        int sm = 0;
        PT_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
        g_noalloc_sms[dev] = sm;
        g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *ptr = g_noalloc_ptr[dev];
    *sms = g_noalloc_sms[dev];
    return PT_OK;
}

}  // namespace bf
}  // namespace pt

extern "C" int pt_bf_accel_f32_noalloc(const float *d_aff, size_t n_aff, const float *d_src, size_t n_src,
                                       float softening, int checked, float *d_out, void *stream) {
    using namespace pt;
    using namespace pt::bf;
    clear_error();
    PT_TRY(validate_sizes("pt_bf_accel_f32_noalloc", n_aff, n_src));
    if (n_src > size_t(PT_NOALLOC_MAX_SOURCES))
        return set_error(PT_ERR_CAPACITY,
                         "pt_bf_accel_f32_noalloc: n_src=%zu exceeds the static scratch limit of %d sources",
                         n_src, PT_NOALLOC_MAX_SOURCES);
    if (n_aff && (!d_aff || !d_out)) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32_noalloc: NULL buffer");
    if (n_src && !d_src) return set_error(PT_ERR_INVALID, "pt_bf_accel_f32_noalloc: NULL affecting buffer");
    if ((n_aff && !aligned16(d_aff)) || (n_src && !aligned16(d_src)))
        return set_error(PT_ERR_INVALID, "pt_bf_accel_f32_noalloc: body buffers must be 16-byte aligned");
    int dev = 0;
    PT_CUDA(cudaGetDevice(&dev));
    unsigned char *scratch = nullptr;
    int sms = 0;
    PT_TRY(noalloc_setup(dev, &scratch, &sms));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n_aff == 0) return PT_OK;
    if (n_src == 0) {
        PT_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * n_aff, st));
        return PT_OK;
    }
    const int na = int(n_aff), ns = int(n_src);
    const float soft2 = softening * softening;
    const bool guard = checked && soft2 == 0.0f;
    pt_ctx shape;  // only carries the SM count into the planner; owns nothing
    shape.sm_count = sms;
    Plan p = plan(&shape, na, ns, guard, g_forced.k, g_forced.s);
    if (p.slices > 1) {
        // Fit the slice partials into their fixed region; one slice needs none.
        const size_t per_slice = sizeof(float4) * 2 * size_t(na);
        const int max_s = int(std::min<size_t>(NOALLOC_PART_BYTES / per_slice, 1 << 20));
        if (max_s < 2) {
            p.slices = 1;
            p.slice_len = (ns + TILE - 1) / TILE * TILE;
        } else if (p.slices > max_s) {
            const int tiles = (ns + TILE - 1) / TILE;
            const int len_tiles = (tiles + max_s - 1) / max_s;
            p.slice_len = len_tiles * TILE;
            p.slices = (ns + p.slice_len - 1) / p.slice_len;
        }
    }
    const int n_pad = (ns + TILE - 1) / TILE * TILE;
    float *soa = reinterpret_cast<float *>(scratch);
    float4 *part = p.slices > 1 ? reinterpret_cast<float4 *>(scratch + NOALLOC_SOA_BYTES) : nullptr;
    bf_to_soa<<<(n_pad + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4 *>(d_src), ns, n_pad, soa);
    PT_CUDA(cudaGetLastError());
    dim3 grid(p.n_ib, p.slices);
    fast_kernel(p.K, guard)<<<grid, THREADS, 0, st>>>(reinterpret_cast<const float4 *>(d_aff), na, soa, ns, n_pad,
                                                      soft2, p.slice_len, part, d_out);
    PT_CUDA(cudaGetLastError());
    if (part) {
        bf_fixup<<<(na + 255) / 256, 256, 0, st>>>(part, na, p.slices, d_out);
        PT_CUDA(cudaGetLastError());
    }
    return PT_OK;
}
