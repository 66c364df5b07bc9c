// Batched ensembles: many independent systems of uneven size, each advanced by
// kick-drift-kick leapfrog with brute-force accelerations inside the system, all
// in ONE persistent cooperative kernel across every step.
//
// The reference evaluates one system per call (particular/src/sequential.rs:181-209);
// an ensemble is a loop of such calls there. Here one launch does
//     for each step:  [work queue] accelerations of every (system, target tile) item
//                     grid barrier
//                     kick + drift of every body
//                     grid barrier
// Items are sorted largest first (longest-processing-time order), so the queue
// balances systems of 64 ... 8192 bodies. Each item stages its system's sources in
// shared memory, in SoA form, one 256-body tile at a time, and evaluates them with
// packed f32x2 math (the brute-force inner loop), compensated across tiles.
// The item's shape -- targets per thread (K) and the number of sources staged per
// shared-memory tile (the j-tile J) -- is chosen per system size class by
// pt_ensemble_tune, which times each candidate.
// Grid barriers spin with an iteration limit: on expiry the kernel records
// PT_ERR_TIMEOUT and every block returns, leaving the context usable.
#include "pt_common.cuh"
#include "pt_f32x2.cuh"

#include <algorithm>
#include <climits>
#include <new>
#include <vector>

namespace pt {
namespace ens {

constexpr int THREADS = 128;
constexpr int TILE = 512;   // the largest j-tile: shared memory holds TILE sources
constexpr int CLASSES = 8;  // size classes by floor(log2(n)) - 6, clamped to [0, 7]

// j-tile codes in an item's word: 0 = 256 (default), 1 = 128, 2 = 512
inline int tile_code(int J) { return J == 128 ? 1 : J == 512 ? 2 : 0; }

inline int size_class(uint32_t n) {
    int c = 0;
    while ((64u << (c + 1)) <= n && c < CLASSES - 1) ++c;
    return c;
}

struct Tile {
    float c[4][TILE + 2];
};

// Accelerations of targets [s0+t0, s0+t0+cnt) from every body of the system [s0, s0+n),
// sources staged J at a time.
template <int K, int J, bool GUARD>
__device__ void accel_item(const float4 *__restrict__ body, float *__restrict__ acc, int s0, int n, int t0, int cnt,
                           float eps2, Tile &T) {
    static_assert(J <= TILE, "j-tile larger than the shared tile");
    const int tid = threadIdx.x;
    f2 xi[K], yi[K], zi[K], ax[K], ay[K], az[K];
    float sx[K], sy[K], sz[K], cx[K], cy[K], cz[K];
    const f2 e2 = pk2(eps2, eps2), zero = pk2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int t = k * THREADS + tid;
        const float4 p = (t < cnt) ? __ldcg(body + s0 + t0 + t) : make_float4(0.f, 0.f, 0.f, 0.f);
        xi[k] = pk2(p.x, p.x);
        yi[k] = pk2(p.y, p.y);
        zi[k] = pk2(p.z, p.z);
        ax[k] = ay[k] = az[k] = zero;
        sx[k] = sy[k] = sz[k] = cx[k] = cy[k] = cz[k] = 0.f;
    }
    for (int j0 = 0; j0 < n; j0 += J) {
        const int cj = min(J, n - j0);
        __syncthreads();  // the previous tile is consumed
        for (int e = tid; e < cj; e += THREADS) {
            const float4 q = __ldcg(body + s0 + j0 + e);
            T.c[0][e] = q.x;
            T.c[1][e] = q.y;
            T.c[2][e] = q.z;
            T.c[3][e] = q.w;
        }
        if ((cj & 1) && tid == 0) {  // massless pad far away: contributes exactly 0
            T.c[0][cj] = T.c[1][cj] = T.c[2][cj] = 1e30f;
            T.c[3][cj] = 0.f;
        }
        __syncthreads();
        const int c2 = (cj + 1) & ~1;
#pragma unroll 4
        for (int e = 0; e < c2; e += 2) {
            const f2 xj = *reinterpret_cast<const f2 *>(&T.c[0][e]);
            const f2 yj = *reinterpret_cast<const f2 *>(&T.c[1][e]);
            const f2 zj = *reinterpret_cast<const f2 *>(&T.c[2][e]);
            const f2 mj = *reinterpret_cast<const f2 *>(&T.c[3][e]);
#pragma unroll
            for (int k = 0; k < K; ++k) interact2<GUARD>(xj, yj, zj, mj, xi[k], yi[k], zi[k], ax[k], ay[k], az[k], e2);
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
            ax[k] = ay[k] = az[k] = zero;
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int t = k * THREADS + tid;
        if (t < cnt) {
            const size_t i = size_t(s0 + t0 + t);
            acc[3 * i + 0] = sx[k] + cx[k];
            acc[3 * i + 1] = sy[k] + cy[k];
            acc[3 * i + 2] = sz[k] + cz[k];
        }
    }
}

template <int K, bool GUARD>
__device__ __forceinline__ void run_item_k(int jc, const int4 w, int cnt, const float4 *__restrict__ body,
                                           float *__restrict__ acc, float eps2, Tile &T) {
    if (jc == 1) accel_item<K, 128, GUARD>(body, acc, w.x, w.y, w.z, cnt, eps2, T);
    else if (jc == 2) accel_item<K, 512, GUARD>(body, acc, w.x, w.y, w.z, cnt, eps2, T);
    else accel_item<K, 256, GUARD>(body, acc, w.x, w.y, w.z, cnt, eps2, T);
}

// item word w = (system start, system size, first target, cnt | K << 24 | j-tile code << 28)
template <bool GUARD>
__device__ __forceinline__ void run_item(const int4 w, const float4 *__restrict__ body, float *__restrict__ acc,
                                         float eps2, Tile &T) {
    const int K = (w.w >> 24) & 7, jc = (w.w >> 28) & 3, cnt = w.w & 0xffffff;
    if (K == 4) run_item_k<4, GUARD>(jc, w, cnt, body, acc, eps2, T);
    else if (K == 2) run_item_k<2, GUARD>(jc, w, cnt, body, acc, eps2, T);
    else run_item_k<1, GUARD>(jc, w, cnt, body, acc, eps2, T);
}

// ctrl: [0] barrier arrivals, [1] barrier generation, [2 + p] queue of phase p.
// Returns false (in every thread) once any block has recorded an error.
__device__ bool grid_sync(unsigned *ctrl, int *err, long long spin_limit, unsigned expected) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = ctrl + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(ctrl, 1u) == expected - 1) {
            atomicExch(ctrl, 0u);
            __threadfence();
            atomicAdd(ctrl + 1, 1u);
        } else {
            long long it = 0;
            while (*gen == g) {
                if (++it > spin_limit || *reinterpret_cast<volatile int *>(err)) {
                    atomicCAS(err, 0, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = *reinterpret_cast<volatile int *>(err) == 0;
    }
    __syncthreads();
    return s_ok;
}

template <bool GUARD>
__global__ void __launch_bounds__(THREADS)
    ens_persistent(const int4 *__restrict__ items, int n_items, float4 *body, float4 *vel, float *acc, int n_bodies,
                   int steps, float dt, float eps2, unsigned *ctrl, int *err, long long spin_limit, int stall) {
    __shared__ __align__(16) Tile T;
    __shared__ int s_item;
    const unsigned expected = gridDim.x + (stall ? 1u : 0u);  // stall: a barrier nothing completes
    for (int phase = 0; phase <= steps; ++phase) {
        for (;;) {
            if (threadIdx.x == 0) s_item = int(atomicAdd(ctrl + 2 + phase, 1u));
            __syncthreads();
            const int it = s_item;
            __syncthreads();
            if (it >= n_items) break;
            run_item<GUARD>(items[it], body, acc, eps2, T);
        }
        if (!grid_sync(ctrl, err, spin_limit, expected)) return;
        const float kick = (phase == 0 || phase == steps) ? 0.5f * dt : dt;
        for (int i = blockIdx.x * THREADS + threadIdx.x; i < n_bodies; i += gridDim.x * THREADS) {
            float4 v = __ldcg(vel + i);
            v.x = fmaf(__ldcg(acc + 3 * size_t(i)), kick, v.x);
            v.y = fmaf(__ldcg(acc + 3 * size_t(i) + 1), kick, v.y);
            v.z = fmaf(__ldcg(acc + 3 * size_t(i) + 2), kick, v.z);
            vel[i] = v;
            if (phase < steps) {
                float4 x = __ldcg(body + i);
                x.x = fmaf(v.x, dt, x.x);
                x.y = fmaf(v.y, dt, x.y);
                x.z = fmaf(v.z, dt, x.z);
                body[i] = x;
            }
        }
        if (phase < steps && !grid_sync(ctrl, err, spin_limit, expected)) return;
    }
}

// One acceleration pass over a list of items (no barrier): the autotuner's probe.
template <bool GUARD>
__global__ void __launch_bounds__(THREADS)
    ens_accel_once(const int4 *__restrict__ items, int n_items, const float4 *__restrict__ body,
                   float *__restrict__ acc, float eps2) {
    __shared__ __align__(16) Tile T;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) run_item<GUARD>(items[it], body, acc, eps2, T);
}

struct State {
    int table[CLASSES] = {0, 0, 0, 0, 0, 0, 0, 0};  // K per size class (0 = default)
    int tiles[CLASSES] = {0, 0, 0, 0, 0, 0, 0, 0};  // j-tile per size class (0 = default 256)
    long long spin_limit = 1ll << 22;
    int stall = 0;
    DevBuf items, ctrl, acc;
    std::vector<int4> host_items;
    std::vector<uint32_t> key;  // offsets + table the items were built for
    int n_items = 0;
    // graph of the last (items, pointers, steps, dt, eps) launch
    cudaGraphExec_t exec = nullptr;
    const void *g_body = nullptr, *g_vel = nullptr;
    int g_steps = 0;
    float g_dt = 0.f, g_eps = 0.f;
    unsigned long long g_epoch = 0;  // the context's buffer addresses it captured
    uint64_t g_kernels = 0;
};

static State *state(pt_ctx *ctx) {
    if (!ctx->ens) ctx->ens = new (std::nothrow) State();
    return static_cast<State *>(ctx->ens);
}

static int default_k(int cls) { return cls >= 5 ? 2 : 1; }  // >= 2048 bodies: 2 targets per thread

// Items sorted by cost (targets x sources), largest first.
static void build_items(const uint32_t *offsets, uint32_t n_sys, const int *table, const int *tiles,
                        std::vector<int4> &out) {
    struct Cost {
        int4 w;
        double c;
    };
    std::vector<Cost> v;
    for (uint32_t k = 0; k < n_sys; ++k) {
        const int s0 = int(offsets[k]), n = int(offsets[k + 1] - offsets[k]);
        if (n <= 0) continue;
        const int cls = size_class(uint32_t(n));
        const int K = table[cls] ? table[cls] : default_k(cls);
        const int jc = tile_code(tiles[cls]);
        const int per = THREADS * K;
        for (int t0 = 0; t0 < n; t0 += per) {
            const int cnt = std::min(per, n - t0);
            v.push_back({make_int4(s0, n, t0, cnt | (K << 24) | (jc << 28)), double(cnt) * n});
        }
    }
    std::stable_sort(v.begin(), v.end(), [](const Cost &a, const Cost &b) { return a.c > b.c; });
    out.resize(v.size());
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i].w;
}

static int upload_items(pt_ctx *ctx, State &S, const uint32_t *offsets, uint32_t n_sys) {
    std::vector<uint32_t> key(offsets, offsets + n_sys + 1);
    key.insert(key.end(), S.table, S.table + CLASSES);
    key.insert(key.end(), S.tiles, S.tiles + CLASSES);
    if (key == S.key && S.items.ptr) return PT_OK;
    build_items(offsets, n_sys, S.table, S.tiles, S.host_items);
    S.n_items = int(S.host_items.size());
    PT_TRY(ensure_buf(ctx, S.items, sizeof(int4) * std::max<size_t>(1, S.host_items.size())));
    PT_CUDA(cudaMemcpyAsync(S.items.ptr, S.host_items.data(), sizeof(int4) * S.host_items.size(),
                            cudaMemcpyHostToDevice, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    S.key.swap(key);
    if (S.exec) {
        cudaGraphExecDestroy(S.exec);
        S.exec = nullptr;
    }
    return PT_OK;
}

static int validate(const char *fn, const uint32_t *offsets, uint32_t n_sys) {
    if (!offsets) return set_error(PT_ERR_INVALID, "%s: offsets is NULL", fn);
    if (offsets[0] != 0) return set_error(PT_ERR_INVALID, "%s: offsets[0] must be 0", fn);
    for (uint32_t k = 0; k < n_sys; ++k)
        if (offsets[k + 1] < offsets[k]) return set_error(PT_ERR_INVALID, "%s: offsets must not decrease", fn);
    if (offsets[n_sys] > uint32_t(INT_MAX / 8)) return set_error(PT_ERR_INVALID, "%s: too many bodies", fn);
    return PT_OK;
}

using PersistentKernel = void (*)(const int4 *, int, float4 *, float4 *, float *, int, int, float, float,
                                  unsigned *, int *, long long, int);

static int launch(pt_ctx *ctx, State &S, float4 *body, float4 *vel, int n_bodies, int steps, float dt,
                  float eps2) {
    const bool guard = eps2 == 0.0f;
    PersistentKernel kern = guard ? ens_persistent<true> : ens_persistent<false>;
    int occ = 0;
    PT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, 0));
    if (occ < 1) return set_error(PT_ERR_CUDA, "ensemble kernel does not fit on an SM");
    int grid = std::max(1, std::min(occ * ctx->sm_count, std::max(S.n_items, 1)));
    PT_CUDA(cudaMemsetAsync(S.ctrl.ptr, 0, sizeof(unsigned) * size_t(steps + 3) + 16, ctx->stream));
    const int4 *items = static_cast<const int4 *>(S.items.ptr);
    float *acc = static_cast<float *>(S.acc.ptr);
    unsigned *ctrl = static_cast<unsigned *>(S.ctrl.ptr);
    int *err = reinterpret_cast<int *>(static_cast<char *>(S.ctrl.ptr) + sizeof(unsigned) * size_t(steps + 3));
    int n_items = S.n_items;
    long long spin = S.spin_limit;
    int stall = S.stall;
    void *args[] = {&items, &n_items, &body, &vel, &acc, &n_bodies, &steps, &dt, &eps2, &ctrl, &err, &spin, &stall};
    PT_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void *>(kern), dim3(grid), dim3(THREADS), args, 0,
                                        ctx->stream));
    return check_launch(ctx, "ens_persistent");
}

}  // namespace ens
}  // namespace pt

void pt_ens_state_free(pt_ctx *ctx) {
    auto *S = static_cast<pt::ens::State *>(ctx->ens);
    if (!S) return;
    if (S->exec) cudaGraphExecDestroy(S->exec);
    pt::free_buf(ctx, S->items);
    pt::free_buf(ctx, S->ctrl);
    pt::free_buf(ctx, S->acc);
    delete S;
    ctx->ens = nullptr;
}

extern "C" int pt_ensemble_run(pt_ctx *ctx, const uint32_t *offsets, uint32_t n_sys, float *d_bodies,
                               float *d_vel, float dt, int steps, float softening, int use_graph) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_ensemble_run: ctx is NULL");
    if (n_sys == 0 || steps <= 0) return PT_OK;
    PT_TRY(ens::validate("pt_ensemble_run", offsets, n_sys));
    if (!d_bodies || !d_vel) return set_error(PT_ERR_INVALID, "pt_ensemble_run: NULL buffer");
    if (!aligned16(d_bodies) || !aligned16(d_vel))
        return set_error(PT_ERR_INVALID, "pt_ensemble_run: bodies and velocities must be 16-byte aligned");
    if (steps > (1 << 20)) return set_error(PT_ERR_INVALID, "pt_ensemble_run: steps=%d too large", steps);
    PT_CUDA(cudaSetDevice(ctx->device));
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    const int n = int(offsets[n_sys]);
    if (n == 0) return PT_OK;
    PT_TRY(ens::upload_items(ctx, *S, offsets, n_sys));
    PT_TRY(ensure_buf(ctx, S->acc, 12 * size_t(n)));
    PT_TRY(ensure_buf(ctx, S->ctrl, sizeof(unsigned) * size_t(steps + 3) + 16));
    float4 *body = reinterpret_cast<float4 *>(d_bodies);
    float4 *vel = reinterpret_cast<float4 *>(d_vel);
    const float eps2 = softening * softening;
    int *err = reinterpret_cast<int *>(static_cast<char *>(S->ctrl.ptr) + sizeof(unsigned) * size_t(steps + 3));
    if (!use_graph) {
        PT_TRY(ens::launch(ctx, *S, body, vel, n, steps, dt, eps2));
    } else {
        if (!(S->exec && S->g_body == d_bodies && S->g_vel == d_vel && S->g_steps == steps && S->g_dt == dt &&
              S->g_eps == softening && S->g_epoch == ctx->buf_epoch)) {
            if (S->exec) {
                cudaGraphExecDestroy(S->exec);
                S->exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            PT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            ctx->capturing = true;
            const uint64_t before = ctx->launches;
            const int rc = ens::launch(ctx, *S, body, vel, n, steps, dt, eps2);
            S->g_kernels = ctx->launches - before;
            ctx->launches = before;
            ctx->capturing = false;
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
            if (rc != PT_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            PT_CUDA(ce);
            const cudaError_t ie = cudaGraphInstantiate(&S->exec, g, 0);
            cudaGraphDestroy(g);
            PT_CUDA(ie);
            S->g_body = d_bodies;
            S->g_vel = d_vel;
            S->g_steps = steps;
            S->g_dt = dt;
            S->g_eps = softening;
            S->g_epoch = ctx->buf_epoch;
        }
        PT_CUDA(cudaGraphLaunch(S->exec, ctx->stream));
        ctx->launches += S->g_kernels;
    }
    // Report a barrier timeout: the step loop is synchronous with its error word.
    int h_err = 0;
    PT_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h_err)
        return set_error(PT_ERR_TIMEOUT, "pt_ensemble_run: a grid barrier gave up after %lld spins; "
                                         "the state is partially advanced", S->spin_limit);
    return PT_OK;
}

// Times every (K, J) in {1, 2, 4} x {128, 256, 512} for every size class present and
// keeps the fastest.
extern "C" int pt_ensemble_tune(pt_ctx *ctx, const uint32_t *offsets, uint32_t n_sys, const float *d_bodies,
                                float softening, int *table_out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_ensemble_tune: ctx is NULL");
    if (n_sys == 0) return PT_OK;
    PT_TRY(ens::validate("pt_ensemble_tune", offsets, n_sys));
    if (!d_bodies || !aligned16(d_bodies))
        return set_error(PT_ERR_INVALID, "pt_ensemble_tune: bodies must be a 16-byte aligned device buffer");
    PT_CUDA(cudaSetDevice(ctx->device));
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    const int n = int(offsets[n_sys]);
    PT_TRY(ensure_buf(ctx, S->acc, 12 * size_t(std::max(n, 1))));
    const float eps2 = softening * softening;
    auto kern = eps2 == 0.0f ? ens::ens_accel_once<true> : ens::ens_accel_once<false>;
    cudaEvent_t e0, e1;
    PT_CUDA(cudaEventCreate(&e0));
    PT_CUDA(cudaEventCreate(&e1));
    int best_table[ens::CLASSES], best_tiles[ens::CLASSES];
    for (int c = 0; c < ens::CLASSES; ++c) {
        std::vector<uint32_t> sub(1, 0);  // the systems of class c, packed as a sub-ensemble
        std::vector<uint32_t> start;
        for (uint32_t k = 0; k < n_sys; ++k) {
            const uint32_t len = offsets[k + 1] - offsets[k];
            if (len && ens::size_class(len) == c) {
                start.push_back(offsets[k]);
                sub.push_back(sub.back() + len);
            }
        }
        best_table[c] = S->table[c];
        best_tiles[c] = S->tiles[c];
        if (start.empty()) continue;
        float best = 1e30f;
        for (int shape = 0; shape < 9; ++shape) {
            const int K = 1 << (shape / 3), J = 128 << (shape % 3);
            int tab[ens::CLASSES] = {K, K, K, K, K, K, K, K};
            int til[ens::CLASSES] = {J, J, J, J, J, J, J, J};
            std::vector<int4> items;
            ens::build_items(sub.data(), uint32_t(start.size()), tab, til, items);
            // map sub-ensemble item starts back to the real system starts
            for (auto &w : items) {
                const auto it = std::upper_bound(sub.begin(), sub.end(), uint32_t(w.x)) - 1;
                w.x = int(start[size_t(it - sub.begin())]);
            }
            PT_TRY(ensure_buf(ctx, S->items, sizeof(int4) * items.size()));
            S->key.clear();  // the item buffer no longer holds a run's items
            PT_CUDA(cudaMemcpyAsync(S->items.ptr, items.data(), sizeof(int4) * items.size(),
                                    cudaMemcpyHostToDevice, ctx->stream));
            const int grid = std::min<int>(int(items.size()), 8 * ctx->sm_count);
            float ms = 0.f;
            for (int rep = 0; rep < 2; ++rep) {  // first run warms up
                cudaEventRecord(e0, ctx->stream);
                kern<<<grid, ens::THREADS, 0, ctx->stream>>>(static_cast<const int4 *>(S->items.ptr),
                                                            int(items.size()),
                                                            reinterpret_cast<const float4 *>(d_bodies),
                                                            static_cast<float *>(S->acc.ptr), eps2);
                PT_TRY(check_launch(ctx, "ens_accel_once"));
                cudaEventRecord(e1, ctx->stream);
                PT_CUDA(cudaEventSynchronize(e1));
                PT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            }
            if (ms < best) {
                best = ms;
                best_table[c] = K;
                best_tiles[c] = J;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::copy(best_table, best_table + ens::CLASSES, S->table);
    std::copy(best_tiles, best_tiles + ens::CLASSES, S->tiles);
    if (S->exec) {
        cudaGraphExecDestroy(S->exec);
        S->exec = nullptr;
    }
    if (table_out) std::copy(best_table, best_table + ens::CLASSES, table_out);
    return PT_OK;
}

extern "C" int pt_ensemble_set_table(pt_ctx *ctx, const int *table) {
    using namespace pt;
    clear_error();
    if (!ctx || !table) return set_error(PT_ERR_INVALID, "pt_ensemble_set_table: NULL argument");
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    for (int c = 0; c < ens::CLASSES; ++c)
        if (table[c] != 0 && table[c] != 1 && table[c] != 2 && table[c] != 4)
            return set_error(PT_ERR_INVALID, "pt_ensemble_set_table: K must be 0, 1, 2 or 4");
    std::copy(table, table + ens::CLASSES, S->table);
    S->key.clear();
    return PT_OK;
}

extern "C" int pt_ensemble_set_barrier(pt_ctx *ctx, long long spin_limit, int stall) {
    using namespace pt;
    clear_error();
    if (!ctx || spin_limit <= 0) return set_error(PT_ERR_INVALID, "pt_ensemble_set_barrier: bad argument");
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    S->spin_limit = spin_limit;
    S->stall = stall ? 1 : 0;
    if (S->exec) {
        cudaGraphExecDestroy(S->exec);
        S->exec = nullptr;
    }
    return PT_OK;
}

extern "C" int pt_ensemble_set_tiles(pt_ctx *ctx, const int *tiles) {
    using namespace pt;
    clear_error();
    if (!ctx || !tiles) return set_error(PT_ERR_INVALID, "pt_ensemble_set_tiles: NULL argument");
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    for (int c = 0; c < ens::CLASSES; ++c)
        if (tiles[c] != 0 && tiles[c] != 128 && tiles[c] != 256 && tiles[c] != 512)
            return set_error(PT_ERR_INVALID, "pt_ensemble_set_tiles: the j-tile must be 0, 128, 256 or 512");
    std::copy(tiles, tiles + ens::CLASSES, S->tiles);
    S->key.clear();
    return PT_OK;
}

extern "C" int pt_ensemble_get_shape(pt_ctx *ctx, int *table, int *tiles) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_ensemble_get_shape: ctx is NULL");
    ens::State *S = ens::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "ensemble state allocation failed");
    for (int c = 0; c < ens::CLASSES; ++c) {
        if (table) table[c] = S->table[c] ? S->table[c] : ens::default_k(c);
        if (tiles) tiles[c] = S->tiles[c] ? S->tiles[c] : 256;
    }
    return PT_OK;
}
