// Exclusive scan and stable LSD radix sort, written for the Barnes-Hut build.
//
// scan_u32: blocks of SCAN_TILE items scan in shared memory and publish their
// totals; the totals are scanned recursively and added back.
// radix_sort_u64: 8-bit digits; per digit a histogram pass (per-tile counts), a row
// scan (one block per digit value over the tiles) and a scatter pass. The scatter
// ranks keys stably inside a tile (each warp its own run of keys, with warp
// match/popc), so equal digits keep their input order, stages the tile in shared
// memory in digit order and writes every digit's run contiguously.
#include "pt_prims.cuh"

namespace pt {
namespace prims {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one tile; writes out[i] and sums[blockIdx.x] = tile total.
__global__ void __launch_bounds__(SCAN_THREADS)
    scan_tiles(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int n, uint32_t *__restrict__ sums) {
    __shared__ uint32_t tile[SCAN_TILE];
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    const size_t base = size_t(blockIdx.x) * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) {
        const size_t i = base + k;
        tile[k] = (i < size_t(n)) ? in[i] : 0u;
    }
    __syncthreads();
    uint32_t local[SCAN_ITEMS];
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        local[k] = acc;
        acc += tile[threadIdx.x * SCAN_ITEMS + k];
    }
    const uint32_t incl = warp_incl_scan(acc);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wi - w;
        if (lane == SCAN_THREADS / 32 - 1) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    const uint32_t off = warp_tot[warp] + incl - acc;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) tile[threadIdx.x * SCAN_ITEMS + k] = off + local[k];
    __syncthreads();
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) {
        const size_t i = base + k;
        if (i < size_t(n)) out[i] = tile[k];
    }
}

__global__ void scan_add(uint32_t *__restrict__ out, int n, const uint32_t *__restrict__ offs) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < size_t(n)) out[i] += offs[i / SCAN_TILE];
}

__global__ void scan_total(uint32_t *__restrict__ out, int n, const uint32_t *__restrict__ sums) {
    out[n] = sums[0];
}

// ---- radix sort ------------------------------------------------------------
constexpr int RS_THREADS = 256;
#ifndef PT_RS_ROUNDS
#define PT_RS_ROUNDS 8
#endif
constexpr int RS_ROUNDS = PT_RS_ROUNDS;  // keys per thread of a tile
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

// Exclusive scan of one value per thread over the 256 threads of a block; wsum holds
// RS_WARPS + 1 words. Every thread of the block must call it.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *wsum, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t incl = warp_incl_scan(v);
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < RS_WARPS ? wsum[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        if (lane < RS_WARPS) wsum[lane] = wi - w;
        if (lane == RS_WARPS - 1) wsum[RS_WARPS] = wi;
    }
    __syncthreads();
    const uint32_t r = wsum[warp] + incl - v;
    if (total) *total = wsum[RS_WARPS];
    __syncthreads();
    return r;
}

// hist[d * nblocks + b] = count of digit d in tile b.
__global__ void __launch_bounds__(RS_THREADS)
    rs_hist(const uint64_t *__restrict__ keys, int n, int shift, uint32_t *__restrict__ hist, int nblocks) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = size_t(blockIdx.x) * RS_TILE;
#pragma unroll 4
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const size_t i = base + size_t(r) * RS_THREADS + threadIdx.x;
        if (i < size_t(n)) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// One block per digit d: offs[d * nblocks + b] = count of digit d in tiles before b,
// rowsum[d] = count of digit d.
__global__ void __launch_bounds__(RS_THREADS)
    rs_rowscan(const uint32_t *__restrict__ hist, uint32_t *__restrict__ offs, uint32_t *__restrict__ rowsum,
               int nblocks) {
    __shared__ uint32_t wsum[RS_WARPS + 1];
    const int d = blockIdx.x;
    const uint32_t *row = hist + size_t(d) * nblocks;
    uint32_t *orow = offs + size_t(d) * nblocks;
    const int q = (nblocks + RS_THREADS - 1) / RS_THREADS;
    const int b0 = min(nblocks, int(threadIdx.x) * q), b1 = min(nblocks, b0 + q);
    uint32_t s = 0;
    for (int b = b0; b < b1; ++b) s += row[b];
    uint32_t total;
    uint32_t acc = block_excl_scan(s, wsum, &total);
    for (int b = b0; b < b1; ++b) {
        const uint32_t h = row[b];
        orow[b] = acc;
        acc += h;
    }
    if (threadIdx.x == 0) rowsum[d] = total;
}

// Ranks the tile's keys stably by digit, stages them in shared memory in digit order,
// then writes each digit's run to its global range (consecutive threads write
// consecutive addresses). Warp w owns the tile's w-th run of 32 * RS_ROUNDS keys and
// ranks them round by round with warp match/popc against its own digit counters (no
// block barrier between rounds); one scan over the warps per digit then orders the
// warps, so equal digits keep their input order.
__global__ void __launch_bounds__(RS_THREADS)
    rs_scatter(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint64_t *__restrict__ kout,
               uint32_t *__restrict__ vout, int n, int shift, const uint32_t *__restrict__ offs,
               const uint32_t *__restrict__ rowsum, int nblocks) {
    __shared__ uint64_t skeys[RS_TILE];
    __shared__ uint32_t svals[RS_TILE];
    __shared__ uint32_t wcnt[RS_WARPS][256];
    __shared__ uint32_t tstart[256], gbase[256];
    __shared__ uint32_t wsum[RS_WARPS + 1];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int b = blockIdx.x;
    // digit t's global start for this tile: all smaller digits, then earlier tiles
    gbase[t] = block_excl_scan(rowsum[t], wsum, nullptr) + offs[size_t(t) * nblocks + b];
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    const size_t wbase = size_t(b) * RS_TILE + size_t(warp) * (32 * RS_ROUNDS);
    uint64_t key[RS_ROUNDS];
    uint32_t val[RS_ROUNDS], rank[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const size_t i = wbase + size_t(r) * 32 + lane;
        const bool valid = i < size_t(n);
        key[r] = valid ? kin[i] : 0ull;
        val[r] = valid ? vin[i] : 0u;
        const uint32_t d = valid ? uint32_t((key[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        // keys of digit d in this warp's earlier rounds, then the lanes below
        const uint32_t before = valid ? wcnt[warp][d] : 0u;
        __syncwarp();
        if (valid && (peers & lt) == 0u) wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = before + __popc(peers & lt);
    }
    __syncthreads();
    // digit t: the warps' starts within the digit, then the digit's start in the tile
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
        const uint32_t c = wcnt[w][t];
        wcnt[w][t] = tot;
        tot += c;
    }
    tstart[t] = block_excl_scan(tot, wsum, nullptr);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const size_t i = wbase + size_t(r) * 32 + lane;
        if (i < size_t(n)) {
            const uint32_t d = uint32_t((key[r] >> shift) & 255u);
            const uint32_t pos = tstart[d] + wcnt[warp][d] + rank[r];
            skeys[pos] = key[r];
            svals[pos] = val[r];
        }
    }
    __syncthreads();
    const int cnt = int(min(size_t(RS_TILE), size_t(n) - size_t(b) * RS_TILE));
    for (int i = t; i < cnt; i += RS_THREADS) {
        const uint64_t k = skeys[i];
        const uint32_t d = uint32_t(k >> shift) & 255u;
        const uint32_t pos = gbase[d] + (uint32_t(i) - tstart[d]);
        kout[pos] = k;
        vout[pos] = svals[i];
    }
}

}  // namespace prims

static int scan_rec(pt_ctx *ctx, uint32_t *tmp, size_t tmp_cap, const uint32_t *in, uint32_t *out, int n) {
    using namespace prims;
    cudaStream_t st = ctx->stream;
    const int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (size_t(2 * nb) > tmp_cap) return set_error(PT_ERR_INVALID, "scan scratch too small");
    uint32_t *sums = tmp;
    uint32_t *sums_scanned = tmp + nb;
    scan_tiles<<<nb, SCAN_THREADS, 0, st>>>(in, out, n, sums);
    PT_TRY(check_launch(ctx, "scan_tiles"));
    if (nb == 1) {
        scan_total<<<1, 1, 0, st>>>(out, n, sums);
        return check_launch(ctx, "scan_total");
    }
    // sums_scanned gets nb + 1 entries: the scanned totals and the grand total.
    PT_TRY(scan_rec(ctx, tmp + 2 * nb + 1, tmp_cap - (2 * nb + 1), sums, sums_scanned, nb));
    scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, n, sums_scanned);
    PT_TRY(check_launch(ctx, "scan_add"));
    scan_total<<<1, 1, 0, st>>>(out, n, sums_scanned + nb);
    return check_launch(ctx, "scan_total");
}

static size_t scan_scratch_words(int n) {
    size_t words = 0;
    int m = n;
    do {
        const int nb = (m + prims::SCAN_TILE - 1) / prims::SCAN_TILE;
        words += 2 * size_t(nb) + 1;
        m = nb;
        if (nb == 1) break;
    } while (true);
    return words + 16;
}

int scan_u32(pt_ctx *ctx, PrimScratch &s, const uint32_t *in, uint32_t *out, int n) {
    if (n <= 0) {
        PT_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), ctx->stream));
        return PT_OK;
    }
    const size_t words = scan_scratch_words(n);
    PT_TRY(ensure_buf(ctx, s.scan, words * sizeof(uint32_t)));
    return scan_rec(ctx, static_cast<uint32_t *>(s.scan.ptr), words, in, out, n);
}

int radix_sort_u64(pt_ctx *ctx, PrimScratch &s, uint64_t *keys, uint32_t *vals, int n, int bits) {
    using namespace prims;
    if (n <= 1) return PT_OK;
    const int nblocks = (n + RS_TILE - 1) / RS_TILE;
    const size_t nhist = 256 * size_t(nblocks);
    PT_TRY(ensure_buf(ctx, s.keys2, sizeof(uint64_t) * size_t(n)));
    PT_TRY(ensure_buf(ctx, s.vals2, sizeof(uint32_t) * size_t(n)));
    PT_TRY(ensure_buf(ctx, s.hist, sizeof(uint32_t) * (2 * nhist + 256)));
    uint32_t *hist = static_cast<uint32_t *>(s.hist.ptr);
    uint32_t *offs = hist + nhist;
    uint32_t *rowsum = offs + nhist;
    uint64_t *ka = keys, *kb = static_cast<uint64_t *>(s.keys2.ptr);
    uint32_t *va = vals, *vb = static_cast<uint32_t *>(s.vals2.ptr);
    const int passes = (bits + 7) / 8;
    cudaStream_t st = ctx->stream;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        rs_hist<<<nblocks, RS_THREADS, 0, st>>>(ka, n, shift, hist, nblocks);
        PT_TRY(check_launch(ctx, "rs_hist"));
        rs_rowscan<<<256, RS_THREADS, 0, st>>>(hist, offs, rowsum, nblocks);
        PT_TRY(check_launch(ctx, "rs_rowscan"));
        rs_scatter<<<nblocks, RS_THREADS, 0, st>>>(ka, va, kb, vb, n, shift, offs, rowsum, nblocks);
        PT_TRY(check_launch(ctx, "rs_scatter"));
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        PT_CUDA(cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * size_t(n), cudaMemcpyDeviceToDevice, st));
        PT_CUDA(cudaMemcpyAsync(vals, va, sizeof(uint32_t) * size_t(n), cudaMemcpyDeviceToDevice, st));
    }
    return PT_OK;
}

void prim_free(pt_ctx *ctx, PrimScratch &s) {
    free_buf(ctx, s.scan);
    free_buf(ctx, s.hist);
    free_buf(ctx, s.keys2);
    free_buf(ctx, s.vals2);
}

}  // namespace pt
