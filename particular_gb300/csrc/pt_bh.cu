// cuda::BarnesHut: the C ABI (include/particular_cuda.h) over the build
// (pt_bh_build.cu) and the walks (pt_bh_walk.cu), the tree export, tree reuse and the
// per-context state.
#include "pt_bh.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

namespace pt {
namespace bh {

int validate(const char *fn, size_t n_aff, size_t n_src, uint32_t flags) {
    const size_t lim = size_t(INT_MAX) / 8;
    if (n_aff > lim || n_src > lim)
        return set_error(PT_ERR_INVALID, "%s: n_aff=%zu n_src=%zu exceed the limit %zu", fn, n_aff, n_src, lim);
    if (flags & ~(PT_BH_QUADRUPOLE | PT_BH_GROUP | PT_BH_LEARNED | PT_BH_LOCAL | PT_BH_RELATIVE))
        return set_error(PT_ERR_INVALID, "%s: unknown flags 0x%x", fn, flags);
    if ((flags & PT_BH_LEARNED) && !(flags & PT_BH_GROUP))
        return set_error(PT_ERR_INVALID, "%s: PT_BH_LEARNED requires PT_BH_GROUP", fn);
    if ((flags & PT_BH_LOCAL) && !(flags & PT_BH_GROUP))
        return set_error(PT_ERR_INVALID, "%s: PT_BH_LOCAL requires PT_BH_GROUP", fn);
    if ((flags & PT_BH_LOCAL) && (flags & PT_BH_LEARNED))
        return set_error(PT_ERR_INVALID, "%s: PT_BH_LOCAL and PT_BH_LEARNED are exclusive", fn);
    if ((flags & PT_BH_RELATIVE) && !(flags & PT_BH_GROUP))
        return set_error(PT_ERR_INVALID, "%s: PT_BH_RELATIVE requires PT_BH_GROUP", fn);
    if ((flags & PT_BH_RELATIVE) && (flags & PT_BH_LEARNED))
        return set_error(PT_ERR_INVALID, "%s: PT_BH_RELATIVE and PT_BH_LEARNED are exclusive", fn);
    return PT_OK;
}

}  // namespace bh
}  // namespace pt

namespace pt {

// The Barnes-Hut settings that captured launches carry as parameters (local ratio,
// error-bound factor, learned inner angle, stack cap, model weights): a CUDA graph
// captured under other values has to be captured again.
BhTuning bh_tuning(pt_ctx *ctx) {
    BhTuning t{};
    const auto *S = static_cast<const bh::State *>(ctx->bh);
    if (S) {
        t.local_ratio = S->local_ratio;
        t.rel_alpha = S->rel_alpha;
        t.theta_inner = S->theta_inner;
        t.stack_cap = S->stack_cap;
        t.learned_cap = S->lcap_fixed;
        t.mlp = S->mlp_w;
    }
    return t;
}

int *bh_error_word(pt_ctx *ctx) {
    auto *S = static_cast<bh::State *>(ctx->bh);
    return (S && S->counters.ptr) ? static_cast<int *>(S->counters.ptr) + 3 : nullptr;
}

int bh_learned_overflow(pt_ctx *ctx, const char *fn) {
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || !S->counters.ptr) return PT_OK;
    int err = 0, used = 0;
    PT_CUDA(cudaMemcpyAsync(&err, static_cast<int *>(S->counters.ptr) + 3, sizeof(int), cudaMemcpyDeviceToHost,
                            ctx->stream));
    if (S->lused.ptr)
        PT_CUDA(cudaMemcpyAsync(&used, S->lused.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!(err & 2)) return PT_OK;
    if (S->lcap_fixed == 0 && used > S->lcap) S->lcap = used + used / 4;
    return set_error(PT_ERR_CAPACITY,
                     "%s: learned-correction records overflowed (%d chunks needed, %d available); the state "
                     "advanced without the corrections that did not fit",
                     fn, used, S->lcap_fixed ? S->lcap_fixed : S->lcap);
}

int bh_build_only(pt_ctx *ctx, const float4 *d_src, int n) {
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    return bh::build(ctx, *S, d_src, n);
}

int bh_tree_view(pt_ctx *ctx, TreeView *out) {
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || !S->nodeA.ptr) return set_error(PT_ERR_INVALID, "no Barnes-Hut tree built yet");
    if (S->f64) return set_error(PT_ERR_INVALID, "the current tree holds DVec3 bodies");
    out->nodeA = static_cast<const float4 *>(S->nodeA.ptr);
    out->nodeB = static_cast<const int4 *>(S->nodeB.ptr);
    out->nodeQ = static_cast<const float4 *>(S->nodeQ.ptr);
    out->nodeG = static_cast<const float4 *>(S->nodeG.ptr);
    out->nodeR = static_cast<const int2 *>(S->nodeR.ptr);
    out->sbody = static_cast<const float4 *>(S->sbody.ptr);
    out->counters = static_cast<const int *>(S->counters.ptr);
    out->n_src = S->last_n_src;
    return PT_OK;
}

int bh_set_mlp(pt_ctx *ctx, const uint32_t *d_tc_weights, const float *d_tc_bias, float theta_inner) {
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->mlp_w = d_tc_weights;
    S->mlp_b = d_tc_bias;
    S->theta_inner = theta_inner;
    return PT_OK;
}

}  // namespace pt

void pt_bh_state_free(pt_ctx *ctx) {
    using namespace pt;
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S) return;
    prim_free(ctx, S->prims);
    DevBuf *all[] = {&S->box_part, &S->box,    &S->keys,   &S->idx,    &S->sbody,   &S->flags,  &S->uscan,
                     &S->ukey,     &S->ufirst, &S->bfirst, &S->blast,  &S->bdelta,  &S->bparent, &S->lparent,
                     &S->top,      &S->oparent, &S->loparent, &S->cnt, &S->pscan,   &S->pre,    &S->nkid, &S->kid, &S->cslot, &S->lslot, &S->levels, &S->by_level,
                     &S->nodeA,  &S->nodeB,  &S->nodeQ,  &S->nodeG, &S->nodeR, &S->mom,     &S->tkeys,  &S->tidx,
                     &S->tbody,    &S->counters, &S->out,  &S->aff_h,  &S->src_h, &S->lrec, &S->lgroup,
                     &S->lnext,    &S->lpart,  &S->lhead, &S->lcentre, &S->lused, &S->sbody64, &S->nodeA64,
                     &S->nodeG64,  &S->tbody64, &S->gscale};
    for (DevBuf *b : all) free_buf(ctx, *b);
    if (S->fork) cudaEventDestroy(S->fork);
    if (S->join) cudaEventDestroy(S->join);
    if (S->aux) cudaStreamDestroy(S->aux);
    delete S;
    ctx->bh = nullptr;
}

extern "C" {

int pt_bh_accel_f32_device(pt_ctx *ctx, const float *d_aff, size_t n_aff, const float *d_src, size_t n_src,
                           float theta, float softening, uint32_t flags, float *d_out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32_device: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_accel_f32_device", n_aff, n_src, flags));
    if (n_aff && (!d_aff || !d_out)) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32_device: NULL buffer");
    if (n_src && !d_src) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32_device: NULL affecting buffer");
    if ((n_aff && !aligned16(d_aff)) || (n_src && !aligned16(d_src)))
        return set_error(PT_ERR_INVALID, "pt_bh_accel_f32_device: body buffers must be 16-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    return bh::run(ctx, reinterpret_cast<const float4 *>(d_aff), int(n_aff), reinterpret_cast<const float4 *>(d_src),
                   int(n_src), theta, softening, flags, d_out);
}

int pt_bh_accel_f32(pt_ctx *ctx, const float *aff, size_t n_aff, const float *src, size_t n_src, float theta,
                    float softening, uint32_t flags, float *out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_accel_f32", n_aff, n_src, flags));
    if (n_aff && (!aff || !out)) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32: NULL buffer");
    if (n_src && !src) return set_error(PT_ERR_INVALID, "pt_bh_accel_f32: NULL affecting buffer");
    if (n_aff == 0) return PT_OK;
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    const bool same = (aff == src) && (n_aff == n_src);
    PT_TRY(ensure_buf(ctx, S->aff_h, 16 * n_aff));
    if (!same && n_src) PT_TRY(ensure_buf(ctx, S->src_h, 16 * n_src));
    PT_TRY(ensure_buf(ctx, S->out, 12 * n_aff));
    float *d_aff = static_cast<float *>(S->aff_h.ptr);
    float *d_src = same ? d_aff : static_cast<float *>(S->src_h.ptr);
    float *d_out = static_cast<float *>(S->out.ptr);
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(d_aff, aff, 16 * n_aff, cudaMemcpyHostToDevice, st));
    if (!same && n_src) PT_CUDA(cudaMemcpyAsync(d_src, src, 16 * n_src, cudaMemcpyHostToDevice, st));
    PT_TRY(bh::run(ctx, reinterpret_cast<const float4 *>(d_aff), int(n_aff), reinterpret_cast<const float4 *>(d_src),
                   int(n_src), theta, softening, flags, d_out));
    PT_CUDA(cudaMemcpyAsync(out, d_out, 12 * n_aff, cudaMemcpyDeviceToHost, st));
    int err = 0;
    if (n_src) PT_CUDA(cudaMemcpyAsync(&err, static_cast<int *>(S->counters.ptr) + 3, sizeof(int),
                                       cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (err & 2)
        return set_error(PT_ERR_CAPACITY, "pt_bh_accel_f32: learned-correction records overflowed");
    return PT_OK;
}

int pt_bh_accel_dvec3_device(pt_ctx *ctx, const double *d_aff, size_t n_aff, const double *d_src, size_t n_src,
                             double theta, double softening, uint32_t flags, double *d_out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3_device: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_accel_dvec3_device", n_aff, n_src, 0));
    if (flags) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3_device: the f64 method takes no flags");
    if (n_aff && (!d_aff || !d_out)) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3_device: NULL buffer");
    if (n_src && !d_src) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3_device: NULL affecting buffer");
    if ((n_aff && reinterpret_cast<uintptr_t>(d_aff) % 32) || (n_src && reinterpret_cast<uintptr_t>(d_src) % 32))
        return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3_device: body buffers must be 32-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    return bh::run64(ctx, reinterpret_cast<const double4_32a *>(d_aff), int(n_aff),
                     reinterpret_cast<const double4_32a *>(d_src), int(n_src), theta, softening, d_out);
}

int pt_bh_accel_dvec3(pt_ctx *ctx, const double *aff, size_t n_aff, const double *src, size_t n_src, double theta,
                      double softening, uint32_t flags, double *out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_accel_dvec3", n_aff, n_src, 0));
    if (flags) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3: the f64 method takes no flags");
    if (n_aff && (!aff || !out)) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3: NULL buffer");
    if (n_src && !src) return set_error(PT_ERR_INVALID, "pt_bh_accel_dvec3: NULL affecting buffer");
    if (n_aff == 0) return PT_OK;
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    const bool same = (aff == src) && (n_aff == n_src);
    PT_TRY(ensure_buf(ctx, S->aff_h, 32 * n_aff));
    if (!same && n_src) PT_TRY(ensure_buf(ctx, S->src_h, 32 * n_src));
    PT_TRY(ensure_buf(ctx, S->out, 24 * n_aff));
    double *d_aff = static_cast<double *>(S->aff_h.ptr);
    double *d_src = same ? d_aff : static_cast<double *>(S->src_h.ptr);
    double *d_out = static_cast<double *>(S->out.ptr);
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(d_aff, aff, 32 * n_aff, cudaMemcpyHostToDevice, st));
    if (!same && n_src) PT_CUDA(cudaMemcpyAsync(d_src, src, 32 * n_src, cudaMemcpyHostToDevice, st));
    PT_TRY(bh::run64(ctx, reinterpret_cast<const double4_32a *>(d_aff), int(n_aff),
                     reinterpret_cast<const double4_32a *>(d_src), int(n_src), theta, softening, d_out));
    PT_CUDA(cudaMemcpyAsync(out, d_out, 24 * n_aff, cudaMemcpyDeviceToHost, st));
    int err = 0;
    if (n_src) PT_CUDA(cudaMemcpyAsync(&err, static_cast<int *>(S->counters.ptr) + 3, sizeof(int),
                                       cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (err & 1) return set_error(PT_ERR_CAPACITY, "pt_bh_accel_dvec3: a warp's stack ran out; its bodies are NaN");
    return PT_OK;
}

int pt_bh_build_device(pt_ctx *ctx, const float *d_src, size_t n_src, uint64_t *generation) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_build_device: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_build_device", 0, n_src, 0));
    if (n_src && !d_src) return set_error(PT_ERR_INVALID, "pt_bh_build_device: NULL affecting buffer");
    if (n_src && !aligned16(d_src))
        return set_error(PT_ERR_INVALID, "pt_bh_build_device: body buffer must be 16-byte aligned");
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    if (n_src == 0) {
        S->last_n_src = 0;
        ++S->generation;
    } else {
        mark(ctx, 0);
        PT_TRY(bh::build(ctx, *S, reinterpret_cast<const float4 *>(d_src), int(n_src)));
    }
    if (generation) *generation = S->generation;
    return PT_OK;
}

int pt_bh_walk_device(pt_ctx *ctx, const float *d_aff, size_t n_aff, float theta, float softening, uint32_t flags,
                      float *d_out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_walk_device: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_walk_device", n_aff, 0, flags));
    if (n_aff && (!d_aff || !d_out)) return set_error(PT_ERR_INVALID, "pt_bh_walk_device: NULL buffer");
    if (n_aff && !aligned16(d_aff))
        return set_error(PT_ERR_INVALID, "pt_bh_walk_device: body buffer must be 16-byte aligned");
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || S->generation == 0)
        return set_error(PT_ERR_INVALID, "pt_bh_walk_device: no tree (call pt_bh_build_device first)");
    PT_CUDA(cudaSetDevice(ctx->device));
    if (n_aff == 0) return PT_OK;
    if (S->last_n_src == 0) {
        PT_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * n_aff, ctx->stream));
        return PT_OK;
    }
    if (S->user_tree && (flags & ~uint32_t(PT_BH_GROUP)))
        return set_error(PT_ERR_INVALID,
                         "pt_bh_walk_device: a caller-built tree carries monopoles only (flags 0 or PT_BH_GROUP)");
    mark(ctx, 0);
    PT_TRY(bh::sort_targets(ctx, *S, reinterpret_cast<const float4 *>(d_aff), int(n_aff)));
    return bh::walk(ctx, *S, bh::as<float4>(S->tbody), bh::as<uint32_t>(S->tidx), int(n_aff), theta, softening,
                    flags, d_out);
}

// A tree the caller built, in the layout of the reference's RootedOrthtree over
// GravitationalField<Vec3, f32> (tree/mod.rs:13-60, storage.rs:10-46): per node its
// eight orthant slots (Option<NodeID>, -1 = None), its bounding box (min, max), whether
// it is Node::Internal, and its data (centre of mass, mass). It is flattened on the
// host into the walk's layout: depth-first preorder in the reference's visiting order
// (sequential.rs:470-505 pushes orthants 0..7 and pops 7..0, so children follow in
// the order 7..0), skip pointers, widths BoundingBox::width() = max.x - min.x in f32.
// External nodes become single-body leaves holding their data. Nothing is collapsed
// or recomputed: the walk accepts, for every body, exactly the nodes the reference's
// walk of this tree accepts.
int pt_bh_load_tree(pt_ctx *ctx, const int32_t *orthant, const float *bbox, const uint8_t *internal,
                    const float *data, size_t n_nodes, int64_t root, uint64_t *generation) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_load_tree: ctx is NULL");
    if (n_nodes > size_t(INT_MAX / 8)) return set_error(PT_ERR_INVALID, "pt_bh_load_tree: %zu nodes", n_nodes);
    if (root < -1 || root >= int64_t(n_nodes))
        return set_error(PT_ERR_INVALID, "pt_bh_load_tree: root %lld outside [-1, %zu)", (long long)root, n_nodes);
    if (n_nodes && (!orthant || !bbox || !internal || !data))
        return set_error(PT_ERR_INVALID, "pt_bh_load_tree: NULL array");
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    std::vector<float4> A, leaves;
    std::vector<int4> B;
    std::vector<uint8_t> seen(n_nodes, 0);
    int cells = 0;
    float box[8] = {-1.f, -1.f, -1.f, 1.f, 1.f, 1.f, 0.f, 0.f};
    if (root >= 0) {
        // stack entries: a node to open (>= 0) or ~k, the end of preorder node k's subtree
        std::vector<int64_t> st{root};
        while (!st.empty()) {
            const int64_t x = st.back();
            st.pop_back();
            if (x < 0) {
                B[size_t(~x)].y = int(A.size());
                continue;
            }
            if (x >= int64_t(n_nodes))
                return set_error(PT_ERR_INVALID, "pt_bh_load_tree: orthant slot names node %lld of %zu",
                                 (long long)x, n_nodes);
            if (seen[size_t(x)])
                return set_error(PT_ERR_INVALID, "pt_bh_load_tree: node %lld is reachable twice (not a tree)",
                                 (long long)x);
            seen[size_t(x)] = 1;
            const int k = int(A.size());
            const float *d = data + 4 * size_t(x);
            A.push_back(make_float4(d[0], d[1], d[2], d[3]));
            if (internal[size_t(x)]) {
                const float *bb = bbox + 6 * size_t(x);
                const float w = bb[3] - bb[0];  // BoundingBox::width(), as the reference computes it
                // the opening factor (M w^3)^(2/5) of the error-bound rule, as built trees keep it
                const float f = std::pow(std::max(d[3], 0.f) * w * w * w, 0.4f);
                int wb, fb;
                std::memcpy(&wb, &w, 4);
                std::memcpy(&fb, &f, 4);
                B.push_back(make_int4(wb, k + 1, -1, fb));
                ++cells;
                if (k == 0)
                    for (int a = 0; a < 6; ++a) box[a] = bb[a];
                st.push_back(~int64_t(k));
                const int32_t *o = orthant + 8 * size_t(x);
                int kids = 0;
                for (int c = 0; c < 8; ++c)  // pushed 0..7: child 7 is opened first
                    if (o[c] >= 0) st.push_back(o[c]), ++kids;
                    else if (o[c] != -1)
                        return set_error(PT_ERR_INVALID, "pt_bh_load_tree: orthant slot %d of node %lld is %d",
                                         c, (long long)x, o[c]);
                if (kids == 0) {
                    // Node::Internal with every slot None: opening it adds nothing. The
                    // walks open a cell into the range of its children, which must not
                    // be empty, so it gets one massless child at its centre of mass
                    // (which contributes exactly zero).
                    B.push_back(make_int4(0, k + 2, int(leaves.size()), 1));
                    A.push_back(make_float4(d[0], d[1], d[2], 0.f));
                    leaves.push_back(A.back());
                }
            } else {
                B.push_back(make_int4(0, k + 1, int(leaves.size()), 1));
                leaves.push_back(A.back());
                if (k == 0)
                    for (int a = 0; a < 3; ++a) box[a] = d[a] - 1.f, box[3 + a] = d[a] + 1.f;
            }
        }
    }
    const size_t T = A.size(), L = leaves.size();
    if (T) {
        PT_TRY(ensure_buf(ctx, S->nodeA, 16 * T));
        PT_TRY(ensure_buf(ctx, S->nodeB, 16 * T));
        PT_TRY(ensure_buf(ctx, S->nodeQ, 32 * T));
        PT_TRY(ensure_buf(ctx, S->sbody, 16 * std::max<size_t>(L, 1)));
    }
    PT_TRY(ensure_buf(ctx, S->counters, sizeof(unsigned long long) * 16));
    PT_TRY(ensure_buf(ctx, S->box, sizeof(float) * 8));
    cudaStream_t st = ctx->stream;
    const int counts[4] = {int(L), int(T), cells, 0};
    if (T) {
        PT_CUDA(cudaMemcpyAsync(S->nodeA.ptr, A.data(), 16 * T, cudaMemcpyHostToDevice, st));
        PT_CUDA(cudaMemcpyAsync(S->nodeB.ptr, B.data(), 16 * T, cudaMemcpyHostToDevice, st));
        PT_CUDA(cudaMemsetAsync(S->nodeQ.ptr, 0, 32 * T, st));
        if (L) PT_CUDA(cudaMemcpyAsync(S->sbody.ptr, leaves.data(), 16 * L, cudaMemcpyHostToDevice, st));
    }
    PT_CUDA(cudaMemsetAsync(S->counters.ptr, 0, sizeof(unsigned long long) * 16, st));
    PT_CUDA(cudaMemcpyAsync(S->counters.ptr, counts, sizeof(counts), cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaMemcpyAsync(S->box.ptr, box, sizeof(box), cudaMemcpyHostToDevice, st));
    PT_CUDA(cudaStreamSynchronize(st));  // the host arrays are freed on return
    S->f64 = false;
    S->user_tree = true;
    S->last_n_src = int(T);  // nonzero when the tree has a node (an internal root alone still adds its data)
    ++S->generation;
    if (generation) *generation = S->generation;
    return PT_OK;
}

int pt_bh_build(pt_ctx *ctx, const float *src, size_t n_src, uint64_t *generation) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_build: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_build", 0, n_src, 0));
    if (n_src && !src) return set_error(PT_ERR_INVALID, "pt_bh_build: NULL affecting buffer");
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    float *d_src = nullptr;
    if (n_src) {
        PT_TRY(ensure_buf(ctx, S->src_h, 16 * n_src));
        d_src = static_cast<float *>(S->src_h.ptr);
        PT_CUDA(cudaMemcpyAsync(d_src, src, 16 * n_src, cudaMemcpyHostToDevice, ctx->stream));
    }
    PT_TRY(pt_bh_build_device(ctx, d_src, n_src, generation));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_bh_walk(pt_ctx *ctx, const float *aff, size_t n_aff, float theta, float softening, uint32_t flags,
               float *out) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_walk: ctx is NULL");
    PT_TRY(bh::validate("pt_bh_walk", n_aff, 0, flags));
    if (n_aff && (!aff || !out)) return set_error(PT_ERR_INVALID, "pt_bh_walk: NULL buffer");
    if (n_aff == 0) return PT_OK;
    PT_CUDA(cudaSetDevice(ctx->device));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    PT_TRY(ensure_buf(ctx, S->aff_h, 16 * n_aff));
    PT_TRY(ensure_buf(ctx, S->out, 12 * n_aff));
    float *d_aff = static_cast<float *>(S->aff_h.ptr);
    float *d_out = static_cast<float *>(S->out.ptr);
    cudaStream_t st = ctx->stream;
    PT_CUDA(cudaMemcpyAsync(d_aff, aff, 16 * n_aff, cudaMemcpyHostToDevice, st));
    PT_TRY(pt_bh_walk_device(ctx, d_aff, n_aff, theta, softening, flags, d_out));
    PT_CUDA(cudaMemcpyAsync(out, d_out, 12 * n_aff, cudaMemcpyDeviceToHost, st));
    int err = 0;
    PT_CUDA(cudaMemcpyAsync(&err, static_cast<int *>(S->counters.ptr) + 3, sizeof(int), cudaMemcpyDeviceToHost,
                            st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (err & 2) return set_error(PT_ERR_CAPACITY, "pt_bh_walk: learned-correction records overflowed");
    return PT_OK;
}

int pt_bh_tree_generation(pt_ctx *ctx, uint64_t *generation) {
    using namespace pt;
    clear_error();
    if (!ctx || !generation) return set_error(PT_ERR_INVALID, "pt_bh_tree_generation: NULL argument");
    auto *S = static_cast<bh::State *>(ctx->bh);
    *generation = S ? S->generation : 0;
    return PT_OK;
}

int pt_bh_set_local_ratio(pt_ctx *ctx, float ratio) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_set_local_ratio: ctx is NULL");
    if (!(ratio > 0.0f && ratio <= 0.5f))
        return set_error(PT_ERR_INVALID, "pt_bh_set_local_ratio: %g outside (0, 0.5]", double(ratio));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->local_ratio = ratio;
    return PT_OK;
}


int pt_bh_set_relative_alpha(pt_ctx *ctx, float alpha) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_set_relative_alpha: ctx is NULL");
    if (!(alpha > 0.0f && alpha <= 1.0f))
        return set_error(PT_ERR_INVALID, "pt_bh_set_relative_alpha: %g outside (0, 1]", double(alpha));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->rel_alpha = alpha;
    return PT_OK;
}

int pt_bh_set_relative_monopole(pt_ctx *ctx, float beta) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_set_relative_monopole: ctx is NULL");
    if (!(beta >= 0.0f && beta <= 1.0f))
        return set_error(PT_ERR_INVALID, "pt_bh_set_relative_monopole: %g outside [0, 1]", double(beta));
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->rel_mono = beta;
    return PT_OK;
}

int pt_bh_set_stack_limit(pt_ctx *ctx, int ranges) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_set_stack_limit: ctx is NULL");
    if (ranges > bh::GW_STACK || (ranges > 0 && ranges < 2))
        return set_error(PT_ERR_INVALID, "pt_bh_set_stack_limit: %d outside [2, %d] (0 = %d)", ranges,
                         bh::GW_STACK, bh::GW_STACK);
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->stack_cap = ranges;
    return PT_OK;
}

int pt_bh_set_learned_capacity(pt_ctx *ctx, int chunks) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_set_learned_capacity: ctx is NULL");
    if (chunks < 0) return set_error(PT_ERR_INVALID, "pt_bh_set_learned_capacity: %d < 0", chunks);
    bh::State *S = bh::state(ctx);
    if (!S) return set_error(PT_ERR_OOM, "Barnes-Hut state allocation failed");
    S->lcap_fixed = chunks;
    if (chunks > 0) S->lcap = chunks;
    return PT_OK;
}

int pt_bh_last_stats(pt_ctx *ctx, pt_bh_stats *out) {
    using namespace pt;
    clear_error();
    if (!ctx || !out) return set_error(PT_ERR_INVALID, "pt_bh_last_stats: NULL argument");
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || !S->counters.ptr) return set_error(PT_ERR_INVALID, "pt_bh_last_stats: no Barnes-Hut call yet");
    PT_CUDA(cudaSetDevice(ctx->device));
    unsigned long long h[11];
    PT_CUDA(cudaMemcpyAsync(h, S->counters.ptr, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA(cudaStreamSynchronize(ctx->stream));
    const int *hi = reinterpret_cast<const int *>(h);
    out->leaves = uint64_t(hi[0]);
    out->nodes = uint64_t(hi[1]);
    out->cells = uint64_t(hi[2]);
    out->overflow = h[8];
    out->local_nodes = h[9];
    out->local_quad_nodes = h[10];
    out->interactions = h[2];
    out->visits = h[3];
    out->warps = h[4];
    out->max_stack = h[5];
    out->learned = h[6];
    out->cell_interactions = h[7];
    return PT_OK;
}

// Copies the last tree (preorder) to host arrays of pt_bh_last_stats().nodes rows.
int pt_bh_export_tree_dvec3(pt_ctx *ctx, double *com_mass, int32_t *links, double *centre_width, size_t rows) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_export_tree_dvec3: ctx is NULL");
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || !S->f64 || !S->nodeA64.ptr)
        return set_error(PT_ERR_INVALID, "pt_bh_export_tree_dvec3: the last Barnes-Hut call was not the f64 method");
    pt_bh_stats st;
    PT_TRY(pt_bh_last_stats(ctx, &st));
    if (rows < st.nodes) return set_error(PT_ERR_INVALID, "pt_bh_export_tree_dvec3: %zu rows < %llu nodes", rows,
                                          (unsigned long long)st.nodes);
    cudaStream_t s = ctx->stream;
    if (com_mass) PT_CUDA(cudaMemcpyAsync(com_mass, S->nodeA64.ptr, 32 * st.nodes, cudaMemcpyDeviceToHost, s));
    if (links) PT_CUDA(cudaMemcpyAsync(links, S->nodeB.ptr, 16 * st.nodes, cudaMemcpyDeviceToHost, s));
    if (centre_width) PT_CUDA(cudaMemcpyAsync(centre_width, S->nodeG64.ptr, 32 * st.nodes, cudaMemcpyDeviceToHost, s));
    PT_CUDA(cudaStreamSynchronize(s));
    return PT_OK;
}

int pt_bh_export_tree(pt_ctx *ctx, float *com_mass, int32_t *links, float *quad, size_t rows) {
    using namespace pt;
    clear_error();
    if (!ctx) return set_error(PT_ERR_INVALID, "pt_bh_export_tree: ctx is NULL");
    auto *S = static_cast<bh::State *>(ctx->bh);
    if (!S || !S->nodeA.ptr) return set_error(PT_ERR_INVALID, "pt_bh_export_tree: no Barnes-Hut call yet");
    if (S->f64) return set_error(PT_ERR_INVALID, "pt_bh_export_tree: the tree holds DVec3 bodies (pt_bh_export_tree_dvec3)");
    pt_bh_stats st;
    PT_TRY(pt_bh_last_stats(ctx, &st));
    if (rows < st.nodes) return set_error(PT_ERR_INVALID, "pt_bh_export_tree: %zu rows < %llu nodes", rows,
                                          (unsigned long long)st.nodes);
    cudaStream_t s = ctx->stream;
    if (com_mass) PT_CUDA(cudaMemcpyAsync(com_mass, S->nodeA.ptr, 16 * st.nodes, cudaMemcpyDeviceToHost, s));
    if (links) PT_CUDA(cudaMemcpyAsync(links, S->nodeB.ptr, 16 * st.nodes, cudaMemcpyDeviceToHost, s));
    if (quad) PT_CUDA(cudaMemcpyAsync(quad, S->nodeQ.ptr, 32 * st.nodes, cudaMemcpyDeviceToHost, s));
    PT_CUDA(cudaStreamSynchronize(s));
    // On the device a cell's last word holds the walk's opening factor and a
    // single-body leaf has no quadrupole: the columns read as documented (body count
    // 0 for cells, a zero quadrupole for single bodies). Single-body rows need the
    // links to be told apart.
    std::vector<int32_t> own;
    if (quad && !links) {
        own.resize(4 * size_t(st.nodes));
        PT_CUDA(cudaMemcpy(own.data(), S->nodeB.ptr, 16 * st.nodes, cudaMemcpyDeviceToHost));
    }
    const int32_t *L = links ? links : own.data();
    for (size_t r = 0; r < st.nodes && (links || quad); ++r) {
        if (L[4 * r + 2] < 0) {
            if (links) links[4 * r + 3] = 0;
        } else if (quad && L[4 * r + 3] == 1) {
            for (int k = 0; k < 8; ++k) quad[8 * r + k] = 0.f;
        }
    }
    return PT_OK;
}

}  // extern "C"
