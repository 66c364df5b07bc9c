/*
 * particular_cuda.h -- C ABI of the GB300 (sm_103a) compute methods for particular.
 *
 * The library adds two compute methods beside particular's `sequential`, `parallel`
 * and `gpu` ones:
 *   cuda::BruteForce        all-pairs acceleration  (replaces gpu::BruteForce's wgpu
 *                           dispatch, particular/src/gpu/mod.rs:179-208, and is the
 *                           GPU counterpart of sequential::BruteForce,
 *                           particular/src/sequential.rs:181-209)
 *   cuda::BarnesHut{theta}  tree acceleration        (GPU counterpart of
 *                           sequential::BarnesHut, particular/src/sequential.rs:456-543)
 *
 * Data layout at the boundary (the layout wgpu's padded types already use,
 * particular/src/gravity/impls/mod.rs:430-434 and gravity/mod.rs:244-272):
 *   affecting (sources) : float[4] per body = (x, y, z, mu)   -- GravitationalField<Vec3, f32>
 *   affected  (targets) : float[4] per body = (x, y, z, unused)
 *   output              : float[3] per affected body = acceleration
 *
 * The interaction is given by (softening, checked), mirroring
 * Acceleration<CHECKED> (softening 0; gravity/newtonian/acceleration.rs:17-58) and
 * AccelerationSoftened<f32, CHECKED> (gravity/newtonian/acceleration_softened.rs:17-63).
 *
 * Every entry point returns PT_OK (0) or a negative PT_ERR_* code and then sets a
 * thread-local message readable with pt_last_error(). There is no CPU fallback: a
 * failed call computes nothing. Calls taking host pointers are synchronous (like
 * gpu::BruteForce, which blocks on the map, particular/src/gpu/mod.rs:200).
 * Edge cases follow particular/src/gpu/resources.rs:272-280: n_aff == 0 computes
 * nothing; n_src == 0 yields zero accelerations (the reference panics there on
 * DynamicBuffer's len != 0 assert, resources.rs:24; this library does not).
 */
#ifndef PARTICULAR_CUDA_H
#define PARTICULAR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_OK 0
#define PT_ERR_INVALID (-1)  /* bad argument (null pointer, size mismatch, bad flag) */
#define PT_ERR_CUDA (-2)     /* a CUDA runtime call or kernel launch failed */
#define PT_ERR_OOM (-3)      /* device or host allocation failed */
#define PT_ERR_CAPACITY (-4) /* request exceeds the context's capacity limit */
#define PT_ERR_TIMEOUT (-5)  /* a bounded device-side wait gave up */
#define PT_ERR_DEPTH (-6)    /* tree deeper than the supported key resolution */

/* Flags for pt_bf_accel_*. */
/* Bit-identical to sequential::BruteForce: per-body sequential sum over j in
 * ascending order, IEEE sqrt and divide, no contraction. Slower; it is the
 * drop-in for callers that need the reference's exact f32 result. */
#define PT_BF_EXACT 0x1u
/* With PT_BF_EXACT: glam Vec3A / Vec4's operand order, a = (d * mu) / (n_s sqrt(n_s))
 * per component (particular/src/gravity/impls/glam.rs:260-275), for callers whose
 * particles use those types. Other 3D f32 vectors (glam Vec3, nalgebra Vector3,
 * ultraviolet Vec3) share the default order; 2D bodies pass z = 0, which gives their
 * 2D results bit for bit (the squared norm adds an exact +0). */
#define PT_BF_VEC3A 0x2u

/* Opaque context: device, stream and grow-only device buffers. It plays the role
 * of gpu::GpuResources (particular/src/gpu/mod.rs:84-143): create it once and
 * reuse it across calls. One context must not be used by two threads at once. */
typedef struct pt_ctx pt_ctx;

/* Creates a context on `device` (a CUDA ordinal). Replaces GpuResources::new
 * (particular/src/gpu/mod.rs:96-98) + the lazy init at :128-142. */
int pt_ctx_create(pt_ctx **ctx, int device);
/* Frees every device buffer the context owns. NULL is accepted. */
void pt_ctx_destroy(pt_ctx *ctx);
/* Message of the last failed call on this thread ("" if none). */
const char *pt_last_error(void);
/* Enqueue subsequent work on `stream` (a cudaStream_t). NULL selects the
 * context's own non-blocking stream, not the legacy default stream. Used to
 * interleave with other CUDA work, e.g. for event timing. */
int pt_ctx_set_stream(pt_ctx *ctx, void *stream);
/* Caps the bytes of device memory the context may hold (0 = unlimited). A call
 * that would grow past it fails with PT_ERR_CAPACITY and computes nothing. */
int pt_ctx_set_capacity_limit(pt_ctx *ctx, size_t bytes);
/* Bytes of device memory currently held by the context. */
size_t pt_ctx_device_bytes(const pt_ctx *ctx);
/* Number of kernels this context has launched so far. */
uint64_t pt_ctx_launch_count(const pt_ctx *ctx);
/* Number of SMs of the context's device. */
int pt_ctx_sm_count(const pt_ctx *ctx);

/* cuda::BruteForce over host buffers: for each affected body i,
 *   out[i] = sum_j a(x_i, affecting_j), a from gravity/impls/mod.rs:150-166.
 * Replaces gpu::BruteForce::compute (particular/src/gpu/mod.rs:186-207), whose
 * per-body result is sequential::BruteForce's fold (sequential.rs:189-193).
 * Default path: FP32 with rsqrt on the FMA pipe and compensated (two-sum) per-tile
 * accumulation; flags = PT_BF_EXACT for the bit-identical path. */
int pt_bf_accel_f32(pt_ctx *ctx, const float *affected, size_t n_aff, const float *affecting,
                    size_t n_src, float softening, int checked, uint32_t flags, float *out_xyz);

/* Same computation on device-resident buffers (no copies, asynchronous on the
 * context's stream). Pointers must be 16-byte aligned device pointers. */
int pt_bf_accel_f32_device(pt_ctx *ctx, const float *d_affected, size_t n_aff,
                           const float *d_affecting, size_t n_src, float softening, int checked,
                           uint32_t flags, float *d_out_xyz);

/* cuda::BruteForce over glam DVec3 bodies: double[4] (x, y, z, mu) in, double[3] out.
 * Replaces the f64 instantiation of the per-pair kernel (impl_acceleration_cpu_scalar!
 * (DVec3, f64), particular/src/gravity/impls/glam.rs:234 over gravity/impls/mod.rs:
 * 150-166) folded as sequential::BruteForce (sequential.rs:189-193): every operation
 * IEEE-rounded in the reference's order, so results equal the reference's bit for bit.
 * Synchronous, host buffers. */
int pt_bf_accel_dvec3(pt_ctx *ctx, const double *affected, size_t n_aff, const double *affecting,
                      size_t n_src, double softening, int checked, double *out_xyz);
/* Same on device buffers (8-byte aligned), asynchronous on the context's stream. */
int pt_bf_accel_dvec3_device(pt_ctx *ctx, const double *d_affected, size_t n_aff,
                             const double *d_affecting, size_t n_src, double softening, int checked,
                             double *d_out_xyz);

/* FP64 brute force of the same formula on device buffers (f32 inputs widened to
 * f64, double accumulation): the error judge for the FP32 methods. It has no
 * counterpart in the reference, which reports no accuracy figures. */
int pt_bf_accel_f64_device(pt_ctx *ctx, const float *d_affected, size_t n_aff,
                           const float *d_affecting, size_t n_src, double softening, int checked,
                           double *d_out_xyz);

/* Overrides the brute-force launch plan of subsequent calls made from this
 * thread: targets per thread (1, 2 or 4) and number of j-slices; 0 restores the
 * automatic choice. Tuning and test knob; results do not depend on it beyond
 * FP32 summation order. */
int pt_bf_set_plan(pt_ctx *ctx, int targets_per_thread, int slices);

/* Measures the device's FP32 FMA-pipe throughput (TFLOP/s, FFMA = 2 flops) with
 * a dependent-chain FFMA kernel over every SM, at the clock the device runs at
 * now. Roofline denominator for the FP32-bound kernels; no reference counterpart. */
int pt_measure_fp32_peak(pt_ctx *ctx, double *tflops);

/* Allocation-free brute force: the same computation as pt_bf_accel_f32_device,
 * for callers that cannot call cudaMalloc -- host programs that own every byte of
 * device memory through their own pool or fixed budget, and time-critical loops
 * where cudaMalloc/cudaFree's implicit device-wide synchronisation is not
 * acceptable. It needs no context: its scratch is one static device array of
 * 16 MiB that every device loading the library holds until the process exits,
 * and no call allocates device memory. The caller passes device inputs and
 * output (16-byte aligned bodies) and a cudaStream_t (NULL = legacy default
 * stream); work is enqueued asynchronously.
 * - n_src above PT_NOALLOC_MAX_SOURCES fails with PT_ERR_CAPACITY.
 * - The first call on a device, with that device current, looks up the scratch
 *   array's device address (cudaGetSymbolAddress); make that first call before
 *   any stream capture.
 * - All calls share the one array and it keeps the last call's contents: calls
 *   whose work overlaps on the GPU (other streams, other threads) race, so
 *   serialise them. Every scratch byte a call reads is written earlier by the
 *   same call; nothing needs clearing.
 * - The address looked up on a device's first call is kept for the process: a
 *   device reset (cudaDeviceReset, or anything else that destroys the primary
 *   context) is not supported afterwards.
 * This entry point has no counterpart in the reference. */
#define PT_NOALLOC_MAX_SOURCES 524288
int pt_bf_accel_f32_noalloc(const float *d_affected, size_t n_aff, const float *d_affecting,
                            size_t n_src, float softening, int checked, float *d_out_xyz,
                            void *stream);

/* ---- cuda::BarnesHut { theta } ------------------------------------------------
 * GPU counterpart of sequential::BarnesHut (particular/src/sequential.rs:456-543):
 * the tree over the affecting bodies is the reference's orthtree
 * (tree/mod.rs:91-138: square root box, cells split at their centre, a leaf per
 * body), built on the device every call; each affected body walks it with the
 * reference's rule: skip a node whose centre of mass coincides with the body, open
 * an internal cell when theta^2 d^2 < w^2 (w = cell width), otherwise add the
 * node's monopole through the per-pair kernel. Because coincident nodes are always
 * skipped, Acceleration's CHECKED flag has no effect on this method, as in the
 * reference. Cell moments are combined bottom-up about each cell's geometric centre
 * (compensated FP32) and stored in f32. */
#define PT_BH_QUADRUPOLE 0x1u /* add the traceless quadrupole of accepted cells */
#define PT_BH_GROUP 0x2u      /* walk per warp of 64 key-adjacent bodies (two per lane):
                                 a cell is opened for all of them when the per-body rule
                                 opens it for any (so never less accurate than that
                                 rule); accepted nodes are evaluated from shared-memory
                                 lists */
#define PT_BH_LOCAL 0x8u      /* with PT_BH_GROUP: far nodes (group radius < ratio x
                                 distance, pt_bh_set_local_ratio, default 0.1) enter
                                 a second-order local expansion about the group's
                                 centre instead of every body's interaction list */
#define PT_BH_RELATIVE 0x10u  /* with PT_BH_GROUP: also open a cell where its truncation
                                 bound M w^3 / d^5 (M w^2 / d^4 without quadrupoles)
                                 exceeds alpha |a| (pt_bh_set_relative_alpha, default
                                 2.5e-3), |a| estimated once per group at its centre by
                                 a coarse walk; theta stays the geometric cap */
#define PT_BH_LEARNED 0x4u    /* with PT_BH_GROUP: add the learned far-field correction
                                 (pt_mlp_*) of every cell accepted at theta that the
                                 model's inner angle would have opened, evaluated once
                                 per warp at the warp's centre */

typedef struct pt_bh_stats {
    uint64_t nodes;        /* cells + leaves of the last tree */
    uint64_t cells;        /* internal cells */
    uint64_t leaves;       /* leaves (bodies with distinct keys) */
    uint64_t interactions; /* accepted nodes summed over bodies, last walk */
    uint64_t visits;       /* nodes visited, summed over bodies, last walk */
    uint64_t warps;        /* warps that walked */
    uint64_t max_stack;    /* deepest shared-memory stack of a PT_BH_GROUP walk */
    uint64_t overflow;     /* warps of a PT_BH_GROUP walk whose shared-memory stack
                              ran out; they took the per-body walk instead (same
                              rule as without PT_BH_GROUP, no error) */
    uint64_t learned;      /* learned corrections evaluated (per warp and cell) */
    uint64_t cell_interactions; /* the accepted nodes of `interactions` that are cells
                                   (the ones a PT_BH_QUADRUPOLE walk adds the
                                   quadrupole term to) */
    uint64_t local_nodes;  /* PT_BH_LOCAL: far nodes added to the groups' local
                              expansions (per group and node) */
    uint64_t local_quad_nodes; /* the far nodes of local_nodes that are cells added with
                                  their quadrupole (PT_BH_QUADRUPOLE; monopole-only
                                  cells of PT_BH_RELATIVE are not) */
} pt_bh_stats;

/* cuda::BarnesHut over host buffers (synchronous). Layouts as pt_bf_accel_f32. */
int pt_bh_accel_f32(pt_ctx *ctx, const float *affected, size_t n_aff, const float *affecting,
                    size_t n_src, float theta, float softening, uint32_t flags, float *out_xyz);
/* Same on 16-byte aligned device buffers, asynchronous on the context's stream. */
int pt_bh_accel_f32_device(pt_ctx *ctx, const float *d_affected, size_t n_aff,
                           const float *d_affecting, size_t n_src, float theta, float softening,
                           uint32_t flags, float *d_out_xyz);
/* Tree reuse: the GPU counterpart of computing with Between(affected, &tree) over a
 * RootedOrthtree built once (particular/src/lib.rs:186-199, sequential.rs:508-522,
 * storage.rs:20-33). pt_bh_build_device builds the reference's orthtree over the
 * affecting bodies (device buffer, asynchronous) and keeps it in the context;
 * *generation (may be NULL) receives its number. pt_bh_walk_device walks the
 * context's current tree for any affected bodies with the same theta rule and flags
 * as pt_bh_accel_f32_device, which gives the same results as one combined call. Every
 * Barnes-Hut call on the context (pt_bh_accel_*, the learned-sample generation)
 * replaces the current tree; pt_bh_tree_generation reports which one is current. */
int pt_bh_build_device(pt_ctx *ctx, const float *d_affecting, size_t n_src, uint64_t *generation);
int pt_bh_walk_device(pt_ctx *ctx, const float *d_affected, size_t n_aff, float theta, float softening,
                      uint32_t flags, float *d_out_xyz);
int pt_bh_tree_generation(pt_ctx *ctx, uint64_t *generation);
/* Makes a tree the caller built the context's current tree, for pt_bh_walk[_device]:
 * the GPU counterpart of computing Between(affected, &tree) over a RootedOrthtree the
 * caller constructed or kept (particular/src/lib.rs:186-199, sequential.rs:466-522,
 * storage.rs:10-46). The arrays are the reference's Orthtree<8, 3, f32,
 * GravitationalField<Vec3, f32>> (tree/mod.rs:13-60) flattened per node:
 *   orthant  int32[8]  SizedOrthant::orthant, child NodeID or -1 for None
 *   bbox     float[6]  SizedOrthant::bbox, min x, y, z then max x, y, z
 *   internal uint8     1 = Node::Internal, 0 = Node::External (orthant, bbox unused)
 *   data     float[4]  the node's GravitationalField: centre of mass x, y, z, mass
 * and root = RootedOrthtree::root() (-1 = None: every acceleration is zero). A walk
 * then accepts, for every affected body, exactly the nodes the reference's walk of this
 * tree accepts (the same opening rule, width = max.x - min.x, skip at d^2 == 0); sums
 * run in list order (rounding-level differences). Such a tree carries monopoles only:
 * walks take flags 0 or PT_BH_GROUP. A node reachable twice from the root is rejected
 * (PT_ERR_INVALID). Synchronous (the host arrays may change after the call). */
int pt_bh_load_tree(pt_ctx *ctx, const int32_t *orthant, const float *bbox, const uint8_t *internal,
                    const float *data, size_t n_nodes, int64_t root, uint64_t *generation);
/* The same over host buffers (synchronous): the bodies are staged in context buffers;
 * the tree keeps its own copy, so `affecting` may change after pt_bh_build returns. */
int pt_bh_build(pt_ctx *ctx, const float *affecting, size_t n_src, uint64_t *generation);
int pt_bh_walk(pt_ctx *ctx, const float *affected, size_t n_aff, float theta, float softening,
               uint32_t flags, float *out_xyz);
/* The far ratio of PT_BH_LOCAL, in (0, 0.5]: smaller is more accurate and slower. */
int pt_bh_set_local_ratio(pt_ctx *ctx, float ratio);
/* The error-bound factor of PT_BH_RELATIVE, in (0, 1]: smaller is more accurate and
 * slower. */
int pt_bh_set_relative_alpha(pt_ctx *ctx, float alpha);
/* PT_BH_RELATIVE with PT_BH_QUADRUPOLE: an accepted cell whose monopole truncation
 * bound M w^2 / d^4 (d from the group's nearest point) stays within beta x alpha |a|
 * is evaluated without its quadrupole term (20 instead of 58 flops per body). beta in
 * [0, 1], 0 = every cell keeps its quadrupole; default 0.1, where the FP64-judged
 * error does not change. */
int pt_bh_set_relative_monopole(pt_ctx *ctx, float beta);
/* Caps the PT_BH_GROUP walk's shared-memory stack at `ranges` entries per warp (2 to
 * the compiled capacity; 0 restores the capacity). A warp that runs out takes the
 * per-body walk instead (counted in pt_bh_stats.overflow): a tuning and test hook. */
int pt_bh_set_stack_limit(pt_ctx *ctx, int ranges);
/* Fixes the record capacity of PT_BH_LEARNED walks at `chunks` chunks of 128 cells
 * (0 restores the automatic capacity, which grows and reruns a walk whose records did
 * not fit). With a fixed capacity, or inside a captured leapfrog graph, a walk whose
 * records overflow keeps the plain result for the cells that did not fit and the call
 * fails with PT_ERR_CAPACITY (pt_bh_accel_f32, pt_bh_walk, pt_leapfrog_device). A
 * tuning and test hook. */
int pt_bh_set_learned_capacity(pt_ctx *ctx, int chunks);
/* cuda::BarnesHut over glam DVec3 bodies: double[4] (x, y, z, mu) in, double[3] out.
 * The reference's BarnesHut over f64 particles (sequential.rs:456-543 with
 * BoundingBox<DVec3>, f64 theta and the f64 per-pair kernel, gravity/impls/glam.rs:234):
 * the orthtree is built by replaying the subdivision in double and walked with the
 * per-body rule in double; accepted sets per body equal the reference's. Monopole
 * only (flags must be 0), as the reference. Synchronous, host buffers. */
int pt_bh_accel_dvec3(pt_ctx *ctx, const double *affected, size_t n_aff, const double *affecting,
                      size_t n_src, double theta, double softening, uint32_t flags, double *out_xyz);
/* Same on 32-byte aligned device buffers, asynchronous on the context's stream. */
int pt_bh_accel_dvec3_device(pt_ctx *ctx, const double *d_affected, size_t n_aff,
                             const double *d_affecting, size_t n_src, double theta, double softening,
                             uint32_t flags, double *d_out_xyz);
/* The last f64 tree in preorder: com_mass = (x, y, z, mass), links as pt_bh_export_tree,
 * centre_width = (cell centre x, y, z, width); NULL skips one. */
int pt_bh_export_tree_dvec3(pt_ctx *ctx, double *com_mass, int32_t *links, double *centre_width,
                            size_t rows);
/* Counters of the last Barnes-Hut call (synchronises the context's stream). */
int pt_bh_last_stats(pt_ctx *ctx, pt_bh_stats *out);
/* Copies the last tree in depth-first preorder (rows >= stats.nodes): per node
 * com_mass = (x, y, z, mass), links = (width bits, skip index, first body or -1 for
 * a cell, body count), quad = (Qxx, Qxy, Qxz, Qyy, Qyz, Qzz, 0, 0). NULL skips one.
 * The tree the reference keeps in RootedOrthtree (particular/src/storage.rs:10-46). */
int pt_bh_export_tree(pt_ctx *ctx, float *com_mass, int32_t *links, float *quad, size_t rows);

/* ---- time integration ------------------------------------------------------
 * Kick-drift-kick leapfrog on device-resident state, around either method:
 *   v += a dt/2; x += v dt; a = accel(x); v += a dt/2      (per step)
 * with the closing half kick of a step fused into the next step's opening kick.
 * The reference integrates with semi-implicit Euler around its methods in its
 * benchmark and tests (particular/benches/benchmark.rs:81,
 * gravity/newtonian/mod.rs:318-330); this driver has no reference counterpart. */
#define PT_METHOD_BRUTE_FORCE 0
#define PT_METHOD_BARNES_HUT 1
/* Host state: bodies float[4] (x, y, z, mu) and velocities float[4] (vx, vy, vz,
 * unused) per body, updated in place after `steps` steps (synchronous). `flags` are
 * the method's flags (PT_BF_* or PT_BH_*); theta is used by Barnes-Hut only. */
int pt_leapfrog(pt_ctx *ctx, float *bodies, float *vel, size_t n, float dt, int steps, int method,
                float theta, float softening, uint32_t flags);
/* Device state (16-byte aligned bodies and velocities; acc = float[3] per body
 * holding the accelerations of the current positions, updated to the final ones).
 * use_graph != 0 captures the whole `steps`-step sequence into a CUDA graph on first
 * use for this (pointers, n, steps, method, dt, theta, softening, flags, stream and,
 * for Barnes-Hut, the context's local ratio, error-bound factor, stack limit and
 * learned model; any reallocation of a context buffer in between) and replays it
 * afterwards; that first call also recomputes `acc` from the positions
 * before capturing, so every buffer is sized outside the capture.
 * With PT_BH_LEARNED the call synchronises at the end and fails with PT_ERR_CAPACITY
 * when any step's learned-correction records overflowed (the state has then advanced
 * with the plain result for those cells); the next call captures again with room for
 * them. The forced brute-force plan (pt_bf_set_plan) is part of the captured shape. */
int pt_leapfrog_device(pt_ctx *ctx, float *d_bodies, float *d_vel, float *d_acc, size_t n, float dt,
                       int steps, int method, float theta, float softening, uint32_t flags,
                       int use_graph);

/* ---- batched ensembles -------------------------------------------------------
 * n_sys independent systems in one device array: system k is bodies
 * [offsets[k], offsets[k+1]) (host array, offsets[0] == 0). Each evolves by the
 * leapfrog above with brute-force accelerations inside the system only, for `steps`
 * steps, all steps in ONE persistent cooperative kernel (work queue over (system,
 * target tile) items, largest first; grid barriers between phases). With use_graph
 * the launch is captured once per (pointers, steps, dt, softening) and replayed.
 * Synchronous. A grid barrier that exceeds its spin limit makes the call fail with
 * PT_ERR_TIMEOUT (the state is then partially advanced); the context stays usable.
 * The reference evaluates one system per call; ensembles have no counterpart. */
int pt_ensemble_run(pt_ctx *ctx, const uint32_t *offsets, uint32_t n_sys, float *d_bodies,
                    float *d_vel, float dt, int steps, float softening, int use_graph);
/* Autotuner: times every item shape -- 1, 2 or 4 targets per thread (128 threads per
 * block) times a j-tile of 128, 256 or 512 sources staged in shared memory -- for each
 * system-size class present (class c: 64*2^c <= n < 64*2^(c+1), c = 0..7, the ends
 * open) and keeps the fastest per class for later runs; table_out (8 ints, may be
 * NULL) receives the targets per thread (pt_ensemble_get_shape reports both). */
int pt_ensemble_tune(pt_ctx *ctx, const uint32_t *offsets, uint32_t n_sys, const float *d_bodies,
                     float softening, int *table_out);
/* Sets the per-class targets per thread directly (8 ints: 0 = default, else 1, 2 or 4). */
int pt_ensemble_set_table(pt_ctx *ctx, const int *table);
/* Sets the per-class j-tile directly (8 ints: 0 = default 256, else 128, 256 or 512). */
int pt_ensemble_set_tiles(pt_ctx *ctx, const int *tiles);
/* The item shape in use per class (8 ints each, defaults resolved; NULL skips one). */
int pt_ensemble_get_shape(pt_ctx *ctx, int *table, int *tiles);
/* Barrier spin limit (iterations of ~64 ns sleeps; default 2^22). stall != 0 makes
 * every barrier wait for one block more than the grid has: a wait nothing ends, to
 * test the timeout path without faulting the GPU. */
int pt_ensemble_set_barrier(pt_ctx *ctx, long long spin_limit, int stall);

/* ---- learned far-field correction ------------------------------------------
 * A 12 -> 64 -> 64 -> 3 MLP (GELU, BF16 weights, FP32 accumulation) predicting the
 * residual between a Barnes-Hut cell's exact field and its monopole + quadrupole, for
 * cells accepted at theta that theta_inner would have opened. Trained on the GPU by
 * this library's kernels from residuals the brute-force pair kernel computes; the
 * reference has no learned part. Parameters: PT_MLP_NPARAM floats (BF16 values). */
#define PT_MLP_NPARAM 5188
/* Random initialisation (seeded). */
int pt_mlp_init(pt_ctx *ctx, uint64_t seed);
/* Loads / reads parameters (host arrays of PT_MLP_NPARAM floats). */
int pt_mlp_set_params(pt_ctx *ctx, const float *params, size_t n, float theta_inner);
int pt_mlp_get_params(pt_ctx *ctx, float *params, size_t n);
/* Builds the tree of one snapshot (device bodies) and appends the samples of
 * n_targets evenly spaced bodies to the dataset (capacity samples at most, kept on
 * the device); *total receives the dataset size. */
int pt_mlp_generate(pt_ctx *ctx, const float *d_bodies, size_t n, int n_targets, float theta_outer,
                    float theta_inner, float softening, size_t capacity, size_t *total);
int pt_mlp_reset_dataset(pt_ctx *ctx);
int pt_mlp_export_dataset(pt_ctx *ctx, float *features, float *targets, size_t n);
/* Adam training for `steps` steps of `batch` random samples; loss_out = mean loss
 * over the last 10% of steps (targets scaled by their RMS). */
int pt_mlp_train(pt_ctx *ctx, int steps, int batch, float lr, uint64_t seed, float *loss_out);
/* Loss and gradient (PT_MLP_NPARAM floats) for host samples: the training kernel's check. */
int pt_mlp_loss_grad(pt_ctx *ctx, const float *features, const float *targets, int batch, float *grad,
                     double *loss_out);
/* Predictions (n x 3) for host features (n x 12). */
int pt_mlp_predict(pt_ctx *ctx, const float *features, int n, float *out);
/* The same predictions through the Barnes-Hut walk's inference path: BF16 tensor-core
 * MMAs (mma.sync m16n8k16) with features and activations rounded to BF16, FP32
 * accumulation. */
int pt_mlp_predict_tc(pt_ctx *ctx, const float *features, int n, float *out);

/* Phase timing of the last pt_bf_* / pt_bh_* call, from CUDA events recorded on
 * the context's stream when enabled: for Barnes-Hut, build = tree construction
 * and moments, walk = the traversal kernel; for the brute force, build = source
 * layout conversion, walk = the pair kernel(s). */
typedef struct pt_timing {
    float build_ms;
    float walk_ms;
} pt_timing;
int pt_ctx_set_timing(pt_ctx *ctx, int enable);
/* Waits for the last call's events and reports its phases. */
int pt_last_timing(pt_ctx *ctx, pt_timing *out);

/* Blocks until all work enqueued by the context has finished; reports any
 * asynchronous kernel error as PT_ERR_CUDA. */
int pt_ctx_synchronize(pt_ctx *ctx);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PARTICULAR_CUDA_H */
