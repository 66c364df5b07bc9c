/*
 * CPU oracle for the particular acceleration hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: only tests/, the smoke
 * check of __graft_entry__.py and the cpu_baseline / reference arm of bench.py
 * may load it. The product path (particular_gb300) never links or calls it.
 *
 * It restates, in plain C with IEEE f32 arithmetic and no FMA contraction
 * (compile with -ffp-contract=off; Rust never contracts), the reference
 * crate's sequential algorithms for 3D f32 bodies (glam::Vec3, f32):
 *
 *   per-pair kernel      particular/src/gravity/impls/mod.rs:150-166
 *                        (reached from gravity/newtonian/acceleration.rs:46-58 and
 *                        acceleration_softened.rs:51-63)
 *   brute force fold     particular/src/sequential.rs:181-194 (start at zero,
 *                        j ascending, self term included)
 *   parallel brute force particular/src/parallel.rs:216-232 (same per-body sum,
 *                        bodies split across threads: bit-identical)
 *   square root box      particular/src/tree/partition.rs:274-292, 295-318
 *   orthtree build       particular/src/tree/mod.rs:91-138 (+ subdivide,
 *                        partition.rs:332-359)
 *   centre of mass       particular/src/gravity/impls/mod.rs:120-134
 *   Barnes-Hut walk      particular/src/sequential.rs:466-505 (LIFO stack,
 *                        skip d2 == 0, open when theta^2 d2 < w^2)
 *   BH distance          particular/src/gravity/newtonian/acceleration.rs:121-126
 *
 * plus an FP64 brute force of the same formula, used as the error judge, the
 * same kernel and fold for glam DVec3 bodies in double (gravity/impls/glam.rs:234),
 * and BruteForcePairs' pairwise fold (sequential.rs:232-304, impls/mod.rs:175-207).
 *
 * Vector arithmetic follows glam's scalar Vec3: component-wise sub/add/mul
 * and length_squared = (x*x + y*y) + z*z evaluated left to right. glam's
 * source is not vendored with the reference (glam >=0.12,<0.33 per
 * particular/Cargo.toml:45); that evaluation order is an assumption, so the
 * bit-level equality with the Rust crate is unpinned at that one step. The
 * restatement is pinned against the reference's own known-answer tests
 * (acceleration_error!, circular_orbit!: particular/src/gravity/newtonian/mod.rs:228-347).
 *
 * Layouts: sources are float[4] (x, y, z, mu); targets are float[4]
 * (x, y, z, ignored); outputs are float[3] (or double[3]).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__FP_FAST_FMAF) && !defined(PT_ORACLE_ALLOW_FMA)
/* Only informative: contraction is controlled by -ffp-contract=off. */
#endif

#define OR_OK 0
#define OR_ERR_INVALID (-1)
#define OR_ERR_OOM (-3)
#define OR_ERR_DEPTH (-6)

static void set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- a1: the per-pair kernel (gravity/impls/mod.rs:150-166) ------------- */
static inline void pair_f32(float xi, float yi, float zi, const float *p2, float softening,
                            int checked, float *ax, float *ay, float *az) {
    float dx = p2[0] - xi;
    float dy = p2[1] - yi;
    float dz = p2[2] - zi;
    float norm = dx * dx + dy * dy + dz * dz;
    if (checked && norm == 0.0f) {
        *ax = dx;
        *ay = dy;
        *az = dz;
        return;
    }
    float norm_s = norm + softening * softening;
    float s = p2[3] / (norm_s * sqrtf(norm_s));
    *ax = dx * s;
    *ay = dy * s;
    *az = dz * s;
}

/* ---- a2/a3: brute force (sequential.rs:181-194, parallel.rs:216-232) ----- */
int oracle_bf_f32(const float *aff, size_t n_aff, const float *src, size_t n_src,
                  float softening, int checked, float *out, int threads) {
    if ((n_aff && (!aff || !out)) || (n_src && !src)) return OR_ERR_INVALID;
    set_threads(threads);
    long long n = (long long)n_aff;
#pragma omp parallel for schedule(dynamic, 16) if (threads != 1)
    for (long long i = 0; i < n; ++i) {
        float xi = aff[4 * i + 0], yi = aff[4 * i + 1], zi = aff[4 * i + 2];
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        for (size_t j = 0; j < n_src; ++j) {
            float ax, ay, az;
            pair_f32(xi, yi, zi, src + 4 * j, softening, checked, &ax, &ay, &az);
            sx = sx + ax;
            sy = sy + ay;
            sz = sz + az;
        }
        out[3 * i + 0] = sx;
        out[3 * i + 1] = sy;
        out[3 * i + 2] = sz;
    }
    return OR_OK;
}

/* The glam Vec3A / Vec4 local kernel (particular/src/gravity/impls/glam.rs:260-275):
 * same as pair_f32 but a = (d * m) / (n_s * sqrt(n_s)) per component. */
static inline void pair_f32_vec3a(float xi, float yi, float zi, const float *p2, float softening,
                                  int checked, float *ax, float *ay, float *az) {
    float dx = p2[0] - xi;
    float dy = p2[1] - yi;
    float dz = p2[2] - zi;
    float norm = dx * dx + dy * dy + dz * dz;
    if (checked && norm == 0.0f) {
        *ax = dx;
        *ay = dy;
        *az = dz;
        return;
    }
    float norm_s = norm + softening * softening;
    float den = norm_s * sqrtf(norm_s);
    *ax = (dx * p2[3]) / den;
    *ay = (dy * p2[3]) / den;
    *az = (dz * p2[3]) / den;
}

int oracle_bf_f32_vec3a(const float *aff, size_t n_aff, const float *src, size_t n_src,
                        float softening, int checked, float *out, int threads) {
    if ((n_aff && (!aff || !out)) || (n_src && !src)) return OR_ERR_INVALID;
    set_threads(threads);
    long long n = (long long)n_aff;
#pragma omp parallel for schedule(dynamic, 16) if (threads != 1)
    for (long long i = 0; i < n; ++i) {
        float xi = aff[4 * i + 0], yi = aff[4 * i + 1], zi = aff[4 * i + 2];
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        for (size_t j = 0; j < n_src; ++j) {
            float ax, ay, az;
            pair_f32_vec3a(xi, yi, zi, src + 4 * j, softening, checked, &ax, &ay, &az);
            sx = sx + ax;
            sy = sy + ay;
            sz = sz + az;
        }
        out[3 * i + 0] = sx;
        out[3 * i + 1] = sy;
        out[3 * i + 2] = sz;
    }
    return OR_OK;
}

/* FP64 judge: the same formula in double, inputs widened from f32. */
int oracle_bf_f64(const float *aff, size_t n_aff, const float *src, size_t n_src,
                  double softening, int checked, double *out, int threads) {
    if ((n_aff && (!aff || !out)) || (n_src && !src)) return OR_ERR_INVALID;
    set_threads(threads);
    long long n = (long long)n_aff;
    double e2 = softening * softening;
#pragma omp parallel for schedule(dynamic, 16) if (threads != 1)
    for (long long i = 0; i < n; ++i) {
        double xi = aff[4 * i + 0], yi = aff[4 * i + 1], zi = aff[4 * i + 2];
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (size_t j = 0; j < n_src; ++j) {
            const float *p = src + 4 * j;
            double dx = (double)p[0] - xi, dy = (double)p[1] - yi, dz = (double)p[2] - zi;
            double norm = dx * dx + dy * dy + dz * dz;
            if (checked && norm == 0.0) continue;
            double ns = norm + e2;
            double s = (double)p[3] / (ns * sqrt(ns));
            sx += dx * s;
            sy += dy * s;
            sz += dz * s;
        }
        out[3 * i + 0] = sx;
        out[3 * i + 1] = sy;
        out[3 * i + 2] = sz;
    }
    return OR_OK;
}

/* ---- f3: glam DVec3 bodies (impl_acceleration_cpu_scalar!(DVec3, f64) at
 * particular/src/gravity/impls/glam.rs:234, the macro at gravity/impls/mod.rs:137-171):
 * the a1 kernel and the a2 fold in double. Bodies are double[4] (x, y, z, mu). */
static inline void pair_f64(double xi, double yi, double zi, const double *p2, double softening,
                            int checked, double *ax, double *ay, double *az) {
    double dx = p2[0] - xi;
    double dy = p2[1] - yi;
    double dz = p2[2] - zi;
    double norm = dx * dx + dy * dy + dz * dz;
    if (checked && norm == 0.0) {
        *ax = dx;
        *ay = dy;
        *az = dz;
        return;
    }
    double norm_s = norm + softening * softening;
    double s = p2[3] / (norm_s * sqrt(norm_s));
    *ax = dx * s;
    *ay = dy * s;
    *az = dz * s;
}

int oracle_bf_dvec3(const double *aff, size_t n_aff, const double *src, size_t n_src,
                    double softening, int checked, double *out, int threads) {
    if ((n_aff && (!aff || !out)) || (n_src && !src)) return OR_ERR_INVALID;
    set_threads(threads);
    long long n = (long long)n_aff;
#pragma omp parallel for schedule(dynamic, 16) if (threads != 1)
    for (long long i = 0; i < n; ++i) {
        double xi = aff[4 * i + 0], yi = aff[4 * i + 1], zi = aff[4 * i + 2];
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (size_t j = 0; j < n_src; ++j) {
            double ax, ay, az;
            pair_f64(xi, yi, zi, src + 4 * j, softening, checked, &ax, &ay, &az);
            sx = sx + ax;
            sy = sy + ay;
            sz = sz + az;
        }
        out[3 * i + 0] = sx;
        out[3 * i + 1] = sy;
        out[3 * i + 2] = sz;
    }
    return OR_OK;
}

/* ---- f4: BruteForcePairs (particular/src/sequential.rs:232-304: RestrictedBruteForce
 * over restrict_len = affecting_len for Ordered storage, the whole slice for a plain
 * one) with the paired kernel of gravity/impls/mod.rs:175-207: for i < restrict_len
 * and j > i, dir = d / (n_s sqrt(n_s)) with d = x_j - x_i (unchecked, mu = 1);
 * out_i gets dir * m_j (summed from zero over j, then added to out[i]) and out[j]
 * gets -dir * m_i as i advances. Bodies are float[4] / double[4]. */
int oracle_bf_pairs_f32(const float *b, size_t n, size_t restrict_len, float softening, float *out) {
    if ((n && (!b || !out)) || restrict_len > n) return OR_ERR_INVALID;
    memset(out, 0, sizeof(float) * 3 * n);
    const float one = 1.0f;
    for (size_t i = 0; i < restrict_len; ++i) {
        float oi[3] = {0.0f, 0.0f, 0.0f};
        for (size_t j = i + 1; j < n; ++j) {
            const float pj[4] = {b[4 * j + 0], b[4 * j + 1], b[4 * j + 2], one};
            float dx, dy, dz;
            pair_f32(b[4 * i + 0], b[4 * i + 1], b[4 * i + 2], pj, softening, 0, &dx, &dy, &dz);
            oi[0] = oi[0] + dx * b[4 * j + 3];
            oi[1] = oi[1] + dy * b[4 * j + 3];
            oi[2] = oi[2] + dz * b[4 * j + 3];
            out[3 * j + 0] = out[3 * j + 0] + (-dx) * b[4 * i + 3];
            out[3 * j + 1] = out[3 * j + 1] + (-dy) * b[4 * i + 3];
            out[3 * j + 2] = out[3 * j + 2] + (-dz) * b[4 * i + 3];
        }
        out[3 * i + 0] = out[3 * i + 0] + oi[0];
        out[3 * i + 1] = out[3 * i + 1] + oi[1];
        out[3 * i + 2] = out[3 * i + 2] + oi[2];
    }
    return OR_OK;
}

int oracle_bf_pairs_f64(const double *b, size_t n, size_t restrict_len, double softening, double *out) {
    if ((n && (!b || !out)) || restrict_len > n) return OR_ERR_INVALID;
    memset(out, 0, sizeof(double) * 3 * n);
    for (size_t i = 0; i < restrict_len; ++i) {
        double oi[3] = {0.0, 0.0, 0.0};
        for (size_t j = i + 1; j < n; ++j) {
            const double pj[4] = {b[4 * j + 0], b[4 * j + 1], b[4 * j + 2], 1.0};
            double dx, dy, dz;
            pair_f64(b[4 * i + 0], b[4 * i + 1], b[4 * i + 2], pj, softening, 0, &dx, &dy, &dz);
            oi[0] = oi[0] + dx * b[4 * j + 3];
            oi[1] = oi[1] + dy * b[4 * j + 3];
            oi[2] = oi[2] + dz * b[4 * j + 3];
            out[3 * j + 0] = out[3 * j + 0] + (-dx) * b[4 * i + 3];
            out[3 * j + 1] = out[3 * j + 1] + (-dy) * b[4 * i + 3];
            out[3 * j + 2] = out[3 * j + 2] + (-dz) * b[4 * i + 3];
        }
        out[3 * i + 0] = out[3 * i + 0] + oi[0];
        out[3 * i + 1] = out[3 * i + 1] + oi[1];
        out[3 * i + 2] = out[3 * i + 2] + oi[2];
    }
    return OR_OK;
}

#define SC float
#define SFX(name) name
#define SC_FMIN fminf
#define SC_FMAX fmaxf
#define PAIR pair_f32
#define BH_NAME oracle_bh_f32
#include "pt_oracle_bh.inc"
#undef SC
#undef SFX
#undef SC_FMIN
#undef SC_FMAX
#undef PAIR
#undef BH_NAME

/* ---- f3: the same tree and walk for glam DVec3 bodies (the reference's BarnesHut
 * over f64 particles: BoundingBox<DVec3>, f64 centre of mass and theta). */
#define SC double
#define SFX(name) name##_dvec3
#define SC_FMIN fmin
#define SC_FMAX fmax
#define PAIR pair_f64
#define BH_NAME oracle_bh_dvec3
#include "pt_oracle_bh.inc"
#undef SC
#undef SFX
#undef SC_FMIN
#undef SC_FMAX
#undef PAIR
#undef BH_NAME

/* ---- precision check of the walk's summation -------------------------------
 * The reference rule over an f32 orthtree exactly as oracle_bh_walk decides it (the
 * same accepted set per body), but every accepted node's term computed in double from
 * its f32 data and summed in double: out = the FP64 sum of the accepted terms, l1 =
 * the sum of the terms' norms (the scale the FP32 summation error is measured
 * against). No reference counterpart: it measures how far an FP32 sum over the
 * reference's accepted set (sequential.rs:497-500 accumulates with +=) strays from the
 * exact sum of the same terms. */
int oracle_bh_walk_sum64(const oracle_tree *t, const float *aff, size_t n_aff, float theta, float softening,
                         int checked, double *out, double *l1, int threads) {
    if (!t || (n_aff && (!aff || !out))) return OR_ERR_INVALID;
    set_threads(threads);
    long long n = (long long)n_aff;
    float th2 = theta * theta;
    int fail = 0;
#pragma omp parallel if (threads != 1)
    {
        size_t cap = 256;
        int32_t *stack = (int32_t *)malloc(cap * sizeof(int32_t));
        if (!stack) {
#pragma omp atomic write
            fail = 1;
        }
#pragma omp for schedule(dynamic, 64)
        for (long long i = 0; i < n; ++i) {
            if (!stack) continue;
            float xi = aff[4 * i + 0], yi = aff[4 * i + 1], zi = aff[4 * i + 2];
            double sx = 0.0, sy = 0.0, sz = 0.0, sa = 0.0;
            size_t sp = 0;
            if (t->root >= 0) stack[sp++] = t->root;
            while (sp) {
                int32_t id = stack[--sp];
                const float *p2 = t->data + 4 * (size_t)id;
                float dx = p2[0] - xi, dy = p2[1] - yi, dz = p2[2] - zi;
                float d2 = dx * dx + dy * dy + dz * dz;
                if (d2 == 0.0f) continue;
                const or_node *nd = &t->nodes[id];
                float w = nd->max[0] - nd->min[0];
                if (nd->internal && th2 * d2 < w * w) {
                    if (sp + 8 > cap) {
                        cap *= 2;
                        int32_t *ns = (int32_t *)realloc(stack, cap * sizeof(int32_t));
                        if (!ns) {
#pragma omp atomic write
                            fail = 1;
                            break;
                        }
                        stack = ns;
                    }
                    for (int c = 0; c < 8; ++c)
                        if (nd->child[c] >= 0) stack[sp++] = nd->child[c];
                } else {
                    const double q[4] = {p2[0], p2[1], p2[2], p2[3]};
                    double ax, ay, az;
                    pair_f64(xi, yi, zi, q, softening, checked, &ax, &ay, &az);
                    sx += ax;
                    sy += ay;
                    sz += az;
                    sa += sqrt(ax * ax + ay * ay + az * az);
                }
            }
            out[3 * i + 0] = sx;
            out[3 * i + 1] = sy;
            out[3 * i + 2] = sz;
            if (l1) l1[i] = sa;
        }
        free(stack);
    }
    return fail ? OR_ERR_OOM : OR_OK;
}
