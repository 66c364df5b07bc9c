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

/* ---- a4/a5: orthtree (tree/mod.rs:91-138, partition.rs, impls/mod.rs:120-134) */
typedef struct {
    int32_t child[8]; /* -1 = None (Option<NodeID>) */
    float min[3], max[3];
    int32_t internal; /* Node::Internal vs Node::External */
    int32_t first, count; /* range in the tree's body permutation */
} or_node;

typedef struct oracle_tree {
    or_node *nodes;
    float *data; /* 4 per node: com x,y,z, mass */
    size_t n_nodes, cap;
    int32_t root; /* -1 when empty */
    uint32_t *perm; /* body permutation: bodies of node k are perm[first..first+count) */
    size_t n_bodies;
    int max_depth;
} oracle_tree;

static int tree_push(oracle_tree *t) {
    if (t->n_nodes == t->cap) {
        size_t nc = t->cap ? t->cap * 2 : 1024;
        or_node *nn = (or_node *)realloc(t->nodes, nc * sizeof(or_node));
        if (!nn) return -1;
        t->nodes = nn;
        float *nd = (float *)realloc(t->data, nc * 4 * sizeof(float));
        if (!nd) return -1;
        t->data = nd;
        t->cap = nc;
    }
    return (int)t->n_nodes++;
}

/* centre_of_mass over the node's bodies in their (input-preserving) order. */
static void centre_of_mass(const float *src, const uint32_t *idx, size_t n, float *out4) {
    float tot = 0.0f;
    for (size_t k = 0; k < n; ++k) tot = tot + src[4 * idx[k] + 3];
    float cx = 0.0f, cy = 0.0f, cz = 0.0f;
    if (tot == 0.0f) {
        for (size_t k = 0; k < n; ++k) {
            const float *p = src + 4 * idx[k];
            cx = cx + p[0];
            cy = cy + p[1];
            cz = cz + p[2];
        }
        float len = (float)n;
        cx = cx / len;
        cy = cy / len;
        cz = cz / len;
    } else {
        for (size_t k = 0; k < n; ++k) {
            const float *p = src + 4 * idx[k];
            float q = p[3] / tot;
            cx = cx + p[0] * q;
            cy = cy + p[1] * q;
            cz = cz + p[2] * q;
        }
    }
    out4[0] = cx;
    out4[1] = cy;
    out4[2] = cz;
    out4[3] = tot;
}

static inline float midpoint(float a, float b) { return (a + b) / 2.0f; }

typedef struct {
    size_t first, count;
    float min[3], max[3];
    int32_t parent; /* node id of parent, -1 for root */
    int slot;       /* child slot in parent */
    int depth;
} build_item;

void oracle_tree_free(oracle_tree *t) {
    if (!t) return;
    free(t->nodes);
    free(t->data);
    free(t->perm);
    free(t);
}

/* Builds the reference's orthtree over the sources. max_depth guards the
 * reference's unbounded recursion (coincident-in-float pathologies). */
oracle_tree *oracle_bh_build(const float *src, size_t n_src, int max_depth) {
    oracle_tree *t = (oracle_tree *)calloc(1, sizeof(oracle_tree));
    if (!t) return NULL;
    t->root = -1;
    t->n_bodies = n_src;
    if (max_depth <= 0) max_depth = 256;
    if (n_src == 0) return t;
    t->perm = (uint32_t *)malloc(n_src * sizeof(uint32_t));
    uint32_t *tmp = (uint32_t *)malloc(n_src * sizeof(uint32_t));
    size_t stack_cap = 1024, sp = 0;
    build_item *stack = (build_item *)malloc(stack_cap * sizeof(build_item));
    if (!t->perm || !tmp || !stack) goto fail;
    for (size_t i = 0; i < n_src; ++i) t->perm[i] = (uint32_t)i;

    /* BoundingBox::square_with (partition.rs:274-292) */
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n_src; ++i)
        for (int a = 0; a < 3; ++a) {
            float v = src[4 * i + a];
            mn[a] = fminf(mn[a], v);
            mx[a] = fmaxf(mx[a], v);
        }
    float center[3], half = 0.0f;
    for (int a = 0; a < 3; ++a) center[a] = midpoint(mn[a], mx[a]);
    for (int a = 0; a < 3; ++a) half = fmaxf(half, mx[a] - mn[a]);
    half = midpoint(half, 0.0f);
    build_item root;
    root.first = 0;
    root.count = n_src;
    for (int a = 0; a < 3; ++a) {
        root.min[a] = center[a] - half;
        root.max[a] = center[a] + half;
    }
    root.parent = -1;
    root.slot = 0;
    root.depth = 0;
    stack[sp++] = root;

    while (sp) {
        build_item it = stack[--sp];
        int id = tree_push(t);
        if (id < 0) goto fail;
        if (it.parent < 0) t->root = id;
        else t->nodes[it.parent].child[it.slot] = id;
        if (it.depth > t->max_depth) t->max_depth = it.depth;
        or_node *nd = &t->nodes[id];
        for (int c = 0; c < 8; ++c) nd->child[c] = -1;
        memcpy(nd->min, it.min, sizeof it.min);
        memcpy(nd->max, it.max, sizeof it.max);
        nd->internal = 0;
        nd->first = (int32_t)it.first;
        nd->count = (int32_t)it.count;
        uint32_t *idx = t->perm + it.first;
        centre_of_mass(src, idx, it.count, t->data + 4 * (size_t)id);

        int differs = 0;
        for (size_t k = 1; k < it.count && !differs; ++k) {
            const float *a = src + 4 * idx[k - 1], *b = src + 4 * idx[k];
            differs = (a[0] != b[0]) || (a[1] != b[1]) || (a[2] != b[2]);
        }
        if (!differs) continue;
        if (it.depth >= max_depth) goto fail_depth;
        nd->internal = 1;
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = midpoint(it.min[a], it.max[a]);
        /* Stable bucketing into the 8 orthants (tree/mod.rs:119-126). */
        size_t cnt[8] = {0};
        unsigned char *oct = (unsigned char *)malloc(it.count);
        if (!oct) goto fail;
        for (size_t k = 0; k < it.count; ++k) {
            const float *p = src + 4 * idx[k];
            int o = (p[0] < c[0]) | ((p[1] < c[1]) << 1) | ((p[2] < c[2]) << 2);
            oct[k] = (unsigned char)o;
            cnt[o]++;
        }
        size_t off[8], acc = 0;
        for (int o = 0; o < 8; ++o) {
            off[o] = acc;
            acc += cnt[o];
        }
        size_t pos[8];
        memcpy(pos, off, sizeof off);
        for (size_t k = 0; k < it.count; ++k) tmp[pos[oct[k]]++] = idx[k];
        memcpy(idx, tmp, it.count * sizeof(uint32_t));
        free(oct);
        /* Children are built depth first in orthant order 0..7 (node ids in
         * preorder, as the reference's recursion assigns them): push 7..0. */
        if (sp + 8 > stack_cap) {
            stack_cap *= 2;
            build_item *ns = (build_item *)realloc(stack, stack_cap * sizeof(build_item));
            if (!ns) goto fail;
            stack = ns;
        }
        for (int o = 7; o >= 0; --o) {
            if (!cnt[o]) continue; /* empty input -> None (tree/mod.rs:104-106) */
            build_item ch;
            ch.first = it.first + off[o];
            ch.count = cnt[o];
            for (int a = 0; a < 3; ++a) {
                if ((o >> a) & 1) { /* subdivide: bit set -> lower half */
                    ch.min[a] = it.min[a];
                    ch.max[a] = c[a];
                } else {
                    ch.min[a] = c[a];
                    ch.max[a] = it.max[a];
                }
            }
            ch.parent = id;
            ch.slot = o;
            ch.depth = it.depth + 1;
            stack[sp++] = ch;
        }
    }
    free(tmp);
    free(stack);
    return t;
fail_depth:
    t->max_depth = -1;
fail:
    free(tmp);
    free(stack);
    if (t && t->max_depth == -1) {
        /* keep the handle so the caller can read the depth failure */
        t->n_nodes = 0;
        t->root = -1;
        return t;
    }
    oracle_tree_free(t);
    return NULL;
}

size_t oracle_tree_node_count(const oracle_tree *t) { return t ? t->n_nodes : 0; }
int oracle_tree_max_depth(const oracle_tree *t) { return t ? t->max_depth : -1; }

/* Exports per node: internal flag, child ids (8), box (6 floats), data (4),
 * body range. Any pointer may be NULL. */
int oracle_tree_export(const oracle_tree *t, int32_t *internal, int32_t *child, float *box,
                       float *data, int32_t *range, uint32_t *perm) {
    if (!t) return OR_ERR_INVALID;
    for (size_t k = 0; k < t->n_nodes; ++k) {
        const or_node *n = &t->nodes[k];
        if (internal) internal[k] = n->internal;
        if (child) memcpy(child + 8 * k, n->child, 8 * sizeof(int32_t));
        if (box) {
            memcpy(box + 6 * k, n->min, 3 * sizeof(float));
            memcpy(box + 6 * k + 3, n->max, 3 * sizeof(float));
        }
        if (data) memcpy(data + 4 * k, t->data + 4 * k, 4 * sizeof(float));
        if (range) {
            range[2 * k] = n->first;
            range[2 * k + 1] = n->count;
        }
    }
    if (perm && t->n_bodies) memcpy(perm, t->perm, t->n_bodies * sizeof(uint32_t));
    return OR_OK;
}

/* ---- a6/a7: the walk (sequential.rs:466-505; parallel.rs:342-367) ------- */
int oracle_bh_walk(const oracle_tree *t, const float *aff, size_t n_aff, float theta,
                   float softening, int checked, float *out, uint32_t *accepted, int threads) {
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
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
            uint32_t nacc = 0;
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
                    float ax, ay, az;
                    pair_f32(xi, yi, zi, p2, softening, checked, &ax, &ay, &az);
                    sx += ax;
                    sy += ay;
                    sz += az;
                    nacc++;
                }
            }
            out[3 * i + 0] = sx;
            out[3 * i + 1] = sy;
            out[3 * i + 2] = sz;
            if (accepted) accepted[i] = nacc;
        }
        free(stack);
    }
    return fail ? OR_ERR_OOM : OR_OK;
}

/* Barnes-Hut over slices: tree over `src`, walk for every target
 * (sequential.rs:526-543 with the walk above). */
int oracle_bh_f32(const float *aff, size_t n_aff, const float *src, size_t n_src, float theta,
                  float softening, int checked, float *out, uint32_t *accepted, int threads) {
    oracle_tree *t = oracle_bh_build(src, n_src, 0);
    if (!t) return OR_ERR_OOM;
    if (t->max_depth < 0) {
        oracle_tree_free(t);
        return OR_ERR_DEPTH;
    }
    int rc = oracle_bh_walk(t, aff, n_aff, theta, softening, checked, out, accepted, threads);
    oracle_tree_free(t);
    return rc;
}
