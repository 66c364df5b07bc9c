/*
 * learned_ceiling.c -- test infrastructure, not part of the product path.
 *
 * Bounds what a learned correction of accepted Barnes-Hut cells can gain, in FP64 on
 * the CPU. It models the GPU's group walk: an octree over the bodies (the reference's
 * subdivision, tree/mod.rs:91-138: square root box, split at the cell centre, a leaf
 * per distinct position), groups of 64 consecutive bodies in tree order, a cell opened
 * for the whole group when any of its bodies opens it, accepted cells evaluated with
 * their monopole + traceless quadrupole about the centre of mass (the
 * PT_BH_QUADRUPOLE term), single bodies exactly.
 *
 * Opening rules, per group:
 *   near cells (centre of mass within kfar x R of the group's box centre, R the box's
 *   half diagonal -- the local expansion's far test at ratio 1/kfar): opened when
 *   theta^2 d^2 < w^2 for a group body, or when M w^3 / d^5 > alpha_near |a|;
 *   far cells: the same with alpha_far.
 * |a| is the FP64 acceleration at the group's box centre.
 *
 * A far accepted cell that the inner rule (theta_in, alpha_in) would open is
 * "marginal": a learned correction would add the residual r(x) = exact(x) - (monopole
 * + quadrupole)(x) of it. For every sampled body the program reports the FP64-judged
 * error of:
 *   plain   no correction;
 *   r0      r(g), the residual at the group's box centre g (one value per group);
 *   r0+J    r(g) + J(g) (x - g), J the residual's Jacobian (central differences);
 *   exact   r(x) at the body itself;
 *   noisy   r0+J with Gaussian noise of NOISE x the outputs' RMS per cell (env NOISE);
 *   net     r0+J predicted by a 12 -> 64 -> 64 -> 8 GELU network (env NET: weights
 *           W1[64][12] b1 W2[64][64] b2 W3[8][64] b3 scale[8], float32), from the
 *           learned correction's features at g (unit offset, w/|r|, quadrupole /
 *           (M w^2), (centre of mass - cell centre) / w).
 * With a dump path it writes, per marginal cell and group, the 12 features, r(g) / (M /
 * |r|^2), the symmetric J(g) / (M / |r|^3) (xx xy xz yy yz zz), the cell's body count,
 * the group index and R / |r| (24 float32) -- training data for such a network.
 *
 * Usage: learned_ceiling bodies.bin n_sample theta theta_in alpha_far alpha_in
 *                       alpha_near kfar [dump.bin]
 *   bodies.bin: float32 (x, y, z, mass) rows; n_sample 0 with env ALLGROUPS walks
 *   every group (one body each) and skips the judge (data generation).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double x, y, z, m;
} Body;

typedef struct {
    double cx, cy, cz, m;  /* centre of mass, mass */
    double q[6];           /* traceless quadrupole about the centre of mass: xx xy xz yy yz zz */
    double gx, gy, gz, w;  /* cell centre, width */
    int first, count, skip, leaf;
} Node;

static Body *B;
static Node *T;
static int NT, CAPT;
static int *perm, *tmp;
static double EPS2 = 1e-4; /* softening 0.01 */

static int push_node(void) {
    if (NT == CAPT) {
        CAPT = CAPT ? 2 * CAPT : 1 << 20;
        T = realloc(T, sizeof(Node) * (size_t)CAPT);
    }
    return NT++;
}

static void moments(Node *n) {
    double m = 0, x = 0, y = 0, z = 0;
    for (int i = n->first; i < n->first + n->count; ++i) {
        Body b = B[perm[i]];
        m += b.m, x += b.x * b.m, y += b.y * b.m, z += b.z * b.m;
    }
    n->m = m, n->cx = x / m, n->cy = y / m, n->cz = z / m;
    memset(n->q, 0, sizeof n->q);
    for (int i = n->first; i < n->first + n->count; ++i) {
        Body b = B[perm[i]];
        double rx = b.x - n->cx, ry = b.y - n->cy, rz = b.z - n->cz, r2 = rx * rx + ry * ry + rz * rz;
        n->q[0] += b.m * (3 * rx * rx - r2), n->q[1] += b.m * 3 * rx * ry, n->q[2] += b.m * 3 * rx * rz;
        n->q[3] += b.m * (3 * ry * ry - r2), n->q[4] += b.m * 3 * ry * rz, n->q[5] += b.m * (3 * rz * rz - r2);
    }
}

static void build(int first, int count, double gx, double gy, double gz, double w, int depth) {
    int id = push_node();
    T[id].first = first, T[id].count = count, T[id].gx = gx, T[id].gy = gy, T[id].gz = gz, T[id].w = w;
    T[id].leaf = 0;
    moments(&T[id]);
    int same = 1;
    for (int i = first + 1; i < first + count && same; ++i) {
        Body a = B[perm[i]], b = B[perm[first]];
        if (a.x != b.x || a.y != b.y || a.z != b.z) same = 0;
    }
    if (count == 1 || same || depth > 40) {
        T[id].leaf = 1;
        T[id].skip = NT;
        return;
    }
    int cnt[8] = {0}, off[8], pos[8], s = 0;
    for (int i = first; i < first + count; ++i) {
        Body b = B[perm[i]];
        cnt[(b.x < gx ? 0 : 1) | (b.y < gy ? 0 : 2) | (b.z < gz ? 0 : 4)]++;
    }
    for (int o = 0; o < 8; ++o) off[o] = pos[o] = s, s += cnt[o];
    for (int i = first; i < first + count; ++i) {
        Body b = B[perm[i]];
        tmp[first + pos[(b.x < gx ? 0 : 1) | (b.y < gy ? 0 : 2) | (b.z < gz ? 0 : 4)]++] = perm[i];
    }
    memcpy(perm + first, tmp + first, sizeof(int) * (size_t)count);
    for (int o = 0; o < 8; ++o)
        if (cnt[o]) {
            double h = w / 4;
            build(first + off[o], cnt[o], gx + ((o & 1) ? h : -h), gy + ((o & 2) ? h : -h), gz + ((o & 4) ? h : -h),
                  w / 2, depth + 1);
        }
    T[id].skip = NT;
}

/* monopole + quadrupole field of node n at t (d = centre of mass - t, softened) */
static void mq(const Node *n, const double *t, double *a) {
    double dx = n->cx - t[0], dy = n->cy - t[1], dz = n->cz - t[2];
    double s = dx * dx + dy * dy + dz * dz + EPS2, inv = 1 / sqrt(s), inv2 = inv * inv, sc = n->m * inv * inv2;
    a[0] = dx * sc, a[1] = dy * sc, a[2] = dz * sc;
    if (!n->leaf) {
        const double *q = n->q;
        double ux = q[0] * dx + q[1] * dy + q[2] * dz, uy = q[1] * dx + q[3] * dy + q[4] * dz,
               uz = q[2] * dx + q[4] * dy + q[5] * dz;
        double c = dx * ux + dy * uy + dz * uz, inv5 = inv2 * inv2 * inv, c7 = 2.5 * c * inv5 * inv2;
        a[0] += c7 * dx - ux * inv5, a[1] += c7 * dy - uy * inv5, a[2] += c7 * dz - uz * inv5;
    }
}

/* exact sum over the bodies of node n at t */
static void exact(const Node *n, const double *t, double *a) {
    double ax = 0, ay = 0, az = 0;
    for (int i = n->first; i < n->first + n->count; ++i) {
        Body b = B[perm[i]];
        double dx = b.x - t[0], dy = b.y - t[1], dz = b.z - t[2], r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == 0) continue;
        double inv = 1 / sqrt(r2 + EPS2), s = b.m * inv * inv * inv;
        ax += dx * s, ay += dy * s, az += dz * s;
    }
    a[0] = ax, a[1] = ay, a[2] = az;
}

static void resid(const Node *n, const double *t, double *r) {
    double e[3], m[3];
    exact(n, t, e);
    mq(n, t, m);
    for (int k = 0; k < 3; ++k) r[k] = e[k] - m[k];
}

static void brute(int n, const double *t, double *a) {
    double ax = 0, ay = 0, az = 0;
    for (int i = 0; i < n; ++i) {
        double dx = B[i].x - t[0], dy = B[i].y - t[1], dz = B[i].z - t[2], r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == 0) continue;
        double inv = 1 / sqrt(r2 + EPS2), s = B[i].m * inv * inv * inv;
        ax += dx * s, ay += dy * s, az += dz * s;
    }
    a[0] = ax, a[1] = ay, a[2] = az;
}

static double gelu(double z) { return 0.5 * z * (1 + tanh(0.7978845608028654 * (z + 0.044715 * z * z * z))); }

static int cmpd(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static void report(const char *name, const double *e, int n) {
    double *c = malloc(sizeof(double) * (size_t)n);
    memcpy(c, e, sizeof(double) * (size_t)n);
    qsort(c, (size_t)n, sizeof(double), cmpd);
    printf("%s p50 %.3e p95 %.3e max %.3e\n", name, c[n / 2], c[(int)(0.95 * (n - 1))], c[n - 1]);
    free(c);
}

static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* standard normal from two hashed uniforms (Box-Muller) */
static double gauss(uint64_t key) {
    double u1 = ((mix(key) >> 11) + 0.5) / 9007199254740992.0;
    double u2 = ((mix(key ^ 0x9E3779B97F4A7C15ull) >> 11) + 0.5) / 9007199254740992.0;
    return sqrt(-2 * log(u1)) * cos(6.283185307179586 * u2);
}

int main(int argc, char **argv) {
    if (argc < 9) {
        fprintf(stderr, "usage: %s bodies.bin n_sample theta theta_in alpha_far alpha_in alpha_near kfar [dump]\n",
                argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    int N = (int)(sz / 16);
    float *raw = malloc((size_t)sz);
    if (fread(raw, 1, (size_t)sz, f) != (size_t)sz) return 2;
    fclose(f);
    B = malloc(sizeof(Body) * (size_t)N);
    for (int i = 0; i < N; ++i) B[i].x = raw[4 * i], B[i].y = raw[4 * i + 1], B[i].z = raw[4 * i + 2], B[i].m = raw[4 * i + 3];
    int ns = atoi(argv[2]);
    double th = atof(argv[3]), thin = atof(argv[4]), alpha = atof(argv[5]), alin = atof(argv[6]),
           alnear = atof(argv[7]), kfar = atof(argv[8]);
    const char *dump = argc > 9 ? argv[9] : NULL;
    const double noise = getenv("NOISE") ? atof(getenv("NOISE")) : 0.0;
    perm = malloc(sizeof(int) * (size_t)N);
    tmp = malloc(sizeof(int) * (size_t)N);
    for (int i = 0; i < N; ++i) perm[i] = i;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; ++i) {
        double v[3] = {B[i].x, B[i].y, B[i].z};
        for (int k = 0; k < 3; ++k) mn[k] = fmin(mn[k], v[k]), mx[k] = fmax(mx[k], v[k]);
    }
    build(0, N, (mn[0] + mx[0]) / 2, (mn[1] + mx[1]) / 2, (mn[2] + mx[2]) / 2,
          fmax(mx[0] - mn[0], fmax(mx[1] - mn[1], mx[2] - mn[2])), 0);
    int all = getenv("ALLGROUPS") != NULL;
    if (all) ns = (N + 63) / 64;
    int *samp = malloc(sizeof(int) * (size_t)ns);
    uint64_t s = 12345;
    for (int i = 0; i < ns; ++i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        samp[i] = all ? 64 * i : (int)((s >> 33) % (uint64_t)N);
    }
    static float NW[12 * 64 + 64 + 64 * 64 + 64 + 8 * 64 + 8 + 8];
    int have_net = 0;
    if (getenv("NET")) {
        FILE *nf = fopen(getenv("NET"), "rb");
        have_net = nf && fread(NW, sizeof NW, 1, nf) == 1;
        if (nf) fclose(nf);
    }
    /* RMS of the outputs (r0 x3, J xx xy xz yy yz) for the noise model */
    static const double rms[8] = {0.0096, 0.0094, 0.0083, 0.043, 0.039, 0.030, 0.045, 0.032};
    double *err[6];
    for (int k = 0; k < 6; ++k) err[k] = calloc((size_t)ns, sizeof(double));
    long long ent = 0, nmarg = 0, vnear = 0, vfar = 0, afar = 0;
    FILE *df = dump ? fopen(dump, "wb") : NULL;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : ent, nmarg, vnear, vfar, afar)
    for (int si = 0; si < ns; ++si) {
        int tpos = samp[si], g0 = tpos / 64 * 64, g1 = g0 + 64 < N ? g0 + 64 : N;
        Body tb = B[perm[tpos]];
        double t[3] = {tb.x, tb.y, tb.z};
        double bmn[3] = {1e300, 1e300, 1e300}, bmx[3] = {-1e300, -1e300, -1e300};
        for (int i = g0; i < g1; ++i) {
            double v[3] = {B[perm[i]].x, B[perm[i]].y, B[perm[i]].z};
            for (int k = 0; k < 3; ++k) bmn[k] = fmin(bmn[k], v[k]), bmx[k] = fmax(bmx[k], v[k]);
        }
        double g[3] = {(bmn[0] + bmx[0]) / 2, (bmn[1] + bmx[1]) / 2, (bmn[2] + bmx[2]) / 2};
        double R = 0.5 * sqrt((bmx[0] - bmn[0]) * (bmx[0] - bmn[0]) + (bmx[1] - bmn[1]) * (bmx[1] - bmn[1]) +
                              (bmx[2] - bmn[2]) * (bmx[2] - bmn[2]));
        double ifar = 0, iin = 0, inear = 0;
        if (alpha > 0 || alin > 0 || alnear > 0) {
            double a[3];
            brute(N, g, a);
            double am = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            ifar = alpha > 0 ? 1 / (alpha * am) : 0;
            iin = alin > 0 ? 1 / (alin * am) : 0;
            inear = alnear > 0 ? 1 / (alnear * am) : 0;
        }
        double dl[3] = {t[0] - g[0], t[1] - g[1], t[2] - g[2]};
        double acc[3] = {0, 0, 0}, cor[6][3];
        memset(cor, 0, sizeof cor);
        for (int node = 0; node < NT;) {
            const Node *n = &T[node];
            int open_far = 0, open_near = 0, open_in = 0;
            if (!n->leaf) {
                double w2 = n->w * n->w, mw3 = n->m * n->w * w2;
                double rf = ifar > 0 ? pow(mw3 * ifar, 0.4) : 0, ri = iin > 0 ? pow(mw3 * iin, 0.4) : 0,
                       rn = inear > 0 ? pow(mw3 * inear, 0.4) : 0;
                for (int i = g0; i < g1; ++i) {
                    double dx = n->cx - B[perm[i]].x, dy = n->cy - B[perm[i]].y, dz = n->cz - B[perm[i]].z;
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 == 0) continue;
                    if (th * th * d2 < w2 || d2 < rf) open_far = 1;
                    if (th * th * d2 < w2 || d2 < rn) open_near = 1;
                    if (thin * thin * d2 < w2 || d2 < ri) open_in = 1;
                }
            }
            double hx = n->cx - g[0], hy = n->cy - g[1], hz = n->cz - g[2];
            int near = hx * hx + hy * hy + hz * hz <= kfar * kfar * R * R;
            int open = near ? open_near : open_far;
            if (near) vnear++;
            else vfar++;
            if (open) {
                node++;
                continue;
            }
            if (!near) afar++;
            double dx = n->cx - t[0], dy = n->cy - t[1], dz = n->cz - t[2];
            if (dx * dx + dy * dy + dz * dz > 0) {
                double a[3];
                if (n->leaf) exact(n, t, a);
                else mq(n, t, a);
                for (int k = 0; k < 3; ++k) acc[k] += a[k];
                ent++;
                if (!n->leaf && !near && open_in && n->m > 0) {
                    nmarg++;
                    double rt[3], r0[3], J[3][3];
                    resid(n, t, rt);
                    resid(n, g, r0);
                    double rx = g[0] - n->cx, ry = g[1] - n->cy, rz = g[2] - n->cz, r = sqrt(rx * rx + ry * ry + rz * rz);
                    double h = 1e-4 * r;
                    for (int c = 0; c < 3; ++c) {
                        double pp[3] = {g[0], g[1], g[2]}, pm[3] = {g[0], g[1], g[2]}, rp[3], rm[3];
                        pp[c] += h, pm[c] -= h;
                        resid(n, pp, rp);
                        resid(n, pm, rm);
                        for (int k = 0; k < 3; ++k) J[k][c] = (rp[k] - rm[k]) / (2 * h);
                    }
                    double sc = n->m / (r * r), sj = sc / r, w2 = n->m * n->w * n->w;
                    double y[8] = {r0[0] / sc, r0[1] / sc, r0[2] / sc, J[0][0] / sj, 0.5 * (J[0][1] + J[1][0]) / sj,
                                   0.5 * (J[0][2] + J[2][0]) / sj, J[1][1] / sj, 0.5 * (J[1][2] + J[2][1]) / sj};
                    float feat[12] = {(float)(rx / r), (float)(ry / r), (float)(rz / r), (float)(n->w / r),
                                      (float)(n->q[0] / w2), (float)(n->q[1] / w2), (float)(n->q[2] / w2),
                                      (float)(n->q[3] / w2), (float)(n->q[4] / w2),
                                      (float)((n->cx - n->gx) / n->w), (float)((n->cy - n->gy) / n->w),
                                      (float)((n->cz - n->gz) / n->w)};
                    double yn[8], yp[8];
                    for (int k = 0; k < 8; ++k) yn[k] = y[k] + noise * rms[k] * gauss(((uint64_t)node << 8) + (uint64_t)k);
                    if (have_net) {
                        const float *W1 = NW, *b1 = W1 + 768, *W2 = b1 + 64, *b2 = W2 + 4096, *W3 = b2 + 64,
                                    *b3 = W3 + 512, *s8 = b3 + 8;
                        double h1[64], h2[64];
                        for (int j = 0; j < 64; ++j) {
                            double z = b1[j];
                            for (int i = 0; i < 12; ++i) z += W1[j * 12 + i] * feat[i];
                            h1[j] = gelu(z);
                        }
                        for (int j = 0; j < 64; ++j) {
                            double z = b2[j];
                            for (int i = 0; i < 64; ++i) z += W2[j * 64 + i] * h1[i];
                            h2[j] = gelu(z);
                        }
                        for (int c = 0; c < 8; ++c) {
                            double z = b3[c];
                            for (int i = 0; i < 64; ++i) z += W3[c * 64 + i] * h2[i];
                            yp[c] = z * s8[c];
                        }
                    }
                    const double *src[2] = {yn, yp};
                    for (int v = 0; v < 2; ++v) {
                        const double *u = src[v];
                        double Jn[3][3] = {{u[3], u[4], u[5]}, {u[4], u[6], u[7]}, {u[5], u[7], -u[3] - u[6]}};
                        for (int k = 0; k < 3; ++k)
                            cor[4 + v][k] += sc * u[k] + sj * (Jn[k][0] * dl[0] + Jn[k][1] * dl[1] + Jn[k][2] * dl[2]);
                    }
                    for (int k = 0; k < 3; ++k) {
                        cor[1][k] += r0[k];
                        cor[2][k] += r0[k] + J[k][0] * dl[0] + J[k][1] * dl[1] + J[k][2] * dl[2];
                        cor[3][k] += rt[k];
                    }
                    if (df) {
                        float rec[24];
                        memcpy(rec, feat, sizeof feat);
                        rec[12] = (float)y[0], rec[13] = (float)y[1], rec[14] = (float)y[2];
                        rec[15] = (float)y[3], rec[16] = (float)y[4], rec[17] = (float)y[5];
                        rec[18] = (float)y[6], rec[19] = (float)y[7], rec[20] = (float)(J[2][2] / sj);
                        rec[21] = (float)n->count, rec[22] = (float)si, rec[23] = (float)(R / r);
#pragma omp critical
                        fwrite(rec, sizeof rec, 1, df);
                    }
                }
            }
            node = n->skip;
        }
        if (all) continue;
        double ref[3];
        brute(N, t, ref);
        double rn = sqrt(ref[0] * ref[0] + ref[1] * ref[1] + ref[2] * ref[2]);
        for (int v = 0; v < 6; ++v) {
            double e2 = 0;
            for (int k = 0; k < 3; ++k) {
                double d = acc[k] + cor[v][k] - ref[k];
                e2 += d * d;
            }
            err[v][si] = sqrt(e2) / rn;
        }
    }
    if (df) fclose(df);
    printf("N %d theta %g theta_in %g alpha_far %g alpha_in %g alpha_near %g kfar %g samples %d\n", N, th, thin, alpha,
           alin, alnear, kfar, ns);
    printf("entries/body %.1f marginal/group %.1f visits near %.1f far %.1f far accepted %.1f\n", (double)ent / ns,
           (double)nmarg / ns, (double)vnear / ns, (double)vfar / ns, (double)afar / ns);
    if (all) return 0;
    const char *names[6] = {"plain ", "r0    ", "r0+J  ", "exact ", "noisy ", "net   "};
    for (int v = 0; v < 6; ++v)
        if ((v != 4 || noise > 0) && (v != 5 || have_net)) report(names[v], err[v], ns);
    return 0;
}
