// The reference's known-answer tests, on the cuda methods, through the C++ host
// mirror (include/particular_cuda.hpp):
//   acceleration_error!  particular/src/gravity/newtonian/mod.rs:228-277
//   circular_orbit!      particular/src/gravity/newtonian/mod.rs:281-347
// run like tests_algorithms_gpu! (mod.rs:474-521): 100 orbits, tolerances 1e-2
// (Barnes-Hut theta 0.5: 5e-1 and 1e-1, mod.rs:415-420).
// Exit status 0 when every case passes; one line per case on stdout.
#include <cmath>
#include <cstdio>
#include <functional>
#include <vector>

#include "particular_cuda.hpp"

using namespace particular;

struct Body {  // what #[derive(Position, Mass)] would accept
    Vec3 position;
    float mu;
};

using Compute = std::function<std::vector<Vec3>(const Reordered<Body> &)>;
using ComputeSlice = std::function<std::vector<Vec3>(const std::vector<Body> &)>;

static bool acceleration_error(const Compute &compute, float epsilon, const char *name) {
    const std::vector<Body> massive = {{Vec3::splat(0.f), 20.f}, {Vec3::splat(1.f), 30.f}, {Vec3::splat(-3.f), 40.f}};
    const std::vector<Body> particles = {{Vec3::splat(10.f), 0.f}, massive[0], massive[1], massive[2],
                                         {Vec3::splat(30.f), 0.f}, {Vec3::splat(-45.f), 0.f}};
    Reordered<Body> reordered{Slice<Body>(particles)};
    const auto computed = compute(reordered);
    bool ok = computed.size() == particles.size();
    float worst = 0.f;
    for (size_t k = 0; ok && k < particles.size(); ++k) {
        Vec3 acc;
        for (const auto &m2 : massive) {
            const Vec3 dir = m2.position - particles[k].position;
            const float mag2 = dir.length_squared();
            if (mag2 != 0.f) acc += dir * m2.mu * std::sqrt(1.f / mag2) * (1.f / mag2);
        }
        const Vec3 c = computed[k];
        const float ex = 1.f - c.x / acc.x, ey = 1.f - c.y / acc.y, ez = 1.f - c.z / acc.z;
        const float err = std::sqrt(ex * ex + ey * ey + ez * ez);
        worst = std::fmax(worst, err);
        ok = ok && err <= epsilon;
    }
    std::printf("%-40s acceleration_error max %.3e (<= %.1e) %s\n", name, worst, epsilon, ok ? "ok" : "FAIL");
    return ok;
}

static bool circular_orbit(const ComputeSlice &compute, int orbit_count, float epsilon, const char *name) {
    const float DT = 1.0f / 60.0f;
    std::vector<Body> particles = {{Vec3(0.f, 0.f, 0.f), 1e6f}, {Vec3(100.f, 0.f, 0.f), 0.f}};
    std::vector<Vec3> velocities = {Vec3(), Vec3(0.f, 100.f, 0.f)};
    auto dist = [&] { return std::sqrt((particles[0].position - particles[1].position).length_squared()); };
    auto energy = [&](float r) { return -(particles[0].mu + particles[1].mu) / (r + r); };
    const float d0 = dist(), e0 = energy(d0);
    const float period = 6.2831853f * std::sqrt((d0 * d0 * d0) / particles[0].mu);
    const int steps = int(std::lround(period / DT));
    for (int s = 0; s < steps * orbit_count; ++s) {
        const auto acc = compute(particles);
        for (size_t i = 0; i < particles.size(); ++i) velocities[i] += acc[i] * DT;
        for (size_t i = 0; i < particles.size(); ++i) particles[i].position += velocities[i] * DT;
    }
    const float d1 = dist(), e1 = energy(d1);
    const float ed = std::fabs(1.f - d0 / d1), ee = std::fabs(1.f - e0 / e1);
    const bool ok = ed < epsilon && ee < epsilon;
    std::printf("%-40s circular_orbit distance %.3e energy %.3e (< %.1e) %s\n", name, ed, ee, epsilon,
                ok ? "ok" : "FAIL");
    return ok;
}

int main() {
    cuda::CudaResources res(0);
    bool ok = true;
    for (bool exact : {false, true}) {
        cuda::BruteForce<Acceleration<true>> bf{res, acceleration_checked(), exact};
        const char *name = exact ? "cuda::BruteForce (exact)" : "cuda::BruteForce";
        ok &= acceleration_error([&](const Reordered<Body> &r) { return bf.compute(r); }, 1e-2f, name);
        ok &= circular_orbit([&](const std::vector<Body> &p) { return bf.compute(p); }, 100, 1e-2f, name);
    }
    struct Case {
        float theta;
        uint32_t flags;
        float err, orbit;
        const char *name;
    };
    const Case cases[] = {{0.f, 0, 1e-2f, 1e-2f, "cuda::BarnesHut(0.0)"},
                          {0.5f, 0, 5e-1f, 1e-1f, "cuda::BarnesHut(0.5)"},
                          {0.5f, PT_BH_GROUP | PT_BH_QUADRUPOLE, 5e-1f, 1e-1f, "cuda::BarnesHut(0.5, quad+group)"},
                          {1.0f, PT_BH_GROUP | PT_BH_QUADRUPOLE | PT_BH_LOCAL | PT_BH_RELATIVE, 5e-1f, 1e-1f,
                           "cuda::BarnesHut(1.0, headline)"}};
    for (const auto &c : cases) {
        cuda::BarnesHut<float, Acceleration<true>> bh{c.theta, res, acceleration_checked(), c.flags, 2.75e-3f};
        ok &= acceleration_error([&](const Reordered<Body> &r) { return bh.compute(r); }, c.err, c.name);
        ok &= circular_orbit([&](const std::vector<Body> &p) { return bh.compute(p); }, 100, c.orbit, c.name);
    }
    // the sugar and the Between storage
    std::vector<Body> few = {{Vec3(0, 0, 0), 1.f}, {Vec3(1, 0, 0), 2.f}, {Vec3(0, 2, 0), 3.f}};
    const auto a1 = cuda::cuda_brute_force(few, res, softened_checked(0.01f));
    const auto a2 = cuda::BruteForce<AccelerationSoftened<float, true>>{res, softened_checked(0.01f)}.compute(
        between(Slice<Body>(few), Slice<Body>(few)));
    bool same = a1.size() == 3;
    for (size_t i = 0; same && i < 3; ++i) same = a1[i].x == a2[i].x && a1[i].y == a2[i].y && a1[i].z == a2[i].z;
    std::printf("%-40s %s\n", "cuda_brute_force == BruteForce(Between)", same ? "ok" : "FAIL");
    ok &= same;

    // DVec3 bodies: the f64 path, equal to the reference's scalar f64 kernel and fold
    // (gravity/impls/mod.rs:150-166, sequential.rs:189-193) evaluated here in double
    struct Body64 {
        DVec3 position;
        double mu;
    };
    std::vector<Body64> b64;
    for (int i = 0; i < 257; ++i)
        b64.push_back({DVec3(std::sin(1.1 * i), std::cos(0.7 * i) * 2.0, 1e-3 * i), 0.5 + (i % 7) * 0.25});
    b64[5].position = b64[3].position;  // a coincident pair (checked: zero)
    const auto g64 = cuda::cuda_brute_force(b64, res, softened_checked(1e-3));
    bool exact64 = g64.size() == b64.size();
    for (size_t i = 0; exact64 && i < b64.size(); ++i) {
        volatile double sx = 0.0, sy = 0.0, sz = 0.0;  // kept in double, no contraction
        for (size_t j = 0; j < b64.size(); ++j) {
            volatile double dx = b64[j].position.x - b64[i].position.x;
            volatile double dy = b64[j].position.y - b64[i].position.y;
            volatile double dz = b64[j].position.z - b64[i].position.z;
            volatile double dxx = dx * dx, dyy = dy * dy, dzz = dz * dz;
            volatile double n2 = dxx + dyy;
            volatile double n = n2 + dzz;
            if (n == 0.0) {
                sx = sx + dx;
                sy = sy + dy;
                sz = sz + dz;
                continue;
            }
            volatile double ns = n + 1e-3 * 1e-3;
            volatile double den = ns * std::sqrt(double(ns));
            volatile double q = b64[j].mu / den;
            volatile double ax = dx * q, ay = dy * q, az = dz * q;
            sx = sx + ax;
            sy = sy + ay;
            sz = sz + az;
        }
        exact64 = g64[i].x == sx && g64[i].y == sy && g64[i].z == sz;
    }
    std::printf("%-40s %s\n", "cuda::BruteForce over DVec3 (bit-exact)", exact64 ? "ok" : "FAIL");
    ok &= exact64;
    // and Barnes-Hut over DVec3 at theta 0: every leaf, the same sums up to order
    cuda::BarnesHut<double, AccelerationSoftened<double, true>> bh64{0.0, res, softened_checked(1e-3)};
    const auto h64 = bh64.compute(b64);
    double worst64 = 0.0, scale64 = 0.0;
    for (size_t i = 0; i < b64.size(); ++i) {
        worst64 = std::fmax(worst64, std::fabs(h64[i].x - g64[i].x) + std::fabs(h64[i].y - g64[i].y) +
                                         std::fabs(h64[i].z - g64[i].z));
        scale64 = std::fmax(scale64, std::fabs(g64[i].x) + std::fabs(g64[i].y) + std::fabs(g64[i].z));
    }
    const bool bhok = h64.size() == b64.size() && worst64 <= 1e-12 * scale64;
    std::printf("%-40s %s (max diff %.1e)\n", "cuda::BarnesHut(0) over DVec3", bhok ? "ok" : "FAIL", worst64);
    ok &= bhok;

    // tree reuse: build once, walk two target sets; equal to the combined calls
    std::vector<Body> srcs, t1, t2;
    for (int i = 0; i < 5000; ++i)
        srcs.push_back({Vec3(std::sin(0.37f * i) * 3.f, std::cos(0.91f * i) * 3.f, std::sin(0.13f * i)), 1.f / 5000});
    for (int i = 0; i < 700; ++i) t1.push_back({Vec3(std::cos(0.5f * i) * 4.f, std::sin(0.3f * i), 0.2f), 0.f});
    for (int i = 0; i < 900; ++i) t2.push_back({Vec3(0.01f * i - 4.f, 0.5f, -0.3f), 0.f});
    cuda::BarnesHut<float, AccelerationSoftened<float, true>> bhq{0.5f, res, softened_checked(0.01f),
                                                                  PT_BH_QUADRUPOLE | PT_BH_GROUP};
    const cuda::CudaTree tree = bhq.build(srcs);
    const auto w1 = bhq.compute(between(Slice<Body>(t1), tree));
    const auto w2 = bhq.compute(between(Slice<Body>(t2), tree));
    const bool current = tree.is_current();
    const auto c1 = bhq.compute(between(Slice<Body>(t1), Slice<Body>(srcs)));
    const auto c2 = bhq.compute(between(Slice<Body>(t2), Slice<Body>(srcs)));
    bool reuse = current && !tree.is_current() && w1.size() == t1.size() && w2.size() == t2.size();
    for (size_t i = 0; reuse && i < t1.size(); ++i) reuse = w1[i].x == c1[i].x && w1[i].y == c1[i].y && w1[i].z == c1[i].z;
    for (size_t i = 0; reuse && i < t2.size(); ++i) reuse = w2[i].x == c2[i].x && w2[i].y == c2[i].y && w2[i].z == c2[i].z;
    bool refused = false;
    try {
        bhq.compute(between(Slice<Body>(t1), tree));
    } catch (const cuda::Error &) {
        refused = true;
    }
    std::printf("%-40s %s\n", "BarnesHut tree reuse (build once, walk)", reuse && refused ? "ok" : "FAIL");
    ok &= reuse && refused;

    // a tree the caller built (a RootedOrthtree flattened per node): root [-4, 4]^3 with
    // an internal child [-4, 0]^3 over two bodies and an external child. At theta 0 its
    // walk sums the leaves (the brute force over them); a far target takes the root's
    // monopole.
    {
        const std::vector<Body> lb = {{Vec3(-3.f, -1.f, -2.f), 2.f}, {Vec3(-1.f, -3.f, -0.5f), 1.f},
                                      {Vec3(2.f, 3.f, 1.f), 4.f}};
        cuda::OrthtreeNodes t;
        t.internal = {1, 1, 0, 0, 0};
        t.orthant.assign(40, -1);
        t.bbox.assign(30, 0.f);
        t.data.assign(20, 0.f);
        for (int c = 0; c < 3; ++c) {
            t.bbox[c] = -4.f, t.bbox[3 + c] = 4.f;      // node 0
            t.bbox[6 + c] = -4.f, t.bbox[9 + c] = 0.f;  // node 1
        }
        t.orthant[0] = 1, t.orthant[7] = 4;
        t.orthant[8 + 0] = 2, t.orthant[8 + 3] = 3;
        auto put = [&](int k, std::initializer_list<int> members) {
            double m = 0, x = 0, y = 0, z = 0;
            for (int i : members) {
                m += lb[i].mu;
                x += double(lb[i].mu) * lb[i].position.x;
                y += double(lb[i].mu) * lb[i].position.y;
                z += double(lb[i].mu) * lb[i].position.z;
            }
            t.data[4 * k] = float(x / m), t.data[4 * k + 1] = float(y / m), t.data[4 * k + 2] = float(z / m);
            t.data[4 * k + 3] = float(m);
        };
        put(0, {0, 1, 2});
        put(1, {0, 1});
        put(2, {0});
        put(3, {1});
        put(4, {2});
        const std::vector<Body> targets = {{Vec3(0.5f, 0.25f, -1.f), 0.f}, {Vec3(-2.f, 2.f, 3.f), 0.f},
                                           {Vec3(100.f, 50.f, -30.f), 0.f}};
        cuda::BarnesHut<float, AccelerationSoftened<float, true>> bh0{0.f, res, softened_checked(0.01f)};
        const cuda::CudaTree ut = bh0.load_tree(t);
        const auto u0 = bh0.compute(between(Slice<Body>(targets), ut));
        const auto d0 = cuda::BruteForce<AccelerationSoftened<float, true>>{res, softened_checked(0.01f)}.compute(
            between(Slice<Body>(targets), Slice<Body>(lb)));
        bool user = u0.size() == 3 && d0.size() == 3;
        for (size_t i = 0; user && i < 3; ++i) {
            const float s = std::fabs(d0[i].x) + std::fabs(d0[i].y) + std::fabs(d0[i].z);
            user = std::fabs(u0[i].x - d0[i].x) + std::fabs(u0[i].y - d0[i].y) + std::fabs(u0[i].z - d0[i].z) <=
                   1e-6f * s;
        }
        cuda::BarnesHut<float, AccelerationSoftened<float, true>> bh1{1.f, res, softened_checked(0.01f)};
        const cuda::CudaTree ut1 = bh1.load_tree(t);
        const auto u1 = bh1.compute(between(Slice<Body>(targets), ut1));
        const double dx = t.data[0] - 100.0, dy = t.data[1] - 50.0, dz = t.data[2] + 30.0;
        const double r2 = dx * dx + dy * dy + dz * dz + 1e-4, q = t.data[3] / (r2 * std::sqrt(r2));
        user = user && u1.size() == 3 && std::fabs(u1[2].x - dx * q) <= 1e-5 * std::fabs(dx * q) &&
               std::fabs(u1[2].y - dy * q) <= 1e-5 * std::fabs(dy * q) &&
               std::fabs(u1[2].z - dz * q) <= 1e-5 * std::fabs(dz * q);
        std::printf("%-40s %s\n", "BarnesHut over a caller-built tree", user ? "ok" : "FAIL");
        ok &= user;
    }
    std::printf("%s\n", ok ? "ALL OK" : "SOME FAILED");
    return ok ? 0 : 1;
}
