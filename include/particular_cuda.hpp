// particular_cuda.hpp -- C++17 host mirror of particular's API over the C ABI.
//
// The reference is a Rust crate; this header restates, for C++ callers, the part of
// its API the cuda compute methods plug into, with the same names and meaning:
//
//   Between<S1, S2>               particular/src/lib.rs:296-300
//   Ordered<P>, Reordered<P, F>   particular/src/storage.rs:48-205
//   GravitationalField<V, S>      particular/src/gravity/mod.rs:12-35
//   Position / Mass               particular/src/gravity/mod.rs:40-148 (a type with a
//                                 `position` member and a `mu` or `mass` member, plus an
//                                 optional `static constexpr G`, as #[derive(Position,
//                                 Mass)] requires, particular_derive/src/gravity.rs)
//   Acceleration<CHECKED>         particular/src/gravity/newtonian/acceleration.rs:17-44
//   AccelerationSoftened<S, C>    particular/src/gravity/newtonian/acceleration_softened.rs:17-49
//   cuda::CudaResources           gpu::GpuResources, particular/src/gpu/mod.rs:84-143
//   cuda::BruteForce<T>           gpu::BruteForce, particular/src/gpu/mod.rs:145-208
//   cuda::BarnesHut<S, T>         sequential::BarnesHut, particular/src/sequential.rs:432-543
//   cuda_brute_force(...) etc.    GpuCompute, particular/src/gpu/mod.rs:13-37
//
// `compute(storage)` accepts a slice (Slice<P>, std::vector<P>), an Ordered, a
// Reordered or a Between, as the storage blanket impls (storage.rs:207-241) do, and
// returns the affected bodies' accelerations in order. A failed call throws
// particular::cuda::Error (the reference panics).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "particular_cuda.h"

namespace particular {

struct Vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
    Vec3() = default;
    Vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    static Vec3 splat(float v) { return {v, v, v}; }
    Vec3 operator+(const Vec3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
    Vec3 operator-(const Vec3 &o) const { return {x - o.x, y - o.y, z - o.z}; }
    Vec3 operator*(float s) const { return {x * s, y * s, z * s}; }
    Vec3 &operator+=(const Vec3 &o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    float length_squared() const { return x * x + y * y + z * z; }
};

// glam DVec3: particles whose position is made of doubles take the f64 path.
struct DVec3 {
    double x = 0.0, y = 0.0, z = 0.0;
    DVec3() = default;
    DVec3(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}
    static DVec3 splat(double v) { return {v, v, v}; }
    DVec3 operator+(const DVec3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
    DVec3 operator-(const DVec3 &o) const { return {x - o.x, y - o.y, z - o.z}; }
    DVec3 operator*(double s) const { return {x * s, y * s, z * s}; }
    DVec3 &operator+=(const DVec3 &o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    double length_squared() const { return x * x + y * y + z * z; }
};

// A view of contiguous particles (the role of `&[P]`).
template <class P>
struct Slice {
    using value_type = P;
    const P *ptr = nullptr;
    size_t len = 0;
    Slice() = default;
    Slice(const P *p, size_t n) : ptr(p), len(n) {}
    Slice(const std::vector<P> &v) : ptr(v.data()), len(v.size()) {}
    const P &operator[](size_t i) const { return ptr[i]; }
    size_t size() const { return len; }
};

template <class S1, class S2>
struct Between {
    S1 affected;
    S2 affecting;
};
template <class S1, class S2>
Between<S1, S2> between(S1 a, S2 b) {
    return Between<S1, S2>{a, b};
}

template <class V, class S>
struct GravitationalField {
    V position;
    S m;
    bool is_affecting() const { return m != S(0); }
};

// ---- Position + Mass detection (the derive's contract) ---------------------
namespace detail {
template <class, class = void>
struct has_mu : std::false_type {};
template <class P>
struct has_mu<P, std::void_t<decltype(std::declval<const P &>().mu)>> : std::true_type {};
template <class, class = void>
struct has_m : std::false_type {};
template <class P>
struct has_m<P, std::void_t<decltype(std::declval<const P &>().m)>> : std::true_type {};
template <class, class = void>
struct has_G : std::false_type {};
template <class P>
struct has_G<P, std::void_t<decltype(P::G)>> : std::true_type {};
}  // namespace detail

template <class P>
inline Vec3 position_of(const P &p) {
    return Vec3(float(p.position.x), float(p.position.y), float(p.position.z));
}
template <class P>
inline double mu64_of(const P &p) {
    if constexpr (detail::has_mu<P>::value) {
        return double(p.mu);
    } else if constexpr (detail::has_m<P>::value) {
        return double(p.m);
    } else if constexpr (detail::has_G<P>::value) {
        return double(P::G * p.mass);
    } else {
        return double(p.mass);
    }
}
template <class P>
inline float mu_of(const P &p) {
    if constexpr (detail::has_mu<P>::value) {
        return float(p.mu);
    } else if constexpr (detail::has_m<P>::value) {
        return float(p.m);
    } else if constexpr (detail::has_G<P>::value) {
        return float(P::G * p.mass);
    } else {
        return float(p.mass);
    }
}
namespace detail {
// particles whose position components are doubles (glam DVec3 and the like)
template <class P>
struct is_f64_position
    : std::is_same<std::decay_t<decltype(std::declval<const P &>().position.x)>, double> {};
}  // namespace detail

// ---- interactions ---------------------------------------------------------
template <bool CHECKED>
struct Acceleration {
    static constexpr bool checked = CHECKED;
    float softening() const { return 0.f; }
    double softening64() const { return 0.0; }
};
inline Acceleration<true> acceleration_checked() { return {}; }
inline Acceleration<false> acceleration_unchecked() { return {}; }

template <class S, bool CHECKED>
struct AccelerationSoftened {
    S softening_;
    static constexpr bool checked = CHECKED;
    float softening() const { return float(softening_); }
    double softening64() const { return double(softening_); }
};
template <class S>
AccelerationSoftened<S, true> softened_checked(S s) {
    return {s};
}

// ---- storages ---------------------------------------------------------------
template <class P>
struct DefaultIsAffecting {
    bool operator()(const P &p) const { return mu_of(p) != 0.f; }
};

template <class P>
class Ordered {
  public:
    template <class F = DefaultIsAffecting<P>>
    static Ordered create(Slice<P> unordered, F is_affecting = F()) {
        Ordered o;
        for (size_t i = 0; i < unordered.size(); ++i)
            if (is_affecting(unordered[i])) o.particles_.push_back(unordered[i]);
        o.affecting_len_ = o.particles_.size();
        for (size_t i = 0; i < unordered.size(); ++i)
            if (!is_affecting(unordered[i])) o.particles_.push_back(unordered[i]);
        return o;
    }
    size_t affecting_len() const { return affecting_len_; }
    Slice<P> affecting() const { return Slice<P>(particles_.data(), affecting_len_); }
    Slice<P> non_affecting() const {
        return Slice<P>(particles_.data() + affecting_len_, particles_.size() - affecting_len_);
    }
    Slice<P> particles() const { return Slice<P>(particles_); }

  private:
    std::vector<P> particles_;
    size_t affecting_len_ = 0;
};

template <class P, class F = DefaultIsAffecting<P>>
class Reordered {
  public:
    Reordered(Slice<P> unordered, F is_affecting = F())
        : unordered(unordered), ordered_(Ordered<P>::create(unordered, is_affecting)) {}
    Slice<P> unordered;
    const Ordered<P> &ordered() const { return ordered_; }
    Slice<P> affecting() const { return ordered_.affecting(); }
    size_t affecting_len() const { return ordered_.affecting_len(); }

  private:
    Ordered<P> ordered_;
};

// storage -> Between(affected, affecting) (storage.rs:207-241)
template <class P>
Between<Slice<P>, Slice<P>> as_between(Slice<P> s) {
    return {s, s};
}
template <class P>
Between<Slice<P>, Slice<P>> as_between(const std::vector<P> &v) {
    return {Slice<P>(v), Slice<P>(v)};
}
template <class P>
Between<Slice<P>, Slice<P>> as_between(const Ordered<P> &o) {
    return {o.particles(), o.affecting()};
}
template <class P, class F>
Between<Slice<P>, Slice<P>> as_between(const Reordered<P, F> &r) {
    return {r.unordered, r.affecting()};
}
template <class P1, class P2>
Between<Slice<P1>, Slice<P2>> as_between(Between<Slice<P1>, Slice<P2>> b) {
    return b;
}

namespace cuda {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != PT_OK) throw Error(rc, std::string("particular cuda: ") + pt_last_error());
}

// One context per device; create once and reuse (gpu/mod.rs:150-151).
class CudaResources {
  public:
    explicit CudaResources(int device = 0) { check(pt_ctx_create(&ctx_, device)); }
    ~CudaResources() { pt_ctx_destroy(ctx_); }
    CudaResources(const CudaResources &) = delete;
    CudaResources &operator=(const CudaResources &) = delete;
    pt_ctx *get() const { return ctx_; }

  private:
    pt_ctx *ctx_ = nullptr;
};

namespace detail {
template <class P>
std::vector<float> pack_fields(Slice<P> s) {
    std::vector<float> out(4 * s.size());
    for (size_t i = 0; i < s.size(); ++i) {
        const Vec3 p = position_of(s[i]);
        out[4 * i] = p.x;
        out[4 * i + 1] = p.y;
        out[4 * i + 2] = p.z;
        out[4 * i + 3] = mu_of(s[i]);
    }
    return out;
}
template <class P>
std::vector<double> pack_fields64(Slice<P> s) {
    std::vector<double> out(4 * s.size());
    for (size_t i = 0; i < s.size(); ++i) {
        out[4 * i] = double(s[i].position.x);
        out[4 * i + 1] = double(s[i].position.y);
        out[4 * i + 2] = double(s[i].position.z);
        out[4 * i + 3] = mu64_of(s[i]);
    }
    return out;
}
inline std::vector<DVec3> unpack64(const std::vector<double> &o) {
    std::vector<DVec3> r(o.size() / 3);
    for (size_t i = 0; i < r.size(); ++i) r[i] = DVec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    return r;
}
inline std::vector<Vec3> unpack(const std::vector<float> &o) {
    std::vector<Vec3> r(o.size() / 3);
    for (size_t i = 0; i < r.size(); ++i) r[i] = Vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    return r;
}
}  // namespace detail

template <class T>
struct BruteForce {
    CudaResources &resources;
    T interaction;
    bool exact = false;  // bit-identical to sequential::BruteForce

    // Accelerations of the affected particles: std::vector<Vec3> for f32 particles,
    // std::vector<DVec3> (the reference's f64 result bit for bit) for DVec3 ones.
    template <class Storage>
    auto compute(const Storage &storage) {
        auto b = as_between(storage);
        using P1 = typename decltype(b.affected)::value_type;
        const bool same = static_cast<const void *>(b.affected.ptr) ==
                              static_cast<const void *>(b.affecting.ptr) &&
                          b.affected.size() == b.affecting.size();
        if constexpr (particular::detail::is_f64_position<P1>::value) {
            const auto aff = detail::pack_fields64(b.affected);
            const auto src = same ? std::vector<double>() : detail::pack_fields64(b.affecting);
            std::vector<double> out(3 * b.affected.size());
            if (out.empty()) return std::vector<DVec3>();
            check(pt_bf_accel_dvec3(resources.get(), aff.data(), b.affected.size(),
                                    same ? aff.data() : src.data(), b.affecting.size(),
                                    interaction.softening64(), T::checked ? 1 : 0, out.data()));
            return detail::unpack64(out);
        } else {
            const auto aff = detail::pack_fields(b.affected);
            const auto src = same ? std::vector<float>() : detail::pack_fields(b.affecting);
            std::vector<float> out(3 * b.affected.size());
            if (out.empty()) return std::vector<Vec3>();
            check(pt_bf_accel_f32(resources.get(), aff.data(), b.affected.size(),
                                  same ? aff.data() : src.data(), b.affecting.size(),
                                  interaction.softening(), T::checked ? 1 : 0, exact ? PT_BF_EXACT : 0u,
                                  out.data()));
            return detail::unpack(out);
        }
    }
};

// A Barnes-Hut tree kept on the device: built once by BarnesHut::build and walked
// through Between(affected, tree), the counterpart of Between(&affected[..], &tree)
// over a RootedOrthtree (lib.rs:186-199). Valid until the next Barnes-Hut call on the
// same resources replaces the context's tree.
struct CudaTree {
    CudaResources *resources = nullptr;
    size_t n_affecting = 0;
    uint64_t generation = 0;
    bool is_current() const {
        uint64_t g = 0;
        check(pt_bh_tree_generation(resources->get(), &g));
        return g == generation;
    }
};

// A tree the caller built: the reference's RootedOrthtree over GravitationalField<Vec3,
// f32> (tree/mod.rs:13-60) flattened per node, as pt_bh_load_tree takes it.
struct OrthtreeNodes {
    std::vector<uint8_t> internal;  // 1 = Node::Internal, 0 = Node::External
    std::vector<int32_t> orthant;   // 8 per node: child NodeID, -1 for None
    std::vector<float> bbox;        // 6 per node: min x, y, z then max x, y, z
    std::vector<float> data;        // 4 per node: centre of mass x, y, z, mass
    int32_t root = 0;               // RootedOrthtree::root(), -1 for None
};

template <class S, class T>
struct BarnesHut {
    S theta;
    CudaResources &resources;
    T interaction;
    uint32_t flags = 0;  // PT_BH_QUADRUPOLE | PT_BH_GROUP | PT_BH_LOCAL | PT_BH_RELATIVE
    float alpha = 0.f;   // PT_BH_RELATIVE: the error-bound factor (0: the resources' current one)
    float local_ratio = 0.f;  // PT_BH_LOCAL: group radius / distance of far nodes (0: current one)
    float monopole = -1.f;    // PT_BH_RELATIVE: monopole-only factor in [0, 1] (< 0: current one)

    // Makes a tree the caller built the resources' current tree (monopoles: walk it
    // with flags 0 or PT_BH_GROUP).
    CudaTree load_tree(const OrthtreeNodes &t) {
        const size_t n = t.internal.size();
        if (t.orthant.size() != 8 * n || t.bbox.size() != 6 * n || t.data.size() != 4 * n)
            throw Error(PT_ERR_INVALID, "particular cuda: OrthtreeNodes arrays of unequal node counts");
        CudaTree tr{&resources, n, 0};
        check(pt_bh_load_tree(resources.get(), t.orthant.data(), t.bbox.data(), t.internal.data(), t.data.data(), n,
                              t.root, &tr.generation));
        return tr;
    }

    // Builds the tree over the affecting particles of `storage` once.
    template <class Storage>
    CudaTree build(const Storage &storage) {
        auto b = as_between(storage);
        const auto src = detail::pack_fields(b.affecting);
        CudaTree t{&resources, b.affecting.size(), 0};
        check(pt_bh_build(resources.get(), src.data(), b.affecting.size(), &t.generation));
        return t;
    }

    // Walks a tree built by `build` for the affected particles.
    template <class P>
    std::vector<Vec3> compute(const Between<Slice<P>, CudaTree> &b) {
        if (b.affecting.resources != &resources) throw Error(PT_ERR_INVALID, "particular cuda: tree of other resources");
        if (!b.affecting.is_current())
            throw Error(PT_ERR_INVALID, "particular cuda: the tree was replaced by a later Barnes-Hut call");
        const auto aff = detail::pack_fields(b.affected);
        std::vector<float> out(3 * b.affected.size());
        if (out.empty()) return {};
        set_alpha();
        check(pt_bh_walk(resources.get(), aff.data(), b.affected.size(), float(theta), interaction.softening(), flags,
                         out.data()));
        return detail::unpack(out);
    }

    // Accelerations of the affected particles: std::vector<Vec3> for f32 particles,
    // std::vector<DVec3> for DVec3 ones (the reference rule in double; flags must be 0).
    template <class Storage>
    auto compute(const Storage &storage) {
        auto b = as_between(storage);
        using P1 = typename decltype(b.affected)::value_type;
        const bool same = static_cast<const void *>(b.affected.ptr) ==
                              static_cast<const void *>(b.affecting.ptr) &&
                          b.affected.size() == b.affecting.size();
        if constexpr (particular::detail::is_f64_position<P1>::value) {
            const auto aff = detail::pack_fields64(b.affected);
            const auto src = same ? std::vector<double>() : detail::pack_fields64(b.affecting);
            std::vector<double> out(3 * b.affected.size());
            if (out.empty()) return std::vector<DVec3>();
            check(pt_bh_accel_dvec3(resources.get(), aff.data(), b.affected.size(),
                                    same ? aff.data() : src.data(), b.affecting.size(), double(theta),
                                    interaction.softening64(), flags, out.data()));
            return detail::unpack64(out);
        } else {
            return compute_f32(b, same);
        }
    }

  private:
    void set_alpha() {
        if ((flags & PT_BH_RELATIVE) && alpha > 0.f) check(pt_bh_set_relative_alpha(resources.get(), alpha));
        if ((flags & PT_BH_RELATIVE) && monopole >= 0.f)
            check(pt_bh_set_relative_monopole(resources.get(), monopole));
        if ((flags & PT_BH_LOCAL) && local_ratio > 0.f) check(pt_bh_set_local_ratio(resources.get(), local_ratio));
    }

    template <class P1, class P2>
    std::vector<Vec3> compute_f32(const Between<Slice<P1>, Slice<P2>> &b, bool same) {
        const auto aff = detail::pack_fields(b.affected);
        const auto src = same ? std::vector<float>() : detail::pack_fields(b.affecting);
        std::vector<float> out(3 * b.affected.size());
        if (out.empty()) return {};
        set_alpha();
        check(pt_bh_accel_f32(resources.get(), aff.data(), b.affected.size(),
                              same ? aff.data() : src.data(), b.affecting.size(), float(theta),
                              interaction.softening(), flags, out.data()));
        return detail::unpack(out);
    }
};

// GpuCompute-style sugar: storage.cuda_brute_force(resources, interaction).
template <class Storage, class T>
auto cuda_brute_force(const Storage &storage, CudaResources &res, T interaction) {
    return BruteForce<T>{res, interaction}.compute(storage);
}
template <class Storage, class S, class T>
std::vector<Vec3> cuda_barnes_hut(const Storage &storage, S theta, CudaResources &res, T interaction,
                                  uint32_t flags = 0) {
    return BarnesHut<S, T>{theta, res, interaction, flags}.compute(storage);
}

}  // namespace cuda
}  // namespace particular
