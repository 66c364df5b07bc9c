"""Seeded synthetic initial conditions for the benchmark workloads (G = 1).

The reference's own benchmark bodies (particular/benches/benchmark.rs:22-37) come
from rand 0.8's StdRng, which is not vendored with it; these generators use their
own counter-based SplitMix64 stream instead, so every array is reproducible on any
machine from (seed, sizes):

* uniform_cube   - N bodies uniform in [-1, 1]^3, masses uniform in [0.5, 1.5]
* plummer        - Plummer sphere (scale a, mass M, equal masses), radii from the
                   inverse cumulative mass profile r = a / sqrt(X^(-2/3) - 1) with X
                   truncated to <= 0.999, isotropic speeds by the rejection method of
                   Aarseth, Henon & Wielen (1974) on g(q) = q^2 (1 - q^2)^(7/2)
* bulge_disk     - 70% Plummer bulge (a = 0.5) + 30% exponential disk (scale length
                   2, sech^2 vertical profile with scale height 0.05) on circular
                   orbits from the enclosed mass of the sampled set; equal masses
                   summing to 1
* ensemble       - many independent Plummer systems of log-uniform sizes
"""
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """Counter-based SplitMix64: draw k returns mix(seed + k * golden)."""

    def __init__(self, seed):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.counter = 0

    def raw(self, n):
        k = np.arange(self.counter + 1, self.counter + 1 + n, dtype=np.uint64)
        self.counter += n
        with np.errstate(over="ignore"):
            z = self.state + k * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))

    def uniform(self, n, lo=0.0, hi=1.0):
        u = (self.raw(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u


def _isotropic(rng, n):
    cos_t = rng.uniform(n, -1.0, 1.0)
    phi = rng.uniform(n, 0.0, 2.0 * math.pi)
    sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
    return np.stack([sin_t * np.cos(phi), sin_t * np.sin(phi), cos_t], axis=1)


def _plummer_q(rng, n):
    """Speed fraction q = v / v_esc by rejection on q^2 (1-q^2)^3.5 (max < 0.1)."""
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x = rng.uniform(todo.size)
        y = rng.uniform(todo.size, 0.0, 0.1)
        ok = y < x * x * (1.0 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    return q


def plummer_raw(rng, n, a, mass):
    """Positions and velocities (float64) of a Plummer sphere; `a` may be per body."""
    a = np.broadcast_to(np.asarray(a, np.float64), (n,))
    mass = np.broadcast_to(np.asarray(mass, np.float64), (n,))
    x = rng.uniform(n) * 0.999
    x = np.maximum(x, 1e-12)
    r = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    pos = _isotropic(rng, n) * r[:, None]
    q = _plummer_q(rng, n)
    v_esc = math.sqrt(2.0) * (1.0 + (r / a) ** 2) ** -0.25 * np.sqrt(mass / a)
    vel = _isotropic(rng, n) * (q * v_esc)[:, None]
    return pos, vel


def _pack(pos, m):
    out = np.empty((pos.shape[0], 4), np.float32)
    out[:, :3] = pos
    out[:, 3] = m
    return out


def _recentre(pos, vel, m):
    mt = m.sum()
    pos = pos - (m[:, None] * pos).sum(0) / mt
    vel = vel - (m[:, None] * vel).sum(0) / mt
    return pos, vel


def uniform_cube(n, seed=1808):
    """N bodies uniform in [-1, 1]^3 with masses uniform in [0.5, 1.5] (mu = m, G = 1)."""
    rng = SplitMix64(seed)
    pos = rng.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    m = rng.uniform(n, 0.5, 1.5)
    return {"bodies": _pack(pos, m), "vel": np.zeros((n, 3), np.float32)}


def criterion_bodies(n, seed=1808):
    """The reference benchmark's bodies (particular/benches/benchmark.rs:22-37,97-105):
    positions uniform in [-5e3, 5e3]^3, every body massive with mu uniform in
    [1e3, 1e9], velocities uniform in [-100, 100]^3. The reference draws them from
    rand's StdRng seeded 1808; this generator cannot reproduce that stream, so the same
    distributions come from SplitMix64 with the same seed."""
    rng = SplitMix64(seed)
    pos = rng.uniform(3 * n, -5e3, 5e3).reshape(n, 3)
    mu = rng.uniform(n, 1e3, 1e9)
    vel = rng.uniform(3 * n, -100.0, 100.0).reshape(n, 3)
    return {"bodies": _pack(pos, mu), "vel": vel.astype(np.float32)}


def plummer(n, a=1.0, total_mass=1.0, seed=1809):
    rng = SplitMix64(seed)
    pos, vel = plummer_raw(rng, n, a, total_mass)
    m = np.full(n, total_mass / n)
    pos, vel = _recentre(pos, vel, m)
    return {"bodies": _pack(pos, m), "vel": vel.astype(np.float32)}


def bulge_disk(n, seed=1810, bulge_fraction=0.7, bulge_a=0.5, disk_rd=2.0, disk_h=0.05):
    rng = SplitMix64(seed)
    nb = int(round(bulge_fraction * n))
    nd = n - nb
    m = np.full(n, 1.0 / n)
    pos_b, vel_b = plummer_raw(rng, nb, bulge_a, nb / n)
    u1 = np.maximum(rng.uniform(nd), 1e-300)
    u2 = np.maximum(rng.uniform(nd), 1e-300)
    R = -disk_rd * np.log(u1 * u2)  # Gamma(2, R_d): surface density ~ exp(-R/R_d)
    phi = rng.uniform(nd, 0.0, 2.0 * math.pi)
    u = rng.uniform(nd, -1.0, 1.0)
    z = disk_h * np.arctanh(np.clip(u, -1 + 1e-12, 1 - 1e-12))  # sech^2(z/h)
    pos_d = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    pos = np.concatenate([pos_b, pos_d])
    # Circular speeds from the enclosed mass of the sampled set (spherical estimate).
    r_all = np.sqrt((pos ** 2).sum(1))
    order = np.argsort(r_all, kind="stable")
    enclosed = np.empty(n)
    enclosed[order] = np.cumsum(m[order])
    r_d = r_all[nb:]
    vc = np.sqrt(enclosed[nb:] / np.maximum(r_d, 1e-6))
    vel_d = np.stack([-np.sin(phi) * vc, np.cos(phi) * vc, np.zeros(nd)], axis=1)
    vel = np.concatenate([vel_b, vel_d])
    pos, vel = _recentre(pos, vel, m)
    return {"bodies": _pack(pos, m), "vel": vel.astype(np.float32)}


def ensemble_sizes(n_sys, lo=64, hi=8192, seed=1811):
    rng = SplitMix64(seed)
    return np.rint(np.exp(rng.uniform(n_sys, math.log(lo), math.log(hi)))).astype(np.int64)


def ensemble(n_sys=4096, lo=64, hi=8192, seed=1811):
    """Independent Plummer systems (mass 1 each, scale radius uniform in [0.5, 2]),
    concatenated; offsets[k]..offsets[k+1] are system k's bodies."""
    sizes = ensemble_sizes(n_sys, lo, hi, seed)
    rng = SplitMix64(seed + 1)
    a_sys = rng.uniform(n_sys, 0.5, 2.0)
    offsets = np.zeros(n_sys + 1, np.int64)
    offsets[1:] = np.cumsum(sizes)
    n = int(offsets[-1])
    sys_of = np.repeat(np.arange(n_sys), sizes)
    pos, vel = plummer_raw(rng, n, a_sys[sys_of], 1.0)
    m = 1.0 / sizes[sys_of]
    for_sums = np.concatenate([[0], offsets[1:]])
    # recentre every system on its own centre of mass
    wsum = np.add.reduceat(m[:, None] * pos, for_sums[:-1], axis=0)
    vsum = np.add.reduceat(m[:, None] * vel, for_sums[:-1], axis=0)
    pos -= wsum[sys_of]
    vel -= vsum[sys_of]
    return {"bodies": _pack(pos, m), "vel": vel.astype(np.float32),
            "offsets": offsets.astype(np.uint32), "scale": a_sys}
