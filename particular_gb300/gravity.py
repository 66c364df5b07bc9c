"""Gravity model and interactions, mirroring particular's `gravity` module.

* GravitationalField  - particular/src/gravity/mod.rs:12-35 (`#[repr(C)] {position, m}`)
* Position / Mass     - gravity/mod.rs:40-46, 133-148: any object with a `position` and
                        a `mu` (or `mass`, times an optional class attribute `G`, as
                        `#[derive(Mass)]` with `#[G = ...]` does, particular_derive/src/gravity.rs:42-108),
                        or a `(position, mu)` tuple (gravity/mod.rs:163-191)
* Acceleration        - gravity/newtonian/acceleration.rs:17-44
* AccelerationSoftened- gravity/newtonian/acceleration_softened.rs:17-49

Particles cross into the library as packed float32 (n, 4) rows (x, y, z, mu), the
layout of GravitationalField<Vec3, f32> that wgpu's padded types also use
(gravity/impls/mod.rs:432).
"""
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class GravitationalField:
    """A point mass: position (3 floats) and standard gravitational parameter m = G*mass."""

    position: tuple
    m: float

    def is_affecting(self):
        """`m != 0` (gravity/mod.rs:29-34)."""
        return self.m != 0.0

    @property
    def mu(self):
        return self.m


def _mu_of(p):
    if hasattr(p, "mu"):
        mu = p.mu
        return mu() if callable(mu) else mu
    if hasattr(p, "m"):
        return p.m
    if hasattr(p, "mass"):
        mass = p.mass
        mass = mass() if callable(mass) else mass
        return getattr(p, "G", 1.0) * mass
    raise TypeError(f"{type(p).__name__} has neither `mu`, `m` nor `mass` (the Mass trait)")


def _position_of(p):
    pos = p.position
    return pos() if callable(pos) else pos


def fields(particles, dtype=np.float32):
    """Packs particles into a C-contiguous (n, 4) array of (x, y, z, mu), float32 by
    default (GravitationalField<Vec3, f32>) or float64 (glam DVec3 bodies).

    Accepts an (n, 4) array (already packed), a (positions (n, 3), mu (n,)) pair, a
    structured array with `position` and `mu`/`mass` fields, or a sequence of objects
    implementing Position + Mass, or of (position, mu) tuples.
    """
    if isinstance(particles, np.ndarray) and particles.dtype.names is None:
        a = np.asarray(particles)
        if a.ndim != 2 or a.shape[1] != 4:
            raise ValueError("a packed particle array must have shape (n, 4): x, y, z, mu")
        return np.ascontiguousarray(a, dtype=dtype)
    if isinstance(particles, np.ndarray):
        names = particles.dtype.names
        mu = particles["mu"] if "mu" in names else particles["mass"]
        pos = particles["position"]
        return _pack(pos, mu, dtype)
    if isinstance(particles, tuple) and len(particles) == 2 and isinstance(particles[0], np.ndarray):
        return _pack(particles[0], particles[1], dtype)
    items = list(particles)
    if not items:
        return np.zeros((0, 4), dtype)
    if isinstance(items[0], tuple) and len(items[0]) == 2:
        pos = [it[0] for it in items]
        mu = [it[1] for it in items]
    else:
        pos = [_position_of(it) for it in items]
        mu = [_mu_of(it) for it in items]
    return _pack(np.asarray(pos, dtype), np.asarray(mu, dtype), dtype)


def positions(particles, dtype=np.float32):
    """Packs the positions of affected particles as (n, 4) rows (w unused)."""
    if isinstance(particles, np.ndarray) and particles.dtype.names is None and particles.ndim == 2 \
            and particles.shape[1] == 3:
        out = np.zeros((particles.shape[0], 4), dtype)
        out[:, :3] = particles
        return out
    return fields(particles, dtype)


def _pack(pos, mu, dtype=np.float32):
    pos = np.asarray(pos, dtype).reshape(-1, 3)
    mu = np.asarray(mu, dtype).reshape(-1)
    if pos.shape[0] != mu.shape[0]:
        raise ValueError("positions and mu differ in length")
    out = np.empty((pos.shape[0], 4), dtype)
    out[:, :3] = pos
    out[:, 3] = mu
    return out


class Acceleration:
    """Newtonian acceleration between point masses (gravity/newtonian/acceleration.rs:17-44).

    `checked` (the default) returns zero for coincident positions; `unchecked` skips
    the test and yields NaN/inf for them, as the reference does.
    """

    softening = 0.0

    def __init__(self, checked=True):
        self.is_checked = bool(checked)

    @classmethod
    def checked(cls):
        return cls(True)

    @classmethod
    def unchecked(cls):
        return cls(False)

    def __repr__(self):
        return f"Acceleration<{'true' if self.is_checked else 'false'}>"


class AccelerationSoftened:
    """Softened acceleration, n_s = |d|^2 + softening^2
    (gravity/newtonian/acceleration_softened.rs:17-49)."""

    def __init__(self, softening, checked=True):
        self.softening = float(np.float32(softening))  # the f32 value the f32 methods use
        self.softening64 = float(softening)            # and the f64 one (DVec3 bodies)
        self.is_checked = bool(checked)

    @classmethod
    def checked(cls, softening):
        return cls(softening, True)

    @classmethod
    def unchecked(cls, softening):
        return cls(softening, False)

    def __repr__(self):
        return f"AccelerationSoftened<{self.softening}, {'true' if self.is_checked else 'false'}>"
