"""CPU-only tests: the C ABI library loads and exports every declared symbol, the
host mirror of particular's storages packs what the reference would pass, and the
argument checks reject bad calls without touching a GPU."""
import ctypes

import numpy as np
import pytest

from particular_gb300 import (Acceleration, AccelerationSoftened, Between, Ordered, Reordered,
                              as_between, fields, ics, positions)
from particular_gb300 import _native as N


def test_library_exports_every_header_symbol(native_lib):
    names = N.header_functions()
    assert "pt_bf_accel_f32" in names and "pt_ctx_create" in names
    for name in names:
        assert hasattr(native_lib, name), name


def test_calls_reject_null_context_without_gpu(native_lib):
    buf = np.zeros((4, 4), np.float32)
    out = np.zeros((4, 3), np.float32)
    rc = native_lib.pt_bf_accel_f32(None, buf.ctypes.data, 4, buf.ctypes.data, 4, 0.0, 1, 0,
                                    out.ctypes.data)
    assert rc == N.PT_ERR_INVALID
    assert "ctx is NULL" in N.last_error()
    assert native_lib.pt_ctx_create(None, 0) == N.PT_ERR_INVALID
    assert native_lib.pt_ctx_set_capacity_limit(None, 0) == N.PT_ERR_INVALID
    assert native_lib.pt_ctx_launch_count(None) == 0
    # the Barnes-Hut settings refuse a NULL context before touching any state
    assert native_lib.pt_bh_set_relative_alpha(None, 2.5e-3) == N.PT_ERR_INVALID
    assert "ctx is NULL" in N.last_error()
    assert native_lib.pt_bh_set_local_ratio(None, 0.1) == N.PT_ERR_INVALID
    assert native_lib.pt_bh_set_stack_limit(None, 0) == N.PT_ERR_INVALID
    native_lib.pt_ctx_destroy(None)


def test_context_creation_fails_loudly_without_device(native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = native_lib.pt_ctx_create(ctypes.byref(h), 0)
    assert rc in (N.PT_ERR_CUDA, N.PT_ERR_INVALID)
    assert N.last_error()
    assert not h.value


class Body:
    def __init__(self, position, mass):
        self.position = position
        self.mass = mass


class Planet:
    G = 2.0

    def __init__(self, position, mass):
        self.position = position
        self.mass = mass


def test_fields_from_particle_kinds():
    want = np.array([[1, 2, 3, 4], [5, 6, 7, 0]], np.float32)
    assert np.array_equal(fields(want), want)
    assert np.array_equal(fields([((1, 2, 3), 4), ((5, 6, 7), 0)]), want)
    assert np.array_equal(fields([Body((1, 2, 3), 4), Body((5, 6, 7), 0)]), want)
    # #[derive(Mass)] with #[G = ...]: mu = G * mass
    assert np.array_equal(fields([Planet((1, 2, 3), 2)])[0], [1, 2, 3, 4])
    st = np.zeros(2, dtype=[("position", np.float32, 3), ("mu", np.float32)])
    st["position"] = want[:, :3]
    st["mu"] = want[:, 3]
    assert np.array_equal(fields(st), want)
    assert np.array_equal(positions(want[:, :3])[:, :3], want[:, :3])


def test_storages_match_reference_semantics():
    # storage.rs:52-95: affecting first, order kept inside each group
    p = np.array([[0, 0, 0, 0], [1, 1, 1, 2], [2, 2, 2, 0], [3, 3, 3, 5]], np.float32)
    o = Ordered.new(p)
    assert o.affecting_len() == 2
    assert np.array_equal(o.affecting()[:, 0], [1, 3])
    assert np.array_equal(o.non_affecting()[:, 0], [0, 2])
    b = as_between(o)
    assert np.array_equal(b.affected[:, 0], [1, 3, 0, 2])      # Between(particles(), affecting())
    r = Reordered(p)
    b = as_between(r)
    assert np.array_equal(b.affected[:, 0], [0, 1, 2, 3])      # Between(unordered, affecting())
    assert np.array_equal(b.affecting[:, 0], [1, 3])
    b = as_between(p)
    assert b.affected is p and b.affecting is p                 # &[P] -> Between(slice, slice)
    x = Between(p[:1], p)
    assert as_between(x) is x
    og = Ordered.with_groups(p[[1, 3]], p[[0, 2]])
    assert og.affecting_len() == 2
    custom = Ordered.new(p, lambda row: row[0] > 1.5)
    assert np.array_equal(custom.affecting()[:, 0], [2, 3])


def test_interactions():
    a = Acceleration.checked()
    assert a.is_checked and a.softening == 0.0
    assert not Acceleration.unchecked().is_checked
    s = AccelerationSoftened.checked(1e-3)
    assert s.softening == float(np.float32(1e-3)) and s.is_checked


def test_ics_are_deterministic():
    a = ics.plummer(1000, seed=3)["bodies"]
    b = ics.plummer(1000, seed=3)["bodies"]
    assert np.array_equal(a, b)
    c = ics.uniform_cube(1024)["bodies"]
    assert c.shape == (1024, 4) and (np.abs(c[:, :3]) <= 1).all()
    assert ((c[:, 3] >= 0.5) & (c[:, 3] <= 1.5)).all()
    sizes = ics.ensemble_sizes(4096)
    assert sizes.min() >= 64 and sizes.max() <= 8192


def test_plummer_is_in_virial_equilibrium():
    d = ics.plummer(20000, seed=11)
    b, v = d["bodies"].astype(np.float64), d["vel"].astype(np.float64)
    K = 0.5 * (b[:, 3] * (v ** 2).sum(1)).sum()
    assert abs(K - 3 * np.pi / 64) / (3 * np.pi / 64) < 0.05


def test_cpp_host_mirror_compiles(native_lib):
    """The C++ mirror of the reference API and its KAT program build (no GPU needed)."""
    import os
    from conftest import load_cpp_build
    assert os.path.exists(load_cpp_build().build())
