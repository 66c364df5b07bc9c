"""Brute-force parity on the GPU, through the C ABI, against the CPU oracle.

* PT_BF_EXACT: bit-identical to the restated sequential::BruteForce (every size,
  softened or not, checked or not, massless and coincident bodies).
* default fast path: within the stated tolerance of the reference f32 result and
  no further from the FP64 judge than the reference's own f32 sum.
* the reference's known-answer tests (mod.rs:228-347, GPU variant at mod.rs:511-518).
"""
import ctypes

import numpy as np
import pytest

import kat
from particular_gb300 import (Acceleration, AccelerationSoftened, Between, Ordered, Reordered,
                              cuda, ics)
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 33, 255, 257, 1023, 1025, 4097]


def rel(a, ref):
    return np.linalg.norm(np.asarray(a, np.float64) - ref, axis=1) / np.maximum(
        np.linalg.norm(ref, axis=1), 1e-30)


def mixed(n, seed):
    b = ics.uniform_cube(n, seed)["bodies"].copy()
    if n > 8:
        b[::7, 3] = 0.0
        b[5] = b[3]
        b[6, :3] = b[3, :3]
    return b


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("softening,checked", [(0.0, True), (1e-3, True), (0.05, False)])
def test_exact_bit_identical(res, oracle, n, softening, checked):
    b = mixed(n, 100 + n) if checked else ics.uniform_cube(n, 200 + n)["bodies"]
    it = AccelerationSoftened(softening, checked)
    got = cuda.BruteForce(res, it, exact=True).compute(b)
    want = oracle.bf_f32(b, b, softening, checked)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("n_aff,n_src", [(37, 1000), (1000, 37), (5000, 3), (3, 70000)])
def test_exact_between_different_sets(res, oracle, n_aff, n_src):
    aff = ics.uniform_cube(n_aff, 1)["bodies"]
    src = ics.plummer(n_src, seed=2)["bodies"]
    got = cuda.BruteForce(res, AccelerationSoftened(0.01), exact=True).compute(Between(aff, src))
    want = oracle.bf_f32(aff, src, 0.01, True)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("n", SIZES + [20000])
def test_fast_within_tolerance(res, oracle, n):
    b = mixed(n, 300 + n)
    got = cuda.BruteForce(res, AccelerationSoftened(1e-3)).compute(b)
    ref32 = oracle.bf_f32(b, b, 1e-3, True)
    ref64 = oracle.bf_f64(b, b, 1e-3, True)
    e_gpu = rel(got, ref64)
    e_ref = rel(ref32, ref64)
    # Compensated sums: never meaningfully less accurate than the reference's f32 sum.
    assert (e_gpu <= e_ref + 2e-6).all(), (e_gpu.max(), e_ref.max())
    assert np.percentile(rel(got, ref32.astype(np.float64)), 99) <= 1e-5


def test_config1_tolerance(res, oracle):
    """N=1024 uniform cube, eps=1e-3: <= 1e-5 relative to the reference f32 result."""
    b = ics.uniform_cube(1024)["bodies"]
    got = cuda.BruteForce(res, AccelerationSoftened(1e-3)).compute(b)
    ref32 = oracle.bf_f32(b, b, 1e-3, True).astype(np.float64)
    e = rel(got, ref32)
    print(f"C1 rel err vs reference f32: p50={np.median(e):.2e} p95={np.percentile(e, 95):.2e} "
          f"max={e.max():.2e}")
    assert e.max() <= 1e-5


@pytest.mark.parametrize("k", [1, 2, 4])
@pytest.mark.parametrize("slices", [1, 2, 7, 0])
def test_launch_plans_agree(res, oracle, k, slices):
    b = ics.plummer(9000, seed=12)["bodies"]
    ref64 = oracle.bf_f64(b, b, 0.01, True)
    N.check(N.lib().pt_bf_set_plan(res.handle, k, slices))
    try:
        got = cuda.BruteForce(res, AccelerationSoftened(0.01)).compute(b)
    finally:
        N.check(N.lib().pt_bf_set_plan(res.handle, 0, 0))
    assert rel(got, ref64).max() < 5e-6


def test_f64_judge_matches_oracle(res, oracle):
    import torch
    b = ics.plummer(3000, seed=13)["bodies"]
    d = torch.from_numpy(b).cuda()
    out = torch.zeros((3000, 3), dtype=torch.float64, device="cuda")
    N.check(N.lib().pt_bf_accel_f64_device(res.handle, d.data_ptr(), 3000, d.data_ptr(), 3000,
                                           0.01, 1, out.data_ptr()))
    res.synchronize()
    want = oracle.bf_f64(b, b, 0.01, True)
    assert rel(out.cpu().numpy(), want).max() < 1e-12


def test_device_api_matches_host_api(res):
    import torch
    b = ics.plummer(5000, seed=14)["bodies"]
    host = cuda.BruteForce(res, AccelerationSoftened(0.01)).compute(b)
    d = torch.from_numpy(b).cuda()
    out = torch.zeros((5000, 3), dtype=torch.float32, device="cuda")
    N.check(N.lib().pt_bf_accel_f32_device(res.handle, d.data_ptr(), 5000, d.data_ptr(), 5000,
                                           0.01, 1, 0, out.data_ptr()))
    res.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


@pytest.mark.parametrize("exact", [False, True])
def test_kat_acceleration_error(res, exact):
    m = cuda.BruteForce(res, Acceleration.checked(), exact=exact)
    kat.acceleration_error(m.compute, 1e-2)


@pytest.mark.parametrize("exact", [False, True])
def test_kat_circular_orbit(res, exact):
    m = cuda.BruteForce(res, Acceleration.checked(), exact=exact)
    kat.circular_orbit(m.compute, 100, 1e-2)  # 100 orbits, as the reference's gpu test


def test_storages(res, oracle):
    p = mixed(2000, 15)
    m = cuda.BruteForce(res, AccelerationSoftened(0.01), exact=True)
    r = Reordered(p)
    want = oracle.bf_f32(p, r.affecting(), 0.01, True)
    assert np.array_equal(m.compute(r), want)
    o = Ordered.new(p)
    want = oracle.bf_f32(o.particles(), o.affecting(), 0.01, True)
    assert np.array_equal(m.compute(o), want)
    assert np.array_equal(cuda.cuda_brute_force(r, res, AccelerationSoftened(0.01), exact=True),
                          m.compute(r))


def test_edge_cases(res):
    m = cuda.BruteForce(res, Acceleration.checked())
    b = ics.uniform_cube(10)["bodies"]
    assert not m.compute(Between(b, np.zeros((0, 4), np.float32))).any()
    assert m.compute(Between(np.zeros((0, 4), np.float32), b)).shape == (0, 3)
    # unchecked with coincident bodies and no softening: NaN, as the reference
    bad = np.array([[0, 0, 0, 1], [0, 0, 0, 1]], np.float32)
    with np.errstate(all="ignore"):
        assert np.isnan(cuda.BruteForce(res, Acceleration.unchecked()).compute(bad)).all()
    assert not np.isnan(m.compute(bad)).any()


def test_capacity_limit_is_reported(res):
    from particular_gb300 import CudaResources
    with CudaResources(0) as r:
        r.set_capacity_limit(1024)
        b = ics.uniform_cube(4096)["bodies"]
        with pytest.raises(N.CudaError) as e:
            cuda.BruteForce(r, Acceleration.checked()).compute(b)
        assert e.value.code == N.PT_ERR_CAPACITY
        r.set_capacity_limit(0)
        assert cuda.BruteForce(r, Acceleration.checked()).compute(b).shape == (4096, 3)


def test_unaligned_device_pointer_rejected(res):
    import torch
    d = torch.zeros(4 * 100 + 1, dtype=torch.float32, device="cuda")
    out = torch.zeros(300, dtype=torch.float32, device="cuda")
    rc = N.lib().pt_bf_accel_f32_device(res.handle, d.data_ptr() + 4, 10, d.data_ptr(), 10, 0.0,
                                        1, 0, out.data_ptr())
    assert rc == N.PT_ERR_INVALID and "aligned" in N.last_error()


def test_full_size_properties(res, oracle):
    """N=131072 Plummer: momentum balance (Newton's third law) and FP64 sample error."""
    b = ics.plummer(131072)["bodies"]
    a = cuda.BruteForce(res, AccelerationSoftened(0.01)).compute(b).astype(np.float64)
    m = b[:, 3].astype(np.float64)[:, None]
    net = np.abs((m * a).sum(0)).max()
    scale = (m * np.abs(a)).sum()
    assert net / scale < 1e-6
    idx = np.random.default_rng(0).choice(131072, 512, replace=False)
    ref = oracle.bf_f64(b[idx], b, 0.01, True)
    e = rel(a[idx], ref)
    assert np.percentile(e, 95) < 1e-6 and e.max() < 1e-5


@pytest.mark.parametrize("softening,checked", [(0.0, True), (1e-3, True)])
def test_exact_vec3a_operand_order(res, oracle, softening, checked):
    """glam Vec3A/Vec4's kernel (d * m / ...): bit-identical to its restatement, and
    not the same bits as the default order (so the flag does something)."""
    b = mixed(3000, 71)
    it = AccelerationSoftened(softening, checked)
    got = cuda.BruteForce(res, it, exact=True, vec3a=True).compute(b)
    want = oracle.bf_f32_vec3a(b, b, softening, checked)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    other = oracle.bf_f32(b, b, softening, checked)
    assert not np.array_equal(got.view(np.uint32), other.view(np.uint32))


def test_two_dimensional_bodies_through_z0(res, oracle):
    """2D particles (glam Vec2) as z = 0: the 2D reference sum (x*x + y*y) is what the
    3D path computes bit for bit, with a zero z acceleration."""
    b = ics.uniform_cube(2000, 72)["bodies"].copy()
    b[:, 2] = 0.0
    got = cuda.BruteForce(res, AccelerationSoftened(1e-3), exact=True).compute(b)
    s = np.float32
    x, y, m = b[:, 0], b[:, 1], b[:, 3]
    acc = np.zeros((2000, 2), np.float32)
    for j in range(2000):  # the 2D restatement, vectorised over targets
        dx, dy = x[j] - x, y[j] - y
        n = dx * dx + dy * dy
        ns = n + s(1e-3) * s(1e-3)
        q = m[j] / (ns * np.sqrt(ns))
        a = np.stack([dx * q, dy * q], 1)
        a = np.where((n == 0)[:, None], np.stack([dx, dy], 1), a)
        acc = acc + a
    assert np.array_equal(got[:, :2].view(np.uint32), acc.view(np.uint32))
    assert not got[:, 2].any()
