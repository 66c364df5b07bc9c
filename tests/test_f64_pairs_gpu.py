"""Rows f3 and f4: glam DVec3 bodies (float64 end to end) and BruteForcePairs
semantics, against the oracle's restatements."""
import numpy as np
import pytest

import kat
from particular_gb300 import (Acceleration, AccelerationSoftened, Between, Ordered, Reordered, cuda, ics)

pytestmark = pytest.mark.gpu


def bodies64(n, seed):
    b = ics.uniform_cube(n, seed)["bodies"].astype(np.float64)
    b[:, :3] += np.random.default_rng(seed).normal(scale=1e-9, size=(n, 3))  # bits below f32
    b[::9, 3] = 0.0
    if n > 7:
        b[6, :3] = b[3, :3]  # coincident pair
    return b


@pytest.mark.parametrize("n", [1, 37, 1000, 4099])
@pytest.mark.parametrize("softening,checked", [(0.0, True), (1e-3, True), (0.05, False)])
def test_dvec3_bit_identical(res, oracle, n, softening, checked):
    b = bodies64(n, 30 + n)
    if not checked:
        b = ics.uniform_cube(n, 31)["bodies"].astype(np.float64)
    it = AccelerationSoftened(softening, checked) if softening else Acceleration(checked)
    got = cuda.BruteForce(res, it, dvec3=True).compute(b)
    want = oracle.bf_dvec3(b, b, softening, checked)
    assert got.dtype == np.float64
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_dvec3_storages(res, oracle):
    b = bodies64(3000, 32)
    m = cuda.BruteForce(res, AccelerationSoftened(1e-3), dvec3=True)
    src = b[b[:, 3] != 0]
    # Ordered and Reordered keep float64 values when built with dtype=np.float64
    o = Ordered.new(b, dtype=np.float64)
    np.testing.assert_array_equal(m.compute(o), oracle.bf_dvec3(o.particles(), o.affecting(), 1e-3, True))
    r = Reordered(b, dtype=np.float64)
    np.testing.assert_array_equal(m.compute(r), oracle.bf_dvec3(b, src, 1e-3, True))
    t = ics.uniform_cube(100, 33)["bodies"].astype(np.float64)
    np.testing.assert_array_equal(m.compute(Between(t, b)), oracle.bf_dvec3(t, b, 1e-3, True))


def test_dvec3_kats(res):
    m = cuda.BruteForce(res, Acceleration.checked(), dvec3=True)
    kat.acceleration_error(m.compute, 1e-2)
    kat.circular_orbit(m.compute, 10, 1e-2)


def test_dvec3_device_entry_point(res, oracle):
    import torch
    from particular_gb300 import _native as N
    b = bodies64(2000, 34)
    d_b = torch.from_numpy(b).cuda()
    d_o = torch.empty((2000, 3), dtype=torch.float64, device="cuda")
    N.check(N.lib().pt_bf_accel_dvec3_device(res.handle, d_b.data_ptr(), 2000, d_b.data_ptr(), 2000, 1e-3, 1,
                                             d_o.data_ptr()))
    res.synchronize()
    np.testing.assert_array_equal(d_o.cpu().numpy(), oracle.bf_dvec3(b, b, 1e-3, True))


@pytest.mark.parametrize("ordered", [False, True])
def test_brute_force_pairs_semantics(res, oracle, ordered):
    """BruteForcePairs (sequential.rs:232-304) sums every pair once; cuda::BruteForce
    sums all of them. The accelerations agree within the summation-order tolerance:
    1e-5 of the largest for f32, 1e-12 for DVec3 bodies."""
    b = ics.plummer(4096, seed=35)["bodies"].copy()
    r = None
    if ordered:
        b[3000:, 3] = 0.0  # massless tail: Ordered's affecting prefix is the first 3000
        r = 3000
        storage = Ordered.new(b)
        storage64 = Ordered.new(b, dtype=np.float64)
    else:
        storage, storage64 = b, b.astype(np.float64)
    want32 = oracle.bf_pairs(b, restrict_len=r, softening=0.01)
    want64 = oracle.bf_pairs(b.astype(np.float64), restrict_len=r, softening=0.01)
    scale = np.abs(want64).max()
    for exact in (False, True):
        got = cuda.BruteForce(res, AccelerationSoftened(0.01), exact=exact).compute(storage)
        assert np.abs(got - want32).max() < 1e-5 * scale, exact
    got64 = cuda.BruteForce(res, AccelerationSoftened(0.01), dvec3=True).compute(storage64)
    assert np.abs(got64 - want64).max() < 1e-12 * scale


def test_in_order_fold_of_the_reference_doctest(res):
    """The fold that particular's brute force documents (lib.rs:212-262: forces[i] is
    the sum of the pair terms in j order from zero, the self term included as zero),
    for that doctest's sun / earth / jupiter bodies (AU, solar masses, G = 4 pi^2)
    with the acceleration interaction (unsoftened, checked) in double, each pair term
    as gravity/impls/mod.rs:150-166 computes it: bit for bit."""
    G = 4.0 * np.pi * np.pi
    b = np.array([[0.0, 0.0, 0.0, 1.0 * G], [1.0, 0.0, 0.0, 3.0027e-6 * G], [5.2, 0.0, 0.0, 0.000954588 * G]],
                 np.float64)
    got = cuda.BruteForce(res, Acceleration.checked(), dvec3=True).compute(b)

    def pair(i, j):
        d = b[j, :3] - b[i, :3]
        n = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
        if n == 0.0:
            return d
        return d * (b[j, 3] / (n * np.sqrt(n)))

    for i in range(3):
        acc = np.zeros(3)
        for j in range(3):
            acc = acc + pair(i, j)
        assert np.array_equal(got[i], acc), (i, got[i], acc)
