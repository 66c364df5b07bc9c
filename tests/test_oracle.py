"""Pins the CPU oracle (oracle/pt_oracle.c) to the reference's own tests.

The reference holds no golden vectors; its known-answer tests are
acceleration_error! and circular_orbit! (particular/src/gravity/newtonian/mod.rs:228-347),
run on sequential::BruteForce, BarnesHut(0.0) and BarnesHut(0.5) with the tolerances
of mod.rs:382-420. The oracle must pass them exactly as the reference's methods do.
"""
import numpy as np
import pytest

import kat
from particular_gb300 import as_between, fields, ics, positions


def oracle_method(O, kind, theta=0.0, softening=0.0, checked=True):
    def compute(storage):
        b = as_between(storage)
        aff, src = positions(b.affected), fields(b.affecting)
        if kind == "bf":
            return O.bf_f32(aff, src, softening, checked, threads=1)
        return O.bh_f32(aff, src, theta, softening, checked, threads=1)
    return compute


KAT_CASES = [("bf", 0.0, 1e-2, 1e-2), ("bh", 0.0, 1e-2, 1e-2), ("bh", 0.5, 5e-1, 1e-1)]


@pytest.mark.parametrize("kind,theta,err_eps,orbit_eps", KAT_CASES)
def test_kat_acceleration_error(oracle, kind, theta, err_eps, orbit_eps):
    kat.acceleration_error(oracle_method(oracle, kind, theta), err_eps)


@pytest.mark.parametrize("kind,theta,err_eps,orbit_eps", KAT_CASES)
def test_kat_circular_orbit(oracle, kind, theta, err_eps, orbit_eps):
    # 1000 orbits, as the reference's CPU tests (mod.rs:386, 412, 419).
    kat.circular_orbit(oracle_method(oracle, kind, theta), 1000, orbit_eps)


def numpy_bf_f32(aff, src, softening, checked):
    """Independent restatement of sequential::BruteForce in numpy float32
    (vectorised over targets, sequential over sources, every op rounded to f32)."""
    s = np.float32
    x = aff[:, :3].astype(s)
    acc = np.zeros_like(x)
    e2 = s(softening) * s(softening)
    with np.errstate(all="ignore"):
        for j in range(src.shape[0]):
            d = src[j, :3][None, :] - x
            n = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            ns = n + e2
            q = src[j, 3] / (ns * np.sqrt(ns))
            a = d * q[:, None]
            if checked:
                a = np.where((n == 0)[:, None], d, a)
            acc = acc + a
    return acc


def mixed_bodies(n, seed):
    b = ics.uniform_cube(n, seed)["bodies"].copy()
    b[::7, 3] = 0.0          # massless bodies
    b[5] = b[3]              # a coincident pair
    b[6, :3] = b[3, :3]
    return b


@pytest.mark.parametrize("softening,checked", [(0.0, True), (1e-3, True), (0.05, False)])
def test_bf_bit_identical_to_numpy_restatement(oracle, softening, checked):
    b = mixed_bodies(300, 7)
    if not checked:
        b = ics.uniform_cube(300, 8)["bodies"]
    got = oracle.bf_f32(b, b, softening, checked, threads=1)
    want = numpy_bf_f32(b, b, softening, checked)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def numpy_bf_dvec3(aff, src, softening, checked):
    """The same restatement in float64 (glam DVec3 bodies)."""
    x = aff[:, :3]
    acc = np.zeros_like(x)
    e2 = softening * softening
    with np.errstate(all="ignore"):
        for j in range(src.shape[0]):
            d = src[j, :3][None, :] - x
            n = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            ns = n + e2
            a = d * (src[j, 3] / (ns * np.sqrt(ns)))[:, None]
            if checked:
                a = np.where((n == 0)[:, None], d, a)
            acc = acc + a
    return acc


@pytest.mark.parametrize("softening,checked", [(0.0, True), (1e-3, True), (0.05, False)])
def test_dvec3_bit_identical_to_numpy_restatement(oracle, softening, checked):
    b = mixed_bodies(300, 10).astype(np.float64)
    b[:, :3] += np.random.default_rng(1).normal(scale=1e-9, size=(300, 3))  # bits below f32
    if not checked:
        b = ics.uniform_cube(300, 11)["bodies"].astype(np.float64)
    got = oracle.bf_dvec3(b, b, softening, checked, threads=1)
    want = numpy_bf_dvec3(b, b, softening, checked)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_pairs_restatement_agrees_with_brute_force(oracle):
    """BruteForcePairs sums each pair once (a_i += dir m_j, a_j -= dir m_i): the same
    accelerations as BruteForce up to summation order; on Ordered storage only the
    affecting prefix acts (restrict_len)."""
    b = ics.uniform_cube(500, 12)["bodies"].copy()
    bf = oracle.bf_f64(b, b, 1e-3, True)
    p32 = oracle.bf_pairs(b, softening=1e-3)
    p64 = oracle.bf_pairs(b.astype(np.float64), softening=1e-3)
    scale = np.abs(bf).max()
    assert np.abs(p64 - bf).max() < 1e-12 * scale
    assert np.abs(p32 - bf).max() < 1e-5 * scale
    # Ordered: 200 massive first, then 300 massless
    b[200:, 3] = 0.0
    p = oracle.bf_pairs(b.astype(np.float64), restrict_len=200, softening=1e-3)
    want = oracle.bf_f64(b, b[:200], 1e-3, True)
    assert np.abs(p - want).max() < 1e-12 * np.abs(want).max()


def test_parallel_bf_bit_identical_to_sequential(oracle):
    b = mixed_bodies(2000, 9)
    one = oracle.bf_f32(b, b, 1e-3, True, threads=1)
    many = oracle.bf_f32(b, b, 1e-3, True, threads=4)
    assert np.array_equal(one.view(np.uint32), many.view(np.uint32))


def test_bh_theta0_is_brute_force_up_to_order(oracle):
    b = ics.plummer(3000, seed=3)["bodies"]
    bf = oracle.bf_f64(b, b, 0.01, True, threads=4)
    bh = oracle.bh_f32(b, b, 0.0, 0.01, True, threads=4)
    rel = np.linalg.norm(bh - bf, axis=1) / np.linalg.norm(bf, axis=1)
    # f32 summation over 3000 terms in another order: the same error the
    # reference's own f32 brute force shows against FP64 (up to a few 1e-5).
    assert rel.max() < 1e-4 and np.median(rel) < 2e-6


def test_bh_error_grows_with_theta(oracle):
    b = ics.plummer(4000, seed=4)["bodies"]
    ref = oracle.bf_f64(b, b, 0.01, True, threads=4)
    p95 = []
    for th in (0.3, 0.5, 0.8):
        a = oracle.bh_f32(b, b, th, 0.01, True, threads=4)
        rel = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
        p95.append(np.percentile(rel, 95))
    assert p95[0] < p95[1] < p95[2] < 0.1


def test_tree_structure(oracle):
    b = mixed_bodies(1500, 10)
    t = oracle.Tree(b)
    e = t.export()
    internal, child, box, rng = e["internal"].astype(bool), e["child"], e["box"], e["range"]
    n = b.shape[0]
    leaves = ~internal
    # every body sits in exactly one leaf
    assert rng[leaves, 1].sum() == n
    # a leaf holds one body or coincident bodies (tree/mod.rs:112-115)
    for k in np.flatnonzero(leaves):
        f, c = rng[k]
        pos = b[e["perm"][f:f + c], :3]
        assert (pos == pos[0]).all()
    # internal nodes: children partition the body range, boxes nest at half width
    for k in np.flatnonzero(internal):
        kids = child[k][child[k] >= 0]
        assert rng[kids, 1].sum() == rng[k, 1]
        w = box[k, 3] - box[k, 0]
        for c in kids:
            assert box[c, 3] - box[c, 0] == np.float32(w / 2) or abs((box[c, 3] - box[c, 0]) - w / 2) <= 1e-6 * w
    # the coincident pair ends up in one leaf
    assert rng[leaves, 1].max() >= 2


def test_bh_walk_threads_identical(oracle):
    b = ics.plummer(3000, seed=5)["bodies"]
    t = oracle.Tree(b)
    a1, c1 = t.walk(b, 0.5, 0.01, True, threads=1, accepted=True)
    a4, c4 = t.walk(b, 0.5, 0.01, True, threads=4, accepted=True)
    assert np.array_equal(a1.view(np.uint32), a4.view(np.uint32))
    assert np.array_equal(c1, c4)


def test_f64_judge_agrees_with_f32(oracle):
    b = ics.plummer(2000, seed=6)["bodies"]
    a32 = oracle.bf_f32(b, b, 0.01, True, threads=4)
    a64 = oracle.bf_f64(b, b, 0.01, True, threads=4)
    rel = np.linalg.norm(a32 - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert rel.max() < 1e-4


def test_empty_inputs(oracle):
    b = ics.uniform_cube(10)["bodies"]
    assert oracle.bf_f32(b, np.zeros((0, 4), np.float32)).shape == (10, 3)
    assert not oracle.bf_f32(b, np.zeros((0, 4), np.float32)).any()
    assert oracle.bh_f32(np.zeros((0, 4), np.float32), b, 0.5).shape == (0, 3)
    assert not oracle.bh_f32(b, np.zeros((0, 4), np.float32), 0.5).any()


def test_mlp_oracle_gradient_by_finite_differences():
    """The FP64 restatement of the learned-correction MLP (the GPU kernels' checker):
    its hand-written gradient agrees with central differences."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(1)
    p = rng.normal(scale=0.3, size=M.NPARAM)
    p[M.SCALE] = 1.7
    f = rng.normal(size=(16, 12))
    t = rng.normal(size=(16, 3))
    _, g = M.loss_grad(p, f, t)
    for k in rng.choice(M.SCALE, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_grad(pp, f, t)[0] - M.loss_grad(pm, f, t)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), k


def test_dvec3_barnes_hut_restatement(oracle):
    """The f64 orthtree and walk: theta 0 is the f64 brute force up to summation order,
    and at theta 0.5 the accepted sets match the f32 walk's on f32-exact positions."""
    b = ics.plummer(3000, seed=12)["bodies"].astype(np.float64)
    ref = oracle.bf_dvec3(b, b, 0.01)
    a0 = oracle.bh_dvec3(b, b, 0.0, 0.01)
    assert np.abs(a0 - ref).max() <= 1e-12 * np.abs(ref).max()
    a64, acc64 = oracle.bh_dvec3(b, b, 0.5, 0.01, accepted=True)
    a32, acc32 = oracle.bh_f32(b.astype(np.float32), b.astype(np.float32), 0.5, 0.01, accepted=True)
    assert np.array_equal(acc64, acc32)
    e = np.linalg.norm(a64 - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.percentile(e, 95) < 2e-2
