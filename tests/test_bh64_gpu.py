"""Row f3 for Barnes-Hut: glam DVec3 bodies through the f64 method, against the
oracle's restatement of the reference's f64 orthtree and walk."""
import numpy as np
import pytest

import kat
from particular_gb300 import Acceleration, AccelerationSoftened, Between, cuda, ics
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def bodies64(kind, n, seed):
    b = {"plummer": lambda: ics.plummer(n, seed=seed)["bodies"],
         "bulge_disk": lambda: ics.bulge_disk(n, seed=seed)["bodies"],
         "cube": lambda: ics.uniform_cube(n, seed)["bodies"]}[kind]().astype(np.float64)
    b[:, :3] += np.random.default_rng(seed).normal(scale=1e-9, size=(n, 3))  # bits below f32
    return b


class _Tree64:
    def __init__(self, e):
        self._e = e

    def export(self):
        return self._e


@pytest.mark.parametrize("kind,n", [("plummer", 3000), ("bulge_disk", 4000)])
def test_f64_tree_matches_reference_orthtree(res, oracle, kind, n):
    from test_bh_gpu import oracle_preorder
    b = bodies64(kind, n, 60)
    m = cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01), dvec3=True)
    m.compute(b)
    g = m.export_tree_dvec3()
    order, e = oracle_preorder(_Tree64(oracle.tree_dvec3_export(b)))
    assert g["links"].shape[0] == order.size
    internal = e["internal"][order].astype(bool)
    assert np.array_equal(internal, g["links"][:, 2] < 0)
    # widths: the reference's f64 subdivision, bit for bit
    w_ref = (e["box"][order, 3] - e["box"][order, 0])[internal]
    assert np.array_equal(g["width"][internal], w_ref)
    # leaves are their body; cells carry the FP64 centre of mass of their bodies
    assert np.array_equal(g["com_mass"][~internal], e["data"][order][~internal])
    cm, ref = g["com_mass"][internal], e["data"][order][internal]
    np.testing.assert_allclose(cm[:, 3], ref[:, 3], rtol=1e-13)
    assert np.abs(cm[:, :3] - ref[:, :3]).max() <= 1e-13 * np.abs(b[:, :3]).max()


@pytest.mark.parametrize("theta", [0.0, 0.3, 0.5, 0.8])
def test_f64_walk_matches_reference(res, oracle, theta):
    b = bodies64("plummer", 20000, 61)
    m = cuda.BarnesHut(theta, res, AccelerationSoftened(0.01), dvec3=True)
    got = m.compute(b)
    st = m.stats()
    ref, acc = oracle.bh_dvec3(b, b, theta, 0.01, True, accepted=True)
    r = rel(got, ref)
    print(f"theta={theta} accepted gpu={st['interactions']} ref={int(acc.sum())} rel diff p50={np.median(r):.2e} "
          f"max={r.max():.2e}")
    assert got.dtype == np.float64
    assert abs(st["interactions"] - int(acc.sum())) <= 1e-4 * acc.sum()
    assert np.median(r) < 1e-13 and r.max() < 1e-8


def test_f64_separate_targets_and_edges(res, oracle):
    src = bodies64("bulge_disk", 8000, 62)
    tgt = bodies64("cube", 1000, 63)
    tgt[:, 3] = 0.0
    m = cuda.BarnesHut(0.5, res, Acceleration.checked(), dvec3=True)
    got = m.compute(Between(tgt, src))
    ref = oracle.bh_dvec3(tgt, src, 0.5, 0.0, True)
    r = rel(got, ref)
    assert np.median(r) < 1e-13 and r.max() < 1e-8
    assert m.compute(Between(np.zeros((0, 4)), src)).shape == (0, 3)
    assert np.array_equal(m.compute(Between(tgt, np.zeros((0, 4)))), np.zeros((1000, 3)))
    with pytest.raises(N.CudaError):
        cuda.BarnesHut(0.5, res, Acceleration.checked(), quadrupole=True, dvec3=True).compute(src)


@pytest.mark.parametrize("theta,err_eps,orbit_eps", [(0.0, 1e-2, 1e-2), (0.5, 5e-1, 1e-1)])
def test_f64_kats(res, theta, err_eps, orbit_eps):
    m = cuda.BarnesHut(theta, res, Acceleration.checked(), dvec3=True)
    kat.acceleration_error(m.compute, err_eps)
    kat.circular_orbit(m.compute, 10, orbit_eps)
