"""Barnes-Hut over a tree the caller built (pt_bh_load_tree): the GPU counterpart of
computing Between(affected, &tree) over a RootedOrthtree (particular/src/lib.rs:186-199,
sequential.rs:466-522). The tree handed over is the oracle's own orthtree, in the
reference's Orthtree layout (orthant slots, bounding boxes, Node::Internal flags,
GravitationalField data), and the walk must accept, body for body, the nodes the
reference's walk of that same tree accepts."""
import numpy as np
import pytest

from particular_gb300 import AccelerationSoftened, Between, cuda, ics
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def rel(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-30)


def load(m, e, root=0):
    return m.load_tree(e["internal"], e["child"], e["box"], e["data"], root)


@pytest.mark.parametrize("theta", [0.3, 0.5, 0.8])
@pytest.mark.parametrize("group", [False, True])
def test_oracle_tree_walked_on_the_gpu(res, oracle, theta, group):
    b = ics.plummer(20000, seed=71)["bodies"]
    t = oracle.Tree(b)
    m = cuda.BarnesHut(theta, res, AccelerationSoftened(0.01), group=group)
    tree = load(m, t.export())
    got = m.compute(Between(b, tree))
    st = m.stats()
    ref, acc = t.walk(b, theta, 0.01, True, accepted=True)
    if not group:
        # the reference rule per body over the very same nodes: the same accepted
        # sets (opening tests on the same f32 data; an FMA in d^2 may flip a decision
        # that sits exactly on the boundary)
        assert abs(int(st["interactions"]) - int(acc.sum())) <= 1e-5 * acc.sum()
        r = rel(got, ref)
        assert np.median(r) < 1e-6 and np.percentile(r, 99) < 1e-5
    else:
        # a group opens a cell whenever one of its bodies would: more nodes, never
        # less accurate against the FP64 judge
        assert st["interactions"] >= acc.sum()
        ref64 = oracle.bf_f64(b[::20], b, 0.01, True)
        e, e_ref = rel(got[::20], ref64), rel(ref[::20], ref64)
        for q in (50, 95):
            assert np.percentile(e, q) <= np.percentile(e_ref, q) * 1.01 + 1e-7


def test_separate_targets_and_the_device_tree(res, oracle):
    """Separate targets walking the oracle's tree on the GPU get the reference walk's
    accelerations; the device's own tree of the same bodies is at least as accurate
    against the FP64 judge (its cell moments are compensated sums, where the
    reference's f32 sums in body order drift by ~sqrt(count) roundings)."""
    src = ics.bulge_disk(30000, seed=72)["bodies"]
    aff = ics.uniform_cube(3000, 73)["bodies"] * np.float32(3.0)
    t = oracle.Tree(src)
    m = cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01))
    got = m.compute(Between(aff, load(m, t.export())))
    r = rel(got, t.walk(aff, 0.5, 0.01, True))
    assert np.median(r) < 1e-6 and np.percentile(r, 99) < 1e-5
    ref64 = oracle.bf_f64(aff, src, 0.01, True)
    own = m.compute(Between(aff, src))
    for q in (50, 95):
        assert np.percentile(rel(own, ref64), q) <= np.percentile(rel(got, ref64), q) * 1.01


def test_edge_cases(res):
    m = cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01))
    aff = ics.uniform_cube(100, 74)["bodies"]
    none = np.zeros((0,), np.uint8)
    # RootedOrthtree with root None: nothing attracts
    tree = m.load_tree(none, np.zeros((0, 8), np.int32), np.zeros((0, 6), np.float32),
                       np.zeros((0, 4), np.float32), root=-1)
    assert not m.compute(Between(aff, tree)).any()
    # one external node: the per-pair kernel with its data
    d = np.array([[3.0, 0.0, 0.0, 2.0]], np.float32)
    tree = m.load_tree(np.zeros(1, np.uint8), -np.ones((1, 8), np.int32), np.zeros((1, 6), np.float32), d)
    p = np.array([[0.0, 0.0, 0.0, 0.0]], np.float32)
    a = m.compute(Between(p, tree))
    np.testing.assert_allclose(a[0], [2.0 / (9.0 + 1e-4) ** 1.5 * 3.0, 0.0, 0.0], rtol=1e-6)
    # an internal node without children: opened it adds nothing, accepted it adds its data
    box = np.array([[-1, -1, -1, 1, 1, 1]], np.float32)
    tree = m.load_tree(np.ones(1, np.uint8), -np.ones((1, 8), np.int32), box, d)
    assert not m.compute(Between(p, tree)).any()  # theta 0.5: 0.25 * 9 < 4, opened
    far = cuda.BarnesHut(2.0, res, AccelerationSoftened(0.01))
    tree = far.load_tree(np.ones(1, np.uint8), -np.ones((1, 8), np.int32), box, d)
    np.testing.assert_allclose(far.compute(Between(p, tree))[0], a[0], rtol=1e-6)


def test_invalid_trees_are_rejected(res):
    L = N.lib()
    m = cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01))
    box = np.tile(np.array([-1, -1, -1, 1, 1, 1], np.float32), (2, 1))
    d = np.array([[0.5, 0, 0, 1], [0.5, 0, 0, 1]], np.float32)
    kids = -np.ones((2, 8), np.int32)
    kids[0, 3] = 5  # no node 5
    with pytest.raises(N.CudaError, match="orthant slot"):
        m.load_tree(np.array([1, 0], np.uint8), kids, box, d)
    kids[0, 3] = 0  # the root as its own child
    with pytest.raises(N.CudaError, match="reachable twice"):
        m.load_tree(np.array([1, 0], np.uint8), kids, box, d)
    with pytest.raises(N.CudaError, match="root"):
        m.load_tree(np.array([1, 0], np.uint8), -np.ones((2, 8), np.int32), box, d, root=2)
    # a caller-built tree carries no quadrupoles
    kids[0, 3] = 1
    tree = m.load_tree(np.array([1, 0], np.uint8), kids, box, d)
    q = cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01), quadrupole=True)
    with pytest.raises(N.CudaError, match="monopoles only"):
        q.compute(Between(np.zeros((4, 4), np.float32), tree))
    assert L.pt_bh_load_tree(None, None, None, None, None, 0, -1, None) == N.PT_ERR_INVALID


@pytest.mark.parametrize("theta", [0.3, 0.8])
def test_walk_sums_are_compensated(res, oracle, theta):
    """Per-body forces are summed with compensation: over the reference's accepted set
    (the oracle's tree walked on the GPU with the reference rule), the GPU result stays
    closer to the FP64 sum of the same terms than the reference's own FP32 sum in visit
    order (sequential.rs:497-500), measured against each body's sum of term norms."""
    b = ics.plummer(20000, seed=75)["bodies"]
    t = oracle.Tree(b)
    s64, l1 = t.walk_sum64(b, theta, 0.01)
    ref32 = t.walk(b, theta, 0.01)
    m = cuda.BarnesHut(theta, res, AccelerationSoftened(0.01))
    got = m.compute(Between(b, load(m, t.export())))
    e_gpu = np.linalg.norm(got - s64, axis=1) / l1
    e_ref = np.linalg.norm(ref32 - s64, axis=1) / l1
    print(f"theta {theta}: |sum - FP64 sum| / sum|term|, p50/p99: GPU {np.median(e_gpu):.2e}/"
          f"{np.percentile(e_gpu, 99):.2e}, reference f32 order {np.median(e_ref):.2e}/{np.percentile(e_ref, 99):.2e}")
    assert np.median(e_gpu) < 0.5 * np.median(e_ref)
    assert np.percentile(e_gpu, 99) < np.percentile(e_ref, 99)
