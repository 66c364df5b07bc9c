"""Kick-drift-kick leapfrog around the cuda methods, eager and CUDA-graph replayed."""
import numpy as np
import pytest

from particular_gb300 import AccelerationSoftened, cuda, ics
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def energy(b, v, eps):
    b = b.astype(np.float64)
    v = v.astype(np.float64)
    m = b[:, 3]
    K = 0.5 * (m * (v[:, :3] ** 2).sum(1)).sum()
    W = 0.0
    for i in range(0, b.shape[0], 512):
        d = b[i:i + 512, None, :3] - b[None, :, :3]
        r = np.sqrt((d ** 2).sum(-1) + eps * eps)
        W -= 0.5 * (m[i:i + 512, None] * m[None, :] / r).sum()
        # remove the self terms m_i^2 / eps
        W += 0.5 * (m[i:i + 512] ** 2 / eps).sum()
    return K + W


def oracle_leapfrog(O, b, v, dt, steps, eps):
    """The same KDK scheme driven by the oracle's brute force (float32 state)."""
    b = b.copy()
    v = v[:, :3].astype(np.float32).copy()
    a = O.bf_f32(b, b, eps, True)
    for s in range(steps):
        k = np.float32(0.5 * dt if s == 0 else dt)
        v = v + a * k
        b[:, :3] = b[:, :3] + v * np.float32(dt)
        a = O.bf_f32(b, b, eps, True)
    v = v + a * np.float32(0.5 * dt)
    return b, v


def test_leapfrog_matches_oracle_integration(res, oracle):
    d = ics.plummer(512, seed=51)
    lf = cuda.Leapfrog(cuda.BruteForce(res, AccelerationSoftened(0.01)), 1e-3)
    b, v = lf.run(d["bodies"], d["vel"], 10)
    rb, rv = oracle_leapfrog(oracle, d["bodies"], d["vel"], 1e-3, 10, 0.01)
    scale = np.abs(rb[:, :3]).max()
    assert np.abs(b[:, :3] - rb[:, :3]).max() < 1e-5 * scale
    assert np.abs(v - rv).max() < 1e-4 * np.abs(rv).max()
    assert np.array_equal(b[:, 3], d["bodies"][:, 3])


@pytest.mark.parametrize("method", ["bf", "bh", "bh_local", "bh_relative", "bh_reference_rule"])
def test_graph_replay_equals_eager(res, method):
    import torch
    d = ics.plummer(20000, seed=52)
    L = N.lib()
    if method == "bf":
        args = (N.PT_METHOD_BRUTE_FORCE, 0.0, 0.01, 0)
    elif method == "bh":
        args = (N.PT_METHOD_BARNES_HUT, 0.5, 0.01, N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP)
    elif method == "bh_local":
        args = (N.PT_METHOD_BARNES_HUT, 0.5, 0.01, N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP | N.PT_BH_LOCAL)
    elif method == "bh_relative":
        args = (N.PT_METHOD_BARNES_HUT, 1.0, 0.01,
                N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP | N.PT_BH_LOCAL | N.PT_BH_RELATIVE)
    else:
        args = (N.PT_METHOD_BARNES_HUT, 0.5, 0.01, 0)
    outs = []
    for use_graph in (0, 1):
        b = torch.from_numpy(d["bodies"]).cuda()
        v = torch.zeros((20000, 4), device="cuda")
        v[:, :3] = torch.from_numpy(d["vel"]).cuda()
        a = torch.zeros((20000, 3), device="cuda")
        m, th, eps, fl = args
        if method == "bf":
            N.check(L.pt_bf_accel_f32_device(res.handle, b.data_ptr(), 20000, b.data_ptr(), 20000,
                                             eps, 1, fl, a.data_ptr()))
        else:
            N.check(L.pt_bh_accel_f32_device(res.handle, b.data_ptr(), 20000, b.data_ptr(), 20000,
                                             th, eps, fl, a.data_ptr()))
        for _ in range(3):  # three calls: capture once, replay twice
            N.check(L.pt_leapfrog_device(res.handle, b.data_ptr(), v.data_ptr(), a.data_ptr(), 20000,
                                         1e-3, 5, m, th, eps, fl, use_graph))
        res.synchronize()
        outs.append((b.cpu().numpy(), v.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_energy_is_conserved(res):
    d = ics.plummer(4096, seed=53)
    eps = 0.01
    e0 = energy(d["bodies"], d["vel"], eps)
    lf = cuda.Leapfrog(cuda.BruteForce(res, AccelerationSoftened(eps)), 1e-3)
    b, v = lf.run(d["bodies"], d["vel"], 200)
    e1 = energy(b, v, eps)
    assert abs(e1 - e0) / abs(e0) < 1e-4


def test_barnes_hut_leapfrog_tracks_brute_force(res):
    d = ics.bulge_disk(30000, seed=54)
    bf = cuda.Leapfrog(cuda.BruteForce(res, AccelerationSoftened(0.01)), 1e-3)
    bh = cuda.Leapfrog(cuda.BarnesHut(0.5, res, AccelerationSoftened(0.01), quadrupole=True,
                                      group=True), 1e-3)
    b1, v1 = bf.run(d["bodies"], d["vel"], 10)
    b2, v2 = bh.run(d["bodies"], d["vel"], 10)
    dv = np.linalg.norm(v2 - v1, axis=1) / np.maximum(np.linalg.norm(v1 - d["vel"], axis=1), 1e-12)
    assert np.percentile(dv, 95) < 5e-3  # velocity change agrees to BH accuracy


def test_graph_recaptured_when_settings_change(res):
    """A captured leapfrog carries the context's Barnes-Hut settings (error-bound
    factor, local ratio) as launch parameters: changing them captures again, so the
    replay equals the eager steps under the new values."""
    import torch
    d = ics.plummer(20000, seed=53)
    L = N.lib()
    fl = N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP | N.PT_BH_LOCAL | N.PT_BH_RELATIVE
    outs = []
    try:
        for use_graph in (0, 1):
            b = torch.from_numpy(d["bodies"]).cuda()
            v = torch.zeros((20000, 4), device="cuda")
            v[:, :3] = torch.from_numpy(d["vel"]).cuda()
            a = torch.zeros((20000, 3), device="cuda")
            for alpha, ratio in ((2.5e-3, 0.1), (1e-3, 0.13)):
                N.check(L.pt_bh_set_relative_alpha(res.handle, alpha))
                N.check(L.pt_bh_set_local_ratio(res.handle, ratio))
                N.check(L.pt_bh_accel_f32_device(res.handle, b.data_ptr(), 20000, b.data_ptr(), 20000,
                                                 1.0, 0.01, fl, a.data_ptr()))
                for _ in range(2):
                    N.check(L.pt_leapfrog_device(res.handle, b.data_ptr(), v.data_ptr(), a.data_ptr(), 20000,
                                                 1e-3, 3, N.PT_METHOD_BARNES_HUT, 1.0, 0.01, fl, use_graph))
            res.synchronize()
            outs.append((b.cpu().numpy(), v.cpu().numpy()))
    finally:
        N.check(L.pt_bh_set_relative_alpha(res.handle, 2.5e-3))
        N.check(L.pt_bh_set_local_ratio(res.handle, 0.1))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_graph_recaptured_when_buffers_grow():
    """A captured leapfrog holds the addresses of the context's grow-only buffers. A
    bigger Barnes-Hut call on the same context between two replays reallocates them
    (every reallocation bumps the context's buffer epoch), so the next replay
    captures again and still equals the eager steps."""
    import torch
    from particular_gb300 import CudaResources
    n, n_big = 20000, 400000
    d = ics.plummer(n, seed=55)
    big = ics.plummer(n_big, seed=56)
    L = N.lib()
    fl = N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP | N.PT_BH_LOCAL
    outs = []
    for use_graph in (0, 1):
        r = CudaResources(0)
        try:
            b = torch.from_numpy(d["bodies"]).cuda()
            v = torch.zeros((n, 4), device="cuda")
            v[:, :3] = torch.from_numpy(d["vel"]).cuda()
            a = torch.zeros((n, 3), device="cuda")
            bb = torch.from_numpy(big["bodies"]).cuda()
            ab = torch.zeros((n_big, 3), device="cuda")
            torch.cuda.synchronize()
            N.check(L.pt_bh_accel_f32_device(r.handle, b.data_ptr(), n, b.data_ptr(), n,
                                             0.5, 0.01, fl, a.data_ptr()))
            for k in range(3):
                N.check(L.pt_leapfrog_device(r.handle, b.data_ptr(), v.data_ptr(), a.data_ptr(), n,
                                             1e-3, 3, N.PT_METHOD_BARNES_HUT, 0.5, 0.01, fl, use_graph))
                if k == 0:  # grows the tree buffers between the capture and the replays
                    N.check(L.pt_bh_accel_f32_device(r.handle, bb.data_ptr(), n_big, bb.data_ptr(),
                                                     n_big, 0.5, 0.01, fl, ab.data_ptr()))
            r.synchronize()
            outs.append((b.cpu().numpy(), v.cpu().numpy()))
        finally:
            r.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
