"""Batched ensembles: one persistent kernel advancing many systems of uneven size."""
import numpy as np
import pytest

from particular_gb300 import ics
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def small_ensemble(n_sys=24, seed=61):
    sizes = ics.ensemble_sizes(n_sys, 20, 900, seed)
    rng = ics.SplitMix64(seed + 7)
    offsets = np.zeros(n_sys + 1, np.uint32)
    offsets[1:] = np.cumsum(sizes)
    bodies, vel = [], []
    for k, n in enumerate(sizes):
        d = ics.plummer(int(n), a=float(rng.uniform(1, 0.5, 2.0)[0]), seed=seed + 100 + k)
        bodies.append(d["bodies"])
        vel.append(d["vel"])
    b = np.concatenate(bodies)
    v = np.zeros((b.shape[0], 4), np.float32)
    v[:, :3] = np.concatenate(vel)
    return offsets, b, v


def run_ensemble(res, offsets, b, v, steps, use_graph=0, dt=1e-3, eps=0.01):
    import torch
    db = torch.from_numpy(b).cuda()
    dv = torch.from_numpy(v).cuda()
    N.check(N.lib().pt_ensemble_run(res.handle, offsets.ctypes.data, len(offsets) - 1, db.data_ptr(),
                                    dv.data_ptr(), dt, steps, eps, use_graph))
    return db.cpu().numpy(), dv.cpu().numpy()


def run_each(res, offsets, b, v, steps, dt=1e-3, eps=0.01):
    import torch
    ob, ov = b.copy(), v.copy()
    for k in range(len(offsets) - 1):
        s, e = int(offsets[k]), int(offsets[k + 1])
        db = torch.from_numpy(b[s:e].copy()).cuda()
        dv = torch.from_numpy(v[s:e].copy()).cuda()
        da = torch.zeros((e - s, 3), device="cuda")
        L = N.lib()
        N.check(L.pt_bf_accel_f32_device(res.handle, db.data_ptr(), e - s, db.data_ptr(), e - s, eps,
                                         1, 0, da.data_ptr()))
        N.check(L.pt_leapfrog_device(res.handle, db.data_ptr(), dv.data_ptr(), da.data_ptr(), e - s,
                                     dt, steps, N.PT_METHOD_BRUTE_FORCE, 0.0, eps, 0, 0))
        res.synchronize()
        ob[s:e], ov[s:e] = db.cpu().numpy(), dv.cpu().numpy()
    return ob, ov


def test_ensemble_matches_per_system_leapfrog(res):
    offsets, b, v = small_ensemble()
    eb, ev = run_ensemble(res, offsets, b, v, 5)
    rb, rv = run_each(res, offsets, b, v, 5)
    assert np.abs(eb[:, :3] - rb[:, :3]).max() < 1e-5 * np.abs(rb[:, :3]).max()
    assert np.abs(ev[:, :3] - rv[:, :3]).max() < 1e-4 * np.abs(rv[:, :3]).max()
    assert np.array_equal(eb[:, 3], b[:, 3])


def large_ensemble(seed=65):
    """Systems in every size class up to 8192 bodies (the autotuner's classes of 2048
    bodies and more included), Plummer spheres of different scale radii."""
    sizes = [64, 130, 300, 700, 1500, 2048, 3000, 4500, 6000, 8192]
    offsets = np.zeros(len(sizes) + 1, np.uint32)
    offsets[1:] = np.cumsum(sizes)
    bodies, vel = [], []
    for k, n in enumerate(sizes):
        d = ics.plummer(n, a=0.5 + 0.15 * k, seed=seed + k)
        bodies.append(d["bodies"])
        vel.append(d["vel"])
    b = np.concatenate(bodies)
    v = np.zeros((b.shape[0], 4), np.float32)
    v[:, :3] = np.concatenate(vel)
    return offsets, b, v


def oracle_kdk(O, b, v, dt, steps, eps):
    """The kick-drift-kick scheme per system with the oracle's sequential::BruteForce
    (float32 state), the closing half kick of a step fused with the next opening one as
    the ensemble kernel does: kicks of dt/2, dt, ..., dt, then dt/2."""
    b = b.copy()
    v = v[:, :3].astype(np.float32).copy()
    a = O.bf_f32(b, b, eps, True)
    for s in range(steps):
        v = v + a * np.float32(0.5 * dt if s == 0 else dt)
        b[:, :3] = b[:, :3] + v * np.float32(dt)
        a = O.bf_f32(b, b, eps, True)
    v = v + a * np.float32(0.5 * dt)
    return b, v


@pytest.mark.parametrize("K,J", [(0, 0), (1, 128), (1, 512), (2, 256), (4, 128), (4, 512)])
def test_large_ensemble_matches_oracle(res, oracle, K, J):
    """Systems up to 8192 bodies against the oracle's integration, per system: with the
    autotuner's shapes (K = 0 runs the tuner first) and with item shapes forced
    (targets per thread K, j-tile J)."""
    import torch
    offsets, b, v = large_ensemble()
    L = N.lib()
    if K == 0:
        table = np.zeros(8, np.int32)
        tiles = np.zeros(8, np.int32)
        db = torch.from_numpy(b).cuda()
        N.check(L.pt_ensemble_tune(res.handle, offsets.ctypes.data, len(offsets) - 1, db.data_ptr(), 0.01,
                                   table.ctypes.data))
        N.check(L.pt_ensemble_get_shape(res.handle, table.ctypes.data, tiles.ctypes.data))
        print(f"autotuned targets per thread {table.tolist()}, j-tiles {tiles.tolist()} per size class")
        assert set(tiles.tolist()) <= {128, 256, 512}
    else:
        N.check(L.pt_ensemble_set_table(res.handle, np.full(8, K, np.int32).ctypes.data))
        N.check(L.pt_ensemble_set_tiles(res.handle, np.full(8, J, np.int32).ctypes.data))
    try:
        eb, ev = run_ensemble(res, offsets, b, v, 3, use_graph=1)
    finally:
        N.check(L.pt_ensemble_set_table(res.handle, np.zeros(8, np.int32).ctypes.data))
        N.check(L.pt_ensemble_set_tiles(res.handle, np.zeros(8, np.int32).ctypes.data))
    for k in range(len(offsets) - 1):
        s, e = int(offsets[k]), int(offsets[k + 1])
        rb, rv = oracle_kdk(oracle, b[s:e], v[s:e], 1e-3, 3, 0.01)
        assert np.abs(eb[s:e, :3] - rb[:, :3]).max() <= 1e-5 * np.abs(rb[:, :3]).max(), (K, e - s)
        assert np.abs(ev[s:e, :3] - rv).max() <= 1e-4 * np.abs(rv).max(), (K, e - s)
        assert np.array_equal(eb[s:e, 3], b[s:e, 3])


def test_graph_equals_eager_and_tuning_keeps_results(res):
    offsets, b, v = small_ensemble(40, 62)
    e1 = run_ensemble(res, offsets, b, v, 8, use_graph=0)
    e2 = run_ensemble(res, offsets, b, v, 8, use_graph=1)
    e3 = run_ensemble(res, offsets, b, v, 8, use_graph=1)  # replay
    assert np.array_equal(e1[0], e2[0]) and np.array_equal(e2[0], e3[0])
    import torch
    db = torch.from_numpy(b).cuda()
    table = np.zeros(8, np.int32)
    N.check(N.lib().pt_ensemble_tune(res.handle, offsets.ctypes.data, len(offsets) - 1,
                                     db.data_ptr(), 0.01, table.ctypes.data))
    assert set(table.tolist()) <= {0, 1, 2, 4}
    e4 = run_ensemble(res, offsets, b, v, 8)
    assert np.abs(e4[0] - e1[0]).max() < 1e-5 * np.abs(e1[0]).max()
    for K in (1, 2, 4):
        t = np.full(8, K, np.int32)
        N.check(N.lib().pt_ensemble_set_table(res.handle, t.ctypes.data))
        e5 = run_ensemble(res, offsets, b, v, 8)
        assert np.abs(e5[0] - e1[0]).max() < 1e-5 * np.abs(e1[0]).max()
    N.check(N.lib().pt_ensemble_set_table(res.handle, np.zeros(8, np.int32).ctypes.data))


def test_barrier_timeout_is_reported_and_context_survives(res):
    """A barrier that no block can complete runs out its (short) spin limit: the call
    fails with PT_ERR_TIMEOUT, nothing hangs, and the next call succeeds."""
    import torch
    offsets, b, v = small_ensemble(8, 63)
    db = torch.from_numpy(b).cuda()
    dv = torch.from_numpy(v).cuda()
    L = N.lib()
    N.check(L.pt_ensemble_set_barrier(res.handle, 2000, 1))
    rc = L.pt_ensemble_run(res.handle, offsets.ctypes.data, len(offsets) - 1, db.data_ptr(),
                           dv.data_ptr(), 1e-3, 3, 0.01, 0)
    assert rc == N.PT_ERR_TIMEOUT and "barrier" in N.last_error()
    N.check(L.pt_ensemble_set_barrier(res.handle, 1 << 22, 0))
    eb, ev = run_ensemble(res, offsets, b, v, 3)
    assert np.isfinite(eb).all()


def test_energy_conserved_per_system(res):
    offsets, b, v = small_ensemble(12, 64)
    eb, ev = run_ensemble(res, offsets, b, v, 100)

    def energy(bb, vv):
        bb = bb.astype(np.float64)
        vv = vv.astype(np.float64)
        d = bb[:, None, :3] - bb[None, :, :3]
        r = np.sqrt((d ** 2).sum(-1) + 1e-4)
        mm = bb[:, 3:4] * bb[:, 3][None, :]
        W = -0.5 * (mm / r).sum() + 0.5 * (bb[:, 3] ** 2 / 0.01).sum()
        return 0.5 * (bb[:, 3] * (vv[:, :3] ** 2).sum(1)).sum() + W

    for k in range(len(offsets) - 1):
        s, e = int(offsets[k]), int(offsets[k + 1])
        e0, e1 = energy(b[s:e], v[s:e]), energy(eb[s:e], ev[s:e])
        assert abs(e1 - e0) / abs(e0) < 1e-4, k
