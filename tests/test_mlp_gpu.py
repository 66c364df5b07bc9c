"""The learned far-field correction: kernels checked against an FP64 restatement,
and what the trained network gains over Barnes-Hut without it."""
import ctypes

import numpy as np
import pytest

from particular_gb300 import AccelerationSoftened, cuda, ics, learned
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_gradient_matches_fp64_restatement(res):
    from oracle import mlp_oracle as M
    learned.init(res, seed=3)
    rng = np.random.default_rng(0)
    f = rng.normal(size=(200, 12)).astype(np.float32)
    t = rng.normal(size=(200, 3)).astype(np.float32)
    g = np.zeros(N.PT_MLP_NPARAM, np.float32)
    loss = ctypes.c_double(0)
    N.check(N.lib().pt_mlp_loss_grad(res.handle, f.ctypes.data, t.ctypes.data, 200, g.ctypes.data,
                                     ctypes.byref(loss)))
    p = learned.get_params(res)
    want_loss, want = M.loss_grad(p, f, t)
    assert abs(loss.value - want_loss) <= 1e-5 * abs(want_loss)
    sl = slice(0, M.SCALE)
    err = np.abs(g[sl] - want[sl]).max() / np.abs(want[sl]).max()
    assert err < 1e-4, err
    # forward pass too
    out = np.zeros((200, 3), np.float32)
    N.check(N.lib().pt_mlp_predict(res.handle, f.ctypes.data, 200, out.ctypes.data))
    np.testing.assert_allclose(out, M.forward(p, f), rtol=1e-4, atol=1e-5)


def test_tensor_core_inference_matches_bf16_restatement(res):
    """pt_mlp_predict_tc (the walk's mma.sync path) against the FP64 forward pass
    with the same BF16 roundings of features and activations. What remains is FP32
    accumulation order and the hardware tanh approximation, whose error can move an
    activation by one BF16 step; relative RMS difference bound 2e-3, and the plain
    FP64 forward within 2e-2 (the BF16 roundings themselves)."""
    from oracle import mlp_oracle as M
    learned.init(res, seed=4)
    p = learned.get_params(res)
    rng = np.random.default_rng(1)
    # trained-model-like weights: the initial output layer is zero, so draw one
    p[M.W3:M.B3] = M.bf16(rng.normal(scale=0.2, size=M.B3 - M.W3))
    p[M.B3:M.SCALE] = [0.01, -0.02, 0.03]
    learned.set_params(res, p.astype(np.float32))
    p = learned.get_params(res)
    f = rng.normal(size=(1000, 12)).astype(np.float32)   # 1000: ragged last batch of 32
    out = np.zeros((1000, 3), np.float32)
    N.check(N.lib().pt_mlp_predict_tc(res.handle, f.ctypes.data, 1000, out.ctypes.data))
    want = M.forward_bf16(p, f)
    rms = np.sqrt((want ** 2).mean())
    err = np.sqrt(((out - want) ** 2).mean()) / rms
    err64 = np.sqrt(((out - M.forward(p, f)) ** 2).mean()) / rms
    print(f"tensor-core inference: rel RMS vs BF16 restatement {err:.2e}, vs FP64 {err64:.2e}")
    assert np.isfinite(out).all()
    assert err < 2e-3 and err64 < 2e-2


@pytest.fixture(scope="module")
def trained(res):
    """A small model: 24 snapshots of 16384 bodies, 400 Adam steps."""
    learned.init(res, seed=1)
    count = learned.generate(res, snapshots=24, n=16384, targets=512, capacity=4_000_000)
    f, t = learned.dataset(res, min(count, 20000))
    first = learned.train(res, steps=20, batch=4096, lr=1e-3, seed=5)
    last = learned.train(res, steps=1500, batch=4096, lr=1e-3, seed=6)
    return {"count": count, "features": f, "targets": t, "first": first, "last": last}


def test_samples_are_marginal_cells(trained):
    f, t = trained["features"], trained["targets"]
    assert trained["count"] > 10000
    assert np.isfinite(f).all() and np.isfinite(t).all()
    np.testing.assert_allclose(np.linalg.norm(f[:, :3], axis=1), 1.0, rtol=1e-5)
    assert (f[:, 3] >= 0.5 - 1e-6).all() and (f[:, 3] <= 1.0 + 1e-6).all()   # w/d in [theta_in, theta_out]
    assert (np.abs(f[:, 9:12]) <= 0.5 + 1e-5).all()                          # COM inside the cell


def test_training_reduces_loss(trained):
    # targets are scaled to unit RMS per component: predicting zero scores 3.0
    print(f"loss after 20 steps {trained['first']:.3f}, after 1520 {trained['last']:.3f} "
          f"(zero predictor: 3.0)")
    assert trained["last"] < trained["first"] and trained["last"] < 2.9


def test_network_gains_on_held_out_cells(res, trained):
    """On samples from snapshots it never saw, the trained network's prediction leaves
    a smaller residual than no correction: what it learned about marginal cells."""
    learned.generate(res, snapshots=2, n=16384, targets=512, seed0=7000, capacity=4_000_000)
    f, t = learned.dataset(res, 20000)
    pred = np.zeros_like(t)
    N.check(N.lib().pt_mlp_predict(res.handle, f.ctypes.data, f.shape[0], pred.ctypes.data))
    before = float((t.astype(np.float64) ** 2).sum(1).mean())
    after = float(((t - pred).astype(np.float64) ** 2).sum(1).mean())
    print(f"held-out marginal cells: residual MSE {before:.4e} -> {after:.4e} "
          f"({100 * (1 - after / before):.1f}% lower)")
    assert after < 0.97 * before


def test_learned_walk_reports_its_effect(res, oracle, trained):
    """theta 1.0, quadrupole + group, with and without the model on a held-out
    snapshot, judged against the FP64 brute force. The walk evaluates the model once
    per warp at the warp's centre; the test records the effect and guards against
    breakage (finite results, corrections applied, error within 2x of plain)."""
    b = ics.bulge_disk(16384, seed=999)["bodies"]
    ref = oracle.bf_f64(b[::8], b, 0.01, True)
    plain = cuda.BarnesHut(1.0, res, AccelerationSoftened(0.01), quadrupole=True, group=True)
    e0 = np.linalg.norm(plain.compute(b)[::8] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    m = cuda.BarnesHut(1.0, res, AccelerationSoftened(0.01), quadrupole=True, group=True, learned=True)
    got = m.compute(b)
    st = m.stats()
    e1 = np.linalg.norm(got[::8] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    print(f"theta 1.0 quad+group p50/p95: plain {np.median(e0):.3e}/{np.percentile(e0, 95):.3e} "
          f"learned {np.median(e1):.3e}/{np.percentile(e1, 95):.3e} ({st['learned']} corrections)")
    assert np.isfinite(got).all() and st["learned"] > 0
    assert np.median(e1) < 2 * np.median(e0)
    # corrections are summed per group in walk order: the result is reproducible
    np.testing.assert_array_equal(m.compute(b), got)


def test_learned_record_overflow_is_reported(res, trained):
    """With room for one chunk of records, a learned walk cannot keep every marginal
    cell: the host call and a graph-replayed leapfrog both fail with PT_ERR_CAPACITY
    instead of dropping corrections silently; with the automatic capacity again the
    same leapfrog replays cleanly."""
    import torch
    L = N.lib()
    d = ics.bulge_disk(16384, seed=998)
    b = np.ascontiguousarray(d["bodies"])
    flags = N.PT_BH_QUADRUPOLE | N.PT_BH_GROUP | N.PT_BH_LEARNED
    out = np.zeros((b.shape[0], 3), np.float32)
    try:
        N.check(L.pt_bh_set_learned_capacity(res.handle, 1))
        rc = L.pt_bh_accel_f32(res.handle, b.ctypes.data, b.shape[0], b.ctypes.data, b.shape[0], 1.0, 0.01,
                               flags, out.ctypes.data)
        assert rc == N.PT_ERR_CAPACITY and "overflowed" in N.last_error()
        vel = np.zeros((b.shape[0], 4), np.float32)
        vel[:, :3] = d["vel"]
        db = torch.from_numpy(b).cuda()
        dv = torch.from_numpy(vel).cuda()
        da = torch.zeros((b.shape[0], 3), device="cuda")
        for _ in range(2):  # the capture call and a replay
            rc = L.pt_leapfrog_device(res.handle, db.data_ptr(), dv.data_ptr(), da.data_ptr(), b.shape[0], 1e-3,
                                      3, N.PT_METHOD_BARNES_HUT, 1.0, 0.01, flags, 1)
            assert rc == N.PT_ERR_CAPACITY and "overflowed" in N.last_error()
    finally:
        N.check(L.pt_bh_set_learned_capacity(res.handle, 0))
    for _ in range(2):
        N.check(L.pt_leapfrog_device(res.handle, db.data_ptr(), dv.data_ptr(), da.data_ptr(), b.shape[0], 1e-3,
                                     3, N.PT_METHOD_BARNES_HUT, 1.0, 0.01, flags, 1))
    assert torch.isfinite(da).all()


def test_shipped_model_gains_at_theta1(res, oracle):
    """The shipped model (256 bulge+disk snapshots of 65536 bodies) on a snapshot it
    never saw at the evaluation size, N = 4,194,304, theta 1.0, quadrupole + 64-body
    groups, against the FP64 brute force on 1024 bodies: the corrected walk is more
    accurate than the same walk without the network at the median and at p95. The gain
    is bounded (one value per group and cell at the group's centre; the bound is
    measured by tests/test_learned_ceiling.py) and it depends on the groups being small
    against the cells they correct: at N = 262144 the same model is neutral."""
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "particular_gb300", "data",
                        "mlp_bulge_disk.npz")
    learned.load(res, path)
    b = ics.bulge_disk(4194304, seed=4242)["bodies"]
    idx = np.random.default_rng(5).choice(b.shape[0], 1024, replace=False)
    ref = oracle.bf_f64(b[idx], b, 0.01, True)
    e = {}
    for lr in (False, True):
        m = cuda.BarnesHut(1.0, res, AccelerationSoftened(0.01), quadrupole=True, group=True, learned=lr)
        e[lr] = np.linalg.norm(m.compute(b)[idx] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    p = {lr: (np.median(e[lr]), np.percentile(e[lr], 95)) for lr in e}
    print(f"shipped model, N=4194304 theta 1.0: p50/p95 plain {p[False][0]:.3e}/{p[False][1]:.3e}, "
          f"learned {p[True][0]:.3e}/{p[True][1]:.3e}")
    assert p[True][0] < p[False][0] and p[True][1] < p[False][1]
