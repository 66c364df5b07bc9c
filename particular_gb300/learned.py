"""The learned far-field correction for cuda::BarnesHut (PT_BH_LEARNED).

generate(): walks seeded bulge+disk snapshots with the reference opening rule at
theta_outer and collects, for every accepted cell that theta_inner would have opened,
its features and the residual of its monopole + quadrupole against the exact sum over
its bodies (brute-force pair kernel). train(): Adam on the GPU with the library's own
fused forward/backward kernel. save()/load(): parameters as .npz.
"""
import ctypes

import numpy as np

from . import _native as N
from . import ics

NPARAM = N.PT_MLP_NPARAM


def init(res, seed=1):
    N.check(N.lib().pt_mlp_init(res.handle, int(seed)))


def generate(res, snapshots=256, n=65536, targets=256, theta_outer=1.0, theta_inner=0.5,
             softening=0.01, capacity=16_000_000, seed0=5000, reset=True):
    """Appends the samples of `snapshots` bulge+disk snapshots; returns the dataset size."""
    import torch
    L = N.lib()
    if reset:
        N.check(L.pt_mlp_reset_dataset(res.handle))
    total = ctypes.c_size_t(0)
    for k in range(snapshots):
        b = ics.bulge_disk(n, seed=seed0 + k)["bodies"]
        d = torch.from_numpy(b).cuda()
        N.check(L.pt_mlp_generate(res.handle, d.data_ptr(), n, targets, theta_outer, theta_inner,
                                  softening, capacity, ctypes.byref(total)))
    return int(total.value)


def dataset(res, count):
    f = np.zeros((count, 12), np.float32)
    t = np.zeros((count, 3), np.float32)
    N.check(N.lib().pt_mlp_export_dataset(res.handle, f.ctypes.data, t.ctypes.data, count))
    return f, t


def train(res, steps=2000, batch=8192, lr=1e-3, seed=7):
    loss = ctypes.c_float(0)
    N.check(N.lib().pt_mlp_train(res.handle, int(steps), int(batch), float(lr), int(seed),
                                 ctypes.byref(loss)))
    return float(loss.value)


def get_params(res):
    p = np.zeros(NPARAM, np.float32)
    N.check(N.lib().pt_mlp_get_params(res.handle, p.ctypes.data, NPARAM))
    return p


def set_params(res, params, theta_inner=0.5):
    p = np.ascontiguousarray(params, np.float32)
    N.check(N.lib().pt_mlp_set_params(res.handle, p.ctypes.data, p.size, float(theta_inner)))


def save(res, path, theta_inner=0.5, **meta):
    np.savez(path, params=get_params(res), theta_inner=np.float32(theta_inner), **meta)


def load(res, path):
    z = np.load(path)
    set_params(res, z["params"], float(z["theta_inner"]))
    return {k: z[k] for k in z.files}


def main(argv=None):
    """Trains the model on the specified data set (256 bulge+disk snapshots of 65536
    bodies, theta 1.0 vs 0.5, softening 0.01) and writes it to --out."""
    import argparse
    import time
    from .cuda import CudaResources
    p = argparse.ArgumentParser()
    p.add_argument("--out", required=True)
    p.add_argument("--snapshots", type=int, default=256)
    p.add_argument("--n", type=int, default=65536)
    p.add_argument("--targets", type=int, default=256)
    p.add_argument("--steps", type=int, default=4000)
    p.add_argument("--batch", type=int, default=8192)
    p.add_argument("--lr", type=float, default=1e-3)
    a = p.parse_args(argv)
    res = CudaResources(0)
    t0 = time.time()
    init(res, seed=1)
    count = generate(res, snapshots=a.snapshots, n=a.n, targets=a.targets)
    t1 = time.time()
    first = train(res, steps=20, batch=a.batch, lr=a.lr, seed=11)
    last = train(res, steps=a.steps, batch=a.batch, lr=a.lr, seed=12)
    t2 = time.time()
    save(res, a.out, theta_inner=0.5, samples=count, snapshots=a.snapshots, n=a.n,
         loss_first=first, loss_last=last, zero_predictor_loss=3.0)
    print(f"samples {count} ({t1 - t0:.1f} s), loss {first:.4f} -> {last:.4f} "
          f"(zero predictor 3.0; {t2 - t1:.1f} s)")


if __name__ == "__main__":
    main()
