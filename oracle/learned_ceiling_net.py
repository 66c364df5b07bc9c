"""Trains the learned correction's network shape on far-cell residuals and judges it
in the FP64 model walk (test infrastructure: the recipe behind the network rows of
the learned-correction bound; oracle/learned_ceiling.c does the walking).

    python -m oracle.learned_ceiling_net [--snapshots 64] [--steps 3000]

1. samples: ALLGROUPS runs of learned_ceiling over `snapshots` bulge+disk snapshots of
   65536 bodies (seeds 5000 + k), far field at alpha 5e-2, inner bound 1e-3, near field
   2.75e-3, far radius 7.1 group radii; per far marginal cell and group the features at
   the group's centre and the exact residual and gradient there;
2. a 12 -> 64 -> 64 -> 8 GELU (tanh form) network fitted with Adam in PyTorch on the CPU
   (outputs r0 x3 and the gradient's xx xy xz yy yz, each scaled to unit RMS), 10 % of
   the samples held out;
3. the model walk on N = 524,288 (seed 1810) at alpha 2e-2 with the network's
   corrections (env NET), beside the exact ones.
"""
import argparse
import os
import subprocess
import tempfile

import numpy as np


def main(argv=None):
    import torch
    from oracle import build
    from particular_gb300 import ics
    p = argparse.ArgumentParser()
    p.add_argument("--snapshots", type=int, default=64)
    p.add_argument("--steps", type=int, default=3000)
    a = p.parse_args(argv)
    exe = build.build_ceiling()
    tmp = tempfile.mkdtemp()
    env = dict(os.environ, ALLGROUPS="1")
    chunks = []
    for k in range(a.snapshots):
        bodies = os.path.join(tmp, "snap.bin")
        dump = os.path.join(tmp, "dump.bin")
        ics.bulge_disk(65536, seed=5000 + k)["bodies"].tofile(bodies)
        subprocess.run([exe, bodies, "0", "1.0", "1.0", "5e-2", "1e-3", "2.75e-3", "7.1", dump], check=True,
                       env=env, capture_output=True)
        chunks.append(np.fromfile(dump, np.float32).reshape(-1, 24))
    d = np.concatenate(chunks)
    X, Y = d[:, :12], d[:, 12:20]
    sc = np.sqrt((Y ** 2).mean(0))
    torch.manual_seed(0)
    m = torch.nn.Sequential(torch.nn.Linear(12, 64), torch.nn.GELU(approximate="tanh"), torch.nn.Linear(64, 64),
                            torch.nn.GELU(approximate="tanh"), torch.nn.Linear(64, 8))
    xt, yt = torch.tensor(X), torch.tensor(Y / sc)
    held = np.arange(len(X)) >= int(0.9 * len(X))
    tr = torch.tensor(np.where(~held)[0])
    opt = torch.optim.Adam(m.parameters(), 1e-3)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, a.steps)
    for _ in range(a.steps):
        idx = tr[torch.randint(len(tr), (8192,))]
        loss = ((m(xt[idx]) - yt[idx]) ** 2).mean()
        opt.zero_grad()
        loss.backward()
        opt.step()
        sched.step()
    with torch.no_grad():
        pred = m(xt[held]).numpy()
    truth = yt[held].numpy()
    r2 = 1 - ((pred - truth) ** 2).sum(0) / (truth ** 2).sum(0)
    print(f"{len(X)} samples; held-out R^2 per output {np.round(r2, 3).tolist()}")
    w = [m[0].weight, m[0].bias, m[2].weight, m[2].bias, m[4].weight, m[4].bias]
    net = os.path.join(tmp, "net.bin")
    np.concatenate([t.detach().numpy().ravel() for t in w] + [sc]).astype(np.float32).tofile(net)
    big = os.path.join(tmp, "bd524288.bin")
    ics.bulge_disk(524288, seed=1810)["bodies"].tofile(big)
    out = subprocess.run([exe, big, "2048", "1.0", "1.0", "2e-2", "1e-3", "2.75e-3", "7.1"], check=True,
                         env=dict(os.environ, NET=net), capture_output=True, text=True).stdout
    print(out)


if __name__ == "__main__":
    main()
