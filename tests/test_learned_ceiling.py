"""What a learned correction of accepted Barnes-Hut cells can gain, bounded in FP64 on
the CPU (oracle/learned_ceiling.c, a model of the GPU's group walk), on the
N = 524,288 bulge+disk mixture (70 % Plummer bulge a = 0.5, 30 % exponential disk),
softening 0.01, 2048 sampled bodies judged against the FP64 brute force.

* theta 1.0 with every marginal cell (one theta 0.5 would open) corrected per group of
  64 bodies: even the EXACT residual at the group's centre leaves p95 where it was,
  and adding its exact gradient makes it far worse (the Taylor series about the
  centre diverges for cells next to the group); only a per-body correction (the
  exact residual at each body) reaches the theta 0.5 accuracy.
* the error-bound walk with the far field (beyond the local expansion's radius) at a
  looser bound: there the exact residual and gradient at the group's centre do
  recover the tight bound's accuracy, but only if the correction is accurate to
  about 10 % of the residuals' RMS per cell: 50 % noise is worse than no correction.
  A network on the learned correction's features (monopole, quadrupole, offset,
  size ratio) reaches R^2 0.5-0.7 on these residuals, i.e. errors of 55-70 % of
  their RMS.
"""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ceiling(tmp_path_factory):
    from oracle import build
    from particular_gb300 import ics
    exe = build.build_ceiling()
    path = str(tmp_path_factory.mktemp("ceiling") / "bulge_disk_524288.bin")
    ics.bulge_disk(524288, seed=1810)["bodies"].tofile(path)

    def run(args, noise=None):
        env = dict(os.environ)
        if noise is not None:
            env["NOISE"] = str(noise)
        out = subprocess.run([exe, path, "2048", *args], check=True, capture_output=True, text=True, env=env).stdout
        rows = {}
        for line in out.splitlines():
            parts = line.split()
            if parts and parts[0] in ("plain", "r0", "r0+J", "exact", "noisy", "net"):
                rows[parts[0]] = {"p50": float(parts[2]), "p95": float(parts[4])}
        print(out)
        return rows
    return run


def test_group_centre_corrections_of_near_cells_cannot_reach_the_bar(ceiling):
    r = ceiling(["1.0", "0.5", "0", "0", "0", "0"])
    assert r["exact"]["p95"] < 0.1 * r["plain"]["p95"]      # per body: the theta 0.5 accuracy
    assert r["r0"]["p95"] > 0.5 * r["plain"]["p95"]         # one value per group: no real gain
    assert r["r0+J"]["p95"] > r["plain"]["p95"]             # its gradient: worse than nothing
    assert r["r0"]["p95"] > 1e-3                            # far from the 1e-3 bar


def test_far_field_corrections_need_ten_percent_accuracy(ceiling):
    args = ["1.0", "1.0", "2e-2", "1e-3", "2.75e-3", "7.1"]
    r = ceiling(args, noise=0.1)
    assert r["plain"]["p95"] > 1e-3                         # the loose far field alone misses the bar
    assert r["r0+J"]["p95"] <= 1.02 * r["exact"]["p95"]     # the expansion about the centre is valid there
    assert r["noisy"]["p95"] < 1e-3                         # 10 % errors per cell keep the bar
    r5 = ceiling(args, noise=0.5)
    assert r5["noisy"]["p95"] > r5["plain"]["p95"]          # 50 % errors: worse than no correction
