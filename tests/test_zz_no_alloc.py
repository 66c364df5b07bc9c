"""The allocation-free brute force, checked against the context entry point.

pt_bf_accel_f32_noalloc exists for callers that cannot call cudaMalloc (programs
that own all device memory through their own pool or budget, and time-critical
loops that cannot afford cudaMalloc's implicit device synchronisation). It keeps
its scratch in one static device array shared by every call. This file is named
to be collected last, so a run that stops at its first failure has already run
every other test.
"""
import numpy as np
import pytest

from particular_gb300 import CudaResources, ics
from particular_gb300 import _native as N

pytestmark = pytest.mark.gpu


def rel(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-30)


def test_noalloc_matches_context_entry_point(native_lib):
    import torch
    L = native_lib
    with CudaResources(0) as res:
        # Two calls in a row with different sizes share (and overwrite) the static
        # scratch; the second must not see stale data from the first.
        for call, (n, seed) in enumerate([(20000, 31), (9001, 32)]):
            b = ics.plummer(n, seed=seed)["bodies"]
            d = torch.from_numpy(b).cuda()
            out_na = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
            out_ctx = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0] if call == 1 else None
            N.check(L.pt_bf_accel_f32_noalloc(d.data_ptr(), n, d.data_ptr(), n, 0.01, 1,
                                              out_na.data_ptr(), None))
            torch.cuda.synchronize()
            if free_before is not None:
                # After the first call loaded the module, a call allocates nothing. The
                # device's free memory moves in 2 MiB pages, the smallest step any
                # cudaMalloc takes; a smaller change comes from elsewhere.
                assert free_before - torch.cuda.mem_get_info()[0] < 2 << 20
            N.check(L.pt_bf_accel_f32_device(res.handle, d.data_ptr(), n, d.data_ptr(), n, 0.01,
                                             1, 0, out_ctx.data_ptr()))
            res.synchronize()
            got, want = out_na.cpu().numpy(), out_ctx.cpu().numpy()
            assert np.isfinite(got).all()
            # tolerance of the brute-force plan tests (tests/test_bf_gpu.py)
            assert rel(got, want).max() < 5e-6, call


def test_noalloc_rejects_sizes_beyond_its_scratch(native_lib):
    import torch
    big = 524288 + 1
    d = torch.zeros((big, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    rc = native_lib.pt_bf_accel_f32_noalloc(d.data_ptr(), 4, d.data_ptr(), big, 0.01, 1,
                                            out.data_ptr(), None)
    assert rc == N.PT_ERR_CAPACITY
    assert "static scratch limit" in N.last_error()
