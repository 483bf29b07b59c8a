"""The no-allocation density entry point (xcgpu_density_fp64_noalloc), called through
the C ABI with device buffers, against the allocating entry point (xcgpu_density):
same kernels, so the results agree to the tolerance of the FP64 stage tests
(1e-12 relative, 1e-14 absolute), on two calls in a row.  It serves callers that
cannot allocate device memory themselves at the point of the call."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_density_matches_allocating_entry_point():
    import torch

    from oracle import pyoracle as po
    from serenity_gb300 import workload as wl
    from serenity_gb300 import xcgpu

    ctx = xcgpu.Context()
    L = ctx.L
    L.xcgpu_density_fp64_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p]
    L.xcgpu_density_fp64_noalloc.restype = ctypes.c_int
    sym, xyz = wl.water_cluster(4, seed=3, jitter=0.2, dims=(2, 2, 1))
    w = wl.Workload(sym, xyz, "DEF2-SVP", "PBE", (20, 19), 30, 110, 3)
    pts, wts = po.becke_grid(w.Z, w.coords, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    P = np.asarray(w.density())
    ref_rho, ref_grad = plan.density(P)  # allocating entry point, host buffers
    n = len(wts)
    Pc = np.ascontiguousarray(np.stack([m.T for m in P]))
    P_dev = torch.from_numpy(Pc).cuda()
    for call in range(2):
        rho = torch.full((2, n), float("nan"), dtype=torch.float64, device="cuda")
        grad = torch.full((2, 3, n), float("nan"), dtype=torch.float64, device="cuda")
        st = L.xcgpu_density_fp64_noalloc(plan.h, 2, ctypes.c_void_p(P_dev.data_ptr()),
                                          ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(grad.data_ptr()))
        assert st == 0, L.xcgpu_last_error(ctx.h)
        np.testing.assert_allclose(rho.cpu().numpy(), ref_rho, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(grad.cpu().numpy(), ref_grad, rtol=1e-12, atol=1e-14)
