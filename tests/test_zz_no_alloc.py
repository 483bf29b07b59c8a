"""The no-allocation density entry point (xcgpu_density_fp64_noalloc), called through
the C ABI with device buffers.  It serves callers that cannot allocate device memory
themselves at the point of the call (a host program that owns all device memory
through its own pool, or a loop whose memory was reserved up front), so it keeps its
scratch in a fixed static device array and calls no allocator.

Held to: the allocating entry point (xcgpu_density, same FP64 kernels: 1e-12 relative,
1e-14 absolute) and the oracle (1e-11 relative, 1e-13 absolute), on two calls in a row,
for two spins with gradients and one spin without; a workload whose block slabs exceed
the 64 MiB array, so the work runs in several chunks; unchanged device memory across a
warm call; and the rejection (XCGPU_ERR_BUDGET) of a block that needs more scratch than
the array holds."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20
MAX_BLOCKS = 4096
XCGPU_ERR_BUDGET = 4


@pytest.fixture(scope="module")
def lib_ctx():
    from serenity_gb300 import xcgpu
    ctx = xcgpu.Context()
    L = ctx.L
    L.xcgpu_density_fp64_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p]
    L.xcgpu_density_fp64_noalloc.restype = ctypes.c_int
    return ctx


def _call(ctx, plan, nspin, P_dev, rho, grad):
    return ctx.L.xcgpu_density_fp64_noalloc(plan.h, nspin, ctypes.c_void_p(P_dev.data_ptr()),
                                            ctypes.c_void_p(rho.data_ptr()),
                                            ctypes.c_void_p(grad.data_ptr()) if grad is not None else None)


@pytest.mark.parametrize("nspin,with_grad", [(2, True), (1, False)])
def test_noalloc_density_matches_allocating_entry_point_and_oracle(lib_ctx, nspin, with_grad):
    import torch

    from oracle import pyoracle as po
    from serenity_gb300 import workload as wl
    from serenity_gb300 import xcgpu

    ctx = lib_ctx
    sym, xyz = wl.water_cluster(4, seed=3, jitter=0.2, dims=(2, 2, 1))
    w = wl.Workload(sym, xyz, "DEF2-SVP", "PBE", (20, 19) if nspin == 2 else 20, 30, 110, 3)
    pts, wts = po.becke_grid(w.Z, w.coords, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    st = plan.stats()
    # the block slabs (4 components x 128 points per active function, FP64) exceed the
    # array, so the call runs in several chunks
    assert 4 * 128 * 8 * st["sum_active"] > SCRATCH_BYTES - 8 * MAX_BLOCKS
    P = np.asarray(w.density()).reshape(nspin, w.nbf, w.nbf)
    ref_rho, ref_grad = plan.density(P if nspin == 2 else P[0])  # allocating entry point
    orc_rho, orc_grad = po.Basis(w.shells).density(pts, P if nspin == 2 else P[0])
    ref_rho = np.asarray(ref_rho).reshape(nspin, -1)
    orc_rho = np.asarray(orc_rho).reshape(nspin, -1)
    n = len(wts)
    P_dev = torch.from_numpy(np.ascontiguousarray(np.stack([m.T for m in P]))).cuda()
    rho = torch.empty((nspin, n), dtype=torch.float64, device="cuda")
    grad = torch.empty((nspin, 3, n), dtype=torch.float64, device="cuda") if with_grad else None
    for call in range(2):
        rho.fill_(float("nan"))
        if grad is not None:
            grad.fill_(float("nan"))
        torch.cuda.synchronize()
        used0, free0 = ctx.bytes_in_use, torch.cuda.mem_get_info()[0]
        assert _call(ctx, plan, nspin, P_dev, rho, grad) == 0, ctx.L.xcgpu_last_error(ctx.h)
        torch.cuda.synchronize()
        if call == 1:  # the first call may load the module's kernels; the second allocates nothing
            assert ctx.bytes_in_use == used0 and torch.cuda.mem_get_info()[0] == free0
        r = rho.cpu().numpy()
        np.testing.assert_allclose(r, ref_rho, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(r, orc_rho, rtol=1e-11, atol=1e-13)
        if grad is not None:
            g = grad.cpu().numpy().reshape(nspin, 3, n)
            np.testing.assert_allclose(g, np.asarray(ref_grad).reshape(nspin, 3, n), rtol=1e-12, atol=1e-14)
            np.testing.assert_allclose(g, np.asarray(orc_grad).reshape(nspin, 3, n), rtol=1e-11, atol=1e-12)


def test_noalloc_rejects_a_block_larger_than_its_scratch(lib_ctx):
    """One block of 128 points spread over a (H2O)400 def2-TZVP cluster: every one of its
    17 200 functions is active, 70 MB of slabs, more than the array holds."""
    import torch

    from serenity_gb300 import workload as wl
    from serenity_gb300 import xcgpu

    ctx = lib_ctx
    sym, xyz = wl.water_cluster(400, seed=1, jitter=0.0)
    w = wl.Workload(sym, xyz, "DEF2-TZVP", "LDA", 5, 10, 14, 1)
    assert w.nbf == 400 * 43
    pts = np.ascontiguousarray(w.coords[np.linspace(0, len(sym) - 1, 128).astype(int)] + 0.1)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, np.ones(128)), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    assert plan.stats()["max_active"] * 4 * 128 * 8 > SCRATCH_BYTES
    P_dev = torch.zeros((w.nbf, w.nbf), dtype=torch.float64, device="cuda")
    rho = torch.zeros(128, dtype=torch.float64, device="cuda")
    assert _call(ctx, plan, 1, P_dev, rho, None) == XCGPU_ERR_BUDGET
    msg = ctx.L.xcgpu_last_error(ctx.h)
    assert b"scratch" in (msg if isinstance(msg, bytes) else str(msg).encode())
