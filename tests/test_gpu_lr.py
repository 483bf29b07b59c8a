"""Linear-response XC kernel (KernelSigmavector<RESTRICTED>::calcF, singlet) on the GPU:
the dual-number kernel of the analytic functionals against the oracle's second-order
differentiation, FP64 and mixed."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300 import workload as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from serenity_gb300 import xcgpu
    return xcgpu.Context()


@pytest.mark.parametrize("func", ["LDA", "PBE", "BLYP"])
def test_lr_kernel_matches_oracle(ctx, func):
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(2, 6, jitter=0.2, dims=(2, 1, 1))
    w = wl.Workload(sym, xyz, "DEF2-SVP", func, 10, 30, 110, 7)
    P0 = w.density()
    rng = np.random.default_rng(9)
    trials = [rng.standard_normal(P0.shape) * 0.05 for _ in range(3)]  # not symmetric: the path symmetrises
    pts, wts = po.becke_grid(w.Z, xyz, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    Fs = plan.lr_kernel(func, P0, trials)
    B = po.Basis(w.shells)
    for D, F in zip(trials, Fs):
        R = po.lr_fock(B, pts, wts, func, P0, D)
        np.testing.assert_allclose(F, R, rtol=0, atol=1e-10 * max(1.0, np.abs(R).max()))
        np.testing.assert_allclose(F, F.T, rtol=0, atol=1e-14 * max(1.0, np.abs(F).max()))
    Fm = plan.lr_kernel(func, P0, trials, precision=xcgpu.PREC_MIXED)
    for F, G in zip(Fs, Fm):
        assert np.abs(G - F).max() <= 2e-6 * max(1.0, np.abs(F).max()), np.abs(G - F).max()


@pytest.mark.parametrize("func", ["LDA", "PBE", "BLYP", "BP86"])
@pytest.mark.parametrize("kind", ["unrestricted", "triplet"])
def test_spin_lr_kernel_matches_oracle(ctx, func, kind):
    """xcgpu_lr_kernel_spin: unrestricted (KernelSigmavector<UNRESTRICTED>) and triplet
    (f_aa - f_ab of the restricted ground state) against the oracle's second-order
    differentiation, 1e-10 of the largest element; mixed against FP64, 2e-6."""
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(2, 6, jitter=0.2, dims=(2, 1, 1))
    w = wl.Workload(sym, xyz, "DEF2-SVP", func, (10, 9) if kind == "unrestricted" else 10, 30, 110, 7)
    P0 = np.asarray(w.density())
    rng = np.random.default_rng(12)
    trials = [rng.standard_normal(P0.shape) * 0.05 for _ in range(2)]  # not symmetric: the path symmetrises
    pts, wts = po.becke_grid(w.Z, xyz, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    Fs = plan.lr_kernel(func, P0, trials, kind=kind)
    B = po.Basis(w.shells)
    for D, F in zip(trials, Fs):
        R = po.lr_fock_spin(B, pts, wts, func, P0, D, kind)
        assert np.abs(R).max() > 1e-2
        np.testing.assert_allclose(F, R, rtol=0, atol=1e-10 * max(1.0, np.abs(R).max()))
        np.testing.assert_allclose(F, np.swapaxes(F, -1, -2), rtol=0, atol=1e-14 * max(1.0, np.abs(F).max()))
    Fm = plan.lr_kernel(func, P0, trials, precision=xcgpu.PREC_MIXED, kind=kind)
    for F, G in zip(Fs, Fm):
        assert np.abs(G - F).max() <= 2e-6 * max(1.0, np.abs(F).max()), np.abs(G - F).max()
