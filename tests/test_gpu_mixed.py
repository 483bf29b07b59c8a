"""GPU parity of the mixed-precision form (FP32 basis values, 3xTF32 tcgen05
contractions with FP32 accumulation; FP64 functional, grid sums and cross-block
Vxc) against the FP64 path and the oracle on the same inputs.

Stated tolerances (water tetramer, def2-SVP / def2-TZVP, 30 x 110 grid): density
relative to max rho 2e-6, adder 2e-6 absolute, E_xc 5e-6 Eh, max|dVxc| 1e-6."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300 import workload as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from serenity_gb300 import xcgpu
    return xcgpu.Context()


def _case(func, unrestricted, max_block=128, seed=3, basis="DEF2-SVP", spherical=True):
    sym, xyz = wl.water_cluster(4, seed, jitter=0.2, dims=(2, 2, 1))
    w = wl.Workload(sym, xyz, basis, func, (20, 19) if unrestricted else 20, 30, 110, seed, spherical=spherical)
    pts, wts = po.becke_grid(w.Z, w.coords, n_rad=30, n_ang=110)
    return w, pts, wts


def _plan(ctx, w, pts, wts, max_block=128):
    from serenity_gb300 import xcgpu
    return xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), max_block, 1e-9)


@pytest.mark.parametrize("max_block", [128, 77])
def test_mixed_density_vs_fp64(ctx, max_block):
    from serenity_gb300 import xcgpu
    w, pts, wts = _case("PBE", False)
    plan = _plan(ctx, w, pts, wts, max_block)
    P = w.density()
    r64, g64 = plan.density(P)
    rmx, gmx = plan.density(P, precision=xcgpu.PREC_MIXED)
    scale = np.abs(r64).max()
    assert np.abs(rmx - r64).max() <= 2e-6 * scale, np.abs(rmx - r64).max() / scale
    assert np.abs(gmx - g64).max() <= 2e-6 * np.abs(g64).max()


def test_mixed_adder_vs_fp64(ctx):
    from serenity_gb300 import xcgpu
    w, pts, wts = _case("PBE", False)
    plan = _plan(ctx, w, pts, wts)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(len(wts))
    g = rng.standard_normal((1, 3, len(wts)))
    F64 = plan.add_scalar(v, g)
    Fmx = plan.add_scalar(v, g, precision=xcgpu.PREC_MIXED)
    assert np.abs(Fmx - F64).max() <= 2e-6 * max(1.0, np.abs(F64).max())
    F64 = plan.add_scalar(v)
    Fmx = plan.add_scalar(v, precision=xcgpu.PREC_MIXED)
    assert np.abs(Fmx - F64).max() <= 2e-6 * max(1.0, np.abs(F64).max())


@pytest.mark.parametrize("func,unrestricted,basis,spherical", [
    ("LDA", False, "DEF2-SVP", True), ("PBE", False, "DEF2-SVP", True), ("BLYP", False, "DEF2-SVP", True),
    ("PBE", True, "DEF2-SVP", True), ("PBE", False, "DEF2-TZVP", True), ("PBE", False, "DEF2-TZVP", False)])
def test_mixed_vxc_vs_oracle(ctx, func, unrestricted, basis, spherical):
    from serenity_gb300 import xcgpu
    w, pts, wts = _case(func, unrestricted, basis=basis, spherical=spherical)
    plan = _plan(ctx, w, pts, wts)
    P = w.density()
    V, exc, nel = plan.vxc(func, P, precision=xcgpu.PREC_MIXED)
    rV, rexc, rnel = po.Basis(w.shells).vxc(pts, wts, func, P)
    assert abs(exc - rexc) <= 5e-6, abs(exc - rexc)
    assert abs(nel - rnel) <= 1e-6 * rnel
    assert np.abs(V - rV).max() <= 1e-6, np.abs(V - rV).max()
    np.testing.assert_allclose(V, np.swapaxes(V, 1, 2), rtol=0, atol=1e-14)
