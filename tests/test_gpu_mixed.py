"""GPU parity of the mixed-precision form (FP32 basis values with FP32-pair
corrections, tcgen05 contractions over fixed-point FP16 slices whose leading products
sum exactly; FP64 functional, grid sums and cross-block Vxc) against the FP64 path and
the oracle on the same inputs.

Stated tolerances (water tetramer, 30 x 110 grid): density relative to max rho 1e-6,
adder 1.5e-6 (random v and g), N_el 1e-8 relative; whole builds against the oracle
E_xc 1e-7 Eh and max|dVxc| 1e-7 with def2-SVP (measured 0.4-1.7e-8 and 0.6-0.9e-7),
1e-7 Eh and 4e-7 with def2-TZVP (measured 3.4-5.2e-8 and 2.7-3.2e-7); on the benchmark grids
1e-7 in both (test_mixed_vxc_benchmark_tolerance)."""
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
    assert np.abs(rmx - r64).max() <= 1e-6 * scale, np.abs(rmx - r64).max() / scale
    assert np.abs(gmx - g64).max() <= 1e-6 * np.abs(g64).max()


def test_mixed_adder_vs_fp64(ctx):
    from serenity_gb300 import xcgpu
    w, pts, wts = _case("PBE", False)
    plan = _plan(ctx, w, pts, wts)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(len(wts))
    g = rng.standard_normal((1, 3, len(wts)))
    F64 = plan.add_scalar(v, g)
    Fmx = plan.add_scalar(v, g, precision=xcgpu.PREC_MIXED)
    assert np.abs(Fmx - F64).max() <= 1.5e-6 * max(1.0, np.abs(F64).max())
    F64 = plan.add_scalar(v)
    Fmx = plan.add_scalar(v, precision=xcgpu.PREC_MIXED)
    assert np.abs(Fmx - F64).max() <= 1.5e-6 * max(1.0, np.abs(F64).max())


# def2-SVP at the benchmark's 1e-7 (measured: |dE_xc| <= 1.7e-8, max|dV| <= 9.2e-8); the
# def2-TZVP tetramer on this coarse grid reaches max|dV| 3.2e-7 (|dE_xc| <= 5.2e-8), so its V
# bound is looser (on the 99 x 434 grid the benchmark-tolerance test below holds TZVP to 1e-7)
@pytest.mark.parametrize("func,unrestricted,basis,spherical,etol,vtol", [
    ("LDA", False, "DEF2-SVP", True, 1e-7, 1e-7), ("PBE", False, "DEF2-SVP", True, 1e-7, 1e-7),
    ("BLYP", False, "DEF2-SVP", True, 1e-7, 1e-7), ("PBE", True, "DEF2-SVP", True, 1e-7, 1e-7),
    ("PBE", False, "DEF2-TZVP", True, 1e-7, 4e-7), ("PBE", False, "DEF2-TZVP", False, 1e-7, 4e-7)])
def test_mixed_vxc_vs_oracle(ctx, func, unrestricted, basis, spherical, etol, vtol):
    from serenity_gb300 import xcgpu
    w, pts, wts = _case(func, unrestricted, basis=basis, spherical=spherical)
    plan = _plan(ctx, w, pts, wts)
    P = w.density()
    V, exc, nel = plan.vxc(func, P, precision=xcgpu.PREC_MIXED)
    rV, rexc, rnel = po.Basis(w.shells).vxc(pts, wts, func, P)
    print("mixed vs oracle %s %s %s: dExc %.3e max dV %.3e" % (func, basis, "U" if unrestricted else "R",
                                                               exc - rexc, np.abs(V - rV).max()))
    assert abs(exc - rexc) <= etol, abs(exc - rexc)
    assert abs(nel - rnel) <= 1e-8 * rnel
    assert np.abs(V - rV).max() <= vtol, np.abs(V - rV).max()
    np.testing.assert_allclose(V, np.swapaxes(V, 1, 2), rtol=0, atol=1e-14)


# The benchmark's own tolerance, |dE_xc| <= 1e-7 Eh and max|dVxc| <= 1e-7 against the
# FP64 oracle, on cut-down forms of the benchmark workloads: (H2O)8 def2-SVP restricted
# PBE on the 75 x 302 grid (543 600 points before the weight cut-off), and a def2-TZVP
# tetramer, unrestricted PBE on the 99 x 434 grid.
@pytest.mark.parametrize("nmol,dims,basis,nocc,n_rad,n_ang", [
    (8, (2, 2, 2), "DEF2-SVP", 40, 75, 302),
    (4, (2, 2, 1), "DEF2-TZVP", (20, 19), 99, 434)])
def test_mixed_vxc_benchmark_tolerance(ctx, nmol, dims, basis, nocc, n_rad, n_ang):
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(nmol, 0, jitter=0.2, dims=dims)
    w = wl.Workload(sym, xyz, basis, "PBE", nocc, n_rad, n_ang, 0)
    pts, wts = po.becke_grid(w.Z, w.coords, n_rad=n_rad, n_ang=n_ang)
    plan = _plan(ctx, w, pts, wts)
    P = w.density()
    V, exc, nel = plan.vxc("PBE", P, precision=xcgpu.PREC_MIXED)
    rV, rexc, rnel = po.Basis(w.shells).vxc(pts, wts, "PBE", P)
    assert abs(exc - rexc) <= 1e-7, abs(exc - rexc)
    assert abs(nel - rnel) <= 1e-8 * rnel, abs(nel - rnel)
    assert np.abs(V - rV).max() <= 1e-7, np.abs(V - rV).max()


def test_pair_functional_matches_fp64(ctx):
    """The mixed build evaluates restricted PBE in FP32 pairs: against the FP64 functional
    on densities 1e-14..1e3 and reduced gradients 0..8.  Bounds: 1e-11 relative above a
    density of 1e-6 (~48-bit pairs; the FP64 form itself rounds to ~1e-15); below it,
    where both forms lose digits to the cancellations of the low-density limit, 1e-7
    relative with a floor of 1e-13 rho^(4/3) (far below the points' weight in E_xc).
    dF/d(grad rho) is measured against the exchange part's size, 1e-2 rho^(-4/3) |grad
    rho|: PBE's mu = beta pi^2 / 3 makes the exchange and correlation parts cancel at
    small reduced gradients (to 2e-8 of each at s = 1e-3), so the sum has fewer correct
    digits than either part in FP64 as well."""
    from serenity_gb300 import xcgpu
    rng = np.random.default_rng(5)
    rho = np.repeat(np.logspace(-14, 3, 171), 12)
    s = np.tile([0.0, 1e-3, 0.01, 0.1, 0.3, 0.7, 1.0, 1.5, 2.0, 3.0, 5.0, 8.0], 171)
    kf = (3 * np.pi ** 2 * rho) ** (1 / 3)
    gnorm = s * 2 * kf * rho
    d = rng.normal(size=(3, rho.size))
    d /= np.linalg.norm(d, axis=0)
    grad = (gnorm * d)[None]
    ref = ctx.functional("PBE", rho[None], grad, skip_block=0, precision=xcgpu.PREC_FP64)
    got = ctx.functional("PBE", rho[None], grad, skip_block=0, precision=xcgpu.PREC_MIXED)
    hi = rho >= 1e-6
    floor = 1e-13 * rho ** (4 / 3)
    for name, a, b, fl_ in [("e", got[0], ref[0], floor), ("vrho", got[1][0], ref[1][0], floor / rho),
                            ("vgrad", got[2][0], ref[2][0], None)]:
        if fl_ is None:  # dF/d(grad rho): relative to the exchange part's size
            nb = np.maximum(np.linalg.norm(b, axis=0), 1e-2 * rho ** (-4 / 3) * gnorm)
            err = np.linalg.norm(a - b, axis=0) / np.maximum(nb, 1e-300)
            err = np.where(gnorm > 0, err, 0.0)
        else:
            err = np.abs(a - b) / np.maximum(np.abs(b), fl_)
        assert err[hi].max() < 1e-11, (name, err[hi].max(), rho[hi][np.argmax(err[hi])])
        assert err[~hi].max() < 1e-7, (name, err[~hi].max(), rho[~hi][np.argmax(err[~hi])])
