"""XC part of the nuclear gradient (FuncPotential<M>::getGeomGradients) on the GPU against
the oracle's restatement of the reference's pair loop (which the CPU tests tie to finite
differences of E_xc on a fixed grid)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300 import workload as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from serenity_gb300 import xcgpu
    return xcgpu.Context()


@pytest.mark.parametrize("func,unrestricted,basis", [("LDA", False, "DEF2-SVP"), ("PBE", False, "DEF2-SVP"),
                                                      ("BLYP", True, "DEF2-SVP"), ("PBE", False, "DEF2-TZVP")])
def test_xc_gradient_matches_oracle(ctx, func, unrestricted, basis):
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(2, 4, jitter=0.2, dims=(2, 1, 1))
    w = wl.Workload(sym, xyz, basis, func, (10, 9) if unrestricted else 10, 30, 110, 4)
    P = w.density()
    pts, wts = po.becke_grid(w.Z, xyz, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, xcgpu.Grid(ctx, pts, wts), xcgpu.Basis(ctx, w.shells), 128, 1e-9)
    sa = w.shells.atom_indices(xyz)
    G = plan.xc_gradient(func, P, sa, len(sym))
    R = po.xc_gradient(po.Basis(w.shells), sa, len(sym), pts, wts, func, P)
    np.testing.assert_allclose(G, R, rtol=0, atol=1e-10 * max(1.0, np.abs(R).max()))


def test_xc_gradient_of_symmetric_h2_is_antisymmetric(ctx):
    from serenity_gb300 import xcgpu
    from serenity_gb300.basis import ANGSTROM_TO_BOHR, Shells
    sym = ["H", "H"]
    xyz = np.array([[0, 0, -0.370424], [0, 0, 0.370424]]) * ANGSTROM_TO_BOHR
    sh = Shells.for_atoms(sym, xyz, "DEF2-TZVP", spherical=False)
    g = xcgpu.Grid.build(ctx, [1, 1], xyz, accuracy=4, partition="ssf")
    plan = xcgpu.Plan(ctx, g, xcgpu.Basis(ctx, sh), 128, 1e-9)
    c = np.zeros(sh.nbf)
    half = sh.nbf // 2
    c[0] = c[half] = 0.5  # a symmetric (sigma_g-like) orbital
    P = 2.0 * np.outer(c, c)
    G = plan.xc_gradient("PBE", P, sh.atom_indices(xyz), 2)
    assert abs(G[0, 2] + G[1, 2]) <= 1e-10 and np.abs(G[:, :2]).max() <= 1e-10
    assert abs(G[0, 2]) > 1e-3
