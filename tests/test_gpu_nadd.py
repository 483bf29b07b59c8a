"""Non-additive XC potential (NAddFuncPotential<M>) on the GPU: the reference's golden
Fock elements, parity with the oracle's composition, spin consistency, the mixed form
against FP64, and the SSF grid partition against the oracle."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300 import workload as wl
from serenity_gb300.basis import ANGSTROM_TO_BOHR, Shells, atomic_number

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from serenity_gb300 import xcgpu
    return xcgpu.Context()


def _pair(ctx, golden):
    from serenity_gb300 import xcgpu
    d = golden("nadd_h2.json")
    sysd = {}
    for role in ["active", "environment"]:
        s = d["systems"][role]
        sym = [a[0] for a in s["atoms_angstrom"]]
        xyz = np.array([a[1:] for a in s["atoms_angstrom"]]) * ANGSTROM_TO_BOHR
        sysd[role] = (sym, xyz, Shells.for_atoms(sym, xyz, d["basis"], spherical=d["spherical"]))
    sym, xyz, _ = sysd["active"]
    gs = d["systems"]["active"]["grid_settings"]
    grid = xcgpu.Grid.build(ctx, [atomic_number(s) for s in sym], xyz, accuracy=int(gs["ACCURACY"]),
                            weight_threshold=float(gs["WEIGHTTHRESHOLD"]), smoothing=int(gs["SMOOTHING"]),
                            partition="ssf")
    plans = {r: xcgpu.Plan(ctx, grid, xcgpu.Basis(ctx, sysd[r][2]), 128, float(gs["BASFUNCRADIALTHRESHOLD"]))
             for r in sysd}
    return d, sysd, grid, plans


def test_ssf_grid_matches_oracle(ctx, golden):
    d, sysd, grid, _ = _pair(ctx, golden)
    sym, xyz, _ = sysd["active"]
    gs = d["systems"]["active"]["grid_settings"]
    pts, w = grid.points()
    rp, rw = po.becke_grid([atomic_number(s) for s in sym], xyz, accuracy=int(gs["ACCURACY"]),
                           weight_threshold=float(gs["WEIGHTTHRESHOLD"]), smoothing=int(gs["SMOOTHING"]),
                           partition="ssf")
    assert pts.shape == rp.shape
    np.testing.assert_allclose(pts, rp, rtol=0, atol=1e-12)
    # cell functions near the polynomial's edges cancel (1 - poly); the GPU's fused
    # multiply-adds round them differently from the host build by ~1e-15 absolute
    np.testing.assert_allclose(w, rw, rtol=1e-11, atol=1e-14)
    # a larger SSF grid (water trimer, explicit 50 x 194) against the oracle
    sym3, xyz3 = wl.water_cluster(3, 1, jitter=0.2, dims=(3, 1, 1))
    from serenity_gb300 import xcgpu
    Z3 = [atomic_number(s) for s in sym3]
    g3 = xcgpu.Grid.build(ctx, Z3, xyz3, n_rad=50, n_ang=194, partition="ssf")
    p3, w3 = g3.points()
    r3, rw3 = po.becke_grid(Z3, xyz3, n_rad=50, n_ang=194, partition="ssf")
    assert p3.shape == r3.shape
    np.testing.assert_allclose(p3, r3, rtol=0, atol=1e-12)
    np.testing.assert_allclose(w3, rw3, rtol=1e-11, atol=1e-14)


def test_nadd_matches_reference_golden_and_oracle(ctx, golden):
    """NAddFuncPotential_test.cpp:58-84 (restricted LDA, 1e-5), and the oracle's
    composition on the same grid to 1e-10."""
    d, sysd, grid, plans = _pair(ctx, golden)
    A, E = np.array(d["systems"]["active"]["P"]), np.array(d["systems"]["environment"]["P"])
    V, e = plans["active"].nadd_vxc("LDA", A, [(plans["environment"], E)])
    for i, j, v in d["F"]:
        assert abs(V[0][i, j] - v) <= d["tolerance"], (i, j, V[0][i, j], v)
    pts, w = grid.points()
    rV, re = po.nadd_vxc(po.Basis(sysd["active"][2]), [po.Basis(sysd["environment"][2])], pts, w, "LDA", A, [E])
    np.testing.assert_allclose(V, rV, rtol=0, atol=1e-10)
    assert abs(e - re) <= 1e-10


@pytest.mark.parametrize("func", ["LDA", "PBE", "BLYP"])
def test_nadd_unrestricted_matches_oracle_and_split(ctx, golden, func):
    d, sysd, grid, plans = _pair(ctx, golden)
    A, E = d["systems"]["active"], d["systems"]["environment"]
    PA = np.array([A["Pa"], A["Pb"]])
    PE = np.array([E["Pa"], E["Pb"]])
    V, e = plans["active"].nadd_vxc(func, PA, [(plans["environment"], PE)])
    pts, w = grid.points()
    rV, re = po.nadd_vxc(po.Basis(sysd["active"][2]), [po.Basis(sysd["environment"][2])], pts, w, func, PA, [PE])
    np.testing.assert_allclose(V, rV, rtol=0, atol=1e-10)
    assert abs(e - re) <= 1e-10
    # P_alpha = P_beta = P / 2 reproduces the restricted build in both channels
    Pr, Er = np.array(A["P"]), np.array(E["P"])
    Vr, er = plans["active"].nadd_vxc(func, Pr, [(plans["environment"], Er)])
    Vu, eu = plans["active"].nadd_vxc(func, np.stack([Pr / 2, Pr / 2]), [(plans["environment"], np.stack([Er / 2, Er / 2]))])
    np.testing.assert_allclose(Vu[0], Vr[0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(Vu[1], Vr[0], rtol=0, atol=1e-12)
    assert abs(eu - er) <= 1e-12


def _water_in_waters(ctx):
    """One water (active) next to a water dimer (two environment subsystems), def2-SVP,
    on a 30 x 110 Becke grid of all atoms (the supersystem grid of an FDE step)."""
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(3, 7, jitter=0.2, dims=(3, 1, 1))
    Z = [atomic_number(s) for s in sym]
    grid = xcgpu.Grid.build(ctx, Z, xyz, n_rad=30, n_ang=110)
    subs = []
    for k in range(3):
        s, x = sym[3 * k:3 * k + 3], xyz[3 * k:3 * k + 3]
        w = wl.Workload(s, x, "DEF2-SVP", "PBE", 5, 30, 110, seed=k)
        subs.append((w, xcgpu.Plan(ctx, grid, xcgpu.Basis(ctx, w.shells), 128, 1e-9), w.density()))
    return grid, subs


@pytest.mark.parametrize("func", ["LDA", "PBE"])
def test_nadd_three_subsystems_fp64_vs_oracle_and_mixed(ctx, func):
    from serenity_gb300 import xcgpu
    grid, subs = _water_in_waters(ctx)
    (wA, pA, PA), env = subs[0], subs[1:]
    V, e = pA.nadd_vxc(func, PA, [(p, P) for _, p, P in env])
    pts, w = grid.points()
    rV, re = po.nadd_vxc(po.Basis(wA.shells), [po.Basis(we.shells) for we, _, _ in env], pts, w, func, PA,
                         [P for _, _, P in env])
    np.testing.assert_allclose(V, rV, rtol=0, atol=1e-10)
    assert abs(e - re) <= 1e-10
    Vm, em = pA.nadd_vxc(func, PA, [(p, P) for _, p, P in env], precision=xcgpu.PREC_MIXED)
    assert np.abs(Vm - V).max() <= 1e-6, np.abs(Vm - V).max()
    assert abs(em - e) <= 5e-6, abs(em - e)


def test_nadd_without_environment_is_zero_and_grid_mismatch_is_rejected(ctx):
    from serenity_gb300 import xcgpu
    grid, subs = _water_in_waters(ctx)
    (wA, pA, PA) = subs[0]
    V, e = pA.nadd_vxc("PBE", PA, [])
    assert np.abs(V).max() == 0.0 and e == 0.0
    other = xcgpu.Grid.build(ctx, wA.Z, wA.coords, n_rad=30, n_ang=110)
    pB = xcgpu.Plan(ctx, other, xcgpu.Basis(ctx, subs[1][0].shells), 128, 1e-9)
    with pytest.raises(xcgpu.XcgpuError):
        pA.nadd_vxc("PBE", PA, [(pB, subs[1][2])])


@pytest.mark.parametrize("precision", [0, 1])
def test_nadd_all_equals_one_call_per_subsystem(ctx, precision):
    """xcgpu_nadd_vxc_all = one xcgpu_nadd_vxc per subsystem with the others as
    environment (each density formed once instead of once per call)."""
    from serenity_gb300 import xcgpu
    grid, subs = _water_in_waters(ctx)
    Vs, e = xcgpu.nadd_vxc_all([(p, P) for _, p, P in subs], "PBE", precision=precision)
    for i, (_, p, P) in enumerate(subs):
        others = [(q, Q) for j, (_, q, Q) in enumerate(subs) if j != i]
        V1, e1 = p.nadd_vxc("PBE", P, others, precision=precision)
        np.testing.assert_allclose(Vs[i], V1, rtol=0, atol=1e-12)
        assert abs(e - e1) <= 1e-12
