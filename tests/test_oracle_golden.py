"""The oracle (CPU restatement of the reference's XC grid path) pinned against
the reference's own golden vectors (tests/golden/, made by make_golden.py)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300.basis import ANGSTROM_TO_BOHR, Shells, atomic_number


def test_basis_values_gradients_hessians(golden):
    g = golden("bf_small_mixed_tiny.json")
    B = po.Basis(Shells(g["shells"]))
    out = B.block(np.array(g["points"]), g["radial_threshold"], deriv=2)
    e = g["expected"]
    tol = g["tolerance"]
    np.testing.assert_allclose(out["values"], e["values"], rtol=0, atol=tol)
    for i, c in enumerate("xyz"):
        np.testing.assert_allclose(out["grad"][i], e[c], rtol=0, atol=tol)
    for i, c in enumerate(["xx", "xy", "xz", "yy", "yz", "zz"]):
        np.testing.assert_allclose(out["hess"][i], e[c], rtol=0, atol=tol)


def test_density_and_gradient(golden):
    d = golden("density_tiny.json")
    B = po.Basis(Shells(d["shells"]))
    rho, grad = B.density(np.array(d["points"]), np.array(d["P"]), max_block=d["max_block_size"],
                          thr=d["radial_threshold"])
    np.testing.assert_allclose(rho[0], d["rho"], rtol=0, atol=d["tolerance"])
    np.testing.assert_allclose(grad[0], d["grad"], rtol=0, atol=d["tolerance"])


def test_scalar_and_gradient_adder(golden):
    a = golden("adder_very_small.json")
    B = po.Basis(Shells(a["shells"]))
    F = B.add_scalar(np.array(a["points"]), a["weights"], a["potential"], np.array(a["gradient_potential"]),
                     max_block=a["max_block_size"], thr=a["radial_threshold"], ave_thr=a["block_ave_threshold"])
    np.testing.assert_allclose(F[0], a["F"], rtol=0, atol=a["tolerance"])


def test_solid_harmonics_match_reference_formulas(golden):
    s = golden("solid_harmonics.json")
    for l, vals in s["Y"].items():
        for pt, v in zip(s["points"], vals):
            np.testing.assert_allclose(po.solid_harmonics(int(l), *pt), v, rtol=1e-13, atol=1e-13)


def _h2(golden):
    d = golden("funcpot_h2.json")
    sym = [a[0] for a in d["atoms_angstrom"]]
    xyz = np.array([a[1:] for a in d["atoms_angstrom"]]) * ANGSTROM_TO_BOHR
    gs = d["grid_settings"]
    pts, w = po.becke_grid([atomic_number(s) for s in sym], xyz, accuracy=int(gs["ACCURACY"]),
                           weight_threshold=float(gs["WEIGHTTHRESHOLD"]), smoothing=int(gs["SMOOTHING"]), sort=True)
    B = po.Basis(Shells.for_atoms(sym, xyz, d["basis"], spherical=d["spherical"]))
    return d, pts, w, B


@pytest.mark.parametrize("func", ["LDA", "BP86"])
@pytest.mark.parametrize("unrestricted", [False, True])
def test_h2_fock_matrix_end_to_end(golden, func, unrestricted):
    """FuncPotential_test.cpp:59-146 (LDA) and :148-232 (BP86 = B88 + P86, the one GGA
    golden vector at this boundary), 1e-6; measured 5e-9 (LDA) and 8e-8 (BP86)."""
    d, pts, w, B = _h2(golden)
    P = np.stack([d["Pa"], d["Pb"]]) if unrestricted else np.array(d["P"])
    V, exc, nel = B.vxc(pts, w, func, P, max_block=int(d["grid_settings"]["BLOCKSIZE"]),
                        thr=float(d["grid_settings"]["BASFUNCRADIALTHRESHOLD"]),
                        ave_thr=float(d["grid_settings"]["BLOCKAVETHRESHOLD"]))
    F = np.array(d["F"][func + "_UNRES" if unrestricted else func])
    for s in range(V.shape[0]):
        np.testing.assert_allclose(V[s], F, rtol=0, atol=d["tolerance"])
    assert abs(nel - 2.0) < 1e-5


def _nadd_pair(golden):
    """Active and environment H2 of the reference's FDE test systems on the active
    system's SSF grid."""
    d = golden("nadd_h2.json")
    out = {}
    for role in ["active", "environment"]:
        s = d["systems"][role]
        sym = [a[0] for a in s["atoms_angstrom"]]
        xyz = np.array([a[1:] for a in s["atoms_angstrom"]]) * ANGSTROM_TO_BOHR
        out[role] = (sym, xyz, po.Basis(Shells.for_atoms(sym, xyz, d["basis"], spherical=d["spherical"])))
    sym, xyz, _ = out["active"]
    gs = d["systems"]["active"]["grid_settings"]
    assert gs["GRIDTYPE"] == "SSF"
    pts, w = po.becke_grid([atomic_number(s) for s in sym], xyz, accuracy=int(gs["ACCURACY"]),
                           weight_threshold=float(gs["WEIGHTTHRESHOLD"]), smoothing=int(gs["SMOOTHING"]),
                           partition="ssf")
    return d, out, pts, w


def test_nadd_lda_fock_matrix_matches_reference(golden):
    """NAddFuncPotential_test.cpp:58-84 (restricted LDA, 1e-5): pins the SSF partition,
    the 6-31G* basis and the non-additive composition."""
    d, sysd, pts, w = _nadd_pair(golden)
    A, E = d["systems"]["active"], d["systems"]["environment"]
    V, _ = po.nadd_vxc(sysd["active"][2], [sysd["environment"][2]], pts, w, d["functional"], np.array(A["P"]),
                       [np.array(E["P"])])
    for i, j, v in d["F"]:
        assert abs(V[0][i, j] - v) <= d["tolerance"], (i, j, V[0][i, j], v)


def test_nadd_unrestricted_split_equals_restricted(golden):
    """Unrestricted input with P_alpha = P_beta = P / 2 gives the restricted potential
    in both spin channels and the same energy (the reference's unrestricted golden values
    of NAddFuncPotential_test.cpp:87-120 need density matrices its test resources do not
    pin, see the fixture)."""
    d, sysd, pts, w = _nadd_pair(golden)
    A, E = np.array(d["systems"]["active"]["P"]), np.array(d["systems"]["environment"]["P"])
    for func in ["LDA", "PBE"]:
        Vr, er = po.nadd_vxc(sysd["active"][2], [sysd["environment"][2]], pts, w, func, A, [E])
        Vu, eu = po.nadd_vxc(sysd["active"][2], [sysd["environment"][2]], pts, w, func, np.stack([A / 2, A / 2]),
                             [np.stack([E / 2, E / 2])])
        np.testing.assert_allclose(Vu[0], Vr[0], rtol=0, atol=1e-12)
        np.testing.assert_allclose(Vu[1], Vr[0], rtol=0, atol=1e-12)
        assert abs(eu - er) <= 1e-12


@pytest.mark.parametrize("func,unrestricted", [("LDA", False), ("PBE", False), ("BLYP", True)])
def test_xc_gradient_is_the_fixed_grid_derivative(func, unrestricted):
    """FuncPotential::getGeomGradients (no grid-weight derivatives) is the exact derivative
    of E_xc on a fixed grid with P fixed and the basis moving with the atom: central
    finite differences agree to O(h^2) (the reference's gradient golden vectors,
    FuncPotential_test.cpp:234-330, need SCF densities its test resources do not hold)."""
    from serenity_gb300 import workload as wl
    sym, xyz = wl.water_cluster(1, 2, jitter=0.1)
    w = wl.Workload(sym, xyz, "DEF2-SVP", func, (5, 4) if unrestricted else 5, 30, 110, 3)
    P = w.density()
    pts, wts = po.becke_grid(w.Z, xyz, n_rad=30, n_ang=110)
    sa = w.shells.atom_indices(xyz)
    G = po.xc_gradient(po.Basis(w.shells), sa, 3, pts, wts, func, P, thr=0.0)
    h = 1e-4
    for atom, k in [(0, 0), (1, 2), (2, 1)]:
        def E(dx):
            x2 = xyz.copy()
            x2[atom, k] += dx
            return po.Basis(Shells.for_atoms(sym, x2, "DEF2-SVP")).vxc(pts, wts, func, P, thr=0.0, ave_thr=0.0)[1]
        fd = (E(h) - E(-h)) / (2 * h)
        assert abs(G[atom, k] - fd) <= 2e-8, (atom, k, G[atom, k], fd)


@pytest.mark.parametrize("func", ["LDA", "PBE", "BLYP"])
def test_lr_kernel_is_the_derivative_of_the_xc_matrix(func):
    """The restricted linear-response kernel contraction (KernelSigmavector<RESTRICTED>
    singlet, second functional derivatives by second-order forward-mode differentiation)
    is the derivative of the XC matrix along the trial density: F(D) = d/de Vxc[P0 + e D]
    for symmetric D (the reference's tests of this path need LRSCF solver runs)."""
    from serenity_gb300 import workload as wl
    sym, xyz = wl.water_cluster(1, 5, jitter=0.1)
    w = wl.Workload(sym, xyz, "DEF2-SVP", func, 5, 30, 110, 6)
    P0 = w.density()
    rng = np.random.default_rng(8)
    D = rng.standard_normal(P0.shape) * 0.05
    D = D + D.T
    pts, wts = po.becke_grid(w.Z, xyz, n_rad=30, n_ang=110)
    B = po.Basis(w.shells)
    F = po.lr_fock(B, pts, wts, func, P0, D, thr=0.0, ave_thr=0.0)
    h = 1e-5
    Vp = B.vxc(pts, wts, func, P0 + h * D, thr=0.0, ave_thr=0.0)[0][0]
    Vm = B.vxc(pts, wts, func, P0 - h * D, thr=0.0, ave_thr=0.0)[0][0]
    fd = (Vp - Vm) / (2 * h)
    assert np.abs(F - fd).max() <= 1e-6 * max(1.0, np.abs(fd).max()), np.abs(F - fd).max()


@pytest.mark.parametrize("func", ["LDA", "PBE", "BLYP", "BP86"])
@pytest.mark.parametrize("kind", ["unrestricted", "triplet"])
def test_spin_lr_kernel_is_the_derivative_of_the_xc_matrix(func, kind):
    """The spin-resolved kernel contraction (KernelSigmavector<UNRESTRICTED>::contractBlock,
    and the triplet's f_aa - f_ab of KernelSigmavector<RESTRICTED>) is the derivative of the
    unrestricted XC matrix along the trial densities: F_s(D) = d/de Vxc_s[P_a + e D_a,
    P_b + e D_b]; the triplet's perturbation is (+D, -D) about (P0/2, P0/2), alpha part."""
    from serenity_gb300 import workload as wl
    sym, xyz = wl.water_cluster(1, 5, jitter=0.1)
    rng = np.random.default_rng(11)
    pts, wts = po.becke_grid([8, 1, 1], xyz, n_rad=30, n_ang=110)
    h = 1e-5
    if kind == "unrestricted":
        w = wl.Workload(sym, xyz, "DEF2-SVP", func, (5, 4), 30, 110, 6)
        P0 = np.asarray(w.density())
        D = rng.standard_normal(P0.shape) * 0.05
        D = D + np.swapaxes(D, 1, 2)
        B = po.Basis(w.shells)
        F = po.lr_fock_spin(B, pts, wts, func, P0, D, kind, thr=0.0, ave_thr=0.0)
        Vp = B.vxc(pts, wts, func, P0 + h * D, thr=0.0, ave_thr=0.0)[0]
        Vm = B.vxc(pts, wts, func, P0 - h * D, thr=0.0, ave_thr=0.0)[0]
    else:
        w = wl.Workload(sym, xyz, "DEF2-SVP", func, 5, 30, 110, 6)
        P0 = np.asarray(w.density())
        D = rng.standard_normal(P0.shape) * 0.05
        D = D + D.T
        B = po.Basis(w.shells)
        F = po.lr_fock_spin(B, pts, wts, func, P0, D, kind, thr=0.0, ave_thr=0.0)
        Vp = B.vxc(pts, wts, func, np.stack([0.5 * P0 + h * D, 0.5 * P0 - h * D]), thr=0.0, ave_thr=0.0)[0][0]
        Vm = B.vxc(pts, wts, func, np.stack([0.5 * P0 - h * D, 0.5 * P0 + h * D]), thr=0.0, ave_thr=0.0)[0][0]
    fd = (Vp - Vm) / (2 * h)
    assert np.abs(fd).max() > 1e-2  # a perturbation that moves the potential
    assert np.abs(F - fd).max() <= 1e-8 * max(1.0, np.abs(fd).max()), np.abs(F - fd).max()
