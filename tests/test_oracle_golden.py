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


@pytest.mark.parametrize("unrestricted", [False, True])
def test_h2_lda_fock_matrix_end_to_end(golden, unrestricted):
    d, pts, w, B = _h2(golden)
    P = np.stack([d["Pa"], d["Pb"]]) if unrestricted else np.array(d["P"])
    V, exc, nel = B.vxc(pts, w, "LDA", P, max_block=int(d["grid_settings"]["BLOCKSIZE"]),
                        thr=float(d["grid_settings"]["BASFUNCRADIALTHRESHOLD"]),
                        ave_thr=float(d["grid_settings"]["BLOCKAVETHRESHOLD"]))
    F = np.array(d["F"]["LDA_UNRES" if unrestricted else "LDA"])
    for s in range(V.shape[0]):
        np.testing.assert_allclose(V[s], F, rtol=0, atol=d["tolerance"])
    assert abs(nel - 2.0) < 1e-5
