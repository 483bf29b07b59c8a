"""Generate the golden fixtures in ``tests/golden/`` from the reference (Serenity)
test sources and test resources.  Run here, where the reference is mounted; the
JSON files it writes are committed and are all the tests read at run time.

Sources (paths inside the reference project):

* ``src/data/grid/BasisFunctionOnGridController_test.cpp:43-484`` -- values,
  gradients and Hessians of the SMALL_MIXED basis on the TINY grid
  (Mathematica results, tolerance 1e-8) -> ``bf_small_mixed_tiny.json``
* ``src/data/grid/DensityOnGridCalculator_test.cpp:43-256`` -- rho and grad rho on
  TINY from a hand-written 10x10 density matrix (5e-8) -> ``density_tiny.json``
* ``src/data/grid/ScalarOperatorToMatrixAdder_test.cpp:41-148`` -- 10x10 matrix
  from scalar + gradient potentials on VERY_SMALL (1e-8) -> ``adder_very_small.json``
* ``src/potentials/FuncPotential_test.cpp:59-232`` -- H2/def2-TZVP LDA and BP86
  Fock matrices, restricted and unrestricted (1e-6), with the density matrices
  read from ``data/testresources/TestSystem_H2_DEF2_TZVP/*.dmat.{res,unres}.h5``
  -> ``funcpot_h2.json``
* ``src/potentials/NAddFuncPotential_test.cpp:58-120`` -- non-additive LDA
  potential of an active H2 next to an environment H2 (6-31G*, SSF grid), restricted
  and unrestricted (1e-5), with the density matrices read from
  ``data/testresources/TestSystem_H2_6_31Gs_{ACTIVE,ENVIRONMENT}_FDE/*.dmat.*.h5``
  -> ``nadd_h2.json``
* ``src/data/grid/BasisFunctionOnGridController.cpp:455-1062`` -- the
  reference's real solid harmonics Y_lm, l = 0..6, evaluated at fixed points by
  reading its formulas as text -> ``solid_harmonics.json``

Fixture definitions (SMALL_MIXED, TINY, VERY_SMALL) follow
``src/testsupply/BasisController__TEST_SUPPLY.cpp:59-84`` and
``src/testsupply/GridController__TEST_SUPPLY.cpp:31-46``.
"""
import json
import math
import os
import re
import struct
import sys

import numpy as np

if len(sys.argv) < 2:
    sys.exit("usage: python tests/golden/make_golden.py <path of the reference source tree>")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))


def _src(rel):
    return open(os.path.join(REF, rel)).read()


def _calls(text, name):
    """Yield the argument lists of every ``name(...)`` call (balanced parentheses)."""
    for m in re.finditer(r"\b%s\(" % name, text):
        i = m.end()
        depth, args, cur = 1, [], ""
        while depth:
            c = text[i]
            if c == "(":
                depth += 1
            elif c == ")":
                depth -= 1
                if depth == 0:
                    break
            if c == "," and depth == 1:
                args.append(cur.strip())
                cur = ""
            else:
                cur += c
            i += 1
        args.append(cur.strip())
        yield args


def _num(expr):
    """Evaluate a C++ numeric expression (literals, + - * /, sqrt) or return None."""
    e = " ".join(expr.split())
    if not re.fullmatch(r"[0-9eE+\-*/(). sqrt]+", e):
        return None
    return float(eval(e, {"__builtins__": {}}, {"sqrt": math.sqrt}))


def _expectations(text):
    out = []
    for args in _calls(text, "EXPECT_NEAR"):
        a, b = args[0], args[1]
        va, vb = _num(a), _num(b)
        if va is not None and vb is None:
            out.append((" ".join(b.split()), va))
        elif vb is not None and va is None:
            out.append((" ".join(a.split()), vb))
    return out


# --- fixtures of the test supply ------------------------------------------------------------
SMALL_MIXED = [  # BasisController__TEST_SUPPLY.cpp:59-84 (Cartesian shells, raw coefficients)
    {"l": 0, "pure": 0, "center": [0.0, 0.0, 0.0], "alpha": [1.0, 2.0], "coef": [1.0, 0.1]},
    {"l": 1, "pure": 0, "center": [1.0, 0.0, 0.0], "alpha": [1.0, 2.0], "coef": [1.0, 0.1]},
    {"l": 2, "pure": 0, "center": [-1.0, 2.5, 1.0], "alpha": [0.5, 1.2], "coef": [0.8, 0.4]},
]
# GridController__TEST_SUPPLY.cpp:31-46; Eigen's comma initialiser fills the 3xN matrix row by row
TINY = np.array([[0.0, 1.0, -2.0, 3.0], [0.0, 0.0, 1.0, 0.5], [0.0, 0.0, 1.0, -1.0]]).T
TINY_W = [1.0, 1.0, 1.0, 1.0]
VERY_SMALL = np.array([[-1.0, 0.0, 0.0, 0.8, 0.1], [0.0, 0.5, -0.4, 0.1, -0.1], [0.0, 0.4, -0.5, -0.1, 0.1]]).T
VERY_SMALL_W = [0.1, 0.2, 0.15, 0.15, 0.4]


def bf_fixture():
    text = _src("src/data/grid/BasisFunctionOnGridController_test.cpp")
    start = text.index("TestBasisFunctionValuesAndDerivatives")
    end = text.index("SphBFOnGridTest")
    exp = _expectations(text[start:end])
    vals = {}
    for key, v in exp:
        m = re.fullmatch(r"(values|derivatives\.(x|y|z)|hessian\.(xx|xy|xz|yy|yz|zz))\((\d+), (\d+)\)", key)
        if not m:
            continue
        comp = m.group(1).split(".")[-1]
        vals.setdefault(comp, np.zeros((4, 10)).tolist())
        vals[comp][int(m.group(4))][int(m.group(5))] = v
    return {
        "source": "src/data/grid/BasisFunctionOnGridController_test.cpp:43-484",
        "tolerance": 1e-8,
        "max_block_size": 10,
        "radial_threshold": 1e-8 * 0.001,
        "shells": SMALL_MIXED,
        "points": TINY.tolist(),
        "expected": vals,  # [point][function], function order = reference's extended index
    }


def density_fixture():
    text = _src("src/data/grid/DensityOnGridCalculator_test.cpp")
    P = np.zeros((10, 10))
    for m in re.finditer(r"densityMatrix\((\d+), (\d+)\) = ([^;]+);", text):
        P[int(m.group(1)), int(m.group(2))] = _num(m.group(3))
    exp = dict(_expectations(text))
    rho = [exp["densOnGrid[%d]" % i] for i in range(4)]
    grad = [[exp["gradOnGrid.%s[%d]" % (c, i)] for i in range(4)] for c in "xyz"]
    return {
        "source": "src/data/grid/DensityOnGridCalculator_test.cpp:43-256",
        "tolerance": 5e-8,
        "max_block_size": 3,
        "radial_threshold": 0.0,
        "shells": SMALL_MIXED,
        "points": TINY.tolist(),
        "P": P.tolist(),
        "rho": rho,
        "grad": grad,
    }


def adder_fixture():
    text = _src("src/data/grid/ScalarOperatorToMatrixAdder_test.cpp")
    start = text.index("IntegrationOfScalarAndGradientPotentialsRestricted")
    body = text[start:]
    body = body[: body.index("TEST_F") if "TEST_F" in body else len(body)]
    pot = [0.0] * 5
    for m in re.finditer(r"pot\[(\d)\] = ([^;]+);", body):
        pot[int(m.group(1))] = _num(m.group(2))
    grad = {c: [0.0] * 5 for c in "xyz"}
    for m in re.finditer(r"gradPot\.(x|y|z)\[(\d)\] = ([^;]+);", body):
        grad[m.group(1)][int(m.group(2))] = _num(m.group(3))
    F = np.full((10, 10), np.nan)
    for key, v in _expectations(body):
        m = re.fullmatch(r"result\((\d+), (\d+)\)", key)
        if m:
            F[int(m.group(1)), int(m.group(2))] = v
    F = np.where(np.isnan(F), F.T, F)
    return {
        "source": "src/data/grid/ScalarOperatorToMatrixAdder_test.cpp:41-148",
        "tolerance": 1e-8,
        "max_block_size": 3,
        "radial_threshold": 1e-8 * 1e-3,
        "block_ave_threshold": 1e-8 * 1e-3,
        "shells": SMALL_MIXED,
        "points": VERY_SMALL.tolist(),
        "weights": VERY_SMALL_W,
        "potential": pot,
        "gradient_potential": [grad["x"], grad["y"], grad["z"]],
        "F": F.tolist(),
    }


def _symmetric_blocks(path, n):
    """Contiguous little-endian n x n FP64 datasets of an HDF5 file: every offset
    where the next n*n doubles form a symmetric, finite, non-zero matrix."""
    raw = open(path, "rb").read()
    nb = n * n * 8
    found = []
    off = 0
    while off + nb <= len(raw):
        a = np.frombuffer(raw[off:off + nb], dtype="<f8").reshape(n, n)
        if (np.all(np.isfinite(a)) and np.abs(a).max() < 1e3 and np.abs(a).max() > 1e-3
                and np.allclose(a, a.T, rtol=0, atol=1e-12) and abs(np.trace(a)) > 1e-6
                and np.count_nonzero(a) > n * n // 2):
            found.append((off, a.copy()))
            off += nb
        else:
            off += 8
    return found


def _fock_matrix(body):
    m = re.search(r"Fref << ([^;]+);", body)
    return np.array([float(x) for x in m.group(1).replace("\n", " ").split(",")]).reshape(12, 12)


def funcpot_fixture():
    text = _src("src/potentials/FuncPotential_test.cpp")
    tests = {}
    for name in ["H2_FockMatrix_LDA", "H2_FockMatrix_LDA_UNRES", "H2_FockMatrix_GGA", "H2_FockMatrix_GGA_UNRES"]:
        i = text.index("TEST_F(FuncPotentialTest, %s)" % name)
        body = text[i:text.index("TEST_F", i + 10)]
        tests[name] = _fock_matrix(body).tolist()
    base = os.path.join(REF, "data/testresources/TestSystem_H2_DEF2_TZVP/TestSystem_H2_DEF2_TZVP")
    res = _symmetric_blocks(base + ".dmat.res.h5", 12)
    unres = _symmetric_blocks(base + ".dmat.unres.h5", 12)
    assert len(res) == 1, [o for o, _ in res]
    assert len(unres) == 2, [o for o, _ in unres]
    settings = open(base + ".settings").read()
    grid = dict(re.findall(r"^(\w+) (\S+)$", settings[settings.index("+grid"):settings.index("-grid")], re.M))
    xyz = [ln.split() for ln in open(base + ".xyz").read().strip().split("\n")[2:]]
    return {
        "source": "src/potentials/FuncPotential_test.cpp:59-232; data/testresources/TestSystem_H2_DEF2_TZVP",
        "tolerance": 1e-6,
        "basis": "DEF2-TZVP",
        "spherical": False,
        "atoms_angstrom": [[a[0], float(a[1]), float(a[2]), float(a[3])] for a in xyz],
        "grid_settings": grid,
        "P": res[0][1].tolist(),
        "P_offset": res[0][0],
        "Pa": unres[0][1].tolist(),
        "Pb": unres[1][1].tolist(),
        "Pab_offsets": [unres[0][0], unres[1][0]],
        "F": {"LDA": tests["H2_FockMatrix_LDA"], "LDA_UNRES": tests["H2_FockMatrix_LDA_UNRES"],
              "BP86": tests["H2_FockMatrix_GGA"], "BP86_UNRES": tests["H2_FockMatrix_GGA_UNRES"]},
    }


def _expect_entries(body, name):
    """EXPECT_NEAR(<name>(i, j), value, tol) lines of a test body -> [[i, j, value]], tol."""
    out, tol = [], None
    for m in re.finditer(r"EXPECT_NEAR\(%s\((\d+), (\d+)\), ([-+0-9.eE]+), ([-+0-9.eE]+)\)" % re.escape(name), body):
        out.append([int(m.group(1)), int(m.group(2)), float(m.group(3))])
        tol = float(m.group(4))
    return out, tol


def _plausible_density(a):
    return bool(np.all(np.isfinite(a)) and np.abs(a).max() < 10 and np.allclose(a, a.T, rtol=0, atol=1e-14)
                and np.all(np.diag(a) > 1e-4))


def nadd_fixture():
    """Non-additive XC potential of the FDE H2 pair (NAddFuncPotential_test.cpp:58-120):
    active H2 in the field of an environment H2, LDA, 6-31G* (Cartesian), on the active
    system's SSF grid (accuracy 4); density matrices from the systems' test resources."""
    text = _src("src/potentials/NAddFuncPotential_test.cpp")
    res_body = text[text.index("TEST_F(NAddFuncPotentialTest, H2Dimer_FockMatrix_LDA)"):]
    res_body = res_body[:res_body.index("TEST_F", 10)]
    unres_body = text[text.index("TEST_F(NAddFuncPotentialTest, H2Dimer_FockMatrix_LDA_UNRES)"):]
    unres_body = unres_body[:unres_body.index("TEST_F", 10)]
    F, tol = _expect_entries(res_body, "F")
    Fa, _ = _expect_entries(unres_body, "F.alpha")
    Fb, _ = _expect_entries(unres_body, "F.beta")
    systems = {}
    for role, name in [("active", "TestSystem_H2_6_31Gs_ACTIVE_FDE"), ("environment", "TestSystem_H2_6_31Gs_ENVIRONMENT_FDE")]:
        base = os.path.join(REF, "data/testresources", name, name)
        res = _symmetric_blocks(base + ".dmat.res.h5", 4)
        raw = open(base + ".dmat.unres.h5", "rb").read()
        # the unrestricted file holds alpha and beta back to back, 128 bytes apart, at the
        # first offset where a symmetric 4x4 block with positive diagonal starts
        ua = next(o for o in range(0, len(raw) - 255, 8)
                  if _plausible_density(np.frombuffer(raw[o:o + 128], dtype="<f8").reshape(4, 4)))
        Pa = np.frombuffer(raw[ua:ua + 128], dtype="<f8").reshape(4, 4)
        Pb = np.frombuffer(raw[ua + 128:ua + 256], dtype="<f8").reshape(4, 4)
        assert np.allclose(Pa, Pa.T) and np.allclose(Pb, Pb.T)
        settings = open(base + ".settings").read()
        grid = dict(re.findall(r"^(\w+) (\S+)$", settings[settings.index("+grid"):settings.index("-grid")], re.M))
        xyz = [ln.split() for ln in open(base + ".xyz").read().strip().split("\n")[2:]]
        res = [(o, a) for o, a in res if np.all(np.diag(a) > 1e-4)]
        assert len(res) == 1, [o for o, _ in res]
        systems[role] = {"atoms_angstrom": [[a[0], float(a[1]), float(a[2]), float(a[3])] for a in xyz],
                         "grid_settings": grid, "P": res[0][1].tolist(), "P_offset": res[0][0],
                         "Pa": Pa.tolist(), "Pb": Pb.tolist(), "Pab_offsets": [ua, ua + 128]}
    return {
        "source": "src/potentials/NAddFuncPotential_test.cpp:58-120; data/testresources/TestSystem_H2_6_31Gs_{ACTIVE,ENVIRONMENT}_FDE",
        "tolerance": tol, "basis": "6-31GS", "spherical": False, "functional": "LDA",
        "systems": systems,
        "F": F, "Fa": Fa, "Fb": Fb,
    }


def solid_harmonics_fixture():
    """Evaluate the reference's Y[m] (value formulas only) for l = 0..6 at fixed points."""
    text = _src("src/data/grid/BasisFunctionOnGridController.cpp")
    lo = text.index("switch (angularMomentumOfMu)")
    text = text[lo:text.index("Common Finalization", lo)]
    cases = re.split(r"\n\s*case (\d):", text)
    pts = [(0.3, -0.7, 1.1), (-1.2, 0.4, 0.25), (0.9, 1.3, -0.6), (2.0, -0.5, -1.5)]
    out = {}
    for i in range(1, len(cases), 2):
        l = int(cases[i])
        body = cases[i + 1]
        body = body[: body.index("if (_highestDerivative")] if "if (_highestDerivative" in body else body
        forms = {}
        for m in re.finditer(r"\bY\[(\d+)\] =\s*([^;]+);", body):
            forms[int(m.group(1))] = " ".join(m.group(2).split())
        vals = []
        for (x, y, z) in pts:
            env = {"sqrt": math.sqrt, "x": [x ** k for k in range(9)], "y": [y ** k for k in range(9)],
                   "z": [z ** k for k in range(9)]}
            vals.append([eval(forms[m], {"__builtins__": {}}, env) for m in range(2 * l + 1)])
        out[str(l)] = vals
    return {"source": "src/data/grid/BasisFunctionOnGridController.cpp:455-1062", "points": pts, "Y": out}


def main():
    fixtures = {
        "bf_small_mixed_tiny.json": bf_fixture(),
        "density_tiny.json": density_fixture(),
        "adder_very_small.json": adder_fixture(),
        "funcpot_h2.json": funcpot_fixture(),
        "solid_harmonics.json": solid_harmonics_fixture(),
        "nadd_h2.json": nadd_fixture(),
    }
    for name, obj in fixtures.items():
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(obj, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
