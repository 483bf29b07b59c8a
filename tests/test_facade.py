"""The C++ facade (include/serenity_xc.hpp): compiles against the C ABI here, and on a
GPU reproduces the reference's golden density and adder vectors; runs the reference's
FuncPotential::getMatrix chain (lazy DensityMatrixDensityOnGridController,
FunctionalLibrary::calcData with the controller, the adder) to the fused build's result;
recomputes the density after the density matrix changes; prints the grid electron count
with gridAccuracyCheck; lists the non-negligible blocks."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out):
    from serenity_gb300 import build
    lib = build.build()
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp",
           "facade_check.cpp"), "-L", os.path.dirname(lib), "-lxcgpu", "-Wl,-rpath," + os.path.dirname(lib),
           "-o", out]
    subprocess.run(cmd, check=True)


def test_facade_compiles(tmp_path):
    _compile(str(tmp_path / "facade_check"))


@pytest.mark.gpu
def test_facade_matches_reference_golden(tmp_path, golden):
    exe = str(tmp_path / "facade_check")
    _compile(exe)
    d = golden("density_tiny.json")
    pfile = tmp_path / "P.txt"
    np.savetxt(pfile, np.array(d["P"]).T.reshape(-1))  # column-major
    out = subprocess.run([exe], check=True, capture_output=True, text=True,
                         env=dict(os.environ, FACADE_P=str(pfile))).stdout
    printed = out[:out.index("{\n")]
    r = json.loads(out[out.index("{\n"):])
    # staged chain = fused build (both FP64)
    np.testing.assert_allclose(r["staged_F"], r["fused_F"], rtol=1e-12, atol=1e-14)
    assert abs(r["staged_E"] - r["fused_E"]) <= 1e-12 * abs(r["fused_E"])
    assert "nElectrons from integration over grid" in printed
    assert abs(r["nel_grid"] - r["nel_sum"]) <= 1e-12 * abs(r["nel_sum"])
    assert not np.allclose(r["rho_before"], r["rho_after"])  # invalidated and recomputed
    assert 0 < r["nonnegligible_blocks"] <= r["nblocks_lazy"] == 2
    np.testing.assert_allclose(r["rho"], d["rho"], rtol=0, atol=d["tolerance"])
    np.testing.assert_allclose(r["grad_x"], d["grad"][0], rtol=0, atol=d["tolerance"])
    assert r["nblocks"] == 2
    a = golden("adder_very_small.json")
    F = np.array(r["F"]).reshape(10, 10).T
    np.testing.assert_allclose(F, a["F"], rtol=0, atol=a["tolerance"])
    assert r["grid_mismatch_throws"]
