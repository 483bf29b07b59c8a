"""The CPU emulation of the mixed density arithmetic (tests/mixed_emulation.py): its exact
part equals the oracle's basis values and gradients; the kernel's pair arithmetic carries
the basis values (high + low part) to about 2^-44 of the shell's largest value, the
former per-operation FP32 form to 1e-10..1e-6 (the error the pairs remove), the exact
mode to FP64; the kernel's gradients carry no per-radial-shell bias; the density's
first three slice accumulators and the adder's leading products sum exactly; and on one
water the emulated mixed density integrates to the FP64 electron count within the
slices' noise."""
import numpy as np
import pytest

from oracle import pyoracle as po
from serenity_gb300 import workload as wl

import mixed_emulation as me


@pytest.fixture(scope="module")
def water():
    sym, xyz = wl.water_cluster(1, seed=0, jitter=0.0)
    w = wl.Workload(sym, xyz, "DEF2-SVP", "PBE", 5, 30, 110, seed=0)
    pts, wts = po.becke_grid(w.Z, w.coords, n_rad=30, n_ang=110)
    return w, pts, wts


def _shells(w):
    sh = w.shells
    b = po.Basis(sh)
    off = np.concatenate([[0], np.cumsum(sh.nprim)])
    cen = np.asarray(sh.centers).reshape(-1, 3)
    return sh, b, off, cen


def test_exact_part_matches_oracle(water):
    w, pts, _ = water
    sh, b, off, cen = _shells(w)
    xyz = pts[::7]
    ref = b.block(xyz, 1e-9, deriv=1)
    j = 0
    for s in range(sh.nshell):
        n = 2 * int(sh.l[s]) + 1
        phi, grad, _, _, _ = me.shell_values(xyz, cen[s], int(sh.l[s]), sh.alpha[off[s]:off[s + 1]], b.shell_coefs(s))
        np.testing.assert_allclose(phi, ref["values"][:, j:j + n], rtol=0, atol=1e-14)
        for ax in range(3):
            np.testing.assert_allclose(grad[ax], ref["grad"][ax][:, j:j + n], rtol=0, atol=1e-13)
        j += n


def test_basis_value_errors_by_mode(water):
    w, pts, _ = water
    sh, b, off, cen = _shells(w)
    xyz = pts[::3]
    worst = {"kernel": 0.0, "fp32": 0.0, "exact": 0.0}
    for s in range(sh.nshell):
        for mode in worst:
            phi, _, V, VL, _ = me.shell_values(xyz, cen[s], int(sh.l[s]), sh.alpha[off[s]:off[s + 1]], b.shell_coefs(s),
                                               mode)
            scale = max(np.abs(phi).max(), 1e-300)
            worst[mode] = max(worst[mode], np.abs(V.astype(np.float64) + VL - phi).max() / scale)
    assert worst["exact"] < 1e-14
    assert worst["kernel"] < 1e-12  # the radial factor's pair and the pair angular part
    assert 1e-10 < worst["fp32"] < 1e-6  # FP32 rounding of the offsets and angular parts


def test_basis_gradient_bias_by_mode(water):
    """On a radial shell of a function's own atom R and R' are one number each: the former
    FP32 gradients carried their rounding as one relative error at every point of the
    shell (a bias, measured as the least-squares relative error over the shell's points);
    the kernel's form R A_i + R' x_i S with the pairs' low parts leaves errors that differ
    from point to point (measured: median bias 2.7e-8 against 2.7e-9)."""
    w, _, _ = water
    sh, b, off, cen = _shells(w)
    rng = np.random.default_rng(1)
    u = rng.normal(size=(302, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    bias = {"fp32": [], "kernel": []}
    for mode in bias:
        for r in [0.3, 0.7, 1.2, 2.0]:
            for s in range(sh.nshell):
                if np.linalg.norm(cen[s] - cen[0]) > 1e-9:  # the oxygen's shells
                    continue
                _, G64, _, _, G32 = me.shell_values(cen[s][None, :] + r * u, cen[s], int(sh.l[s]),
                                                    sh.alpha[off[s]:off[s + 1]], b.shell_coefs(s), mode)
                for m in range(G64.shape[2]):
                    g = G64[:, :, m].ravel()
                    if not np.abs(g).max() > 0:  # below the radial threshold at this distance
                        continue
                    e = G32[:, :, m].astype(np.float64).ravel() - g
                    bias[mode].append(abs((e * g).sum() / (g * g).sum()))
    fp32, kern = np.median(bias["fp32"]), np.median(bias["kernel"])
    assert fp32 > 1e-8
    assert kern < 0.25 * fp32 and kern < 6e-9, (kern, fp32)


def test_emulated_mixed_density_of_one_water(water):
    w, pts, wts = water
    P = np.asarray(w.density()).reshape(w.nbf, w.nbf)
    dN, dE, N = me.density_errors(w.shells, pts, wts, P, "PBE", "kernel")
    assert N == pytest.approx(10.0, abs=1e-3)
    assert abs(dN) < 2e-7 and abs(dE) < 2e-7
    # the exact basis values leave only the slices' and the epilogue's noise
    dNx, dEx, _ = me.density_errors(w.shells, pts, wts, P, "PBE", "exact")
    assert abs(dNx) < 2e-7 and abs(dEx) < 2e-7


def test_adder_slices_are_fp16_exact_and_leading_products_sum_exactly():
    """The adder's operands: every slice is an FP16 number, the three reconstruct the value
    and its low part to about half a unit of 2^-16 of the row's scale, and the leading products
    (integers below 2^14) sum over a block's 128 points below 2^24, so their FP32 sum is
    exact in any order."""
    rng = np.random.default_rng(3)
    for _ in range(50):
        mag = np.exp(rng.uniform(-12.0, 3.0)) * np.exp(rng.normal(0.0, 2.0, 128))
        v = mag * rng.choice([-1.0, 1.0], 128)
        vh = v.astype(np.float32)
        vl = (v - vh.astype(np.float64)).astype(np.float32)
        f0, f1, f2, sc = me.adder_slices(vh, vl)
        for sl in (f0, f1, f2):
            assert np.array_equal(sl.astype(np.float16).astype(np.float32), sl)
        assert np.abs(f0).max() <= 128 and np.abs(f1).max() <= 0.5 and np.abs(f2).max() <= 2.0 ** -9
        x = (vh.astype(np.float64) + vl.astype(np.float64)) / sc
        rec = f0.astype(np.float64) + f1.astype(np.float64) + f2.astype(np.float64)
        # half a unit of 2^-16 from the last slice's rounding, plus the FP32 rounding of
        # the low part's addition to the remainder
        assert np.abs(rec - x).max() <= 2.0 ** -17 + 2.0 ** -23
        g0 = me.adder_slices(vh[::-1].copy(), vl[::-1].copy())[0]
        prods = f0.astype(np.float64) * g0.astype(np.float64)
        exact = prods.sum()
        assert np.abs(prods).sum() < 2.0 ** 24
        acc = np.float32(0)
        for q in rng.permutation(128):
            acc = np.float32(acc + np.float32(prods[q]))
        assert float(acc) == exact



def test_density_slice_products_sum_exactly_in_the_first_three_accumulators():
    """The density's operands: a point's basis values (row scale below 2^8, slices of 9 bits,
    the last dithered) against P's columns (the same digits).  Over a 128-function window
    the accumulators s0t0, s0t1 + s1t0 and s1t1, each in its unit, sum absolute values of at
    most 2^24, so their FP32 sums are exact in any order; the fourth (s0t2 + s2t0 + s1t2 +
    s2t1, 2^-18 of the first) is not bounded so and is summed to FP32."""
    rng = np.random.default_rng(11)
    worst = [0.0, 0.0, 0.0]
    for _ in range(40):
        v = np.exp(rng.normal(0.0, 2.5, 128)) * rng.choice([-1.0, 1.0], 128)
        vh = v.astype(np.float32)
        vl = (v - vh.astype(np.float64)).astype(np.float32)
        m = np.abs(vh).max()
        _, inva = me.row_scale(np.array([m], dtype=np.float32))
        h0, h1, h2 = me.slice_digits(vh * inva[0], vl * inva[0], rng.uniform(size=128).astype(np.float32))
        Pm = rng.normal(size=(128, 128)) * np.exp(rng.normal(0.0, 2.0, (128, 1)))
        T0, T1, T2, _ = me.split_p(Pm)  # (square, as P is; four of its columns are used)
        for j in range(4):
            # each accumulator's terms in its unit (1, 2^-9, 2^-18) and the sum of the
            # absolute values of the products that form them
            terms = [h0 * T0[:, j], (h0 * T1[:, j] + h1 * T0[:, j]) * 512.0, h1 * T1[:, j] * 512.0 ** 2]
            mags = [np.abs(terms[0]).sum(), (np.abs(h0 * T1[:, j]) + np.abs(h1 * T0[:, j])).sum() * 512.0,
                    np.abs(terms[2]).sum()]
            for k, t in enumerate(terms):
                assert np.array_equal(t, np.rint(t))  # integers in the accumulator's unit
                worst[k] = max(worst[k], mags[k])
                acc = np.float32(0)
                for q in rng.permutation(128):
                    acc = np.float32(acc + np.float32(t[q]))
                assert float(acc) == t.sum()
    assert max(worst) <= 2.0 ** 24
