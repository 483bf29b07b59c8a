"""CPU emulation of the mixed-precision density arithmetic (test and analysis tool).

Restates, operation by operation in numpy float32 (FMAs through float64, exact for FP32
products), what the mixed build kernel computes for rho and grad rho, so that its errors
against FP64 can be attributed stage by stage without a GPU:

  * basis values (serenity_gb300/csrc/xc_mixed_kernel.cuh: shell_rec_at; basis_eval.cuh:
    shell_functions_px): point and centre as FP32 high + remainder, the point-centre
    offset as an FP32 pair (two-sum), r^2 and alpha r^2 as FP32 pairs, the radial sum and
    its derivative as pairs (the exponential taken exact: the kernel's pair exponential is
    accurate to 2e-11), the monomials, the coefficients and the solid-harmonic sums as
    FP32 pairs, the value's low part fma(v, R_lo / R, v_low), the gradients as
    R A_i + R' x_i S in FP32 with the low parts of R and R' (A_i the FP32 sum of the
    coefficients times the monomials' derivatives, S the angular pair sum);
  * the plan's screening (xc_fp64.cu: screen_kernel) and 128-point blocks;
  * the fixed-point slices of A (density_slices: row scale from the point's largest |phi|,
    dithered last digit, point_dither / function_dither) and of P (split_p_kernel);
  * the four accumulators of issue_density_chunk per 128-function window (s0t0,
    s0t1 + s1t0, s1t1, s0t2 + s2t0 + s1t2 + s2t1), their FP32 combination, and the
    epilogue's per-quarter FP32 sums over 8 columns with the low parts summed apart.

On (H2O)32 def2-SVP PBE its former FP32 form ("fp32", the angular part and the offset
rounded once per operation) reproduced the GPU's N_el error to four digits and named
the pair arithmetic the kernel now uses.  The oracle (oracle/pyoracle.py) supplies the
exact basis values check and the functional derivatives for the first-order E_xc error.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

f32, f64 = np.float32, np.float64


def fl(x):
    return np.asarray(x, dtype=f64).astype(f32)


def fma(a, b, c):
    """FP32 fused multiply-add (the FP32 product is exact in FP64; one rounding of the sum,
    double rounding aside)."""
    return (np.asarray(a, f32).astype(f64) * np.asarray(b, f32).astype(f64) + np.asarray(c, f32).astype(f64)).astype(f32)


def two_sum(a, b):
    s = a + b
    bp = s - a
    return s, (a - (s - bp)) + (b - bp)


def _fact(n):
    return 1.0 if n <= 1 else n * _fact(n - 1)


def _binom(n, k):
    return 0.0 if (k < 0 or k > n) else _fact(n) / (_fact(k) * _fact(n - k))


def solid_table(l):
    """Real solid harmonics m = -l..l over Cartesian monomials (a from l down, b from l-a
    down): the closed form of basis_eval.cuh cx::solid."""
    T = np.zeros((2 * l + 1, (l + 1) * (l + 2) // 2))
    for m in range(-l, l + 1):
        am, tv0 = abs(m), (1 if m < 0 else 0)
        N = math.sqrt(2.0 * _fact(l + am) * _fact(l - am) / (2.0 if m == 0 else 1.0)) / (2 ** am * _fact(l))
        for t in range((l - am) // 2 + 1):
            for u in range(t + 1):
                for tv in range(tv0, am + 1, 2):
                    se = t + (tv - tv0) // 2
                    C = ((-1.0 if se % 2 else 1.0) * 0.25 ** t * _binom(l, t) * _binom(l - t, am + t) * _binom(t, u) *
                         _binom(am, tv))
                    py = 2 * u + tv
                    px = 2 * t + am - py
                    k = sum(l - aa + 1 for aa in range(l, px, -1)) + (l - px - py)
                    T[m + l, k] += N * C
    return T


TS = [solid_table(l) for l in range(7)]


def shell_values(xyz, A, l, alpha, coef, mode="kernel", thr=1e-9):
    """Pure shell l at points xyz [n, 3]: (exact values [n, 2l+1], exact gradients [3, n, 2l+1],
    FP32 values, their FP32 low parts, FP32 gradients [3, n, 2l+1]).

    mode "kernel": the kernel's arithmetic, the offset and the whole angular part
    (powers, monomials, the solid-harmonic sums) carried as FP32 pairs (error-free
    products by FMA, two-sum); "fp32": the kernel's former arithmetic, offset and angular
    part rounded to FP32 at every operation (values and gradients); "exact": the exact
    value split into FP32 high and low parts, the gradients in the kernel's form with the
    exact angular sum."""
    ethr = -math.log(thr)
    d = xyz - A[None, :]
    r2e = (d * d).sum(1)
    R64 = np.zeros(len(xyz))
    dR64 = np.zeros(len(xyz))
    for a, c in zip(alpha, coef):
        e = np.where(a * r2e < ethr, c * np.exp(-a * r2e), 0.0)
        R64 += e
        dR64 += -2.0 * a * e
    ks = [(a, b, l - a - b) for a in range(l, -1, -1) for b in range(l - a, -1, -1)]
    mono = np.stack([d[:, 0] ** a * d[:, 1] ** b * d[:, 2] ** c for a, b, c in ks], 1)
    S64 = mono @ TS[l].T
    phi64 = S64 * R64[:, None]
    G64 = np.zeros((3, len(xyz), 2 * l + 1))
    for ax in range(3):
        dm = []
        for e in ks:
            if e[ax] == 0:
                dm.append(np.zeros(len(xyz)))
            else:
                e2 = list(e)
                e2[ax] -= 1
                dm.append(e[ax] * d[:, 0] ** e2[0] * d[:, 1] ** e2[1] * d[:, 2] ** e2[2])
        G64[ax] = (np.stack(dm, 1) @ TS[l].T) * R64[:, None] + S64 * (dR64 * d[:, ax])[:, None]
    # FP32: point and centre as high + remainder
    qh = fl(xyz)
    ql = fl(xyz - qh.astype(f64))
    ah = fl(A)
    al = fl(A - ah.astype(f64))
    X = [(qh[:, i] - ah[i]) + (ql[:, i] - al[i]) for i in range(3)]
    XL = None
    if mode == "kernel":
        XL = []
        for i in range(3):
            s, e = two_sum(qh[:, i], -np.full_like(qh[:, i], ah[i]))
            dl = (ql[:, i] - al[i]) + e
            X[i] = s + dl
            XL.append(dl - (X[i] - s))
    x, y, z = X
    r2 = x * x
    r2l = fma(x, x, -r2)
    yy, zz = y * y, z * z
    s1 = r2 + yy
    b1 = s1 - r2
    e1 = (r2 - (s1 - b1)) + (yy - b1)
    s2 = s1 + zz
    b2 = s2 - s1
    e2 = (s1 - (s2 - b2)) + (zz - b2)
    r2l = (r2l + (e1 + e2)) + (fma(y, y, -yy) + fma(z, z, -zz))
    if XL is not None:
        r2l = r2l + f32(2) * fma(x, XL[0], fma(y, XL[1], z * XL[2]))
    r2 = s2
    Rv = np.zeros_like(x)
    Rl = np.zeros_like(x)
    dR = np.zeros_like(x)
    Dh = np.zeros_like(x)  # D = sum alpha c exp(-alpha r^2) = -R'/2 as a pair (kernel mode)
    Dl = np.zeros_like(x)
    for a, c in zip(alpha, coef):
        a_h, c_h = f32(a), f32(c)
        a_l, c_l = f32(a - float(a_h)), f32(c - float(c_h))
        one = np.ones_like(r2)
        t = a_h * r2
        tl = fma(a_h * one, r2l, fma(a_l * one, r2, fma(a_h * one, r2, -t)))
        on = t < f32(ethr)
        E = np.exp(-t.astype(f64))
        Eh = fl(E)
        El = fma(-Eh, tl, fl(E - Eh.astype(f64)))
        eh = c_h * Eh
        el = fma(c_h * one, El, fma(c_l * one, Eh, fma(c_h * one, Eh, -eh)))
        s = Rv + eh
        bp = s - Rv
        err = (Rv - (s - bp)) + (eh - bp)
        Rl = np.where(on, Rl + (err + el), Rl)
        Rv = np.where(on, s, Rv)
        dR = np.where(on, fma(f32(-2) * a_l * one, eh, fma(f32(-2) * a_h * one, eh, dR)), dR)
        ph = a_h * eh
        pl = fma(a_h * one, el, fma(a_l * one, eh, fma(a_h * one, eh, -ph)))
        sd, ed = two_sum(Dh, ph)
        Dl = np.where(on, Dl + (ed + pl), Dl)
        Dh = np.where(on, sd, Dh)
    zero = ~(np.abs(Rv) >= f32(thr))
    rlo = np.where(Rv != 0, Rl / np.where(Rv != 0, Rv, f32(1)), f32(0)).astype(f32)
    px, py, pz = [np.ones_like(x)], [np.ones_like(x)], [np.ones_like(x)]
    for _ in range(l + 1):
        px.append(px[-1] * x)
        py.append(py[-1] * y)
        pz.append(pz[-1] * z)
    NS = 2 * l + 1
    sv = [np.zeros_like(x) for _ in range(NS)]
    svl = [np.zeros_like(x) for _ in range(NS)]
    sg = [[np.zeros_like(x) for _ in range(NS)] for _ in range(3)]
    sa = [[np.zeros_like(x) for _ in range(NS)] for _ in range(3)]  # sum t d_i(monomial)
    for k, (a, b, c) in enumerate(ks):
        m_ = (px[a] * py[b]) * pz[c]
        v = m_ * Rv
        md = m_ * dR
        dmx = ((f32(a) * px[max(a - 1, 0)]) * py[b]) * pz[c] if a else np.zeros_like(x)
        dmy = ((f32(b) * px[a]) * py[max(b - 1, 0)]) * pz[c] if b else np.zeros_like(x)
        dmz = ((f32(c) * px[a]) * py[b]) * pz[max(c - 1, 0)] if c else np.zeros_like(x)
        g = [fma(dmx, Rv, md * x), fma(dmy, Rv, md * y), fma(dmz, Rv, md * z)]
        for m in range(NS):
            T = TS[l][m, k]
            if T == 0.0:
                continue
            t, tl = f32(T), f32(T - float(f32(T)))
            sv[m] = fma(t * np.ones_like(v), v, sv[m])
            if tl != 0:
                svl[m] = fma(tl * np.ones_like(v), v, svl[m])
            for ax in range(3):
                sg[ax][m] = fma(t * np.ones_like(v), g[ax], sg[ax][m])
                sa[ax][m] = fma(t * np.ones_like(v), (dmx, dmy, dmz)[ax], sa[ax][m])
    if mode == "kernel":
        def pmul(ah_, al_, bh_, bl_):
            h = ah_ * bh_
            return h, fma(ah_, bh_, -h) + fma(ah_, bl_, al_ * bh_)
        qx = [[np.ones_like(x), np.zeros_like(x)]]
        qy = [[np.ones_like(x), np.zeros_like(x)]]
        qz = [[np.ones_like(x), np.zeros_like(x)]]
        for _ in range(l):
            qx.append(list(pmul(qx[-1][0], qx[-1][1], x, XL[0])))
            qy.append(list(pmul(qy[-1][0], qy[-1][1], y, XL[1])))
            qz.append(list(pmul(qz[-1][0], qz[-1][1], z, XL[2])))
        # the angular sum S as a pair, then the value S R (pair times FP32)
        sh_ = [np.zeros_like(x) for _ in range(NS)]
        sl_ = [np.zeros_like(x) for _ in range(NS)]
        for k, (a, b, c) in enumerate(ks):
            mh, ml = pmul(qx[a][0], qx[a][1], qy[b][0], qy[b][1])
            mh, ml = pmul(mh, ml, qz[c][0], qz[c][1])
            for m in range(NS):
                T = TS[l][m, k]
                if T == 0.0:
                    continue
                t, tl = f32(T), f32(T - float(f32(T)))
                ph, pl = pmul(t * np.ones_like(mh), tl * np.ones_like(mh), mh, ml)
                sh_[m], e = two_sum(sh_[m], ph)
                sl_[m] = sl_[m] + (e + pl)
        sv, svl = [], []
        for m in range(NS):
            vh, vl_ = pmul(sh_[m], sl_[m], Rv, np.zeros_like(Rv))
            sv.append(vh)
            svl.append(vl_)
            # gradient R A_i + R' x_i S, R and R' with their low parts
            u = (f32(-2) * Dh) * sh_[m]
            ul = (f32(-2) * Dl) * sh_[m]
            for ax in range(3):
                A_ = sa[ax][m]
                sg[ax][m] = fma(Rv, A_, fma(u, X[ax], fma(Rl, A_, ul * X[ax])))
    if mode == "exact":
        for m in range(NS):
            Sh = fl(S64[:, m])
            u = (f32(-2) * Dh) * Sh
            ul = (f32(-2) * Dl) * Sh
            for ax in range(3):
                A_ = sa[ax][m]
                sg[ax][m] = fma(Rv, A_, fma(u, X[ax], fma(Rl, A_, ul * X[ax])))
    V = np.zeros((len(xyz), NS), f32)
    VL = np.zeros_like(V)
    G32 = np.zeros((3, len(xyz), NS), f32)
    for m in range(NS):
        lo = fma(sv[m], rlo, svl[m])
        hi = sv[m]
        if mode == "exact":
            val = S64[:, m] * R64
            hi = fl(val)
            lo = fl(val - hi.astype(f64))
        V[:, m] = np.where(zero, f32(0), hi)
        VL[:, m] = np.where(zero, f32(0), lo)
        for ax in range(3):
            G32[ax, :, m] = np.where(zero, f32(0), sg[ax][m])
    zr = zero[:, None]
    return np.where(zr, 0.0, phi64), np.where(zr[None], 0.0, G64), V, VL, G32


def point_dither(g):
    M = np.uint64(0xFFFFFFFF)
    g = g.astype(np.uint64) & M
    g ^= g >> np.uint64(16)
    g = (g * np.uint64(0x7FEB352D)) & M
    g ^= g >> np.uint64(15)
    g = (g * np.uint64(0x846CA68B)) & M
    g ^= g >> np.uint64(16)
    return ((g >> np.uint64(8)).astype(f64) / 16777216.0).astype(f32)


def row_scale(m):
    """fixed_scale<8>: (scale, 1/scale) powers of two with m / scale < 256."""
    e = np.frexp(m.astype(f64))[1]
    ok = m > 0
    return np.where(ok, np.ldexp(1.0, e - 8), 0.0).astype(f32), np.where(ok, np.ldexp(1.0, 8 - e), 0.0).astype(f32)


def slice_digits(vh, vl, u):
    """density_slices: stored FP16 slices (s0, s1 / 512, s2 / 512) of vh + vl."""
    s0 = np.rint(vh)
    r1 = ((vh - s0) + vl) * f32(512)
    s1 = np.rint(r1)
    s2 = np.floor(((r1 - s1) * f32(512)) + u)
    return s0.astype(f64), s1.astype(f64) / 512, s2.astype(f64) / 512


def adder_slices(vh, vl):
    """fixed_scale<7> and fixed_slices2<7, 8> (the adder's operands, a function's values over
    a block's points): a power-of-two scale with max|x| / scale < 128, then three 8-bit
    slices, the last rounded to nearest.  Returns (f0, f1, f2, scale): x ~ (f0 + f1 + f2) scale,
    f0 an integer, f1 a multiple of 2^-8, f2 of 2^-16."""
    m = float(np.abs(vh).max())
    if not m > 0:
        z = np.zeros_like(vh)
        return z, z, z, 0.0
    e = np.frexp(m)[1]
    inv = f32(np.ldexp(1.0, 7 - e))
    x, xl = (vh * inv).astype(f32), (vl * inv).astype(f32)
    f0 = np.rint(x)
    r1 = ((x - f0) + xl) * f32(256)
    s1 = np.rint(r1)
    f2 = np.rint((r1 - s1) * f32(256)) * f32(1.0 / 65536)
    return f0, s1 * f32(1.0 / 256), f2.astype(f32), float(np.ldexp(1.0, e - 7))


def split_p(P, exact=False):
    """split_p_kernel: per column a power-of-two scale and three stored slices (exact: the
    scaled column itself as the leading slice, for bounding what the slicing costs)."""
    n = P.shape[0]
    T0, T1, T2, sc = np.empty_like(P), np.empty_like(P), np.empty_like(P), np.empty(n)
    for j in range(n):
        e = np.frexp(np.abs(P[:, j]).max())[1]
        v = P[:, j] * 2.0 ** (8 - e)
        if exact:
            T0[:, j], T1[:, j], T2[:, j], sc[j] = v, 0.0, 0.0, 2.0 ** (e - 8)
            continue
        s0 = np.rint(v)
        r1 = (v - s0) * 512
        s1 = np.rint(r1)
        T0[:, j], T1[:, j], T2[:, j], sc[j] = s0, s1 / 512, np.rint((r1 - s1) * 512) / 512, 2.0 ** (e - 8)
    return T0, T1, T2, sc


def screen(pb, centres, alpha, coef, thr=1e-9):
    """screen_kernel: shells kept for the block of points pb."""
    c = pb.sum(0) / len(pb)
    spread = np.sqrt(((pb - c) ** 2).sum(1)).max()
    keep = []
    for s in range(len(centres)):
        d = math.sqrt(((c - centres[s]) ** 2).sum()) - spread
        if d < 1.0 or abs((coef[s] * np.exp(-alpha[s] * d * d)).sum()) >= thr:
            keep.append(s)
    return keep


def block_density(V, VL, G32, Psl, g0):
    """rho and grad rho of one block by the kernel's arithmetic: V, VL [npts, nact] FP32 values
    and low parts, G32 [3, npts, nact], Psl = (T0, T1, T2, column scales) of P_b, g0 the global
    index of the block's first point."""
    npts, nact = V.shape
    T0, T1, T2, bs = Psl
    sa, inva = row_scale(np.abs(V).max(1))
    up = point_dither(np.arange(g0, g0 + npts))
    x = (np.arange(nact)[None, :].astype(f64) * f64(f32(0.6180339887)) + up[:, None].astype(f64)).astype(f32)
    h0, h1, h2 = slice_digits(V * inva[:, None], VL * inva[:, None], (x - np.floor(x)).astype(f32))
    rq, gq = np.zeros((4, npts)), np.zeros((4, 3, npts))
    rlo = np.zeros((4, npts), f32)
    for nu0 in range(0, nact, 128):
        jn = slice(nu0, min(nu0 + 128, nact))
        nn = jn.stop - nu0
        for w0 in range(0, nact, 128):
            wk = slice(w0, min(w0 + 128, nact))
            a0 = h0[:, wk] @ T0[wk, jn]
            a1 = h0[:, wk] @ T1[wk, jn] + h1[:, wk] @ T0[wk, jn]
            ar = h1[:, wk] @ T1[wk, jn]
            a3 = h0[:, wk] @ T2[wk, jn] + h2[:, wk] @ T0[wk, jn] + h1[:, wk] @ T2[wk, jn] + h2[:, wk] @ T1[wk, jn]
            X = (a0.astype(f32) + a1.astype(f32)) + fma(a3.astype(f32), np.full(a3.shape, f32(1 / 512)), ar.astype(f32))
            xv = (X * (sa[:, None] * bs[None, jn].astype(f32))).astype(f32)
            for q in range(4):
                for cb in range(32 * q, min(32 * q + 32, nn), 8):
                    rr = np.zeros(npts, f32)
                    gx = np.zeros((3, npts), f32)
                    for c in range(cb, min(cb + 8, nn)):
                        rr = fma(xv[:, c], V[:, nu0 + c], rr)
                        rlo[q] = fma(xv[:, c], VL[:, nu0 + c], rlo[q])
                        for ax in range(3):
                            gx[ax] = fma(xv[:, c], G32[ax, :, nu0 + c], gx[ax])
                    rq[q] += rr.astype(f64)
                    gq[q] += gx.astype(f64)
    rq += rlo.astype(f64)
    return ((rq[0] + rq[1]) + rq[2]) + rq[3], 2.0 * (((gq[0] + gq[1]) + gq[2]) + gq[3])


def density_errors(sh, pts, wts, P, func="PBE", basis_mode="kernel", chunk=8192, blocks=None, log=None,
                   chunk_stride=1, p_exact=False):
    """(dN_el, first-order dE_xc, N_el) of the emulated mixed density against FP64 for the
    density matrix P ([nbf, nbf] restricted, or [nspin, nbf, nbf] per spin) on the points
    (Hilbert-ordered, 128-point blocks).  With chunk_stride k only every k-th chunk of points
    is emulated and the sums are scaled by k (a sampled estimate for large workloads)."""
    from oracle import pyoracle as po
    P = np.asarray(P, dtype=f64)
    Ps = P.reshape(-1, P.shape[-1], P.shape[-1])
    nspin = Ps.shape[0]
    b = po.Basis(sh)
    coefs = [b.shell_coefs(s) for s in range(sh.nshell)]
    off = np.concatenate([[0], np.cumsum(sh.nprim)])
    first = np.concatenate([[0], np.cumsum(2 * sh.l + 1)])
    alpha = [sh.alpha[off[s]:off[s + 1]] for s in range(sh.nshell)]
    cen = np.asarray(sh.centers).reshape(-1, 3)
    Psl = [split_p(Ps[i], p_exact) for i in range(nspin)]
    dN = dE = N = 0.0
    nblk = 0
    for ci_, c0 in enumerate(range(0, len(pts), chunk)):
        if ci_ % chunk_stride:
            continue
        xyz = pts[c0:c0 + chunk]
        n = len(xyz)
        keeps = [screen(xyz[bb:bb + 128], cen, alpha, coefs) for bb in range(0, n, 128)]
        act = sorted(set(s for k in keeps for s in k))
        if not act:
            continue
        cols = np.concatenate([np.arange(first[s], first[s + 1]) for s in act])
        pos = {c: i for i, c in enumerate(cols)}
        F = np.zeros((n, len(cols)))
        G64 = np.zeros((3, n, len(cols)))
        V = np.zeros((n, len(cols)), f32)
        VL = np.zeros_like(V)
        G32 = np.zeros((3, n, len(cols)), f32)
        j = 0
        for s in act:
            k = 2 * int(sh.l[s]) + 1
            F[:, j:j + k], G64[:, :, j:j + k], V[:, j:j + k], VL[:, j:j + k], G32[:, :, j:j + k] = shell_values(
                xyz, cen[s], int(sh.l[s]), alpha[s], coefs[s], basis_mode)
            j += k
        r64, g64 = np.zeros((nspin, n)), np.zeros((nspin, 3, n))
        rm, gm = np.zeros((nspin, n)), np.zeros((nspin, 3, n))
        for bi, bb in enumerate(range(0, n, 128)):
            if not keeps[bi] or (blocks is not None and nblk >= blocks):
                continue
            fl_ = np.concatenate([np.arange(first[s], first[s + 1]) for s in keeps[bi]])
            ci = np.array([pos[f] for f in fl_])
            sl = slice(bb, bb + 128)
            Fb = F[sl][:, ci]
            for sp in range(nspin):
                X64 = Fb @ Ps[sp][np.ix_(fl_, fl_)]
                r64[sp, sl] = (X64 * Fb).sum(1)
                g64[sp, :, sl] = 2 * np.einsum("knj,nj->kn", G64[:, sl][:, :, ci], X64)
                sub = tuple(t[np.ix_(fl_, fl_)] for t in Psl[sp][:3]) + (Psl[sp][3][fl_],)
                rm[sp, sl], gm[sp, :, sl] = block_density(V[sl][:, ci], VL[sl][:, ci], G32[:, sl][:, :, ci], sub,
                                                          c0 + bb)
            nblk += 1
        ww = wts[c0:c0 + n]
        _, vr, vg = po.functional(func, r64, g64)
        dN += chunk_stride * (ww * (rm - r64).sum(0)).sum()
        dE += chunk_stride * sum((ww * (vr[sp] * (rm[sp] - r64[sp]) + (vg[sp] * (gm[sp] - g64[sp])).sum(0))).sum()
                                 for sp in range(nspin))
        N += chunk_stride * (ww * r64.sum(0)).sum()
        if log:
            log("%d/%d points  dN %+.4e  dE %+.4e" % (c0 + n, len(pts), dN, dE))
        if blocks is not None and nblk >= blocks:
            break
    return dN, dE, N
