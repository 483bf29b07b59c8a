"""The FP32-pair (double-float) algorithms of serenity_gb300/csrc/df32.cuh, restated in
numpy float32 with the same operation order (FMA through exact float64 products), and
held to the accuracy the mixed build's PBE relies on: ~1e-13 relative against float64
references for sums, products, quotients, square and cube roots, exp, expm1 and log.
The GPU test tests/test_gpu_mixed.py::test_pair_functional_matches_fp64 holds the device
code itself against the FP64 functional."""
import math

import numpy as np

f32 = np.float32


def fl(x):
    return np.float32(x)


def fma(a, b, c):  # a*b is exact in float64 for float32 a, b
    return fl(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = fl(a + b)
    bb = fl(s - a)
    return s, fl(fl(a - fl(s - bb)) + fl(b - bb))


def fast_two_sum(a, b):
    s = fl(a + b)
    return s, fl(b - fl(s - a))


def add(a, b):
    sh, sl = two_sum(a[0], b[0])
    th, tl = two_sum(a[1], b[1])
    sh, sl = fast_two_sum(sh, fl(sl + th))
    return fast_two_sum(sh, fl(sl + tl))


def sub(a, b):
    return add(a, (-b[0], -b[1]))


def mul(a, b):
    p = fl(a[0] * b[0])
    return fast_two_sum(p, fma(a[0], b[1], fma(a[1], b[0], fma(a[0], b[0], -p))))


def seed(x, ulps, rng):  # an FP32 approximation a few ulp off, as the device's fast functions
    v = fl(x)
    return fl(v * fl(1 + ulps * 2.0 ** -23 * rng.uniform(-1, 1)))


def div(a, b, rng):
    rb = seed(1.0 / np.float64(b[0]), 2, rng)
    q1 = fl(a[0] * rb)
    r = sub(a, mul(b, (q1, f32(0))))
    q2 = fl(r[0] * rb)
    r = sub(r, mul(b, (q2, f32(0))))
    q3 = fl(r[0] * rb)
    return add(fast_two_sum(q1, q2), (q3, f32(0)))


def val(a):
    return np.float64(a[0]) + np.float64(a[1])


def pair(x):
    h = fl(x)
    return h, fl(x - np.float64(h))


TAB = [pair(2.0 ** (j / 32)) for j in range(32)]
C1, C2, C3 = f32(float.fromhex("0x1.63p-6")), f32(float.fromhex("-0x1.bd0106p-18")), f32(float.fromhex("0x1.cf79acp-45"))


def expm1_small(r):
    r2 = mul(r, r)
    r3s = mul(mul(r2, r), pair(1.0 / 6.0))
    t = fl(fl(r2[0] * r2[0]) * fma(r[0], fma(r[0], f32(1 / 720), f32(1 / 120)), f32(1 / 24)))
    return add(add(r, (fl(0.5 * r2[0]), fl(0.5 * r2[1]))), add(r3s, (t, f32(0))))


def exp(a):
    x = min(a[0], f32(88))
    kf = f32(np.rint(fl(x * f32(46.16624))))
    k = int(kf)
    j, m = k & 31, k >> 5
    r1 = fma(-kf, C1, x)
    ph = fl(kf * C2)
    pl = fma(kf, C2, -ph)
    rh, rhl = two_sum(r1, -ph)
    rl = fl(fma(-kf, C3, fl(rhl - pl)) + a[1])
    q = expm1_small(fast_two_sum(rh, rl))
    v = add(TAB[j], mul(TAB[j], q))
    sc = f32(2.0 ** m)
    return fl(v[0] * sc), fl(v[1] * sc)


def expm1(a):
    if abs(a[0]) <= 0.0108:
        return expm1_small(a)
    return sub(exp(a), (f32(1), f32(0)))


def log(a, rng):
    y0 = fl(math.log(np.float64(a[0])) + 2.0 ** -22 * rng.uniform(-1, 1))  # FP32 log, ~2^-22 absolute
    t = sub(mul(a, exp((-y0, f32(0)))), (f32(1), f32(0)))
    c = fl(fl(t[0] * t[0]) * fma(t[0], f32(1 / 3), f32(-0.5)))
    return add(add((y0, f32(0)), t), (c, f32(0)))


def sqrt(a, rng):
    x = seed(1 / math.sqrt(a[0]), 2, rng)
    ax = fl(a[0] * x)
    d = sub(a, (fl(ax * ax), fma(ax, ax, -fl(ax * ax))))
    return two_sum(ax, fl(d[0] * fl(x * f32(0.5))))


def cbrt(a, rng):
    y = seed(np.float64(a[0]) ** (1 / 3), 1, rng)
    y2 = (fl(y * y), fma(y, y, -fl(y * y)))
    r = sub(mul(y2, (y, f32(0))), a)
    return two_sum(y, -fl(r[0] / fl(3 * y2[0])))


def test_pair_arithmetic_accuracy():
    rng = np.random.default_rng(1)
    worst = {}

    def note(name, err):
        worst[name] = max(worst.get(name, 0.0), err)

    for _ in range(400):
        x = float(np.exp(rng.uniform(-32, 10)))
        a = pair(x)
        xv = val(a)
        note("sqrt", abs(val(sqrt(a, rng)) - math.sqrt(xv)) / math.sqrt(xv))
        note("cbrt", abs(val(cbrt(a, rng)) - xv ** (1 / 3)) / xv ** (1 / 3))
        lg = math.log(xv)
        note("log", abs(val(log(a, rng)) - lg) / max(abs(lg), 1.0))
        b = pair(rng.uniform(-60, 60))
        note("exp", abs(val(exp(b)) - math.exp(val(b))) / math.exp(val(b)))
        z = pair(rng.uniform(-0.3, 0.3) * 10 ** rng.uniform(-8, 0))
        note("expm1", abs(val(expm1(z)) - math.expm1(val(z))) / abs(math.expm1(val(z))))
        d = pair(float(np.exp(rng.uniform(-20, 20))) * rng.choice([-1, 1]))
        note("div", abs(val(div(a, d, rng)) - xv / val(d)) / abs(xv / val(d)))
        e = pair(rng.normal() * 10 ** rng.uniform(-5, 5))
        note("mul", abs(val(mul(a, e)) - xv * val(e)) / abs(xv * val(e)))
    bounds = {"sqrt": 5e-13, "cbrt": 2e-13, "log": 5e-14, "exp": 1e-13, "expm1": 2e-12, "div": 5e-14, "mul": 5e-14}
    for name, bound in bounds.items():
        assert worst[name] < bound, (name, worst[name])
