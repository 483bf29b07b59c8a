// FP32-pair ("double-float") arithmetic for the functional of the mixed build.
//
// A value is an unevaluated sum h + l of two FP32 numbers with |l| <= ulp(h) / 2, about 48
// significant bits.  GB300 executes FP32 at 64 times its FP64 rate, so a functional
// evaluated in pairs costs a fraction of the FP64 one at ~1e-14 relative accuracy (the
// FP32 exponent range limits it to the densities the functional cut-offs admit).
//
// Error-free transformations after Knuth (two-sum) and Dekker (product, here by FMA);
// addition, multiplication and division follow the double-double algorithms of Hida,
// Li & Bailey ("Algorithms for quad-double precision floating point arithmetic", ARITH
// 15, 2001).  Elementary functions: square root by one Karp-Markstein step from the FP32
// reciprocal square root; cube root by one Newton step from the FP32 cube root;
// exponential after P. T. P. Tang (ACM TOMS 15, 1989) with the 32-entry table of
// exp_tang.cuh and exp(r) - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720) for
// |r| <= ln2/64; logarithm by one Newton step y + (x e^-y - 1) - (...)^2/2 on the FP32
// logarithm.  Roundings are explicit (__fadd_rn, ...) so no contraction changes the
// error-free steps.
#pragma once
#include <cuda_runtime.h>

#include "exp_tang.cuh"

namespace xcgpu {

struct DF {
  float h, l;
  DF() = default;
  __host__ __device__ constexpr DF(float a, float b) : h(a), l(b) {}
  // from a double (folded at compile time for constants)
  __host__ __device__ constexpr DF(double x)
      : h(static_cast<float>(x)), l(static_cast<float>(x - static_cast<double>(static_cast<float>(x)))) {}
  __host__ __device__ constexpr DF(int x) : DF(static_cast<double>(x)) {}
};

namespace dfo {
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return DF(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  const float s = __fadd_rn(a, b);
  return DF(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ DF two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return DF(p, fmaf(a, b, -p));
}
}  // namespace dfo

__device__ __forceinline__ DF operator+(DF a, DF b) {
  DF s = dfo::two_sum(a.h, b.h);
  const DF t = dfo::two_sum(a.l, b.l);
  s = dfo::fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return dfo::fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}
__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.h, -a.l); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
  return dfo::fast_two_sum(p, e);
}
__device__ __forceinline__ DF operator/(DF a, DF b) {
  const float rb = __fdividef(1.f, b.h);  // ~2^-22; the two corrections make the quotient ~2^-44
  const float q1 = __fmul_rn(a.h, rb);
  DF r = a - b * DF(q1, 0.f);
  const float q2 = __fmul_rn(r.h, rb);
  r = r - b * DF(q2, 0.f);
  const float q3 = __fmul_rn(r.h, rb);
  return dfo::fast_two_sum(q1, q2) + DF(q3, 0.f);
}

__device__ __forceinline__ DF df_from_double(double x) {
  const float h = __double2float_rn(x);
  return DF(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.h + (double)a.l; }

// sqrt(a), a >= 0
__device__ __forceinline__ DF df_sqrt(DF a) {
  if (!(a.h > 0.f)) return DF(0.f, 0.f);
  const float x = rsqrtf(a.h), ax = __fmul_rn(a.h, x);
  const DF d = a - dfo::two_prod(ax, ax);
  return dfo::two_sum(ax, __fmul_rn(d.h, __fmul_rn(x, 0.5f)));
}

// a^(1/3), a > 0
__device__ __forceinline__ DF df_cbrt(DF a) {
  const float y = cbrtf(a.h);
  const DF y2 = dfo::two_prod(y, y);
  const DF r = y2 * DF(y, 0.f) - a;
  return dfo::two_sum(y, -__fdividef(r.h, __fmul_rn(3.f, y2.h)));
}

// exp(r) - 1 for |r| <= ln2/64: r + r^2/2 + r^3/6 in pairs, r^4/24 + r^5/120 + r^6/720 in
// FP32 (the r^7 term, below 2^-52 relative, is left out)
__device__ __forceinline__ DF df_expm1_small(DF r) {
  const DF r2 = r * r;
  const DF r3s = r2 * r * DF(1.0 / 6.0);
  const float t = __fmul_rn(__fmul_rn(r2.h, r2.h), fmaf(r.h, fmaf(r.h, 1.f / 720.f, 1.f / 120.f), 1.f / 24.f));
  return (r + DF(__fmul_rn(0.5f, r2.h), __fmul_rn(0.5f, r2.l))) + (r3s + DF(t, 0.f));
}

// exp(a) = 2^m 2^(j/32) exp(r), a = (32 m + j) ln2/32 + r, ln2/32 in three parts (the first
// of 9 bits, so k ln2/32 is exact for |k| < 2^15)
__device__ __forceinline__ DF df_exp(DF a) {
  if (a.h < -87.f) return DF(0.f, 0.f);  // below the FP32 normal range
  const float x = fminf(a.h, 88.f);
  const float kf = rintf(__fmul_rn(x, 46.16624f));  // 32 / ln2
  const int k = (int)kf;
  const int j = k & 31, m = k >> 5;
  const float r1 = fmaf(-kf, 0x1.63p-6f, x);  // exact
  const DF p = dfo::two_prod(kf, -0x1.bd0106p-18f);
  const DF rh = dfo::two_sum(r1, -p.h);
  const float rl = __fadd_rn(fmaf(-kf, 0x1.cf79acp-45f, __fsub_rn(rh.l, p.l)), a.l);
  const DF q = df_expm1_small(dfo::fast_two_sum(rh.h, rl));
  const float2 T2 = __ldg(kExp2Tab + j);
  const DF T(T2.x, T2.y);
  const DF v = T + T * q;
  const float sc = __int_as_float((m + 127) << 23);  // 2^m, m in [-126, 127]
  return DF(__fmul_rn(v.h, sc), __fmul_rn(v.l, sc));
}

// exp(a) - 1 without the cancellation of exp(a) - 1 near a = 0
__device__ __forceinline__ DF df_expm1(DF a) {
  if (fabsf(a.h) <= 0.0108f) return df_expm1_small(a);
  return df_exp(a) - DF(1.f, 0.f);
}

// log(a), a > 0: y0 = log(a_hi) in FP32, t = a e^-y0 - 1 (|t| ~ 2^-21), log(a) = y0 +
// log(1 + t) = y0 + t - t^2/2 + t^3/3
__device__ __forceinline__ DF df_log(DF a) {
  const float y0 = __logf(a.h);
  const DF t = a * df_exp(DF(-y0, 0.f)) - DF(1.f, 0.f);
  const float c = __fmul_rn(__fmul_rn(t.h, t.h), fmaf(t.h, 1.f / 3.f, -0.5f));
  return (DF(y0, 0.f) + t) + DF(c, 0.f);
}

}  // namespace xcgpu
