// FP32 exponential without a mean error, for the FP32 basis-function evaluation.
#pragma once
#include <cuda_runtime.h>

namespace xcgpu {

// exp(x) for x <= 0 with a mean error of zero: table-driven, after P. T. P. Tang, "Table-
// driven implementation of the exponential function in IEEE floating-point arithmetic",
// ACM TOMS 15 (1989) 144-157.  x = (32 m + j) ln2/32 + r with |r| <= ln2/64 (ln2/32 in
// three parts: the first, 9 bits, makes k ln2/32 exact for |k| < 2^15), exp(x) =
// 2^m 2^(j/32) exp(r), 2^(j/32) as an FP32 pair (kExp2Tab), exp(r) - 1 - r by its Taylor
// terms to r^4 (the rest is below 2^-40).  Before the final rounding the value carries
// ~30 bits, so the result is the correctly rounded exp except next to rounding
// boundaries and its errors average to zero.  (The library expf averages 0.07-0.15 ulp
// high, which raises every basis function by ~1e-8 and the density by twice that.)
__device__ const float2 kExp2Tab[32] = {
    {0x1.0000000000000p+0f, 0x0p+0f}, {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f}, {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f}, {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f}, {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f}, {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f}, {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f}, {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f}, {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f}, {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f}, {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f}, {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f}, {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f}, {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f}, {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f}, {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f}, {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f}};

__device__ __forceinline__ float exp_tang(float x) {
  x = fmaxf(x, -104.f);  // exp(-104) is below the FP32 range: the result is 0
  const float kf = rintf(__fmul_rn(x, 46.16624f));  // 32 / ln2
  const int k = (int)kf;
  const int j = k & 31, m = k >> 5;  // floor division
  float r = fmaf(-kf, 0x1.63p-6f, x);  // exact
  r = fmaf(-kf, -0x1.bd0106p-18f, r);
  r = fmaf(-kf, 0x1.cf79acp-45f, r);
  const float q = __fmul_rn(__fmul_rn(r, r), fmaf(r, fmaf(r, 1.f / 24.f, 1.f / 6.f), 0.5f));
  const float u = __fadd_rn(r, q);
  const float2 T = __ldg(kExp2Tab + j);
  const float v = __fadd_rn(T.x, fmaf(T.x, u, T.y));
  return m < -125 ? 0.f : __fmul_rn(v, __int_as_float((m + 127) << 23));
}

// the same value as an FP32 pair, exp(x) = hi + lo to ~2^-36: hi is the rounded value,
// lo the remainder (|lo| <= ulp(hi) / 2); for sums that must not inherit the rounding of
// each exp.  The reduced argument is kept as a pair (kf ln2/32 by an exact product and
// a two-sum), T_hi r as an exact product, and the pieces are added largest first.
__device__ __forceinline__ void exp_tang2(float x, float& hi, float& lo) {
  x = fmaxf(x, -104.f);
  const float kf = rintf(__fmul_rn(x, 46.16624f));
  const int k = (int)kf;
  const int j = k & 31, m = k >> 5;
  const float r1 = fmaf(-kf, 0x1.63p-6f, x);  // exact
  const float p = __fmul_rn(kf, -0x1.bd0106p-18f), pe = fmaf(kf, -0x1.bd0106p-18f, -p);
  const float rh = __fsub_rn(r1, p);  // two-sum r1 - p
  const float bp = __fsub_rn(rh, r1);
  const float re = __fadd_rn(__fsub_rn(r1, __fsub_rn(rh, bp)), __fsub_rn(-p, bp));
  const float rl = fmaf(-kf, 0x1.cf79acp-45f, __fsub_rn(re, pe));  // r = rh + rl
  const float q = __fmul_rn(__fmul_rn(rh, rh), fmaf(rh, fmaf(rh, 1.f / 24.f, 1.f / 6.f), 0.5f));
  const float2 T = __ldg(kExp2Tab + j);
  // T (1 + r + q) = T.x + T.x rh + [T.x (rl + q) + T.y (1 + rh + q)]
  const float ph = __fmul_rn(T.x, rh), phe = fmaf(T.x, rh, -ph);
  const float small = fmaf(T.x, __fadd_rn(rl, q), fmaf(T.y, __fadd_rn(rh, q), T.y));
  const float h = __fadd_rn(T.x, ph);
  const float l = __fadd_rn(__fsub_rn(ph, __fsub_rn(h, T.x)), __fadd_rn(phe, small));
  const float h2 = __fadd_rn(h, l);
  const float l2 = __fsub_rn(l, __fsub_rn(h2, h));
  const float sc = m < -125 ? 0.f : __int_as_float((m + 127) << 23);
  hi = __fmul_rn(h2, sc);
  lo = __fmul_rn(l2, sc);
}

}  // namespace xcgpu
