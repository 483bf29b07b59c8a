// Contracted Gaussian shells on a grid point: radial part, Cartesian monomials and
// the transform to real solid harmonics, with gradients (and Hessians).
//
// Follows BasisFunctionOnGridController.cpp:259-1097: per point and shell the
// radial sum R = sum_i c_i exp(-a_i r^2) skips primitives with a_i r^2 beyond
// -ln(threshold) (:298-307); if |R| < threshold every function of the shell is
// zero at this point (:312-329); Cartesian functions run (l,0,0) ... (0,0,l)
// (:359-362); spherical ones are real solid harmonics m = -l..l (:455-1062);
// gradients use R' = -2 sum a c exp(.) (:1068-1080).
#pragma once
#include <cuda_runtime.h>

namespace xcgpu {

__host__ __device__ __forceinline__ int ncart_d(int l) { return (l + 1) * (l + 2) / 2; }

// ---- compile-time real solid harmonic coefficients -----------------------------------
// Same closed form as the host tables (Helgaker, Joergensen & Olsen, sec. 6.4):
// S_lm = N_lm sum_{t,u,v} C_tuv x^(2t+|m|-2(u+v)) y^(2(u+v)) z^(l-2t-|m|), m = -l..l,
// evaluated by constexpr code so the device kernels multiply by literal constants.
namespace cx {
constexpr double fact(int n) { return n <= 1 ? 1.0 : n * fact(n - 1); }
constexpr double binom(int n, int k) { return (k < 0 || k > n) ? 0.0 : fact(n) / (fact(k) * fact(n - k)); }
constexpr double sqrt_newton(double x, double g, int it) { return it == 0 ? g : sqrt_newton(x, 0.5 * (g + x / g), it - 1); }
constexpr double sqrt(double x) { return x <= 0 ? 0.0 : sqrt_newton(x, x > 1 ? x : 1.0, 60); }
constexpr double pow2(int n) { return n == 0 ? 1.0 : 2.0 * pow2(n - 1); }
constexpr double pow025(int n) { return n == 0 ? 1.0 : 0.25 * pow025(n - 1); }
struct Table {
  double c[13][28];
};
constexpr int cart_index(int l, int a, int b) {
  int k = 0;
  for (int aa = l; aa > a; --aa) k += l - aa + 1;
  return k + (l - a - b);
}
constexpr Table solid(int l) {
  Table T{};
  for (int m = -l; m <= l; ++m) {
    const int am = m < 0 ? -m : m;
    const int tv0 = m < 0 ? 1 : 0;
    const double N = sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0)) / (pow2(am) * fact(l));
    for (int t = 0; t <= (l - am) / 2; ++t)
      for (int u = 0; u <= t; ++u)
        for (int tv = tv0; tv <= am; tv += 2) {
          const int se = t + (tv - tv0) / 2;
          const double C = (se % 2 ? -1.0 : 1.0) * pow025(t) * binom(l, t) * binom(l - t, am + t) * binom(t, u) *
                           binom(am, tv);
          const int py = 2 * u + tv, px = 2 * t + am - py;
          T.c[m + l][cart_index(l, px, py)] += N * C;
        }
  }
  return T;
}
constexpr double dfact(int n) { return n <= 1 ? 1.0 : n * dfact(n - 2); }
// per solid harmonic m of a table, the first monomial k with a nonzero coefficient
struct FirstTerms {
  int k[13];
};
constexpr FirstTerms first_terms(const Table& T, int ns, int nc) {
  FirstTerms f{};
  for (int m = 0; m < 13; ++m) f.k[m] = -1;
  for (int m = 0; m < ns; ++m)
    for (int k = 0; k < nc; ++k)
      if (T.c[m][k] != 0.0 && f.k[m] < 0) f.k[m] = k;
  return f;
}
constexpr Table cartesian(int l) {
  Table T{};
  int k = 0;
  for (int a = l; a >= 0; --a)
    for (int b = l - a; b >= 0; --b, ++k)
      T.c[0][k] = sqrt(dfact(2 * l - 1) / (dfact(2 * a - 1) * dfact(2 * b - 1) * dfact(2 * (l - a - b) - 1)));
  return T;
}
}  // namespace cx

template <class R> __device__ __forceinline__ R dexp(R x);
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
// FP32 exponential of the mixed-precision basis: the accurate expf by default;
// XCGPU_FAST_EXP selects the approximate __expf.
#ifdef XCGPU_FAST_EXP
template <> __device__ __forceinline__ float dexp<float>(float x) { return __expf(x); }
#else
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
#endif

// radial part of shell s at squared distance r2; returns false if negligible
template <class R, int DERIV>
__device__ __forceinline__ bool shell_radial(const double* __restrict__ alpha, const double* __restrict__ coef, int np,
                                             R r2, R expthr, R thr, R& Rv, R& dR, R& ddR) {
  Rv = R(0);
  dR = R(0);
  ddR = R(0);
  for (int i = 0; i < np; ++i) {
    const R a = (R)__ldg(alpha + i);
    const R t = a * r2;
    if (t < expthr) {
      const R e = (R)__ldg(coef + i) * dexp<R>(-t);
      Rv += e;
      if (DERIV >= 1) dR -= R(2) * a * e;
      if (DERIV >= 2) ddR += R(4) * a * a * e;
    }
  }
  return fabs(Rv) >= thr;
}

// Emit(f, value, gx, gy, gz, h) for the nfunc functions of an l = L shell.
// T: solid-harmonic matrix (2L+1) x ncart(L) (pure) ; cn: Cartesian factors (ncart(L)).
template <class R, int L, int DERIV, class Emit>
__device__ __forceinline__ void shell_functions(R x, R y, R z, R Rv, R dR, R ddR, bool pure,
                                                const double* __restrict__ T, const double* __restrict__ cn,
                                                Emit&& emit) {
  constexpr int NC = (L + 1) * (L + 2) / 2;
  constexpr int NS = 2 * L + 1;
  R px[L + 3], py[L + 3], pz[L + 3];
  px[0] = py[0] = pz[0] = R(1);
#pragma unroll
  for (int k = 1; k < L + 3; ++k) {
    px[k] = px[k - 1] * x;
    py[k] = py[k - 1] * y;
    pz[k] = pz[k - 1] * z;
  }
  R sv[NS], sg[DERIV >= 1 ? 3 * NS : 1], sh[DERIV >= 2 ? 6 * NS : 1];
  if (pure) {
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      sv[m] = R(0);
      if (DERIV >= 1) sg[3 * m] = sg[3 * m + 1] = sg[3 * m + 2] = R(0);
      if (DERIV >= 2)
#pragma unroll
        for (int h = 0; h < 6; ++h) sh[6 * m + h] = R(0);
    }
  }
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; --a) {
#pragma unroll
    for (int b = L - a; b >= 0; --b, ++k) {
      const int c = L - a - b;
      const R mono = px[a] * py[b] * pz[c];
      const R v = mono * Rv;
      R g[3] = {R(0), R(0), R(0)};
      R hh[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
      if (DERIV >= 1) {
        const R dmx = a > 0 ? R(a) * px[a > 0 ? a - 1 : 0] * py[b] * pz[c] : R(0);
        const R dmy = b > 0 ? R(b) * px[a] * py[b > 0 ? b - 1 : 0] * pz[c] : R(0);
        const R dmz = c > 0 ? R(c) * px[a] * py[b] * pz[c > 0 ? c - 1 : 0] : R(0);
        g[0] = dmx * Rv + mono * dR * x;
        g[1] = dmy * Rv + mono * dR * y;
        g[2] = dmz * Rv + mono * dR * z;
        if (DERIV >= 2) {
          const R r[3] = {x, y, z};
          const R dm[3] = {dmx, dmy, dmz};
          const int e[3] = {a, b, c};
          const int hi[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            const int i = hi[q][0], j = hi[q][1];
            int f[3] = {e[0], e[1], e[2]};
            R coefm = R(f[i]);
            f[i] -= 1;
            coefm *= R(f[j]);
            f[j] -= 1;
            R d2 = R(0);
            if (f[0] >= 0 && f[1] >= 0 && f[2] >= 0 && coefm != R(0)) d2 = coefm * px[f[0]] * py[f[1]] * pz[f[2]];
            hh[q] = d2 * Rv + dm[i] * dR * r[j] + dm[j] * dR * r[i] + mono * (ddR * r[i] * r[j] + (i == j ? dR : R(0)));
          }
        }
      }
      if (pure) {
#pragma unroll
        for (int m = 0; m < NS; ++m) {
          const R t = (R)__ldg(T + m * NC + k);
          sv[m] += t * v;
          if (DERIV >= 1) {
            sg[3 * m] += t * g[0];
            sg[3 * m + 1] += t * g[1];
            sg[3 * m + 2] += t * g[2];
          }
          if (DERIV >= 2)
#pragma unroll
            for (int q = 0; q < 6; ++q) sh[6 * m + q] += t * hh[q];
        }
      } else {
        const R t = (R)__ldg(cn + k);
        R ht[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) ht[q] = t * hh[q];
        emit(k, t * v, t * g[0], t * g[1], t * g[2], ht);
      }
    }
  }
  if (pure) {
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      R ht[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) ht[q] = DERIV >= 2 ? sh[6 * m + q] : R(0);
      emit(m, sv[m], DERIV >= 1 ? sg[3 * m] : R(0), DERIV >= 1 ? sg[3 * m + 1] : R(0),
           DERIV >= 1 ? sg[3 * m + 2] : R(0), ht);
    }
  }
}

// FP32 pairs (h + l, |l| about an ulp of h) and their error-free transformations:
// products by FMA, sums by Knuth's two-sum (Ogita, Rump & Oishi, SIAM J. Sci. Comput.
// 26 (2005) 1955), with explicit roundings so no contraction changes them.
struct F2 {
  float h, l;
};
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float h = __fmul_rn(a.h, b.h);
  return {h, fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -h)))};
}
__device__ __forceinline__ F2 f2_mul1(F2 a, float b) {  // pair times an FP32 number
  const float h = __fmul_rn(a.h, b);
  return {h, fmaf(a.l, b, fmaf(a.h, b, -h))};
}
__device__ __forceinline__ void f2_acc(F2& s, F2 p) {  // s += p
  const float t = __fadd_rn(s.h, p.h), bp = __fsub_rn(t, s.h);
  const float e = __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bp)), __fsub_rn(p.h, bp));
  s.l = __fadd_rn(s.l, __fadd_rn(e, p.l));
  s.h = t;
}

// Values and gradients of an l = L shell with the transform coefficients as
// compile-time constants, the value carried as an FP32 pair.
// Emit(f, value, value_lo, dx, dy, dz).  The point-centre offset comes as pairs (x + xl,
// ...), and the monomials, the coefficients (with their FP32 rounding) and the
// solid-harmonic sums are pair products and two-sums, so value + value_lo is the FP32
// radial value Rv times the exact angular factor to about 2^-44: every FP32 rounding of
// the angular part would otherwise be one relative error repeated wherever the same
// offset recurs (on a radial shell of the function's own atom, at every atom of an
// element), a bias rather than noise.
// The gradients are FP32 numbers formed as d_i phi = R A_i + R' x_i S, with A_i the
// FP32 sum of the coefficients times d_i of the monomials and S the angular sum above
// (the value before R): R = Rv + Rl and R' = dR + dRl enter with their low parts, as on
// a radial shell of the function's own atom they are one number each, and their FP32
// roundings would be the same relative error of the gradient at every point of the
// shell; what is left rounds differently from point to point.
template <int L, int DERIV, class Emit>
__device__ __forceinline__ void shell_functions_px(F2 x, F2 y, F2 z, float Rv, float Rl, float dR, float dRl,
                                                   bool pure, Emit&& emit) {
  constexpr int NS = 2 * L + 1;
  constexpr cx::Table TS = cx::solid(L);
  constexpr cx::Table TC = cx::cartesian(L);
  constexpr cx::FirstTerms FK = cx::first_terms(TS, NS, (L + 1) * (L + 2) / 2);
  F2 px[L + 1], py[L + 1], pz[L + 1];
  px[0] = py[0] = pz[0] = F2{1.f, 0.f};
#pragma unroll
  for (int k = 1; k <= L; ++k) {
    px[k] = f2_mul(px[k - 1], x);
    py[k] = f2_mul(py[k - 1], y);
    pz[k] = f2_mul(pz[k - 1], z);
  }
  F2 sv[NS];
  float sg[3 * NS];
#pragma unroll
  for (int m = 0; m < NS; ++m) {
    sv[m] = F2{0.f, 0.f};
    sg[3 * m] = sg[3 * m + 1] = sg[3 * m + 2] = 0.f;
  }
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; --a) {
#pragma unroll
    for (int b = L - a; b >= 0; --b, ++k) {
      const int c = L - a - b;
      F2 mono = px[a];
      if (b > 0) mono = a > 0 ? f2_mul(mono, py[b]) : py[b];
      if (c > 0) mono = (a > 0 || b > 0) ? f2_mul(mono, pz[c]) : pz[c];
      // d_i of the monomial (FP32)
      float g0 = 0.f, g1 = 0.f, g2 = 0.f;
      if (DERIV >= 1) {
        g0 = a > 0 ? float(a) * px[a > 0 ? a - 1 : 0].h * py[b].h * pz[c].h : 0.f;
        g1 = b > 0 ? float(b) * px[a].h * py[b > 0 ? b - 1 : 0].h * pz[c].h : 0.f;
        g2 = c > 0 ? float(c) * px[a].h * py[b].h * pz[c > 0 ? c - 1 : 0].h : 0.f;
      }
      // (the coefficient tests below are on compile-time tables and fold away: a unit
      // coefficient multiplies nothing, a function's first term starts its sum)
      if (pure) {
#pragma unroll
        for (int m = 0; m < NS; ++m) {
          if (TS.c[m][k] != 0.0) {
            const float t = float(TS.c[m][k]);
            const float tl = float(TS.c[m][k] - (double)float(TS.c[m][k]));
            F2 p = mono;
            if (t != 1.f || tl != 0.f) {
              p = f2_mul1(mono, t);
              if (tl != 0.f) p.l = fmaf(tl, mono.h, p.l);
            }
            if (k == FK.k[m]) {
              sv[m] = p;
              if (DERIV >= 1) {
                sg[3 * m] = t == 1.f ? g0 : t * g0;
                sg[3 * m + 1] = t == 1.f ? g1 : t * g1;
                sg[3 * m + 2] = t == 1.f ? g2 : t * g2;
              }
            } else {
              f2_acc(sv[m], p);
              if (DERIV >= 1) {
                sg[3 * m] += t * g0;
                sg[3 * m + 1] += t * g1;
                sg[3 * m + 2] += t * g2;
              }
            }
          }
        }
      } else {
        const float t = float(TC.c[0][k]);
        const float tl = float(TC.c[0][k] - (double)float(TC.c[0][k]));
        F2 p = mono;
        if (t != 1.f || tl != 0.f) {
          p = f2_mul1(mono, t);
          if (tl != 0.f) p.l = fmaf(tl, mono.h, p.l);
        }
        const F2 v = f2_mul1(p, Rv);
        if (DERIV >= 1) {
          const float u = dR * p.h, ul = dRl * p.h;
          const float a0 = t == 1.f ? g0 : t * g0, a1 = t == 1.f ? g1 : t * g1, a2 = t == 1.f ? g2 : t * g2;
          emit(k, v.h, v.l, fmaf(Rv, a0, fmaf(u, x.h, fmaf(Rl, a0, ul * x.h))),
               fmaf(Rv, a1, fmaf(u, y.h, fmaf(Rl, a1, ul * y.h))), fmaf(Rv, a2, fmaf(u, z.h, fmaf(Rl, a2, ul * z.h))));
        } else {
          emit(k, v.h, v.l, 0.f, 0.f, 0.f);
        }
      }
    }
  }
  if (pure) {
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      const F2 v = f2_mul1(sv[m], Rv);
      if (DERIV >= 1) {
        const float u = dR * sv[m].h, ul = dRl * sv[m].h;
        const float* A = sg + 3 * m;
        emit(m, v.h, v.l, fmaf(Rv, A[0], fmaf(u, x.h, fmaf(Rl, A[0], ul * x.h))),
             fmaf(Rv, A[1], fmaf(u, y.h, fmaf(Rl, A[1], ul * y.h))),
             fmaf(Rv, A[2], fmaf(u, z.h, fmaf(Rl, A[2], ul * z.h))));
      } else {
        emit(m, v.h, v.l, 0.f, 0.f, 0.f);
      }
    }
  }
}

// dispatch on l <= MAXL at run time (the callers select MAXL from the basis)
template <int DERIV, int MAXL, class Emit>
__device__ __forceinline__ void shell_functions_px_l(int l, F2 x, F2 y, F2 z, float Rv, float Rl, float dR, float dRl,
                                                     bool pure, Emit&& emit) {
  switch (l) {
    case 0: shell_functions_px<0, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
    case 1: shell_functions_px<1, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
    case 2: shell_functions_px<2, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
    case 3: shell_functions_px<3, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
    default:
      if constexpr (MAXL >= 4) {
        switch (l) {
          case 4: shell_functions_px<4, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
          case 5: shell_functions_px<5, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
          case 6: shell_functions_px<6, DERIV>(x, y, z, Rv, Rl, dR, dRl, pure, emit); break;
          default: break;
        }
      }
      break;
  }
}

// dispatch on l at run time
template <class R, int DERIV, class Emit>
__device__ __forceinline__ void shell_functions_l(int l, R x, R y, R z, R Rv, R dR, R ddR, bool pure,
                                                  const double* T, const double* cn, Emit&& emit) {
  switch (l) {
    case 0: shell_functions<R, 0, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 1: shell_functions<R, 1, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 2: shell_functions<R, 2, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 3: shell_functions<R, 3, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 4: shell_functions<R, 4, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 5: shell_functions<R, 5, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    case 6: shell_functions<R, 6, DERIV>(x, y, z, Rv, dR, ddR, pure, T, cn, emit); break;
    default: break;
  }
}

}  // namespace xcgpu
