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

// Same as shell_functions, with the transform coefficients as compile-time constants.
// Emit(f, value, value_lo, dx, dy, dz): value_lo carries the rounding of the coefficients
// to R (c - R(c) times the term), which is the same relative error of a function at
// every point (sqrt(3) of the d functions, for one) and would otherwise bias it.
template <class R, int L, int DERIV, class Emit>
__device__ __forceinline__ void shell_functions_cx(R x, R y, R z, R Rv, R dR, bool pure, Emit&& emit) {
  constexpr int NS = 2 * L + 1;
  constexpr cx::Table TS = cx::solid(L);
  constexpr cx::Table TC = cx::cartesian(L);
  R px[L + 2], py[L + 2], pz[L + 2];
  px[0] = py[0] = pz[0] = R(1);
#pragma unroll
  for (int k = 1; k < L + 2; ++k) {
    px[k] = px[k - 1] * x;
    py[k] = py[k - 1] * y;
    pz[k] = pz[k - 1] * z;
  }
  R sv[NS], svl[NS], sg[3 * NS];
#pragma unroll
  for (int m = 0; m < NS; ++m) {
    sv[m] = svl[m] = R(0);
    sg[3 * m] = sg[3 * m + 1] = sg[3 * m + 2] = R(0);
  }
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; --a) {
#pragma unroll
    for (int b = L - a; b >= 0; --b, ++k) {
      const int c = L - a - b;
      const R mono = px[a] * py[b] * pz[c];
      const R v = mono * Rv;
      R g0 = R(0), g1 = R(0), g2 = R(0);
      if (DERIV >= 1) {
        const R dmx = a > 0 ? R(a) * px[a > 0 ? a - 1 : 0] * py[b] * pz[c] : R(0);
        const R dmy = b > 0 ? R(b) * px[a] * py[b > 0 ? b - 1 : 0] * pz[c] : R(0);
        const R dmz = c > 0 ? R(c) * px[a] * py[b] * pz[c > 0 ? c - 1 : 0] : R(0);
        const R md = mono * dR;
        g0 = dmx * Rv + md * x;
        g1 = dmy * Rv + md * y;
        g2 = dmz * Rv + md * z;
      }
      if (pure) {
#pragma unroll
        for (int m = 0; m < NS; ++m) {
          const R t = R(TS.c[m][k]);
          const R tl = R(TS.c[m][k] - (double)R(TS.c[m][k]));
          if (TS.c[m][k] != 0.0) {
            sv[m] += t * v;
            if (tl != R(0)) svl[m] = fmaf(tl, v, svl[m]);
            if (DERIV >= 1) {
              sg[3 * m] += t * g0;
              sg[3 * m + 1] += t * g1;
              sg[3 * m + 2] += t * g2;
            }
          }
        }
      } else {
        const R t = R(TC.c[0][k]);
        const R tl = R(TC.c[0][k] - (double)R(TC.c[0][k]));
        emit(k, t * v, tl * v, t * g0, t * g1, t * g2);
      }
    }
  }
  if (pure) {
#pragma unroll
    for (int m = 0; m < NS; ++m) emit(m, sv[m], svl[m], sg[3 * m], sg[3 * m + 1], sg[3 * m + 2]);
  }
}

template <class R, int DERIV, class Emit>
__device__ __forceinline__ void shell_functions_cx_l(int l, R x, R y, R z, R Rv, R dR, bool pure, Emit&& emit) {
  switch (l) {
    case 0: shell_functions_cx<R, 0, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 1: shell_functions_cx<R, 1, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 2: shell_functions_cx<R, 2, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 3: shell_functions_cx<R, 3, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 4: shell_functions_cx<R, 4, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 5: shell_functions_cx<R, 5, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    case 6: shell_functions_cx<R, 6, DERIV>(x, y, z, Rv, dR, pure, emit); break;
    default: break;
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
