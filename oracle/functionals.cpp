/*
 * ORACLE -- test infrastructure only (see oracle.h).
 *
 * Exchange-correlation energy densities written from the literature and
 * differentiated by forward-mode automatic differentiation (dual numbers), the
 * same strategy xcfun uses (Taylor arithmetic; the reference evaluates through
 * xcfun by default, XCFun.cpp:129-153, CMakeLists.txt:38).  The GPU product
 * uses hand-derived analytic derivatives instead, so the two are independent.
 *
 *   Slater exchange        Dirac (1930), spin-scaled
 *   VWN5 correlation       Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980), fit "V"
 *   PW92 correlation       Perdew, Wang, PRB 45, 13244 (1992), original digits
 *                          (A = 0.031091, 0.015545, 0.016887; f''(0) = 1.709921)
 *   PBE exchange/corr.     Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)
 *   B88 exchange           Becke, PRA 38, 3098 (1988)
 *   LYP correlation        Lee, Yang, Parr, PRB 37, 785 (1988), Miehlich et al. form
 *                          (CPL 157, 200 (1989))
 *   PZ81 correlation       Perdew, Zunger, PRB 23, 5048 (1981), their parametrisation of
 *                          the Ceperley-Alder correlation energy (Table XII / eqs. C1, C3)
 *   P86 correlation        Perdew, PRB 33, 8822 (1986), erratum PRB 34, 7406 (1986):
 *                          PZ81 plus the gradient correction of eqs. (6), (8), (9)
 *                          (the reference's BP86 = X_B88 + C_P86, CompositeFunctionals.cpp:244)
 *
 * Density cut-offs: a point whose total density is below 1e-14 contributes
 * nothing (the reference sets libxc's dens_threshold to 1e-14, LibXC.cpp:86-97);
 * a spin channel below 0.5e-14 contributes no exchange; |zeta| is capped at
 * 1 - 1e-12 in the correlation functionals.
 */
#include <cmath>

#include "oracle_internal.h"

namespace orc {

template <int N>
struct D {
  double v;
  double d[N];
  D(double x = 0.0) : v(x) {
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  static D var(double x, int i) {
    D r(x);
    r.d[i] = 1.0;
    return r;
  }
};
template <int N>
D<N> chain(const D<N>& a, double f, double df) {
  D<N> r(f);
  for (int i = 0; i < N; ++i) r.d[i] = df * a.d[i];
  return r;
}
template <int N>
D<N> operator+(const D<N>& a, const D<N>& b) {
  D<N> r(a.v + b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
D<N> operator-(const D<N>& a, const D<N>& b) {
  D<N> r(a.v - b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
D<N> operator-(const D<N>& a) {
  return chain(a, -a.v, -1.0);
}
template <int N>
D<N> operator*(const D<N>& a, const D<N>& b) {
  D<N> r(a.v * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
D<N> operator/(const D<N>& a, const D<N>& b) {
  D<N> r(a.v / b.v);
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
  return r;
}
template <int N> D<N> operator+(const D<N>& a, double b) { return a + D<N>(b); }
template <int N> D<N> operator+(double a, const D<N>& b) { return D<N>(a) + b; }
template <int N> D<N> operator-(const D<N>& a, double b) { return a - D<N>(b); }
template <int N> D<N> operator-(double a, const D<N>& b) { return D<N>(a) - b; }
template <int N> D<N> operator*(const D<N>& a, double b) { return chain(a, a.v * b, b); }
template <int N> D<N> operator*(double a, const D<N>& b) { return chain(b, a * b.v, a); }
template <int N> D<N> operator/(const D<N>& a, double b) { return chain(a, a.v / b, 1.0 / b); }
template <int N> D<N> operator/(double a, const D<N>& b) { return D<N>(a) / b; }

template <int N> D<N> sqrt(const D<N>& a) { const double s = std::sqrt(a.v); return chain(a, s, 0.5 / s); }
template <int N> D<N> cbrt(const D<N>& a) { const double s = std::cbrt(a.v); return chain(a, s, s / (3.0 * a.v)); }
template <int N> D<N> pow(const D<N>& a, double p) { return chain(a, std::pow(a.v, p), p * std::pow(a.v, p - 1.0)); }
template <int N> D<N> exp(const D<N>& a) { const double e = std::exp(a.v); return chain(a, e, e); }
template <int N> D<N> log(const D<N>& a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template <int N> D<N> atan(const D<N>& a) { return chain(a, std::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
// x*asinh(x) as a function of u = x^2 (smooth at u = 0, where the derivative is 1)
template <int N> D<N> xasinhx_of_sq(const D<N>& u) {
  const double x = std::sqrt(u.v);
  const double f = x * std::asinh(x);
  double df;
  if (u.v < 1e-8) df = 1.0 - u.v / 3.0;
  else df = 0.5 * (std::asinh(x) / x + 1.0 / std::sqrt(1.0 + u.v));
  return chain(u, f, df);
}
template <int N> double val(const D<N>& a) { return a.v; }

// Second-order forward-mode numbers (value, gradient, Hessian over N variables), for
// the second functional derivatives of the linear-response kernel.
template <int N>
struct H {
  double v;
  double d[N];
  double h[N][N];
  H(double x = 0.0) : v(x) {
    for (int i = 0; i < N; ++i) {
      d[i] = 0.0;
      for (int j = 0; j < N; ++j) h[i][j] = 0.0;
    }
  }
  static H var(double x, int i) {
    H r(x);
    r.d[i] = 1.0;
    return r;
  }
};
template <int N>
H<N> chain2(const H<N>& a, double f, double df, double ddf) {
  H<N> r(f);
  for (int i = 0; i < N; ++i) {
    r.d[i] = df * a.d[i];
    for (int j = 0; j < N; ++j) r.h[i][j] = df * a.h[i][j] + ddf * a.d[i] * a.d[j];
  }
  return r;
}
template <int N>
H<N> operator+(const H<N>& a, const H<N>& b) {
  H<N> r(a.v + b.v);
  for (int i = 0; i < N; ++i) {
    r.d[i] = a.d[i] + b.d[i];
    for (int j = 0; j < N; ++j) r.h[i][j] = a.h[i][j] + b.h[i][j];
  }
  return r;
}
template <int N> H<N> operator-(const H<N>& a) { return chain2(a, -a.v, -1.0, 0.0); }
template <int N> H<N> operator-(const H<N>& a, const H<N>& b) { return a + (-b); }
template <int N>
H<N> operator*(const H<N>& a, const H<N>& b) {
  H<N> r(a.v * b.v);
  for (int i = 0; i < N; ++i) {
    r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    for (int j = 0; j < N; ++j)
      r.h[i][j] = a.h[i][j] * b.v + a.d[i] * b.d[j] + a.d[j] * b.d[i] + a.v * b.h[i][j];
  }
  return r;
}
template <int N> H<N> inv(const H<N>& b) {
  const double q = 1.0 / b.v;
  return chain2(b, q, -q * q, 2.0 * q * q * q);
}
template <int N> H<N> operator/(const H<N>& a, const H<N>& b) { return a * inv(b); }
template <int N> H<N> operator+(const H<N>& a, double b) { return a + H<N>(b); }
template <int N> H<N> operator+(double a, const H<N>& b) { return H<N>(a) + b; }
template <int N> H<N> operator-(const H<N>& a, double b) { return a - H<N>(b); }
template <int N> H<N> operator-(double a, const H<N>& b) { return H<N>(a) - b; }
template <int N> H<N> operator*(const H<N>& a, double b) { return chain2(a, a.v * b, b, 0.0); }
template <int N> H<N> operator*(double a, const H<N>& b) { return chain2(b, a * b.v, a, 0.0); }
template <int N> H<N> operator/(const H<N>& a, double b) { return chain2(a, a.v / b, 1.0 / b, 0.0); }
template <int N> H<N> operator/(double a, const H<N>& b) { return a * inv(b); }
template <int N> H<N> sqrt(const H<N>& a) {
  const double s = std::sqrt(a.v);
  return chain2(a, s, 0.5 / s, -0.25 / (s * s * s));
}
template <int N> H<N> cbrt(const H<N>& a) {
  const double s = std::cbrt(a.v);
  return chain2(a, s, s / (3.0 * a.v), -2.0 * s / (9.0 * a.v * a.v));
}
template <int N> H<N> pow(const H<N>& a, double p) {
  return chain2(a, std::pow(a.v, p), p * std::pow(a.v, p - 1.0), p * (p - 1.0) * std::pow(a.v, p - 2.0));
}
template <int N> H<N> exp(const H<N>& a) {
  const double e = std::exp(a.v);
  return chain2(a, e, e, e);
}
template <int N> H<N> log(const H<N>& a) { return chain2(a, std::log(a.v), 1.0 / a.v, -1.0 / (a.v * a.v)); }
template <int N> H<N> atan(const H<N>& a) {
  const double q = 1.0 / (1.0 + a.v * a.v);
  return chain2(a, std::atan(a.v), q, -2.0 * a.v * q * q);
}
// x asinh(x) of u = x^2: f'(u) = (asinh x / x + 1/sqrt(1+u)) / 2,
// f''(u) = (1 / (2u sqrt(1+u)) - asinh x / (2 u x) - (1+u)^(-3/2) / 2) / 2; series below 1e-4
template <int N> H<N> xasinhx_of_sq(const H<N>& u) {
  const double x = std::sqrt(u.v);
  const double f = x * std::asinh(x);
  double df, ddf;
  if (u.v < 1e-4) {
    df = 1.0 - u.v / 3.0 + 9.0 * u.v * u.v / 40.0;
    ddf = -1.0 / 3.0 + 9.0 * u.v / 20.0;
  } else {
    const double sq = std::sqrt(1.0 + u.v);
    df = 0.5 * (std::asinh(x) / x + 1.0 / sq);
    ddf = 0.5 * (1.0 / (2.0 * u.v * sq) - std::asinh(x) / (2.0 * u.v * x) - 0.5 / (sq * sq * sq));
  }
  return chain2(u, f, df, ddf);
}

static const double kDensTiny = 1e-14;
static const double kZetaMax = 1.0 - 1e-12;

template <class T> T clamp_zeta(const T& z) {
  if (z.v > kZetaMax) return T(kZetaMax);
  if (z.v < -kZetaMax) return T(-kZetaMax);
  return z;
}
template <class T> T pow43(const T& x) { return x * cbrt(x); }

/* ---- LDA exchange ---- */
template <class T> T slater(const T& na, const T& nb) {
  const double C = 0.75 * std::cbrt(6.0 / M_PI);
  T e(0.0);
  if (na.v > 0.5 * kDensTiny) e = e - C * pow43(na);
  if (nb.v > 0.5 * kDensTiny) e = e - C * pow43(nb);
  return e;
}

/* ---- spin interpolation ---- */
template <class T> T fzeta(const T& z) {
  return (pow(1.0 + z, 4.0 / 3.0) + pow(1.0 - z, 4.0 / 3.0) - 2.0) / (std::pow(2.0, 4.0 / 3.0) - 2.0);
}

/* ---- VWN5 ---- */
template <class T> T vwn_g(const T& x, double A, double x0, double b, double c) {
  const double Q = std::sqrt(4.0 * c - b * b);
  const double X0 = x0 * x0 + b * x0 + c;
  T X = x * x + b * x + c;
  T at = atan(Q / (2.0 * x + b));
  return A * (log(x * x / X) + (2.0 * b / Q) * at -
              (b * x0 / X0) * (log((x - x0) * (x - x0) / X) + (2.0 * (b + 2.0 * x0) / Q) * at));
}
template <class T> T vwn5(const T& na, const T& nb) {
  T n = na + nb;
  T rs = cbrt(3.0 / (4.0 * M_PI * n));
  T x = sqrt(rs);
  T z = clamp_zeta((na - nb) / n);
  T eP = vwn_g(x, 0.0310907, -0.10498, 3.72744, 12.9352);
  T eF = vwn_g(x, 0.01554535, -0.32500, 7.06042, 18.0578);
  T ac = vwn_g(x, -1.0 / (6.0 * M_PI * M_PI), -0.0047584, 1.13107, 13.0045);
  const double fpp0 = 4.0 / (9.0 * (std::cbrt(2.0) - 1.0));
  T f = fzeta(z);
  T z4 = z * z * z * z;
  T eps = eP + ac * f / fpp0 * (1.0 - z4) + (eF - eP) * f * z4;
  return n * eps;
}

/* ---- PW92 ---- */
template <class T> T pw92_g(const T& rs, double A, double a1, double b1, double b2, double b3, double b4) {
  T srs = sqrt(rs);
  T den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return -2.0 * A * (1.0 + a1 * rs) * log(1.0 + 1.0 / den);
}
template <class T> T pw92_eps(const T& rs, const T& z) {
  T ec0 = pw92_g(rs, 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  T ec1 = pw92_g(rs, 0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  T mac = pw92_g(rs, 0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671);
  const double fpp0 = 1.709921;
  T f = fzeta(z);
  T z4 = z * z * z * z;
  return ec0 - mac * f / fpp0 * (1.0 - z4) + (ec1 - ec0) * f * z4;
}
template <class T> T pw92(const T& na, const T& nb) {
  T n = na + nb;
  T rs = cbrt(3.0 / (4.0 * M_PI * n));
  return n * pw92_eps(rs, clamp_zeta((na - nb) / n));
}

/* ---- PBE ---- */
static const double kPbeKappa = 0.804;
static const double kPbeBeta = 0.06672455060314922;
static const double kPbeMu = kPbeBeta * M_PI * M_PI / 3.0;
static const double kPbeGamma = (1.0 - 0.69314718055994530942) / (M_PI * M_PI);

template <class T> T pbex_unpol(const T& n, const T& sigma) {
  T kF = cbrt(3.0 * M_PI * M_PI * n);
  T s2 = sigma / (4.0 * kF * kF * n * n);
  T Fx = 1.0 + kPbeKappa - kPbeKappa / (1.0 + kPbeMu * s2 / kPbeKappa);
  return -0.75 * std::cbrt(3.0 / M_PI) * pow43(n) * Fx;
}
template <class T> T pbex(const T& na, const T& nb, const T& saa, const T& sbb) {
  T e(0.0);
  if (na.v > 0.5 * kDensTiny) e = e + 0.5 * pbex_unpol(2.0 * na, 4.0 * saa);
  if (nb.v > 0.5 * kDensTiny) e = e + 0.5 * pbex_unpol(2.0 * nb, 4.0 * sbb);
  return e;
}
template <class T> T pbec(const T& na, const T& nb, const T& saa, const T& sab, const T& sbb) {
  T n = na + nb;
  T z = clamp_zeta((na - nb) / n);
  T rs = cbrt(3.0 / (4.0 * M_PI * n));
  T eu = pw92_eps(rs, z);
  T phi = 0.5 * (pow(1.0 + z, 2.0 / 3.0) + pow(1.0 - z, 2.0 / 3.0));
  T kF = cbrt(3.0 * M_PI * M_PI * n);
  T ks2 = 4.0 * kF / M_PI;
  T sigma = saa + 2.0 * sab + sbb;
  T t2 = sigma / (4.0 * phi * phi * ks2 * n * n);
  T phi3 = phi * phi * phi;
  T A = (kPbeBeta / kPbeGamma) / (exp(-eu / (kPbeGamma * phi3)) - 1.0);
  T At2 = A * t2;
  T H = kPbeGamma * phi3 * log(1.0 + (kPbeBeta / kPbeGamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return n * (eu + H);
}

/* ---- B88 (includes the Slater part) ---- */
template <class T> T b88(const T& na, const T& nb, const T& saa, const T& sbb) {
  const double beta = 0.0042;
  T e = slater(na, nb);
  const T* ns[2] = {&na, &nb};
  const T* ss[2] = {&saa, &sbb};
  for (int s = 0; s < 2; ++s) {
    if (ns[s]->v <= 0.5 * kDensTiny) continue;
    T n43 = pow43(*ns[s]);
    T x2 = *ss[s] / (n43 * n43);
    e = e - beta * n43 * x2 / (1.0 + 6.0 * beta * xasinhx_of_sq(x2));
  }
  return e;
}

/* ---- LYP ---- */
template <class T> T lyp(const T& na, const T& nb, const T& saa, const T& sab, const T& sbb) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double CF = 0.3 * std::pow(3.0 * M_PI * M_PI, 2.0 / 3.0);
  T n = na + nb;
  T nm13 = 1.0 / cbrt(n);
  T dn = 1.0 + d * nm13;
  T omega = exp(-c * nm13) / dn * pow(n, -11.0 / 3.0);
  T delta = c * nm13 + d * nm13 / dn;
  T sigma = saa + 2.0 * sab + sbb;
  T n2 = n * n;
  T t1 = -a * 4.0 / dn * na * nb / n;
  T inner = na * nb *
                (std::pow(2.0, 11.0 / 3.0) * CF * (pow(na, 8.0 / 3.0) + pow(nb, 8.0 / 3.0)) +
                 (47.0 / 18.0 - 7.0 / 18.0 * delta) * sigma - (2.5 - delta / 18.0) * (saa + sbb) -
                 (delta - 11.0) / 9.0 * (na / n * saa + nb / n * sbb)) -
            2.0 / 3.0 * n2 * sigma + (2.0 / 3.0 * n2 - na * na) * sbb + (2.0 / 3.0 * n2 - nb * nb) * saa;
  return t1 - a * b * omega * inner;
}

/* ---- PZ81: eps_c(rs) of the unpolarised (U) and fully polarised (P) gas ---- */
template <class T> T pz81_eps(const T& rs, double g, double b1, double b2, double A, double B, double C, double D) {
  if (rs.v >= 1.0) return g / (1.0 + b1 * sqrt(rs) + b2 * rs);
  T l = log(rs);
  return A * l + B + C * rs * l + D * rs;
}
template <class T> T pz81(const T& na, const T& nb) {
  T n = na + nb;
  T rs = cbrt(3.0 / (4.0 * M_PI * n));
  T z = clamp_zeta((na - nb) / n);
  T eU = pz81_eps(rs, -0.1423, 1.0529, 0.3334, 0.0311, -0.048, 0.0020, -0.0116);
  T eP = pz81_eps(rs, -0.0843, 1.3981, 0.2611, 0.01555, -0.0269, 0.0007, -0.0048);
  return n * (eU + fzeta(z) * (eP - eU));
}

/* ---- P86 gradient correction: e = exp(-Phi) C(n) |grad n|^2 / (d n^(4/3)) ----
 *   C(n) = 0.001667 + (0.002568 + a rs + b rs^2) / (1 + g rs + h rs^2 + 1e4 b rs^3),
 *   Phi = (9 pi)^(1/6) f (C(inf) / C(n)) |grad n| / n^(7/6), f = 0.11, C(inf) = 0.004235
 *         (the paper's 1.745 is (9 pi)^(1/6) = 1.745415 rounded; the unrounded factor
 *         reproduces the reference's BP86 Fock matrices, the rounded one misses by 8e-6),
 *   d = 2^(1/3) sqrt(((1 + z)/2)^(5/3) + ((1 - z)/2)^(5/3)) */
template <class T> T p86_corr(const T& na, const T& nb, const T& saa, const T& sab, const T& sbb) {
  const double a = 0.023266, b = 7.389e-6, g = 8.723, h = 0.472, c1 = 0.001667, c2 = 0.002568;
  T n = na + nb;
  T rs = cbrt(3.0 / (4.0 * M_PI * n));
  T Cn = c1 + (c2 + a * rs + b * rs * rs) / (1.0 + g * rs + h * rs * rs + 1e4 * b * rs * rs * rs);
  T sigma = saa + 2.0 * sab + sbb;
  // |grad n| = sqrt(sigma); floored so the derivative of sqrt stays finite at sigma = 0
  // (sigma exp(-Phi) itself has a finite first derivative there)
  T gn = sigma.v > 1e-300 ? sqrt(sigma) : T(0.0);
  T n16 = pow(n, 1.0 / 6.0);
  T phi = (std::pow(9.0 * M_PI, 1.0 / 6.0) * 0.11 * (c1 + c2)) / Cn * gn / (n * n16);
  T z = clamp_zeta((na - nb) / n);
  T d = std::cbrt(2.0) * sqrt(pow(0.5 * (1.0 + z), 5.0 / 3.0) + pow(0.5 * (1.0 - z), 5.0 / 3.0));
  return exp(-phi) * Cn * sigma / (d * pow43(n));
}

template <class T> T energy(int func, const T& na, const T& nb, const T& saa, const T& sab, const T& sbb) {
  switch (func) {
    case ORC_FUNC_LDA: return slater(na, nb) + vwn5(na, nb);
    case ORC_FUNC_PBE: return pbex(na, nb, saa, sbb) + pbec(na, nb, saa, sab, sbb);
    case ORC_FUNC_BLYP: return b88(na, nb, saa, sbb) + lyp(na, nb, saa, sab, sbb);
    case ORC_FUNC_SLATER: return slater(na, nb);
    case ORC_FUNC_VWN5: return vwn5(na, nb);
    case ORC_FUNC_PBEX: return pbex(na, nb, saa, sbb);
    case ORC_FUNC_PBEC: return pbec(na, nb, saa, sab, sbb);
    case ORC_FUNC_B88: return b88(na, nb, saa, sbb);
    case ORC_FUNC_LYP: return lyp(na, nb, saa, sab, sbb);
    case ORC_FUNC_PW92: return pw92(na, nb);
    case ORC_FUNC_BP86: return b88(na, nb, saa, sbb) + pz81(na, nb) + p86_corr(na, nb, saa, sab, sbb);
    case ORC_FUNC_P86: return pz81(na, nb) + p86_corr(na, nb, saa, sab, sbb);
    case ORC_FUNC_PZ81: return pz81(na, nb);
  }
  return T(0.0);
}

bool functional_is_gga(int func) {
  switch (func) {
    case ORC_FUNC_PBE: case ORC_FUNC_BLYP: case ORC_FUNC_PBEX: case ORC_FUNC_PBEC: case ORC_FUNC_B88: case ORC_FUNC_LYP:
    case ORC_FUNC_BP86: case ORC_FUNC_P86:
      return true;
  }
  return false;
}

// Restricted linear-response kernel contracted with a perturbed density (the pp, pg, gg
// kernel products of KernelSigmavector.cpp:363-392 with p = rho1, g = grad rho1, weights
// left to the adder): with F(n, sigma) and sigma1 = 2 grad n . grad rho1,
//   v1 = F_nn rho1 + F_n,sigma sigma1,
//   g1 = 2 (F_sigma,n rho1 + F_sigma,sigma sigma1) grad n + 2 F_sigma grad rho1.
void lr_kernel_point(int func, double n0, const double* g0, double n1, const double* g1, double* v1, double* gg1) {
  const bool gga = functional_is_gga(func);
  *v1 = 0.0;
  if (gga)
    for (int k = 0; k < 3; ++k) gg1[k] = 0.0;
  if (!(n0 >= kDensTiny)) return;
  double sig0 = 0.0, sig1 = 0.0;
  if (gga)
    for (int k = 0; k < 3; ++k) {
      sig0 += g0[k] * g0[k];
      sig1 += 2.0 * g0[k] * g1[k];
    }
  typedef H<2> T;
  T n = T::var(n0, 0), s = T::var(sig0, 1);
  T half = 0.5 * n, q = 0.25 * s;
  T e = energy(func, half, half, q, q, q);
  *v1 = e.h[0][0] * n1 + e.h[0][1] * sig1;
  if (gga)
    for (int k = 0; k < 3; ++k) gg1[k] = 2.0 * (e.h[1][0] * n1 + e.h[1][1] * sig1) * g0[k] + 2.0 * e.d[1] * g1[k];
}

// Spin-resolved kernel contraction (KernelSigmavector<UNRESTRICTED>::contractBlock,
// KernelSigmavector.cpp:422-499; the triplet's f_aa - f_ab of :367-391 is the alpha part of
// the perturbation (+rho1, -rho1) about (rho0/2, rho0/2)): with x = (n_a, n_b, s_aa, s_ab,
// s_bb) and x1 its first-order change, dd_i = sum_j E_ij x1_j, and
//   v1_a = dd_0, v1_b = dd_1,
//   g1_a = 2 dd_2 grad n_a + 2 E_2 grad n1_a + dd_3 grad n_b + E_3 grad n1_b, alike for b.
// n0[2], g0[2][3] (ground state per spin), n1[2], g1[2][3]; v1[2], gg1[2][3] out.
void lr_kernel_spin_point(int func, const double* n0, const double* g0, const double* n1, const double* g1,
                          double* v1, double* gg1) {
  const bool gga = functional_is_gga(func);
  for (int s = 0; s < 2; ++s) {
    v1[s] = 0.0;
    for (int k = 0; k < 3; ++k) gg1[3 * s + k] = 0.0;
  }
  const double na0 = n0[0] > 0 ? n0[0] : 0.0, nb0 = n0[1] > 0 ? n0[1] : 0.0;
  if (!(na0 + nb0 >= kDensTiny)) return;
  const double na1 = n0[0] > 0 ? n1[0] : 0.0, nb1 = n0[1] > 0 ? n1[1] : 0.0;
  double x1[5] = {na1, nb1, 0.0, 0.0, 0.0}, s[3] = {0.0, 0.0, 0.0};
  const double *ga = g0, *gb = g0 + 3, *da = g1, *db = g1 + 3;
  if (gga)
    for (int k = 0; k < 3; ++k) {
      s[0] += ga[k] * ga[k];
      s[1] += ga[k] * gb[k];
      s[2] += gb[k] * gb[k];
      x1[2] += 2.0 * ga[k] * da[k];
      x1[3] += ga[k] * db[k] + da[k] * gb[k];
      x1[4] += 2.0 * gb[k] * db[k];
    }
  typedef H<5> T;
  T e = energy(func, T::var(na0, 0), T::var(nb0, 1), T::var(s[0], 2), T::var(s[1], 3), T::var(s[2], 4));
  double dd[5];
  for (int i = 0; i < 5; ++i) {
    dd[i] = 0.0;
    for (int j = 0; j < 5; ++j) dd[i] += e.h[i][j] * x1[j];
  }
  v1[0] = dd[0];
  v1[1] = dd[1];
  if (gga)
    for (int k = 0; k < 3; ++k) {
      gg1[k] = 2.0 * dd[2] * ga[k] + 2.0 * e.d[2] * da[k] + dd[3] * gb[k] + e.d[3] * db[k];
      gg1[3 + k] = 2.0 * dd[4] * gb[k] + 2.0 * e.d[4] * db[k] + dd[3] * ga[k] + e.d[3] * da[k];
    }
}

void functional_point(int func, int nspin, const double* in, double* out) {
  const bool gga = functional_is_gga(func);
  if (nspin == 1) {
    for (int i = 0; i < 5; ++i) out[i] = 0.0;
    if (!(in[0] >= kDensTiny)) return;
    const double sig = gga ? in[1] * in[1] + in[2] * in[2] + in[3] * in[3] : 0.0;
    typedef D<2> T;
    T n = T::var(in[0], 0), s = T::var(sig, 1);
    T half = 0.5 * n, q = 0.25 * s;
    T e = energy(func, half, half, q, q, q);
    out[0] = e.v;
    out[1] = e.d[0];
    if (gga)
      for (int k = 0; k < 3; ++k) out[2 + k] = 2.0 * e.d[1] * in[1 + k];
  } else {
    for (int i = 0; i < 9; ++i) out[i] = 0.0;
    const double na0 = in[0] > 0 ? in[0] : 0.0, nb0 = in[1] > 0 ? in[1] : 0.0;
    if (!(na0 + nb0 >= kDensTiny)) return;
    const double* ga = in + 2;
    const double* gb = in + 5;
    double saa = 0, sab = 0, sbb = 0;
    if (gga)
      for (int k = 0; k < 3; ++k) {
        saa += ga[k] * ga[k];
        sab += ga[k] * gb[k];
        sbb += gb[k] * gb[k];
      }
    typedef D<5> T;
    T na = T::var(na0, 0), nb = T::var(nb0, 1), Saa = T::var(saa, 2), Sab = T::var(sab, 3), Sbb = T::var(sbb, 4);
    T e = energy(func, na, nb, Saa, Sab, Sbb);
    out[0] = e.v;
    out[1] = e.d[0];
    out[2] = e.d[1];
    if (gga)
      for (int k = 0; k < 3; ++k) {
        out[3 + k] = 2.0 * e.d[2] * ga[k] + e.d[3] * gb[k];
        out[6 + k] = 2.0 * e.d[4] * gb[k] + e.d[3] * ga[k];
      }
  }
}

}  // namespace orc
