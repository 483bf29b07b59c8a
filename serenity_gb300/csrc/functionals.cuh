// Exchange-correlation functionals with hand-derived first derivatives, for the
// GRADIENTS data type at order 1 (XCFun.cpp:39-158): the energy per volume e and
// de/drho_s, de/dsigma_ss'.  Written from the literature:
//   Slater        Dirac exchange, spin-scaled
//   VWN5          Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980), fit "V"
//   PW92          Perdew, Wang, PRB 45, 13244 (1992), original parameters
//                 (A = 0.031091/0.015545/0.016887, f''(0) = 1.709921)
//   PBE x, c      Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)
//   B88           Becke, PRA 38, 3098 (1988) (includes the Slater part)
//   LYP           Lee, Yang, Parr, PRB 37, 785 (1988), Miehlich et al. form,
//                 CPL 157, 200 (1989)
//   PZ81          Perdew, Zunger, PRB 23, 5048 (1981), their fit of the Ceperley-Alder
//                 correlation energy
//   P86           Perdew, PRB 33, 8822 (1986): PZ81 plus a gradient correction (BP86 =
//                 B88 + P86, CompositeFunctionals.cpp:244)
// Cut-offs: no contribution below a total density of 1e-14 (the reference sets
// libxc's dens_threshold to 1e-14, LibXC.cpp:86-97); a spin channel below 0.5e-14
// carries no exchange; |zeta| <= 1 - 1e-12 in the correlation functionals.
#pragma once
#include <cuda_runtime.h>

#include "../../include/xcgpu.h"
#include "df32.cuh"

namespace xcgpu {
namespace xc {

template <class R> __device__ __forceinline__ R cbrt_(R x);
template <> __device__ __forceinline__ double cbrt_<double>(double x) { return cbrt(x); }
template <> __device__ __forceinline__ float cbrt_<float>(float x) { return cbrtf(x); }
template <class R> __device__ __forceinline__ R log_(R x);
template <> __device__ __forceinline__ double log_<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float log_<float>(float x) { return logf(x); }
template <class R> __device__ __forceinline__ R exp_(R x);
template <> __device__ __forceinline__ double exp_<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float exp_<float>(float x) { return expf(x); }
template <class R> __device__ __forceinline__ R atan_(R x);
template <> __device__ __forceinline__ double atan_<double>(double x) { return atan(x); }
template <> __device__ __forceinline__ float atan_<float>(float x) { return atanf(x); }
template <class R> __device__ __forceinline__ R asinh_(R x);
template <> __device__ __forceinline__ double asinh_<double>(double x) { return asinh(x); }
template <> __device__ __forceinline__ float asinh_<float>(float x) { return asinhf(x); }
template <class R> __device__ __forceinline__ R sqrt_(R x);
template <> __device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float sqrt_<float>(float x) { return sqrtf(x); }
template <class R> __device__ __forceinline__ R pow_(R x, R p);
template <> __device__ __forceinline__ double pow_<double>(double x, double p) { return pow(x, p); }
template <> __device__ __forceinline__ float pow_<float>(float x, float p) { return powf(x, p); }
// E = exp(x) and Em1 = E - 1 (FP32 pairs: Em1 from expm1, free of the cancellation)
template <class R> __device__ __forceinline__ void exp_em1_(R x, R& E, R& Em1) {
  E = exp_<R>(x);
  Em1 = E - R(1);
}
// FP32 pairs (df32.cuh): the functions restricted PBE needs
template <> __device__ __forceinline__ DF cbrt_<DF>(DF x) { return df_cbrt(x); }
template <> __device__ __forceinline__ DF sqrt_<DF>(DF x) { return df_sqrt(x); }
template <> __device__ __forceinline__ DF log_<DF>(DF x) { return df_log(x); }
template <> __device__ __forceinline__ DF exp_<DF>(DF x) { return df_exp(x); }
template <> __device__ __forceinline__ void exp_em1_<DF>(DF x, DF& E, DF& Em1) {
  Em1 = df_expm1(x);
  E = Em1 + DF(1.f, 0.f);
}

constexpr double kPi = 3.14159265358979323846;
constexpr double kTiny = 1e-14;
constexpr double kZetaMax = 1.0 - 1e-12;

// ---- Slater: e_s = -C (n_s)^(4/3) per spin, C = (3/4)(6/pi)^(1/3) ----
template <class R>
__device__ __forceinline__ void slater_spin(R ns, R& e, R& v) {
  if (!(ns > R(0.5 * kTiny))) return;
  const R C = R(0.9305257363491000);  // (3/4)(6/pi)^(1/3)
  const R c = cbrt_<R>(ns);
  e -= C * ns * c;
  v -= R(4.0 / 3.0) * C * c;
}

// ---- VWN: G(x) and dG/dx, x = sqrt(rs) ----
template <class R>
__device__ __forceinline__ void vwn_g(R x, double A, double x0, double b, double c, R& g, R& dg) {
  const double Q = sqrt(4.0 * c - b * b);
  const double X0 = x0 * x0 + b * x0 + c;
  const R X = x * x + R(b) * x + R(c);
  const R at = atan_<R>(R(Q) / (R(2) * x + R(b)));
  const R t = R(b * x0 / X0);
  g = R(A) * (log_<R>(x * x / X) + R(2.0 * b / Q) * at -
              t * (log_<R>((x - R(x0)) * (x - R(x0)) / X) + R(2.0 * (b + 2.0 * x0) / Q) * at));
  const R tx = (R(2) * x + R(b)) / X;
  dg = R(A) * (R(2) / x - tx - R(b) / X - t * (R(2) / (x - R(x0)) - tx - R(b + 2.0 * x0) / X));
}

template <class R>
__device__ __forceinline__ void fzeta(R z, R& f, R& df) {
  const R k = R(1.0 / (2.5198420997897464 - 2.0));  // 1/(2^(4/3)-2)
  const R a = cbrt_<R>(R(1) + z), b = cbrt_<R>(R(1) - z);
  f = ((R(1) + z) * a + (R(1) - z) * b - R(2)) * k;
  df = R(4.0 / 3.0) * (a - b) * k;
}

// zeta == 0 exactly: the spin-polarised formulas then reduce to the unpolarised ones.
// A number type that also carries derivatives (the response kernel's dual numbers)
// specialises this to require a zero derivative as well: along a spin-flip
// perturbation zeta is 0 but its derivative is not, and the zeta terms matter.
template <class R>
__device__ __forceinline__ bool zeta_is_zero(R z) {
  return z == R(0);
}

// |zeta| is capped at 1 - 1e-12; where the cap applies, zeta no longer depends on
// the spin densities, so the zeta-derivative terms vanish (scale = 0).
template <class R>
__device__ __forceinline__ R clampz(R z, R& scale) {
  scale = R(1);
  if (z > R(kZetaMax)) {
    scale = R(0);
    return R(kZetaMax);
  }
  if (z < R(-kZetaMax)) {
    scale = R(0);
    return R(-kZetaMax);
  }
  return z;
}

// VWN5 correlation, spin-polarised; adds e and de/dna, de/dnb
template <class R>
__device__ __forceinline__ void vwn5(R na, R nb, R& e, R& va, R& vb) {
  const R n = na + nb;
  const R rs = cbrt_<R>(R(3.0 / (4.0 * kPi)) / n);
  const R x = sqrt_<R>(rs);
  R eP, dP, eF, dF, ac, dac;
  vwn_g(x, 0.0310907, -0.10498, 3.72744, 12.9352, eP, dP);
  R zs;
  const R z = clampz((na - nb) / n, zs);
  if (zeta_is_zero(z)) {
    const R deps_drs = dP / (R(2) * x);
    e += n * eP;
    const R v = eP - rs / R(3) * deps_drs;
    va += v;
    vb += v;
    return;
  }
  vwn_g(x, 0.01554535, -0.32500, 7.06042, 18.0578, eF, dF);
  vwn_g(x, -1.0 / (6.0 * kPi * kPi), -0.0047584, 1.13107, 13.0045, ac, dac);
  const R fpp0 = R(1.7099209341613657);  // 4/(9(2^(1/3)-1))
  R f, df;
  fzeta(z, f, df);
  const R z3 = z * z * z, z4 = z3 * z;
  const R eps = eP + ac * f / fpp0 * (R(1) - z4) + (eF - eP) * f * z4;
  const R dx = dP + dac * f / fpp0 * (R(1) - z4) + (dF - dP) * f * z4;
  const R deps_drs = dx / (R(2) * x);
  const R deps_dz = zs * (ac / fpp0 * (df * (R(1) - z4) - R(4) * z3 * f) + (eF - eP) * (df * z4 + R(4) * z3 * f));
  e += n * eps;
  const R base = eps - rs / R(3) * deps_drs;
  va += base + (R(1) - z) * deps_dz;
  vb += base - (R(1) + z) * deps_dz;
}

// ---- PW92 ----
template <class R>
__device__ __forceinline__ void pw92_g(R rs, R srs, double A, double a1, double b1, double b2, double b3, double b4,
                                       R& g, R& dg) {
  const R Q1 = R(2 * A) * (R(b1) * srs + R(b2) * rs + R(b3) * rs * srs + R(b4) * rs * rs);
  const R dQ1 = R(2 * A) * (R(0.5 * b1) / srs + R(b2) + R(1.5 * b3) * srs + R(2 * b4) * rs);
  const R L = log_<R>(R(1) + R(1) / Q1);
  g = R(-2 * A) * (R(1) + R(a1) * rs) * L;
  dg = R(-2 * A * a1) * L + R(2 * A) * (R(1) + R(a1) * rs) * dQ1 / (Q1 * Q1 + Q1);
}

// eps_c(rs, zeta) with derivatives
template <class R>
__device__ __forceinline__ void pw92_eps(R rs, R z, R& eps, R& deps_drs, R& deps_dz) {
  const R srs = sqrt_<R>(rs);
  R e0, d0;
  pw92_g(rs, srs, 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294, e0, d0);
  if (zeta_is_zero(z)) {
    eps = e0;
    deps_drs = d0;
    deps_dz = R(0);
    return;
  }
  R e1, d1, ma, dma;
  pw92_g(rs, srs, 0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517, e1, d1);
  pw92_g(rs, srs, 0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671, ma, dma);
  const R fpp0 = R(1.709921);
  R f, df;
  fzeta(z, f, df);
  const R z3 = z * z * z, z4 = z3 * z;
  eps = e0 - ma * f / fpp0 * (R(1) - z4) + (e1 - e0) * f * z4;
  deps_drs = d0 - dma * f / fpp0 * (R(1) - z4) + (d1 - d0) * f * z4;
  deps_dz = -ma / fpp0 * (df * (R(1) - z4) - R(4) * z3 * f) + (e1 - e0) * (df * z4 + R(4) * z3 * f);
}

template <class R>
__device__ __forceinline__ void pw92(R na, R nb, R& e, R& va, R& vb) {
  const R n = na + nb;
  const R rs = cbrt_<R>(R(3.0 / (4.0 * kPi)) / n);
  R zs;
  const R z = clampz((na - nb) / n, zs);
  R eps, dr, dz;
  pw92_eps(rs, z, eps, dr, dz);
  dz *= zs;
  e += n * eps;
  const R base = eps - rs / R(3) * dr;
  va += base + (R(1) - z) * dz;
  vb += base - (R(1) + z) * dz;
}

// ---- PBE exchange, unpolarised form e(n, sigma) ----
constexpr double kKappa = 0.804;
constexpr double kBeta = 0.06672455060314922;
constexpr double kMu = kBeta * kPi * kPi / 3.0;
constexpr double kGamma = (1.0 - 0.69314718055994530942) / (kPi * kPi);

template <class R>
__device__ __forceinline__ void pbex_unpol(R n, R sigma, R& e, R& vn, R& vs) {
  const R Cx = R(0.7385587663820224);        // (3/4)(3/pi)^(1/3)
  const R c2 = R(1.0 / (4.0 * 9.570780000627305));  // 1/(4 (3 pi^2)^(2/3))
  const R n13 = cbrt_<R>(n);
  const R n43 = n * n13;
  const R n83 = n43 * n43;
  const R s2 = sigma * c2 / n83;
  const R den = R(1) + R(kMu / kKappa) * s2;
  const R Fx = R(1 + kKappa) - R(kKappa) / den;
  const R dFx = R(kMu) / (den * den);
  e = -Cx * n43 * Fx;
  vn = -Cx * (R(4.0 / 3.0) * n13 * Fx - n43 * dFx * R(8.0 / 3.0) * s2 / n);
  vs = -Cx * n43 * dFx * c2 / n83;
}

// ---- PBE correlation (spin-polarised) ----
template <class R>
__device__ __forceinline__ void pbec(R na, R nb, R saa, R sab, R sbb, R& e, R& va, R& vb, R& vsaa, R& vsab, R& vsbb) {
  const R n = na + nb;
  R zs;
  const R z = clampz((na - nb) / n, zs);
  const R rs = cbrt_<R>(R(3.0 / (4.0 * kPi)) / n);
  R eps, deps_drs, deps_dz;
  pw92_eps(rs, z, eps, deps_drs, deps_dz);
  R phi = R(1), dphi = R(0);
  if (!zeta_is_zero(z)) {
    const R a = cbrt_<R>(R(1) + z), b = cbrt_<R>(R(1) - z);
    phi = R(0.5) * (a * a + b * b);
    dphi = R(1.0 / 3.0) * (R(1) / a - R(1) / b);
  }
  const R sigma = saa + R(2) * sab + sbb;
  const R kF = cbrt_<R>(R(3.0 * kPi * kPi) * n);
  const R phi2 = phi * phi, phi3 = phi2 * phi;
  const R dt2_dsig = R(kPi / 16.0) / (phi2 * kF * n * n);
  const R t2 = sigma * dt2_dsig;
  const R gphi3 = R(kGamma) * phi3;
  const R E = exp_<R>(-eps / gphi3);
  const R A = R(kBeta / kGamma) / (E - R(1));
  const R y = A * t2;
  const R N = R(1) + y, Dn = R(1) + y + y * y;
  const R Q = t2 * N / Dn;
  const R arg = R(1) + R(kBeta / kGamma) * Q;
  const R H = gphi3 * log_<R>(arg);
  const R pref = gphi3 * R(kBeta / kGamma) / arg;
  const R dQ_dt2 = N / Dn - y * y * (R(2) + y) / (Dn * Dn);
  const R dQ_dA = -t2 * t2 * y * (R(2) + y) / (Dn * Dn);
  const R dH_dt2 = pref * dQ_dt2;
  const R dH_dA = pref * dQ_dA;
  const R dA_deps = A * A * E / (R(kBeta) * phi3);
  const R dA_dphi = -R(3) * A * A * E * eps / (R(kBeta) * phi3 * phi);
  const R deps_dn = -rs / (R(3) * n) * deps_drs;
  const R dH_dn = dH_dt2 * (-R(7.0 / 3.0) * t2 / n) + dH_dA * dA_deps * deps_dn;
  const R dH_dz = (R(3) * H / phi + dH_dt2 * (-R(2) * t2 / phi) + dH_dA * dA_dphi) * dphi + dH_dA * dA_deps * deps_dz;
  e += n * (eps + H);
  const R base = eps + H + n * (deps_dn + dH_dn);
  const R dz = zs * (deps_dz + dH_dz);
  va += base + (R(1) - z) * dz;
  vb += base - (R(1) + z) * dz;
  const R vs = n * dH_dt2 * dt2_dsig;
  vsaa += vs;
  vsab += R(2) * vs;
  vsbb += vs;
}

// ---- PBE exchange + correlation of an unpolarised density in one pass: the same
// expressions as pbex_unpol + pbec at zeta = 0 (phi = 1), with n^(1/3) taken once and
// the divisions shared (FP64 division and the cube root dominate the functional's cost
// on a GPU whose FP64 rate is a small fraction of its FP32 rate) ----
template <class R>
__device__ __forceinline__ void pbe_unpol(R n, R sigma, R& e, R& vn, R& vs) {
  constexpr double A0 = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const R n13 = cbrt_<R>(n);
  const R r13 = R(1) / n13, rn = r13 * r13 * r13;
  // exchange: e = -Cx n^(4/3) Fx(s^2), s^2 = sigma / (4 (3 pi^2)^(2/3) n^(8/3))
  const R n43 = n * n13;
  const R k8 = R(1.0 / (4.0 * 9.570780000627305)) * (rn * rn * r13 * r13);  // 1 / (4 (3 pi^2)^(2/3) n^(8/3))
  const R s2 = sigma * k8;
  const R rden = R(1) / (R(1) + R(kMu / kKappa) * s2);
  const R Fx = R(1 + kKappa) - R(kKappa) * rden;
  const R dFx = R(kMu) * rden * rden;
  const R Cx = R(0.7385587663820224);  // (3/4)(3/pi)^(1/3)
  e = -Cx * n43 * Fx;
  vn = -Cx * (R(4.0 / 3.0) * n13 * Fx - R(8.0 / 3.0) * n13 * dFx * s2);
  vs = -Cx * n43 * dFx * k8;
  // correlation: PW92 eps(rs) and the PBE gradient term H(t^2)
  const R rs = R(0.6203504908994001) * r13;  // (3 / (4 pi n))^(1/3)
  const R srs = sqrt_<R>(rs);
  const R Q1 = R(2 * A0) * (R(b1) * srs + R(b2) * rs + R(b3) * rs * srs + R(b4) * rs * rs);
  const R dQ1 = R(2 * A0) * (R(0.5 * b1) * srs * (n13 * R(1.0 / 0.6203504908994001)) + R(b2) + R(1.5 * b3) * srs +
                              R(2 * b4) * rs);
  const R rq = R(1) / (Q1 * (Q1 + R(1)));  // 1 / (Q1^2 + Q1)
  const R L = log_<R>(R(1) + rq * (Q1 + R(1)));
  const R eps = R(-2 * A0) * (R(1) + R(a1) * rs) * L;
  const R deps_drs = R(-2 * A0 * a1) * L + R(2 * A0) * (R(1) + R(a1) * rs) * dQ1 * rq;
  const R dt2_dsig = R(kPi / 16.0 / 3.0936677262801355) * r13 * rn * rn;  // pi / (16 kF n^2)
  const R t2 = sigma * dt2_dsig;
  R E, Em1;
  exp_em1_<R>(-eps * R(1.0 / kGamma), E, Em1);
  const R rE = R(1) / Em1;
  const R A = R(kBeta / kGamma) * rE;
  const R y = A * t2;
  const R N = R(1) + y;
  const R rD = R(1) / (R(1) + y + y * y);
  const R Q = t2 * N * rD;
  const R arg = R(1) + R(kBeta / kGamma) * Q;
  const R rarg = R(1) / arg;
  const R H = R(kGamma) * log_<R>(arg);
  const R pref = R(kBeta) * rarg;
  const R y2y = y * (R(2) + y) * rD * rD;
  const R dH_dt2 = pref * (N * rD - y * y2y);
  const R dH_dA = -pref * t2 * t2 * y2y;
  const R dA_deps = A * A * E * R(1.0 / kBeta);
  const R deps_dn = R(-1.0 / 3.0) * rs * rn * deps_drs;
  const R dH_dn = dH_dt2 * (R(-7.0 / 3.0) * t2 * rn) + dH_dA * dA_deps * deps_dn;
  e += n * (eps + H);
  vn += eps + H + n * (deps_dn + dH_dn);
  vs += n * dH_dt2 * dt2_dsig;
}

// restricted PBE in FP32 pairs (the mixed build's functional): the same expressions as
// pbe_unpol<double> to ~1e-13 relative, at FP32 instruction rates.  Above the density
// cut-off every intermediate stays inside the FP32 range (n^-8/3 <= 2e37 at n = 1e-14).
__device__ __forceinline__ void pbe_restricted_pair(double n, double sigma, double& e, double& vn, double& vs) {
  e = vn = vs = 0.0;
  if (!(n >= kTiny)) return;
  DF E = DF(0.f, 0.f), VN = DF(0.f, 0.f), VS = DF(0.f, 0.f);
  pbe_unpol<DF>(df_from_double(n), df_from_double(sigma), E, VN, VS);
  e = df_to_double(E);
  vn = df_to_double(VN);
  vs = df_to_double(VS);
}

// ---- B88 gradient correction per spin (without the Slater part) ----
template <class R>
__device__ __forceinline__ void b88_spin(R ns, R sss, R& e, R& vn, R& vs) {
  if (!(ns > R(0.5 * kTiny))) return;
  const R beta = R(0.0042);
  const R n13 = cbrt_<R>(ns);
  const R n43 = ns * n13;
  const R x = sqrt_<R>(sss) / n43;
  const R as = asinh_<R>(x);
  const R D = R(1) + R(6) * beta * x * as;
  const R g = x * x / D;
  const R sq = sqrt_<R>(R(1) + x * x);
  const R gp_over_x = (R(2) + R(6) * beta * x * as - R(6) * beta * x * x / sq) / (D * D);  // g'(x)/x
  e -= beta * n43 * g;
  vn -= beta * R(4.0 / 3.0) * n13 * (g - x * x * gp_over_x);
  vs -= beta * gp_over_x / (R(2) * n43);
}

// ---- LYP (spin-polarised, Miehlich form) ----
template <class R>
__device__ __forceinline__ void lyp(R na, R nb, R saa, R sab, R sbb, R& e, R& va, R& vb, R& vsaa, R& vsab, R& vsbb) {
  const R a = R(0.04918), b = R(0.132), c = R(0.2533), d = R(0.349);
  const R CF = R(2.8712340001881915);  // (3/10)(3 pi^2)^(2/3)
  const R c2113 = R(12.699208415745595);  // 2^(11/3)
  const R n = na + nb;
  const R m = R(1) / cbrt_<R>(n);  // n^(-1/3)
  const R dn = R(1) + d * m;
  const R n113 = pow_<R>(n, R(-11.0 / 3.0));
  const R omega = exp_<R>(-c * m) / dn * n113;
  const R delta = c * m + d * m / dn;
  const R domega = omega / (R(3) * n) * (c * m - R(11) + d * m / dn);
  const R ddelta = -c * m / (R(3) * n) - d * m / (R(3) * n * dn * dn);
  const R S = saa + R(2) * sab + sbb;
  const R Ss = saa + sbb;
  const R na83 = pow_<R>(na, R(8.0 / 3.0)), nb83 = pow_<R>(nb, R(8.0 / 3.0));
  const R na53 = pow_<R>(na, R(5.0 / 3.0)), nb53 = pow_<R>(nb, R(5.0 / 3.0));
  const R A1 = R(47.0 / 18.0) - R(7.0 / 18.0) * delta;
  const R A2 = R(2.5) - delta / R(18);
  const R A3 = (delta - R(11)) / R(9);
  const R mix = (na * saa + nb * sbb) / n;
  const R W = c2113 * CF * (na83 + nb83) + A1 * S - A2 * Ss - A3 * mix;
  const R n2 = n * n;
  const R inner = na * nb * W - R(2.0 / 3.0) * n2 * S + (R(2.0 / 3.0) * n2 - na * na) * sbb +
                  (R(2.0 / 3.0) * n2 - nb * nb) * saa;
  // derivatives of W
  const R dW_common = ddelta * (-R(7.0 / 18.0) * S + Ss / R(18) - mix / R(9));
  const R dWa = c2113 * CF * R(8.0 / 3.0) * na53 + dW_common - A3 * (saa / n - mix / n);
  const R dWb = c2113 * CF * R(8.0 / 3.0) * nb53 + dW_common - A3 * (sbb / n - mix / n);
  const R dIa = nb * W + na * nb * dWa - R(4.0 / 3.0) * n * S + (R(4.0 / 3.0) * n - R(2) * na) * sbb +
                R(4.0 / 3.0) * n * saa;
  const R dIb = na * W + na * nb * dWb - R(4.0 / 3.0) * n * S + R(4.0 / 3.0) * n * sbb +
                (R(4.0 / 3.0) * n - R(2) * nb) * saa;
  const R dIsaa = na * nb * (A1 - A2 - A3 * na / n) - nb * nb;
  const R dIsbb = na * nb * (A1 - A2 - A3 * nb / n) - na * na;
  const R dIsab = R(2) * na * nb * A1 - R(4.0 / 3.0) * n2;
  // first term
  const R t1 = -R(4) * a * na * nb / (n * dn);
  const R k1 = d * m / (R(3) * dn);
  const R dt1a = -R(4) * a * nb / (n * dn) * (nb / n + k1 * na / n);
  const R dt1b = -R(4) * a * na / (n * dn) * (na / n + k1 * nb / n);
  const R ab = a * b;
  e += t1 - ab * omega * inner;
  va += dt1a - ab * (domega * inner + omega * dIa);
  vb += dt1b - ab * (domega * inner + omega * dIb);
  vsaa -= ab * omega * dIsaa;
  vsab -= ab * omega * dIsab;
  vsbb -= ab * omega * dIsbb;
}

// ---- PZ81: eps(rs) of one spin state and d eps / d rs ----
template <class R>
__device__ __forceinline__ void pz81_g(R rs, double g, double b1, double b2, double A, double B, double C, double D,
                                       R& eps, R& deps) {
  if (rs >= R(1)) {
    const R srs = sqrt_<R>(rs);
    const R den = R(1) + R(b1) * srs + R(b2) * rs;
    eps = R(g) / den;
    deps = -R(g) * (R(0.5 * b1) / srs + R(b2)) / (den * den);
  } else {
    const R l = log_<R>(rs);
    eps = R(A) * l + R(B) + R(C) * rs * l + R(D) * rs;
    deps = R(A) / rs + R(C) * (l + R(1)) + R(D);
  }
}

// PZ81 correlation, spin-polarised (f(zeta) interpolation); adds e and de/dna, de/dnb
template <class R>
__device__ __forceinline__ void pz81(R na, R nb, R& e, R& va, R& vb) {
  const R n = na + nb;
  const R rs = cbrt_<R>(R(3.0 / (4.0 * kPi)) / n);
  R zs;
  const R z = clampz((na - nb) / n, zs);
  R eps, dr, dz = R(0);
  pz81_g(rs, -0.1423, 1.0529, 0.3334, 0.0311, -0.048, 0.0020, -0.0116, eps, dr);
  if (!zeta_is_zero(z)) {
    R eP, dP, f, df;
    pz81_g(rs, -0.0843, 1.3981, 0.2611, 0.01555, -0.0269, 0.0007, -0.0048, eP, dP);
    fzeta(z, f, df);
    dz = zs * df * (eP - eps);
    eps += f * (eP - eps);
    dr += f * (dP - dr);
  }
  e += n * eps;
  const R base = eps - rs / R(3) * dr;
  va += base + (R(1) - z) * dz;
  vb += base - (R(1) + z) * dz;
}

// ---- P86 gradient correction, e = exp(-Phi) C(n) sigma / (d(zeta) n^(4/3)):
//   C(n) = c1 + (c2 + a rs + b rs^2) / (1 + g rs + h rs^2 + 1e4 b rs^3),
//   Phi = (9 pi)^(1/6) 0.11 (C(inf) / C(n)) sigma^(1/2) / n^(7/6), C(inf) = c1 + c2,
//   d = 2^(1/3) sqrt(((1 + z)/2)^(5/3) + ((1 - z)/2)^(5/3)).
// The paper prints (9 pi)^(1/6) rounded to 1.745; the unrounded factor reproduces the
// reference's BP86 Fock matrices (FuncPotential_test.cpp:148-232).  de/dsigma =
// e (1 - Phi/2) / sigma has no singularity at sigma = 0.
template <class R>
__device__ __forceinline__ void p86corr(R na, R nb, R saa, R sab, R sbb, R& e, R& va, R& vb, R& vsaa, R& vsab,
                                        R& vsbb) {
  constexpr double a = 0.023266, b = 7.389e-6, g = 8.723, h = 0.472, c1 = 0.001667, c2 = 0.002568;
  constexpr double K = 0.19199566167376364 * (c1 + c2);  // (9 pi)^(1/6) 0.11 C(inf)
  const R n = na + nb;
  const R rs = cbrt_<R>(R(3.0 / (4.0 * kPi)) / n);
  const R num = R(c2) + R(a) * rs + R(b) * rs * rs;
  const R den = R(1) + R(g) * rs + R(h) * rs * rs + R(1e4 * b) * rs * rs * rs;
  const R C = R(c1) + num / den;
  const R dC_drs = ((R(a) + R(2 * b) * rs) * den - num * (R(g) + R(2 * h) * rs + R(3e4 * b) * rs * rs)) / (den * den);
  const R sigma = saa + R(2) * sab + sbb;
  const R sg = sigma > R(0) ? sqrt_<R>(sigma) : R(0);
  const R n13 = cbrt_<R>(n);
  const R n16 = sqrt_<R>(n13);
  const R phi = R(K) / C * sg / (n * n16);
  const R E = exp_<R>(-phi);
  R zs;
  const R z = clampz((na - nb) / n, zs);
  R dinv = R(1), dlog = R(0);  // 1/d and d'(z)/d
  if (!zeta_is_zero(z)) {
    const R up = R(0.5) * (R(1) + z), dn = R(0.5) * (R(1) - z);
    const R u23 = cbrt_<R>(up * up), d23 = cbrt_<R>(dn * dn);
    const R A = up * u23 + dn * d23;
    dinv = R(1) / (R(1.2599210498948732) * sqrt_<R>(A));  // 2^(1/3)
    dlog = zs * R(5.0 / 6.0) * (u23 - d23) / (R(2) * A);
  }
  const R pre = E * C * dinv / (n * n13);  // exp(-Phi) C / (d n^(4/3))
  const R ec = pre * sigma;
  const R dC_dn = -rs / (R(3) * n) * dC_drs;
  const R den_ = ec * ((R(1) + phi) * dC_dn / C + (R(7.0 / 6.0) * phi - R(4.0 / 3.0)) / n);
  const R dez = -ec * dlog;  // de/dzeta
  e += ec;
  va += den_ + (R(1) - z) / n * dez;
  vb += den_ - (R(1) + z) / n * dez;
  const R vs = pre * (R(1) - R(0.5) * phi);
  vsaa += vs;
  vsab += R(2) * vs;
  vsbb += vs;
}

__host__ __device__ inline bool is_gga(int func) {
  return func == XCGPU_FUNC_PBE || func == XCGPU_FUNC_BLYP || func == XCGPU_FUNC_PBEX || func == XCGPU_FUNC_PBEC ||
         func == XCGPU_FUNC_B88 || func == XCGPU_FUNC_LYP || func == XCGPU_FUNC_BP86 || func == XCGPU_FUNC_P86;
}
__host__ __device__ inline bool is_known(int func) {
  return (func >= XCGPU_FUNC_LDA && func <= XCGPU_FUNC_BP86) || (func >= 16 && func <= 24);
}

// restricted point: e, de/dn, de/dsigma
template <class R>
__device__ __forceinline__ void eval_restricted(int func, R n, R sigma, R& e, R& vn, R& vs) {
  e = vn = vs = R(0);
  if (!(n >= R(kTiny))) return;
  const R h = R(0.5) * n;
  switch (func) {
    case XCGPU_FUNC_LDA:
    case XCGPU_FUNC_SLATER:
    case XCGPU_FUNC_VWN5:
    case XCGPU_FUNC_PW92: {
      R va = R(0), vb = R(0);
      if (func != XCGPU_FUNC_VWN5 && func != XCGPU_FUNC_PW92) {
        slater_spin(h, e, va);
        slater_spin(h, e, vb);
      }
      if (func == XCGPU_FUNC_LDA || func == XCGPU_FUNC_VWN5) vwn5(h, h, e, va, vb);
      if (func == XCGPU_FUNC_PW92) pw92(h, h, e, va, vb);
      vn = R(0.5) * (va + vb);
      break;
    }
    case XCGPU_FUNC_PBE:
      pbe_unpol(n, sigma, e, vn, vs);
      break;
    case XCGPU_FUNC_PBEX:
    case XCGPU_FUNC_PBEC: {
      if (func != XCGPU_FUNC_PBEC && n > R(kTiny)) {
        R ex, vx, sx;
        pbex_unpol(n, sigma, ex, vx, sx);
        e += ex;
        vn += vx;
        vs += sx;
      }
      if (func != XCGPU_FUNC_PBEX) {
        R va = R(0), vb = R(0), vaa = R(0), vab = R(0), vbb = R(0);
        const R q = R(0.25) * sigma;
        pbec(h, h, q, q, q, e, va, vb, vaa, vab, vbb);
        vn += R(0.5) * (va + vb);
        vs += R(0.25) * (vaa + vab + vbb);
      }
      break;
    }
    case XCGPU_FUNC_PZ81:
    case XCGPU_FUNC_P86: {
      R va = R(0), vb = R(0), vaa = R(0), vab = R(0), vbb = R(0);
      const R q = R(0.25) * sigma;
      pz81(h, h, e, va, vb);
      if (func == XCGPU_FUNC_P86) p86corr(h, h, q, q, q, e, va, vb, vaa, vab, vbb);
      vn += R(0.5) * (va + vb);
      vs += R(0.25) * (vaa + vab + vbb);
      break;
    }
    case XCGPU_FUNC_BLYP:
    case XCGPU_FUNC_BP86:
    case XCGPU_FUNC_B88:
    case XCGPU_FUNC_LYP: {
      if (func != XCGPU_FUNC_LYP) {
        R es = R(0), vns = R(0), vss = R(0);
        slater_spin(h, es, vns);
        b88_spin(h, R(0.25) * sigma, es, vns, vss);
        e += R(2) * es;
        vn += vns;
        vs += R(0.5) * vss;
      }
      if (func == XCGPU_FUNC_BP86) {
        R va = R(0), vb = R(0), vaa = R(0), vab = R(0), vbb = R(0);
        const R q = R(0.25) * sigma;
        pz81(h, h, e, va, vb);
        p86corr(h, h, q, q, q, e, va, vb, vaa, vab, vbb);
        vn += R(0.5) * (va + vb);
        vs += R(0.25) * (vaa + vab + vbb);
      } else if (func != XCGPU_FUNC_B88) {
        R va = R(0), vb = R(0), vaa = R(0), vab = R(0), vbb = R(0);
        const R q = R(0.25) * sigma;
        lyp(h, h, q, q, q, e, va, vb, vaa, vab, vbb);
        vn += R(0.5) * (va + vb);
        vs += R(0.25) * (vaa + vab + vbb);
      }
      break;
    }
    default:
      break;
  }
}

// unrestricted point: e, de/dna, de/dnb, de/dsaa, de/dsab, de/dsbb
template <class R>
__device__ __forceinline__ void eval_unrestricted(int func, R na, R nb, R saa, R sab, R sbb, R& e, R& va, R& vb,
                                                  R& vaa, R& vab, R& vbb) {
  e = va = vb = vaa = vab = vbb = R(0);
  na = na > R(0) ? na : R(0);
  nb = nb > R(0) ? nb : R(0);
  if (!(na + nb >= R(kTiny))) return;
  switch (func) {
    case XCGPU_FUNC_LDA:
    case XCGPU_FUNC_SLATER:
    case XCGPU_FUNC_VWN5:
    case XCGPU_FUNC_PW92:
      if (func != XCGPU_FUNC_VWN5 && func != XCGPU_FUNC_PW92) {
        slater_spin(na, e, va);
        slater_spin(nb, e, vb);
      }
      if (func == XCGPU_FUNC_LDA || func == XCGPU_FUNC_VWN5) vwn5(na, nb, e, va, vb);
      if (func == XCGPU_FUNC_PW92) pw92(na, nb, e, va, vb);
      break;
    case XCGPU_FUNC_PBE:
    case XCGPU_FUNC_PBEX:
    case XCGPU_FUNC_PBEC:
      if (func != XCGPU_FUNC_PBEC) {
        R ex, vx, sx;
        if (na > R(0.5 * kTiny)) {
          pbex_unpol(R(2) * na, R(4) * saa, ex, vx, sx);
          e += R(0.5) * ex;
          va += vx;
          vaa += R(2) * sx;
        }
        if (nb > R(0.5 * kTiny)) {
          pbex_unpol(R(2) * nb, R(4) * sbb, ex, vx, sx);
          e += R(0.5) * ex;
          vb += vx;
          vbb += R(2) * sx;
        }
      }
      if (func != XCGPU_FUNC_PBEX) pbec(na, nb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
      break;
    case XCGPU_FUNC_PZ81:
    case XCGPU_FUNC_P86:
      pz81(na, nb, e, va, vb);
      if (func == XCGPU_FUNC_P86) p86corr(na, nb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
      break;
    case XCGPU_FUNC_BLYP:
    case XCGPU_FUNC_BP86:
    case XCGPU_FUNC_B88:
    case XCGPU_FUNC_LYP:
      if (func != XCGPU_FUNC_LYP) {
        slater_spin(na, e, va);
        slater_spin(nb, e, vb);
        b88_spin(na, saa, e, va, vaa);
        b88_spin(nb, sbb, e, vb, vbb);
      }
      if (func == XCGPU_FUNC_BP86) {
        pz81(na, nb, e, va, vb);
        p86corr(na, nb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
      } else if (func != XCGPU_FUNC_B88) {
        lyp(na, nb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
      }
      break;
    default:
      break;
  }
}

}  // namespace xc
}  // namespace xcgpu
