/*
 * ORACLE -- test infrastructure only (see oracle.h).
 *
 * Basis normalisation, real solid harmonics, basis functions on a block of grid
 * points, and the atom-centred Becke grid, restated from the reference:
 *   Shell.cpp:30-47 + libint2 2.7.0-beta.6 Shell::renorm (published convention:
 *     primitives normalised for the x^l component, then the contraction to unit
 *     self-overlap) and Normalization.h:82-87 (Cartesian factors);
 *   BasisFunctionOnGridController.cpp:150-1107 (screening, radial cut-offs,
 *     Cartesian order, real solid harmonics, gradients, Hessians);
 *   AtomGridFactory.cpp:78-290 (Ahlrichs radial rule, pruning by accuracy);
 *   GridFactory.cpp:52-346 (Becke cells with size adjustment and smoothing);
 *   HilbertRTreeSorting.cpp:29-216 (Hilbert ordering of the points).
 */
#include "oracle_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace orc {

static double dfact(int n) {  // n!! with (-1)!! = 0!! = 1
  double r = 1.0;
  for (int k = n; k > 1; k -= 2) r *= k;
  return r;
}
static double fact(int n) {
  double r = 1.0;
  for (int k = 2; k <= n; ++k) r *= k;
  return r;
}
static double binom(int n, int k) {
  if (k < 0 || k > n) return 0.0;
  return fact(n) / (fact(k) * fact(n - k));
}

int ncart(int l) { return (l + 1) * (l + 2) / 2; }

void cart_exponents(int l, std::vector<int>& ax, std::vector<int>& ay, std::vector<int>& az) {
  ax.clear(); ay.clear(); az.clear();
  for (int a = l; a >= 0; --a)
    for (int b = l - a; b >= 0; --b) {
      ax.push_back(a); ay.push_back(b); az.push_back(l - a - b);
    }
}

// Real solid harmonics S_lm as Cartesian polynomials (Helgaker, Joergensen, Olsen,
// "Molecular Electronic-Structure Theory", eqs. 6.4.47-6.4.50):
//   S_lm = N_lm sum_t sum_u sum_v C_tuv x^(2t+|m|-2(u+v)) y^(2(u+v)) z^(l-2t-|m|)
// m = -l..l; row m+l, column = Cartesian index in the reference's order.
std::vector<double> solid_harmonic_matrix(int l) {
  std::vector<int> ax, ay, az;
  cart_exponents(l, ax, ay, az);
  const int nc = ncart(l);
  std::vector<double> T((2 * l + 1) * nc, 0.0);
  for (int m = -l; m <= l; ++m) {
    const int am = std::abs(m);
    const double vm = (m < 0) ? 0.5 : 0.0;
    const double N = std::sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0)) / (std::pow(2.0, am) * fact(l));
    for (int t = 0; t <= (l - am) / 2; ++t)
      for (int u = 0; u <= t; ++u) {
        // v runs over vm, vm+1, ... <= floor(|m|/2 - vm) + vm
        const int vmax2 = 2 * (int)std::floor(am / 2.0 - vm) + (int)(2 * vm);
        for (int v2 = (int)(2 * vm); v2 <= vmax2; v2 += 2) {
          const double v = 0.5 * v2;
          const double sgn = ((int)std::lround(t + v - vm) % 2 == 0) ? 1.0 : -1.0;
          const double C = sgn * std::pow(0.25, t) * binom(l, t) * binom(l - t, am + t) * binom(t, u) *
                           binom(am, (int)std::lround(2 * v));
          const int px = 2 * t + am - (int)std::lround(2 * (u + v));
          const int py = (int)std::lround(2 * (u + v));
          const int pz = l - 2 * t - am;
          for (int k = 0; k < nc; ++k)
            if (ax[k] == px && ay[k] == py && az[k] == pz) T[(m + l) * nc + k] += N * C;
        }
      }
  }
  return T;
}

Basis::Basis(int nshell, const int* l, const int* pure, const int* nprim, const double* centers, const double* alpha,
             const double* coef) {
  const double pi32 = std::pow(M_PI, 1.5);
  int off = 0;
  nbf = 0;
  for (int s = 0; s < nshell; ++s) {
    Shell sh;
    sh.l = l[s];
    sh.pure = pure[s] != 0;
    for (int k = 0; k < 3; ++k) sh.O[k] = centers[3 * s + k];
    sh.alpha.assign(alpha + off, alpha + off + nprim[s]);
    sh.coef.assign(coef + off, coef + off + nprim[s]);
    off += nprim[s];
    const int L = sh.l;
    // primitive normalisation for the x^L component
    for (size_t p = 0; p < sh.alpha.size(); ++p) {
      const double ta = 2.0 * sh.alpha[p];
      sh.coef[p] *= std::sqrt(std::pow(2.0, L) * std::pow(ta, L + 1.5) / (pi32 * dfact(2 * L - 1)));
    }
    // contraction normalisation to unit self-overlap
    double norm = 0.0;
    for (size_t p = 0; p < sh.alpha.size(); ++p)
      for (size_t q = 0; q < sh.alpha.size(); ++q) {
        const double g = sh.alpha[p] + sh.alpha[q];
        norm += dfact(2 * L - 1) * pi32 * sh.coef[p] * sh.coef[q] / (std::pow(2.0, L) * std::pow(g, L + 1.5));
      }
    for (auto& c : sh.coef) c /= std::sqrt(norm);
    sh.nfunc = sh.pure ? 2 * L + 1 : ncart(L);
    sh.first = nbf;
    nbf += sh.nfunc;
    cart_exponents(L, sh.ax, sh.ay, sh.az);
    sh.cartnorm.resize(ncart(L));
    for (int k = 0; k < ncart(L); ++k)  // Normalization.h:82-87 relative to (L,0,0)
      sh.cartnorm[k] = std::sqrt(dfact(2 * L - 1) / (dfact(2 * sh.ax[k] - 1) * dfact(2 * sh.ay[k] - 1) * dfact(2 * sh.az[k] - 1)));
    if (sh.pure) sh.sph = solid_harmonic_matrix(L);
    shells.push_back(sh);
  }
}

// Values (and derivatives) of every function of a block; screening as in
// BasisFunctionOnGridController.cpp:192-255, point loop :259-1097.
void block_on_grid(const Basis& B, const double* xyz, int npts, double thr, int deriv, double* val, double* grad,
                   double* hess, int* negligible) {
  const int nbf = B.nbf;
  std::memset(val, 0, sizeof(double) * npts * nbf);
  if (deriv >= 1) std::memset(grad, 0, sizeof(double) * 3 * npts * nbf);
  if (deriv >= 2) std::memset(hess, 0, sizeof(double) * 6 * npts * nbf);
  double c[3] = {0, 0, 0};
  for (int p = 0; p < npts; ++p)
    for (int k = 0; k < 3; ++k) c[k] += xyz[3 * p + k];
  for (int k = 0; k < 3; ++k) c[k] /= npts;
  double spread = 0.0;
  for (int p = 0; p < npts; ++p) {
    const double dx = xyz[3 * p] - c[0], dy = xyz[3 * p + 1] - c[1], dz = xyz[3 * p + 2] - c[2];
    spread = std::max(spread, std::sqrt(dx * dx + dy * dy + dz * dz));
  }
  for (int i = 0; i < nbf; ++i) negligible[i] = 0;
  for (const auto& sh : B.shells) {
    const double dx = c[0] - sh.O[0], dy = c[1] - sh.O[1], dz = c[2] - sh.O[2];
    double d = std::sqrt(dx * dx + dy * dy + dz * dz) - spread;
    if (d < 1.0) continue;
    d = d * d;
    double radial = 0.0;
    for (size_t q = 0; q < sh.alpha.size(); ++q) radial += sh.coef[q] * std::exp(-sh.alpha[q] * d);
    if (std::fabs(radial) < thr)
      for (int i = 0; i < sh.nfunc; ++i) negligible[sh.first + i] = 1;
  }
  const double expthr = -std::log(thr);
  std::vector<double> cv, cg, ch;
  for (int p = 0; p < npts; ++p) {
    for (const auto& sh : B.shells) {
      if (negligible[sh.first]) continue;
      const double x = xyz[3 * p] - sh.O[0], y = xyz[3 * p + 1] - sh.O[1], z = xyz[3 * p + 2] - sh.O[2];
      const double r2 = x * x + y * y + z * z;
      double R = 0.0, dR = 0.0, ddR = 0.0;
      for (size_t q = 0; q < sh.alpha.size(); ++q) {
        const double t = sh.alpha[q] * r2;
        if (t < expthr) {
          const double e = std::exp(-t);
          R += sh.coef[q] * e;
          dR -= 2.0 * sh.alpha[q] * sh.coef[q] * e;
          ddR += 4.0 * sh.alpha[q] * sh.alpha[q] * sh.coef[q] * e;
        }
      }
      if (std::fabs(R) < thr) continue;  // stays zero
      const int L = sh.l, nc = ncart(L);
      cv.assign(nc, 0.0);
      cg.assign(3 * nc, 0.0);
      ch.assign(6 * nc, 0.0);
      const double r[3] = {x, y, z};
      for (int k = 0; k < nc; ++k) {
        const int e[3] = {sh.ax[k], sh.ay[k], sh.az[k]};
        auto pw = [](double b, int n) { return n < 0 ? 0.0 : std::pow(b, n); };
        double mono = pw(x, e[0]) * pw(y, e[1]) * pw(z, e[2]);
        double dm[3], d2m[3][3];
        for (int a = 0; a < 3; ++a) {
          int f[3] = {e[0], e[1], e[2]};
          f[a] -= 1;
          dm[a] = e[a] == 0 ? 0.0 : e[a] * pw(x, f[0]) * pw(y, f[1]) * pw(z, f[2]);
          for (int b2 = 0; b2 < 3; ++b2) {
            int g[3] = {e[0], e[1], e[2]};
            double coef = 1.0;
            coef *= g[a]; g[a] -= 1;
            coef *= g[b2]; g[b2] -= 1;
            d2m[a][b2] = (coef == 0.0 || g[0] < 0 || g[1] < 0 || g[2] < 0) ? 0.0 : coef * pw(x, g[0]) * pw(y, g[1]) * pw(z, g[2]);
          }
        }
        cv[k] = mono * R;
        for (int a = 0; a < 3; ++a) cg[3 * k + a] = dm[a] * R + mono * dR * r[a];
        const int hi[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
        for (int h = 0; h < 6; ++h) {
          const int a = hi[h][0], b2 = hi[h][1];
          ch[6 * k + h] = d2m[a][b2] * R + dm[a] * dR * r[b2] + dm[b2] * dR * r[a] +
                          mono * (ddR * r[a] * r[b2] + (a == b2 ? dR : 0.0));
        }
      }
      for (int f = 0; f < sh.nfunc; ++f) {
        double v = 0.0, g3[3] = {0, 0, 0}, h6[6] = {0, 0, 0, 0, 0, 0};
        if (sh.pure) {
          for (int k = 0; k < nc; ++k) {
            const double t = sh.sph[f * nc + k];
            if (t == 0.0) continue;
            v += t * cv[k];
            for (int a = 0; a < 3; ++a) g3[a] += t * cg[3 * k + a];
            for (int h = 0; h < 6; ++h) h6[h] += t * ch[6 * k + h];
          }
        } else {
          const double t = sh.cartnorm[f];
          v = t * cv[f];
          for (int a = 0; a < 3; ++a) g3[a] = t * cg[3 * f + a];
          for (int h = 0; h < 6; ++h) h6[h] = t * ch[6 * f + h];
        }
        const long idx = (long)(sh.first + f) * npts + p;
        val[idx] = v;
        if (deriv >= 1)
          for (int a = 0; a < 3; ++a) grad[(long)a * npts * nbf + idx] = g3[a];
        if (deriv >= 2)
          for (int h = 0; h < 6; ++h) hess[(long)h * npts * nbf + idx] = h6[h];
      }
    }
  }
}

// Values (and, deriv = 1, gradients) of the block's non-negligible functions only, with
// the screening and cut-offs of block_on_grid: act[] receives their global indices in
// order, val[f * npts + p], grad[(3 f + k) * npts + p].  Monomials by repeated products
// and no Hessians: the lean form of the reference's per-l unrolled point loop
// (BasisFunctionOnGridController.cpp:259-1097) that the CPU baseline times.
int block_active(const Basis& B, const double* xyz, int npts, double thr, int deriv, int* act, double* val,
                 double* grad) {
  std::vector<int> negl(B.nbf);
  double c[3] = {0, 0, 0};
  for (int p = 0; p < npts; ++p)
    for (int k = 0; k < 3; ++k) c[k] += xyz[3 * p + k];
  for (int k = 0; k < 3; ++k) c[k] /= npts;
  double spread = 0.0;
  for (int p = 0; p < npts; ++p) {
    const double dx = xyz[3 * p] - c[0], dy = xyz[3 * p + 1] - c[1], dz = xyz[3 * p + 2] - c[2];
    spread = std::max(spread, std::sqrt(dx * dx + dy * dy + dz * dz));
  }
  const double expthr = -std::log(thr);
  int nact = 0;
  double mono[28], dmono[3][28];
  for (const auto& sh : B.shells) {
    const double dx = c[0] - sh.O[0], dy = c[1] - sh.O[1], dz = c[2] - sh.O[2];
    double d = std::sqrt(dx * dx + dy * dy + dz * dz) - spread;
    if (d >= 1.0) {
      d = d * d;
      double radial = 0.0;
      for (size_t q = 0; q < sh.alpha.size(); ++q) radial += sh.coef[q] * std::exp(-sh.alpha[q] * d);
      if (std::fabs(radial) < thr) continue;
    }
    const int f0 = nact;
    for (int i = 0; i < sh.nfunc; ++i) act[nact++] = sh.first + i;
    const int L = sh.l, nc = ncart(L), np = (int)sh.alpha.size();
    for (int p = 0; p < npts; ++p) {
      const double x = xyz[3 * p] - sh.O[0], y = xyz[3 * p + 1] - sh.O[1], z = xyz[3 * p + 2] - sh.O[2];
      const double r2 = x * x + y * y + z * z;
      double R = 0.0, dR = 0.0;
      for (int q = 0; q < np; ++q) {
        const double t = sh.alpha[q] * r2;
        if (t < expthr) {
          const double e = sh.coef[q] * std::exp(-t);
          R += e;
          dR -= 2.0 * sh.alpha[q] * e;
        }
      }
      if (std::fabs(R) < thr) {
        for (int f = 0; f < sh.nfunc; ++f) {
          val[(size_t)(f0 + f) * npts + p] = 0.0;
          if (deriv >= 1)
            for (int k = 0; k < 3; ++k) grad[((size_t)3 * (f0 + f) + k) * npts + p] = 0.0;
        }
        continue;
      }
      double px[8], py[8], pz[8];
      px[0] = py[0] = pz[0] = 1.0;
      for (int k = 1; k <= L; ++k) {
        px[k] = px[k - 1] * x;
        py[k] = py[k - 1] * y;
        pz[k] = pz[k - 1] * z;
      }
      for (int k = 0; k < nc; ++k) {
        const int a = sh.ax[k], b = sh.ay[k], cc = sh.az[k];
        mono[k] = px[a] * py[b] * pz[cc];
        if (deriv >= 1) {
          dmono[0][k] = a ? a * px[a - 1] * py[b] * pz[cc] : 0.0;
          dmono[1][k] = b ? b * px[a] * py[b - 1] * pz[cc] : 0.0;
          dmono[2][k] = cc ? cc * px[a] * py[b] * pz[cc - 1] : 0.0;
        }
      }
      const double r[3] = {x, y, z};
      for (int f = 0; f < sh.nfunc; ++f) {
        double s = 0.0, sd[3] = {0.0, 0.0, 0.0};
        if (sh.pure) {
          const double* T = &sh.sph[(size_t)f * nc];
          for (int k = 0; k < nc; ++k) {
            if (T[k] == 0.0) continue;
            s += T[k] * mono[k];
            if (deriv >= 1)
              for (int q = 0; q < 3; ++q) sd[q] += T[k] * dmono[q][k];
          }
        } else {
          s = sh.cartnorm[f] * mono[f];
          if (deriv >= 1)
            for (int q = 0; q < 3; ++q) sd[q] = sh.cartnorm[f] * dmono[q][f];
        }
        val[(size_t)(f0 + f) * npts + p] = s * R;
        if (deriv >= 1)
          for (int q = 0; q < 3; ++q) grad[((size_t)3 * (f0 + f) + q) * npts + p] = sd[q] * R + s * dR * r[q];
      }
    }
  }
  return nact;
}

/* ------------------------------------------------------------------------------------------ */
/* grids                                                                                      */

// Treutler-Ahlrichs alpha values for Z = 1..36 (AtomGridFactory.cpp:39-52).
static const double kAhlrichsAlpha[37] = {1.1, 0.8, 0.9, 1.8, 1.4, 1.3, 1.1, 0.9, 0.9, 0.9, 0.9, 1.4, 1.3,
                                          1.3, 1.2, 1.1, 1.0, 1.0, 1.0, 1.5, 1.4, 1.3, 1.2, 1.2, 1.2, 1.2,
                                          1.2, 1.2, 1.1, 1.1, 1.1, 1.1, 1.0, 0.9, 0.9, 0.9, 0.9};
// Clementi radii for Z = 1..36 (AtomGridFactory.cpp:53-62), used by the pruning zones.
static const double kClementi[37] = {1.00, 1.00, 0.59, 3.16, 2.12, 1.64, 1.27, 1.06, 0.91, 0.79, 0.72, 3.59, 2.74,
                                     2.23, 2.10, 1.85, 1.66, 1.49, 1.34, 4.59, 3.67, 3.48, 3.33, 3.23, 3.14, 3.04,
                                     2.95, 2.87, 2.82, 2.74, 2.68, 2.57, 2.36, 2.15, 1.95, 1.78, 1.66};
// Bragg-Slater radii in Angstrom for Z = 1..36 (AtomicParameters.h:454-462,
// hydrogen 0.25 A per AtomTypeFactory.cpp:105-108).  Only ratios enter.
static const double kBraggSlater[37] = {-1.0, 0.25, 1.20, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50, 0.38, 1.80, 1.50,
                                        1.25, 1.10, 1.00, 1.00, 1.00, 0.71, 2.20, 1.80, 1.60, 1.40, 1.35, 1.40, 1.40,
                                        1.40, 1.35, 1.35, 1.35, 1.35, 1.30, 1.25, 1.15, 1.15, 1.15, 0.88};

static int period_row(int Z) { return Z <= 2 ? 1 : Z <= 10 ? 2 : Z <= 18 ? 3 : Z <= 36 ? 4 : 5; }

void ahlrichs_radial(double alpha, int n, double* r, double* w) {
  for (int i = 1; i <= n; ++i) {
    const double log2 = std::log(2.0);
    const double tmp = alpha / log2;
    const double x = std::cos(i * M_PI / (n + 1.0));
    const double ri = tmp * std::pow(x + 1.0, 0.6) * std::log(2.0 / (1.0 - x));
    const double ln = std::log((1.0 - x) / 2.0);
    const double sq = std::sqrt((1.0 + x) / (1.0 - x));
    const double wi = (M_PI / (n + 1.0)) * std::pow(1.0 + x, 3 * 0.6) * tmp * tmp * tmp * (sq * ln * ln - 0.6 * ln * ln * ln / sq);
    w[n - i] = wi;
    r[n - i] = ri;
  }
}

struct Lebedev {
  std::map<int, std::vector<double>> rules;  // order -> x,y,z,w interleaved
  explicit Lebedev(const char* path) {
    std::ifstream f(path);
    std::string tok;
    int order = 0;
    while (f >> tok) {
      if (tok == "order") {
        f >> order;
        auto& v = rules[order];
        v.resize(4 * order);
        for (int i = 0; i < 4 * order; ++i) f >> v[i];
      }
    }
  }
};

static const int kLebedevOrders[18] = {6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302, 350, 434, 590, 770};

// one atom's reference grid (not yet shifted)
static void atom_grid(const Lebedev& leb, int Z, int n_rad, int n_ang, int acc, std::vector<double>& pts,
                      std::vector<double>& w) {
  const double alpha = kAhlrichsAlpha[Z];
  const int row = period_row(Z);
  int nr = n_rad;
  if (acc > 0) {
    static const int radAcc[7] = {13, 13, 13, 14, 15, 16, 17};
    nr = (int)(5.0 * (radAcc[acc - 1] + row - 8));
  }
  std::vector<double> r(nr), rw(nr);
  ahlrichs_radial(alpha, nr, r.data(), rw.data());
  static const int ldval[7][5] = {{4, 4, 4, 4, 4},     {4, 4, 4, 7, 4},      {4, 4, 7, 10, 7},    {4, 7, 10, 13, 10},
                                  {7, 10, 13, 15, 13}, {10, 13, 15, 16, 15}, {13, 15, 16, 17, 16}};
  static const double ranges[3][4] = {{0.25, 0.5, 1.0, 4.5}, {0.1667, 0.5, 0.9, 3.5}, {0.1, 0.4, 0.8, 2.5}};
  const int zrow = (row > 3) ? 2 : row - 1;
  const int redp1 = (row == 1 && acc > 1) ? 2 : 1;
  double rr[4];
  for (int i = 0; i < 4; ++i) rr[i] = ranges[zrow][i] * kClementi[Z];
  int sphAcc = 0;
  for (int i = 0; i < nr; ++i) {
    int order = n_ang;
    if (acc > 0) {
      if (sphAcc < 4)
        if (r[i] > rr[sphAcc]) ++sphAcc;
      order = kLebedevOrders[ldval[acc - redp1][sphAcc]];
    }
    const auto& rule = leb.rules.at(order);
    for (int k = 0; k < order; ++k) {
      w.push_back(rule[4 * k + 3] * rw[i] * 4.0 * M_PI);
      pts.push_back(rule[4 * k + 0] * r[i]);
      pts.push_back(rule[4 * k + 1] * r[i]);
      pts.push_back(rule[4 * k + 2] * r[i]);
    }
  }
}

static double becke_p(double nu, int k) {  // GridFactory.cpp:324-340
  for (int i = 0; i < k; ++i) nu = (3.0 - nu * nu) * nu / 2.0;
  return nu;
}

void hilbert_sort(std::vector<double>& pts, std::vector<double>& w) {
  const long n = (long)w.size();
  int depth = 1;
  long length = 2, nvert = 8;
  while (n * 8 > nvert) {
    depth += 1;
    length *= 2;
    nvert *= 8;
  }
  double mn[3], spread[3];
  for (int k = 0; k < 3; ++k) {
    double lo = 1e300, hi = -1e300;
    for (long i = 0; i < n; ++i) {
      lo = std::min(lo, pts[3 * i + k]);
      hi = std::max(hi, pts[3 * i + k]);
    }
    mn[k] = lo;
    spread[k] = double(length) / (hi - lo);
  }
  static const int trans[8][8] = {{0, 7, 6, 1, 2, 5, 4, 3}, {0, 3, 4, 6, 7, 5, 2, 1}, {0, 3, 4, 6, 7, 5, 2, 1},
                                  {2, 3, 0, 1, 6, 7, 4, 5}, {2, 3, 0, 1, 6, 7, 4, 5}, {6, 5, 2, 1, 0, 3, 4, 7},
                                  {6, 5, 2, 1, 0, 3, 4, 7}, {4, 3, 2, 5, 6, 1, 0, 7}};
  static const int val[2][2][2] = {{{5, 6}, {4, 7}}, {{2, 1}, {3, 0}}};
  std::vector<long> key(n);
  for (long i = 0; i < n; ++i) {
    int pt[3];
    for (int k = 0; k < 3; ++k) pt[k] = int((pts[3 * i + k] - mn[k]) * spread[k]);
    int l = (int)(length / 2);
    int gx = pt[0] > l, gy = pt[1] > l, gz = pt[2] > l;
    int v = val[gx][gy][gz];
    long idx = v;
    while (l > 1) {
      idx *= 8;
      if (gx) pt[0] -= l;
      if (gy) pt[1] -= l;
      if (gz) pt[2] -= l;
      l /= 2;
      gx = pt[0] > l; gy = pt[1] > l; gz = pt[2] > l;
      v = trans[v][val[gx][gy][gz]];
      idx += v;
    }
    key[i] = idx;
  }
  // descending Hilbert index; equal keys keep their input order (the reference's
  // single-thread selection order, HilbertRTreeSorting.cpp:121-133)
  std::vector<long> order(n);
  for (long i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](long a, long b) { return key[a] > key[b]; });
  std::vector<double> p2(3 * n), w2(n);
  for (long i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) p2[3 * i + k] = pts[3 * order[i] + k];
    w2[i] = w[order[i]];
  }
  pts.swap(p2);
  w.swap(w2);
}

// Stratmann-Scuseria-Frisch weight of a point of atom k (GridFactory.cpp:209-268): untouched
// inside 0.5 (1 - a) of the nearest-neighbour distance, zero once some nu_kj >= a, otherwise
// the cell products with the piecewise polynomial of SSF Eq. (14), a = 0.64, no size
// adjustment, over all atoms.  Returns false when the point is screened out.
static bool ssf_weight(int natoms, int k, const std::vector<double>& rd, const std::vector<double>& dist,
                       double min_dist, double& weight) {
  constexpr double a = 0.64;
  if (!(rd[k] >= 0.5 * (1.0 - a) * min_dist)) return true;
  for (int j = 0; j < natoms; ++j) {
    const double nu = (rd[k] - rd[j]) / dist[k + natoms * j];  // j == k: 0/0, compares false
    if (nu >= a) return false;
  }
  double sum = 0.0;
  for (int i = 0; i < natoms; ++i) {
    double cell = 1.0;
    for (int j = 0; j < natoms; ++j) {
      if (i == j) continue;
      double nu = (rd[i] - rd[j]) / dist[i + natoms * j];
      if (nu <= -a) continue;
      if (nu >= a) {
        cell = 0.0;
        break;
      }
      nu /= a;
      const double n3 = nu * nu * nu;
      const double poly = (-5.0 * n3 * n3 * nu + 21.0 * n3 * nu * nu - 35.0 * n3 + 35.0 * nu) / 16.0;
      cell *= 0.5 * (1 - poly);
    }
    if (i == k) weight *= cell;
    sum += cell;
  }
  weight /= sum;
  return true;
}

long becke_grid(int natoms, const int* Z, const double* xyz, int n_rad, int n_ang, int acc, double wthr, int smoothing,
                int sort, const char* lebedev_path, std::vector<double>& outp, std::vector<double>& outw, int partition) {
  Lebedev leb(lebedev_path);
  std::vector<double> dist(natoms * natoms);
  for (int i = 0; i < natoms; ++i)
    for (int j = 0; j < natoms; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += (xyz[3 * i + k] - xyz[3 * j + k]) * (xyz[3 * i + k] - xyz[3 * j + k]);
      dist[i + natoms * j] = std::sqrt(s);
    }
  // size adjustments, GridFactory.cpp:84-110 (column-major a(j, i), chi = sqrt(R_j / R_i))
  std::vector<double> a(natoms * natoms);
  for (int i = 0; i < natoms; ++i)
    for (int j = 0; j < natoms; ++j) {
      const double q = std::sqrt(kBraggSlater[Z[j]] / kBraggSlater[Z[i]]);
      const double u = (q - 1) / (q + 1);
      double v = u / (u * u - 1);
      v = std::min(0.5, std::max(-0.5, v));
      a[j + natoms * i] = v;
    }
  std::vector<std::vector<double>> apts(natoms), aw(natoms);
#pragma omp parallel for schedule(dynamic)
  for (int k = 0; k < natoms; ++k) {
    std::vector<double> rp, rw;
    atom_grid(leb, Z[k], n_rad, n_ang, acc, rp, rw);
    std::vector<int> sig;
    double min_dist = 999999999.9;
    for (int l = 0; l < natoms; ++l) {
      if (dist[l + natoms * k] < 40.0) sig.push_back(l);
      if (l != k) min_dist = std::min(min_dist, dist[l + natoms * k]);
    }
    std::vector<double> rd(natoms);
    for (size_t i = 0; i < rw.size(); ++i) {
      const double g[3] = {rp[3 * i] + xyz[3 * k], rp[3 * i + 1] + xyz[3 * k + 1], rp[3 * i + 2] + xyz[3 * k + 2]};
      double weight = rw[i];
      for (int l = 0; l < natoms; ++l) {
        double s = 0;
        for (int c = 0; c < 3; ++c) s += (xyz[3 * l + c] - g[c]) * (xyz[3 * l + c] - g[c]);
        rd[l] = std::sqrt(s);
      }
      if (partition == 1) {
        if (!ssf_weight(natoms, k, rd, dist, min_dist, weight)) continue;
      } else {
        double sum = 0.0;
        for (int l : sig) {
          double cell = 1.0;
          for (int j : sig) {
            if (l == j) continue;
            const double mu = (rd[l] - rd[j]) / dist[l + natoms * j];
            const double nu = mu + a[j + natoms * l] * (1.0 - mu * mu);
            cell *= 0.5 * (1 - becke_p(nu, smoothing));
          }
          if (l == k) weight *= cell;
          sum += cell;
        }
        weight /= sum;
      }
      if (weight > wthr) {
        aw[k].push_back(weight);
        apts[k].insert(apts[k].end(), g, g + 3);
      }
    }
  }
  outp.clear();
  outw.clear();
  for (int k = 0; k < natoms; ++k) {
    outp.insert(outp.end(), apts[k].begin(), apts[k].end());
    outw.insert(outw.end(), aw[k].begin(), aw[k].end());
  }
  if (sort) hilbert_sort(outp, outw);
  return (long)outw.size();
}

}  // namespace orc

extern "C" {

void* orc_basis_create(int nshell, const int* l, const int* pure, const int* nprim, const double* centers,
                       const double* alpha, const double* coef) {
  return new orc::Basis(nshell, l, pure, nprim, centers, alpha, coef);
}
void orc_basis_free(void* b) { delete static_cast<orc::Basis*>(b); }
int orc_basis_nbf(const void* b) { return static_cast<const orc::Basis*>(b)->nbf; }
void orc_basis_shell_coefs(const void* b, int s, double* out) {
  const auto& sh = static_cast<const orc::Basis*>(b)->shells[s];
  for (size_t i = 0; i < sh.coef.size(); ++i) out[i] = sh.coef[i];
}

int orc_block_on_grid(const void* basis, const double* xyz, int npts, double thr, int deriv, double* values,
                      double* grad, double* hess, int* negligible) {
  orc::block_on_grid(*static_cast<const orc::Basis*>(basis), xyz, npts, thr, deriv, values, grad, hess, negligible);
  return 0;
}

long orc_becke_grid(int natoms, const int* Z, const double* xyz, int n_rad, int n_ang, int accuracy,
                    double weight_threshold, int smoothing, int sort, const char* lebedev_path, double* out_xyz,
                    double* out_w, long capacity, int partition) {
  std::vector<double> p, w;
  long n = orc::becke_grid(natoms, Z, xyz, n_rad, n_ang, accuracy, weight_threshold, smoothing, sort, lebedev_path, p, w,
                           partition);
  if (n > capacity) return -1;
  std::memcpy(out_xyz, p.data(), sizeof(double) * 3 * n);
  std::memcpy(out_w, w.data(), sizeof(double) * n);
  return n;
}

void orc_ahlrichs_radial(double alpha, int n, double* r, double* w) { orc::ahlrichs_radial(alpha, n, r, w); }

void orc_solid_harmonics(int l, double x, double y, double z, double* out) {
  auto T = orc::solid_harmonic_matrix(l);
  std::vector<int> ax, ay, az;
  orc::cart_exponents(l, ax, ay, az);
  const int nc = orc::ncart(l);
  for (int m = 0; m < 2 * l + 1; ++m) {
    double s = 0;
    for (int k = 0; k < nc; ++k) s += T[m * nc + k] * std::pow(x, ax[k]) * std::pow(y, ay[k]) * std::pow(z, az[k]);
    out[m] = s;
  }
}

}  // extern "C"
