/*
 * ORACLE -- test infrastructure only (see oracle.h).
 *
 * Density on the grid, functional evaluation over blocks, the scalar-operator
 * adder and the whole XC build, restated from the reference:
 *   MatrixOperatorToGridTransformer.cpp:37-198   (rho = rowsum((phi P_b) o phi),
 *                                                 grad rho = 2 rowsum((phi P_b) o grad phi))
 *   XCFun.cpp:39-158, 751-765                    (block skip, GRADIENTS outputs, E_xc)
 *   ScalarOperatorToMatrixAdder.cpp:51-113,178-303 (per-thread matrices, block
 *                                                 thresholds, F_b = tmp + tmp^T)
 *   FuncPotential.cpp:74-110                     (the wiring: FunctionalLibrary(128),
 *                                                 LDA -> scalar adder, GGA -> gradient adder)
 * The three phases run one after the other over all blocks, with the basis
 * evaluated again in the adder phase, as the reference does.
 */
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle_internal.h"

namespace orc {

// Basis data of one block restricted to its non-negligible functions:
// phi[f*npts + p], grad[(3*f + k)*npts + p]; idx[f] = global function index.
struct ActiveBlock {
  int npts = 0, nact = 0;
  std::vector<int> idx;
  std::vector<double> phi, grad;
};

static void eval_active(const Basis& B, const double* xyz, int npts, double thr, int deriv, ActiveBlock& out) {
  const int nbf = B.nbf;
  out.idx.resize(nbf);
  out.phi.resize((size_t)nbf * npts);
  if (deriv >= 1) out.grad.resize((size_t)3 * nbf * npts);
  out.npts = npts;
  out.nact = block_active(B, xyz, npts, thr, deriv, out.idx.data(), out.phi.data(), deriv >= 1 ? out.grad.data() : nullptr);
  out.idx.resize(out.nact);
}

// C (m x n, row stride ldc) = A (m x k, row stride lda) B (k x n, row stride ldb), all
// row-major, m a multiple of 4 and n of 8 (callers pad with zeros).  Register tiles of
// 4 x 8 accumulators over the whole k, the 8-wide rows of B contiguous: the per-block
// GEMMs of the reference's Eigen path (MatrixOperatorToGridTransformer.cpp:131-146,
// ScalarOperatorToMatrixAdder.cpp:224-303) in portable, auto-vectorised C++.
static void gemm_nn(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc) {
  for (int j0 = 0; j0 < n; j0 += 8)
    for (int i0 = 0; i0 < m; i0 += 4) {
      double acc[4][8] = {};
      const double* a0 = A + (size_t)i0 * lda;
      for (int kk = 0; kk < k; ++kk) {
        const double* b = B + (size_t)kk * ldb + j0;
        for (int i = 0; i < 4; ++i) {
          const double a = a0[(size_t)i * lda + kk];
          for (int j = 0; j < 8; ++j) acc[i][j] += a * b[j];
        }
      }
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) C[(size_t)(i0 + i) * ldc + j0 + j] = acc[i][j];
    }
}

static inline int pad4(int x) { return (x + 3) & ~3; }
static inline int pad8(int x) { return (x + 7) & ~7; }

// X = P_b Phi (P_b the block's active rows and columns of P, symmetric), then
// rho = rowsum(X o Phi), grad rho = 2 rowsum(X o grad Phi)
static void density_block(const ActiveBlock& A, int nbf, const double* P, double* rho, double* grad, long gstride) {
  const int n = A.npts, m = A.nact;
  if (m == 0) {
    for (int p = 0; p < n; ++p) rho[p] = 0.0;
    if (grad)
      for (int k = 0; k < 3; ++k)
        for (int p = 0; p < n; ++p) grad[k * gstride + p] = 0.0;
    return;
  }
  const int mp = pad4(m), np = pad8(n);
  std::vector<double> Pb((size_t)mp * m, 0.0), Ph((size_t)m * np, 0.0), X((size_t)mp * np);
  for (int nu = 0; nu < m; ++nu) {
    const double* Pcol = P + (size_t)A.idx[nu] * nbf;
    for (int mu = 0; mu < m; ++mu) Pb[(size_t)nu * m + mu] = Pcol[A.idx[mu]];
    std::memcpy(&Ph[(size_t)nu * np], &A.phi[(size_t)nu * n], sizeof(double) * n);
  }
  gemm_nn(mp, np, m, Pb.data(), m, Ph.data(), np, X.data(), np);
  for (int p = 0; p < n; ++p) rho[p] = 0.0;
  for (int nu = 0; nu < m; ++nu) {
    const double* x = &X[(size_t)nu * np];
    const double* ph = &A.phi[(size_t)nu * n];
    for (int p = 0; p < n; ++p) rho[p] += x[p] * ph[p];
  }
  if (grad) {
    for (int k = 0; k < 3; ++k) {
      double* g = grad + k * gstride;
      for (int p = 0; p < n; ++p) g[p] = 0.0;
      for (int nu = 0; nu < m; ++nu) {
        const double* x = &X[(size_t)nu * np];
        const double* gp = &A.grad[((size_t)3 * nu + k) * n];
        for (int p = 0; p < n; ++p) g[p] += x[p] * gp[p];
      }
      for (int p = 0; p < n; ++p) g[p] *= 2.0;
    }
  }
}

// adds the block's contribution of one spin into F (nbf x nbf, column-major):
// tmp = Phi^T G by one GEMM over the block's points, F_b = tmp (LDA, G = w v Phi) or
// tmp + tmp^T (GGA, G = w (v/2 Phi + g . grad Phi))
static void adder_block(const ActiveBlock& A, int nbf, const double* wv, const double* wg /*3*npts or null*/,
                        double* F) {
  const int n = A.npts, m = A.nact;
  if (m == 0) return;
  const int mp4 = pad4(m), mp8 = pad8(m);
  std::vector<double> Ph((size_t)mp4 * n, 0.0), GT((size_t)n * mp8, 0.0), T((size_t)mp4 * mp8);
  for (int f = 0; f < m; ++f) {
    const double* ph = &A.phi[(size_t)f * n];
    std::memcpy(&Ph[(size_t)f * n], ph, sizeof(double) * n);
    if (wg) {
      const double* gx = &A.grad[((size_t)3 * f + 0) * n];
      const double* gy = &A.grad[((size_t)3 * f + 1) * n];
      const double* gz = &A.grad[((size_t)3 * f + 2) * n];
      for (int p = 0; p < n; ++p)
        GT[(size_t)p * mp8 + f] = wg[p] * gx[p] + wg[n + p] * gy[p] + wg[2 * n + p] * gz[p] + 0.5 * wv[p] * ph[p];
    } else {
      for (int p = 0; p < n; ++p) GT[(size_t)p * mp8 + f] = wv[p] * ph[p];
    }
  }
  gemm_nn(mp4, mp8, n, Ph.data(), n, GT.data(), mp8, T.data(), mp8);
  for (int a = 0; a < m; ++a) {
    double* Fcol = F + (size_t)A.idx[a] * nbf;
    const double* t = &T[(size_t)a * mp8];
    if (wg) {
      for (int b = 0; b < m; ++b) {
        Fcol[A.idx[b]] += t[b];
        F[(size_t)A.idx[b] * nbf + A.idx[a]] += t[b];
      }
    } else {
      for (int b = 0; b < m; ++b) Fcol[A.idx[b]] += t[b];
    }
  }
}

static int block_size(long b, long nblocks, long npts, int maxb) {
  if (b == nblocks - 1) {
    int r = (int)(npts % maxb);
    return r == 0 ? maxb : r;
  }
  return maxb;
}

static void add_scalar(const Basis& B, const double* xyz, const double* w, long npts, int maxb, double thr,
                       double ave_thr, int nspin, const double* v, const double* g, double* F) {
  const int nbf = B.nbf;
  const long nblocks = (npts + maxb - 1) / maxb;
  const int nthreads = omp_get_max_threads();
  std::vector<std::vector<double>> Ft(nthreads, std::vector<double>((size_t)nspin * nbf * nbf, 0.0));
#pragma omp parallel
  {
    ActiveBlock A;
    std::vector<double> wv, wg;
    double* myF = Ft[omp_get_thread_num()].data();
#pragma omp for schedule(dynamic)
    for (long b = 0; b < nblocks; ++b) {
      const long first = b * maxb;
      const int n = block_size(b, nblocks, npts, maxb);
      eval_active(B, xyz + 3 * first, n, thr, g ? 1 : 0, A);
      for (int s = 0; s < nspin; ++s) {
        wv.resize(n);
        double ave = 0.0;
        for (int p = 0; p < n; ++p) {
          wv[p] = v[s * npts + first + p] * w[first + p];
          ave += std::fabs(wv[p]);
        }
        if (g) {
          wg.resize(3 * n);
          for (int k = 0; k < 3; ++k)
            for (int p = 0; p < n; ++p) {
              wg[k * n + p] = w[first + p] * g[(s * 3 + k) * npts + first + p];
              ave += std::fabs(wg[k * n + p]);
            }
        }
        if (ave / n < ave_thr) continue;
        adder_block(A, nbf, wv.data(), g ? wg.data() : nullptr, myF + (size_t)s * nbf * nbf);
      }
    }
  }
  for (auto& m : Ft)
    for (size_t i = 0; i < m.size(); ++i) F[i] += m[i];
}

static void density(const Basis& B, const double* xyz, long npts, int maxb, double thr, int nspin, const double* P,
                    double* rho, double* grad) {
  const int nbf = B.nbf;
  const long nblocks = (npts + maxb - 1) / maxb;
#pragma omp parallel
  {
    ActiveBlock A;
#pragma omp for schedule(dynamic)
    for (long b = 0; b < nblocks; ++b) {
      const long first = b * maxb;
      const int n = block_size(b, nblocks, npts, maxb);
      eval_active(B, xyz + 3 * first, n, thr, 1, A);
      for (int s = 0; s < nspin; ++s)
        density_block(A, nbf, P + (size_t)s * nbf * nbf, rho + s * npts + first,
                      grad ? grad + (size_t)s * 3 * npts + first : nullptr, npts);
    }
  }
}

static void functional(int func, int nspin, long npts, int maxb, const double* rho, const double* grad, double* epuv,
                       double* dfdrho, double* dfdgrad) {
  const bool gga = functional_is_gga(func);
  const long blk = maxb > 0 ? maxb : npts;
  const long nblocks = (npts + blk - 1) / blk;
#pragma omp parallel for schedule(dynamic)
  for (long b = 0; b < nblocks; ++b) {
    const long first = b * blk;
    const long n = std::min(blk, npts - first);
    bool skip = maxb > 0;
    for (int s = 0; s < nspin && skip; ++s) {
      double sum = 0.0;
      for (long p = 0; p < n; ++p) sum += std::fabs(rho[s * npts + first + p]);
      skip = skip && (sum < n * 1e-12);
    }
    for (long p = first; p < first + n; ++p) {
      double in[8] = {0, 0, 0, 0, 0, 0, 0, 0}, out[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      if (!skip) {
        if (nspin == 1) {
          in[0] = rho[p];
          if (gga)
            for (int k = 0; k < 3; ++k) in[1 + k] = grad[k * npts + p];
        } else {
          in[0] = rho[p];
          in[1] = rho[npts + p];
          if (gga)
            for (int k = 0; k < 3; ++k) {
              in[2 + k] = grad[k * npts + p];
              in[5 + k] = grad[(3 + k) * npts + p];
            }
        }
        functional_point(func, nspin, in, out);
      }
      epuv[p] = out[0];
      if (nspin == 1) {
        dfdrho[p] = out[1];
        if (gga && dfdgrad)
          for (int k = 0; k < 3; ++k) dfdgrad[k * npts + p] = out[2 + k];
      } else {
        dfdrho[p] = out[1];
        dfdrho[npts + p] = out[2];
        if (gga && dfdgrad)
          for (int k = 0; k < 3; ++k) {
            dfdgrad[k * npts + p] = out[3 + k];
            dfdgrad[(3 + k) * npts + p] = out[6 + k];
          }
      }
    }
  }
}

// XC contribution to the nuclear gradient, FuncPotential<M>::getGeomGradients
// (FuncPotential.cpp:113-241), loop for loop: per block and pair (mu, nu) of
// non-negligible functions, the atom of nu collects
//   -2 P_mu,nu sum_p w v phi_mu d_k phi_nu
//   -2 P_mu,nu sum_p w sum_j g_j (phi_mu d_j d_k phi_nu + d_j phi_mu d_k phi_nu)   (GGA)
// per spin (restricted: the total density and its potential).  No weight derivatives,
// as in the reference.  out: natoms x 3, column-major (atom + natoms * k).
static void xc_gradient(const Basis& B, const int* shell_atom, int natoms, const double* xyz, const double* w,
                        long npts, int maxb, double thr, int func, int nspin, const double* P, double* out) {
  const int nbf = B.nbf;
  const bool gga = functional_is_gga(func);
  std::vector<int> fatom(nbf);
  for (size_t s = 0; s < B.shells.size(); ++s)
    for (int f = 0; f < B.shells[s].nfunc; ++f) fatom[B.shells[s].first + f] = shell_atom[s];
  std::vector<double> rho((size_t)nspin * npts), grad(gga ? (size_t)nspin * 3 * npts : 0);
  density(B, xyz, npts, maxb, thr, nspin, P, rho.data(), gga ? grad.data() : nullptr);
  std::vector<double> epuv(npts), v((size_t)nspin * npts), g(gga ? (size_t)nspin * 3 * npts : 0);
  functional(func, nspin, npts, 128, rho.data(), gga ? grad.data() : nullptr, epuv.data(), v.data(),
             gga ? g.data() : nullptr);
  const long nblocks = (npts + maxb - 1) / maxb;
  const int nthreads = omp_get_max_threads();
  std::vector<std::vector<double>> Gt(nthreads, std::vector<double>((size_t)3 * natoms, 0.0));
#pragma omp parallel
  {
    std::vector<double> val, gr, he;
    std::vector<int> negl(nbf);
    double* G = Gt[omp_get_thread_num()].data();
#pragma omp for schedule(dynamic)
    for (long b = 0; b < nblocks; ++b) {
      const long first = b * maxb;
      const int n = block_size(b, nblocks, npts, maxb);
      val.assign((size_t)n * nbf, 0.0);
      gr.assign((size_t)3 * n * nbf, 0.0);
      he.assign(gga ? (size_t)6 * n * nbf : 0, 0.0);
      block_on_grid(B, xyz + 3 * first, n, thr, gga ? 2 : 1, val.data(), gr.data(), gga ? he.data() : nullptr,
                    negl.data());
      auto phi = [&](int mu, int p) { return val[(size_t)mu * n + p]; };
      auto d = [&](int k, int mu, int p) { return gr[(size_t)k * n * nbf + (size_t)mu * n + p]; };
      // Hessian component of the pair (j, k): xx xy xz yy yz zz
      static const int hc[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
      auto dd = [&](int j, int k, int mu, int p) { return he[(size_t)hc[j][k] * n * nbf + (size_t)mu * n + p]; };
      for (int s = 0; s < nspin; ++s) {
        const double* Ps = P + (size_t)s * nbf * nbf;
        for (int mu = 0; mu < nbf; ++mu) {
          if (negl[mu]) continue;
          for (int nu = 0; nu < nbf; ++nu) {
            if (negl[nu]) continue;
            const double pref = 2.0 * Ps[(size_t)nu * nbf + mu];  // P(mu, nu), column-major
            const int A = fatom[nu];
            for (int k = 0; k < 3; ++k) {
              double t = 0.0;
              for (int p = 0; p < n; ++p) t += w[first + p] * v[s * npts + first + p] * phi(mu, p) * d(k, nu, p);
              G[A + natoms * k] -= pref * t;
            }
            if (gga) {
              for (int k = 0; k < 3; ++k) {
                double t = 0.0;
                for (int j = 0; j < 3; ++j)
                  for (int p = 0; p < n; ++p)
                    t += w[first + p] * g[((size_t)s * 3 + j) * npts + first + p] *
                         (phi(mu, p) * dd(j, k, nu, p) + d(j, mu, p) * d(k, nu, p));
                G[A + natoms * k] -= pref * t;
              }
            }
          }
        }
      }
    }
  }
  for (int i = 0; i < 3 * natoms; ++i) {
    out[i] = 0.0;
    for (auto& t : Gt) out[i] += t[i];
  }
}

}  // namespace orc

extern "C" {

int orc_density(const void* basis, const double* xyz, long npts, int max_block, double thr, int nspin, const double* P,
                double* rho, double* grad) {
  orc::density(*static_cast<const orc::Basis*>(basis), xyz, npts, max_block, thr, nspin, P, rho, grad);
  return 0;
}

int orc_functional(int func, int nspin, long npts, int max_block, const double* rho, const double* grad, double* epuv,
                   double* dfdrho, double* dfdgrad) {
  orc::functional(func, nspin, npts, max_block, rho, grad, epuv, dfdrho, dfdgrad);
  return 0;
}

int orc_functional_is_gga(int func) { return orc::functional_is_gga(func) ? 1 : 0; }

long orc_active_functions(const void* basis, const double* xyz, long npts, int max_block, double thr) {
  const orc::Basis& B = *static_cast<const orc::Basis*>(basis);
  const long nblocks = (npts + max_block - 1) / max_block;
  long total = 0;
#pragma omp parallel reduction(+ : total)
  {
    std::vector<int> act(B.nbf);
    std::vector<double> val;
#pragma omp for schedule(dynamic)
    for (long b = 0; b < nblocks; ++b) {
      const long first = b * max_block;
      const int n = (int)std::min((long)max_block, npts - first);
      val.resize((size_t)B.nbf * n);
      total += orc::block_active(B, xyz + 3 * first, n, thr, 0, act.data(), val.data(), nullptr);
    }
  }
  return total;
}

int orc_add_scalar(const void* basis, const double* xyz, const double* w, long npts, int max_block, double thr,
                   double ave_thr, int nspin, const double* v, const double* g, double* F) {
  orc::add_scalar(*static_cast<const orc::Basis*>(basis), xyz, w, npts, max_block, thr, ave_thr, nspin, v, g, F);
  return 0;
}

int orc_vxc(const void* basis, const double* xyz, const double* w, long npts, int max_block, double thr,
            double ave_thr, int func, int nspin, const double* P, double* V, double* Exc, double* Nel, int threads) {
  const orc::Basis& B = *static_cast<const orc::Basis*>(basis);
  const int saved = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
  const bool gga = orc::functional_is_gga(func);
  std::vector<double> rho((size_t)nspin * npts), grad(gga ? (size_t)nspin * 3 * npts : 0);
  orc::density(B, xyz, npts, max_block, thr, nspin, P, rho.data(), gga ? grad.data() : nullptr);
  std::vector<double> epuv(npts), dfdrho((size_t)nspin * npts), dfdgrad(gga ? (size_t)nspin * 3 * npts : 0);
  // FunctionalLibrary(128): the functional's block size is fixed at 128 (FuncPotential.cpp:86)
  orc::functional(func, nspin, npts, 128, rho.data(), gga ? grad.data() : nullptr, epuv.data(), dfdrho.data(),
                  gga ? dfdgrad.data() : nullptr);
  double e = 0.0, ne = 0.0;
#pragma omp parallel for reduction(+ : e, ne)
  for (long p = 0; p < npts; ++p) {
    e += epuv[p] * w[p];
    double r = 0.0;
    for (int s = 0; s < nspin; ++s) r += rho[s * npts + p];
    ne += r * w[p];
  }
  const int nbf = B.nbf;
  std::memset(V, 0, sizeof(double) * nspin * nbf * nbf);
  orc::add_scalar(B, xyz, w, npts, max_block, thr, ave_thr, nspin, dfdrho.data(), gga ? dfdgrad.data() : nullptr, V);
  *Exc = e;
  *Nel = ne;
  if (threads > 0) omp_set_num_threads(saved);
  return 0;
}

}  // extern "C"

extern "C" int orc_xc_gradient(const void* basis, const int* shell_atom, int natoms, const double* xyz,
                               const double* w, long npts, int max_block, double thr, int func, int nspin,
                               const double* P, double* out) {
  orc::xc_gradient(*static_cast<const orc::Basis*>(basis), shell_atom, natoms, xyz, w, npts, max_block, thr, func,
                   nspin, P, out);
  return 0;
}

// Restricted linear-response kernel on points (KernelSigmavector<RESTRICTED> singlet
// contraction before the numerical integration): blocks of 128 points whose ground-state
// density sums below 128e-12 give zero (the functional data's block skip); grad0/grad1
// are [3][npts] (GGA only), g1 [3][npts].
extern "C" int orc_lr_kernel(int func, long npts, const double* rho0, const double* grad0, const double* rho1,
                             const double* grad1, double* v1, double* g1) {
  const bool gga = orc::functional_is_gga(func);
#pragma omp parallel for schedule(static)
  for (long b = 0; b < (npts + 127) / 128; ++b) {
    const long first = b * 128, n = std::min<long>(128, npts - first);
    double sum = 0.0;
    for (long p = first; p < first + n; ++p) sum += std::fabs(rho0[p]);
    const bool skip = sum < n * 1e-12;
    for (long p = first; p < first + n; ++p) {
      double a0[3] = {0, 0, 0}, a1[3] = {0, 0, 0}, out[3] = {0, 0, 0};
      double v = 0.0;
      if (!skip) {
        if (gga)
          for (int k = 0; k < 3; ++k) {
            a0[k] = grad0[k * npts + p];
            a1[k] = grad1[k * npts + p];
          }
        orc::lr_kernel_point(func, rho0[p], a0, rho1[p], a1, &v, out);
      }
      v1[p] = v;
      if (gga)
        for (int k = 0; k < 3; ++k) g1[k * npts + p] = out[k];
    }
  }
  return 0;
}


// The spin-resolved kernel contraction on points, the layout of the GPU's: kind 2
// (unrestricted) rho0, rho1 [2][n], grad0, grad1 [2][3][n], v1 [2][n], g1 [2][3][n];
// kind 1 (triplet) rho0, grad0 the restricted total density (each spin half), rho1, grad1
// one perturbation taken as (+, -), v1 [n], g1 [3][n] the alpha parts.  Blocks of 128
// points whose spin densities all sum below n 1e-12 give zero (XCFun.cpp:136-140).
extern "C" int orc_lr_kernel_spin(int func, int kind, long npts, const double* rho0, const double* grad0,
                                  const double* rho1, const double* grad1, double* v1, double* g1) {
  const bool gga = orc::functional_is_gga(func), trip = kind == 1;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < (npts + 127) / 128; ++b) {
    const long first = b * 128, n = std::min<long>(128, npts - first);
    double sa = 0.0, sb = 0.0;
    for (long p = first; p < first + n; ++p) {
      sa += std::fabs(trip ? 0.5 * rho0[p] : rho0[p]);
      sb += std::fabs(trip ? 0.5 * rho0[p] : rho0[npts + p]);
    }
    const bool skip = sa < n * 1e-12 && sb < n * 1e-12;
    for (long p = first; p < first + n; ++p) {
      double n0[2], n1[2], a0[6] = {0, 0, 0, 0, 0, 0}, a1[6] = {0, 0, 0, 0, 0, 0}, v[2] = {0, 0},
                               out[6] = {0, 0, 0, 0, 0, 0};
      if (!skip) {
        n0[0] = trip ? 0.5 * rho0[p] : rho0[p];
        n0[1] = trip ? n0[0] : rho0[npts + p];
        n1[0] = rho1[p];
        n1[1] = trip ? -n1[0] : rho1[npts + p];
        if (gga)
          for (int k = 0; k < 3; ++k) {
            a0[k] = trip ? 0.5 * grad0[k * npts + p] : grad0[k * npts + p];
            a0[3 + k] = trip ? a0[k] : grad0[(3 + k) * npts + p];
            a1[k] = grad1[k * npts + p];
            a1[3 + k] = trip ? -a1[k] : grad1[(3 + k) * npts + p];
          }
        orc::lr_kernel_spin_point(func, n0, a0, n1, a1, v, out);
      }
      const int nout = trip ? 1 : 2;
      for (int s = 0; s < nout; ++s) {
        v1[s * npts + p] = v[s];
        if (gga)
          for (int k = 0; k < 3; ++k) g1[(s * 3 + k) * npts + p] = out[3 * s + k];
      }
    }
  }
  return 0;
}
