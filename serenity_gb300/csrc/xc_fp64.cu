// FP64 kernels of the XC build (the drop-in precision): block screening, basis
// functions on a block, rho / grad rho, the functional, and the Vxc adder.
//
// Work decomposition: one CTA of 128 threads per grid block, thread t <-> point t
// (a block holds at most 128 points).  Basis values of a chunk of blocks live in
// a scratch slab per block, laid out [component][active function][128 points]
// (component 0 = value, 1..3 = x, y, z derivatives), so every access of a warp
// to a slab is 32 consecutive doubles.  On GB300 the FP64 pipe is the bound for
// this precision; the kernels keep DFMA issue dense and move little data.
#include <cuda_runtime.h>

#include "basis_eval.cuh"
#include "functionals.cuh"
#include "internal.h"

namespace xcgpu {

// ------------------------------------------------------------------------------------
// Screening (BasisFunctionOnGridController.cpp:192-255): block centre = mean of the
// points, spread = max distance from it; a shell is kept if |c - A| - spread < 1 or
// if |sum_i c_i exp(-a_i d^2)| >= threshold at d = |c - A| - spread.
__global__ void __launch_bounds__(128) screen_kernel(DevBasis B, const double* __restrict__ xyz, long npoints,
                                                     int max_block, double thr, unsigned char* __restrict__ flags,
                                                     int* __restrict__ nfn) {
  const int b = blockIdx.x;
  const long first = (long)b * max_block;
  const int n = (int)min((long)max_block, npoints - first);
  __shared__ double red[3][128];
  __shared__ double c[3];
  __shared__ int cnt;
  double s[3] = {0, 0, 0};
  for (int p = threadIdx.x; p < n; p += blockDim.x)
    for (int k = 0; k < 3; ++k) s[k] += xyz[3 * (first + p) + k];
  for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = s[k];
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) c[k] = red[k][0] / n;
  __syncthreads();
  double sp = 0.0;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const double dx = xyz[3 * (first + p)] - c[0], dy = xyz[3 * (first + p) + 1] - c[1],
                 dz = xyz[3 * (first + p) + 2] - c[2];
    sp = fmax(sp, sqrt(dx * dx + dy * dy + dz * dz));
  }
  __syncthreads();
  red[0][threadIdx.x] = sp;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + w]);
    __syncthreads();
  }
  const double spread = red[0][0];
  int mine = 0;
  for (int sh = threadIdx.x; sh < B.nshell; sh += blockDim.x) {
    const double dx = c[0] - B.center[3 * sh], dy = c[1] - B.center[3 * sh + 1], dz = c[2] - B.center[3 * sh + 2];
    double d = sqrt(dx * dx + dy * dy + dz * dz) - spread;
    bool keep = true;
    if (!(d < 1.0)) {
      d = d * d;
      double r = 0.0;
      const int o = B.prim_off[sh];
      for (int i = 0; i < B.nprim[sh]; ++i) r += B.coef[o + i] * exp(-B.alpha[o + i] * d);
      keep = fabs(r) >= thr;
    }
    flags[(long)b * B.nshell + sh] = keep ? 1 : 0;
    if (keep) mine += B.pure[sh] ? 2 * B.l[sh] + 1 : ncart_d(B.l[sh]);
  }
  atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0) nfn[b] = cnt;
}

xcgpu_status launch_screen(Ctx* c, const DevBasis& B, const double* xyz, long npoints, int max_block, int nblocks,
                           double thr, unsigned char* flags, int* nfn) {
  if (nblocks == 0) return XCGPU_OK;
  KernelTimer kt(c, kOther);
  screen_kernel<<<nblocks, 128, 0, c->stream>>>(B, xyz, npoints, max_block, thr, flags, nfn);
  return c->check_launch("screen_kernel");
}

// ------------------------------------------------------------------------------------
// Basis functions of the active shells of block b at point p.
// Emit(local function index f within the block's active list, v, gx, gy, gz, h[6]).
template <class R, int DERIV, class Emit>
__device__ __forceinline__ void eval_point(const DevBasis& B, const DevPlan& P, int b, double px, double py, double pz,
                                           Emit&& emit) {
  const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
  int f0 = 0;
  for (int si = s0; si < s1; ++si) {
    const int sh = P.sh_list[si];
    const int l = B.l[sh];
    const bool pure = B.pure[sh] != 0;
    const int nf = pure ? 2 * l + 1 : ncart_d(l);
    const R x = (R)(px - B.center[3 * sh]), y = (R)(py - B.center[3 * sh + 1]), z = (R)(pz - B.center[3 * sh + 2]);
    const R r2 = x * x + y * y + z * z;
    R Rv, dR, ddR;
    const int o = B.prim_off[sh];
    const bool sig = shell_radial<R, DERIV>(B.alpha + o, B.coef + o, B.nprim[sh], r2, (R)P.exponent_threshold,
                                            (R)P.radial_threshold, Rv, dR, ddR);
    if (!sig) {
      R hz[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
      for (int f = 0; f < nf; ++f) emit(f0 + f, R(0), R(0), R(0), R(0), hz);
    } else {
      const double* T = B.trans + B.trans_off[l];
      const double* cn = B.cnorm + B.cnorm_off[l];
      shell_functions_l<R, DERIV>(l, x, y, z, Rv, dR, ddR, pure, T, cn,
                                  [&](int f, R v, R gx, R gy, R gz, const R* h) { emit(f0 + f, v, gx, gy, gz, h); });
    }
    f0 += nf;
  }
}

// Dense block data for the getBlockOnGridData API: out[c][mu][p] (ld = npts) with
// c = value, then 3 gradient, then 6 Hessian components; zero for negligible ones.
template <int DERIV>
__global__ void __launch_bounds__(128) block_values_kernel(DevBasis B, DevPlan P, int b, double* __restrict__ out,
                                                           int ld) {
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const long plane = (long)ld * B.nbf;
  const int* fn = P.fn_list + P.fn_off[b];
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const double* q = P.xyz + 3 * (first + p);
    eval_point<double, DERIV>(B, P, b, q[0], q[1], q[2],
                              [&](int f, double v, double gx, double gy, double gz, const double* h) {
                                const long o = (long)fn[f] * ld + p;
                                out[o] = v;
                                if (DERIV >= 1) {
                                  out[plane + o] = gx;
                                  out[2 * plane + o] = gy;
                                  out[3 * plane + o] = gz;
                                }
                                if (DERIV >= 2)
                                  for (int k = 0; k < 6; ++k) out[(4 + k) * plane + o] = h[k];
                              });
  }
}

xcgpu_status launch_block_values(Ctx* c, const DevBasis& B, const DevPlan& P, int block, int deriv, double* out,
                                 int ld) {
  if (deriv == 0) block_values_kernel<0><<<1, 128, 0, c->stream>>>(B, P, block, out, ld);
  else if (deriv == 1) block_values_kernel<1><<<1, 128, 0, c->stream>>>(B, P, block, out, ld);
  else block_values_kernel<2><<<1, 128, 0, c->stream>>>(B, P, block, out, ld);
  return c->check_launch("block_values_kernel");
}

// ------------------------------------------------------------------------------------
// Values + gradients of the active functions of blocks [b0, b1) into their slabs.
__global__ void __launch_bounds__(128) fp64_eval_kernel(DevBasis B, DevPlan P, int b0, const long* __restrict__ slab_off,
                                                        double* __restrict__ scratch) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  double* slab = scratch + slab_off[blockIdx.x];
  const int p = threadIdx.x;
  if (p < n) {
    const double* q = P.xyz + 3 * (first + p);
    eval_point<double, 1>(B, P, b, q[0], q[1], q[2], [&](int f, double v, double gx, double gy, double gz, const double*) {
      slab[(long)f * kBlockPoints + p] = v;
      slab[(long)(nact + f) * kBlockPoints + p] = gx;
      slab[(long)(2 * nact + f) * kBlockPoints + p] = gy;
      slab[(long)(3 * nact + f) * kBlockPoints + p] = gz;
    });
  } else {
    for (int f = 0; f < 4 * nact; ++f) slab[(long)f * kBlockPoints + p] = 0.0;
  }
}

xcgpu_status fp64_eval_chunk(Ctx* c, const DevBasis& B, const DevPlan& P, int b0, int b1, const long* slab_off,
                             double* scratch, int /*deriv*/) {
  if (b1 <= b0) return XCGPU_OK;
  KernelTimer kt(c, kEval);
  fp64_eval_kernel<<<b1 - b0, kBlockPoints, 0, c->stream>>>(B, P, b0, slab_off, scratch);
  return c->check_launch("fp64_eval_kernel");
}

// ------------------------------------------------------------------------------------
// rho_p = sum_nu X_p,nu phi_p,nu ; grad rho_p = 2 sum_nu X_p,nu grad phi_p,nu ;
// X = phi P_b (MatrixOperatorToGridTransformer.cpp:137-164).
constexpr int kDNu = 16, kDMu = 32;
__global__ void __launch_bounds__(128) fp64_density_kernel(DevPlan P, int b0, const long* __restrict__ slab_off,
                                                           const double* __restrict__ scratch, int nspin,
                                                           const double* __restrict__ Pm, double* __restrict__ rho,
                                                           double* __restrict__ grad) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  const int* fn = P.fn_list + P.fn_off[b];
  const double* slab = scratch + slab_off[blockIdx.x];
  const int p = threadIdx.x;
  const int nbf = P.nbf;
  __shared__ double Ps[kDMu][kDNu];
  for (int s = 0; s < nspin; ++s) {
    const double* Pmat = Pm + (long)s * nbf * nbf;
    double r = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int nu0 = 0; nu0 < nact; nu0 += kDNu) {
      double acc[kDNu];
#pragma unroll
      for (int j = 0; j < kDNu; ++j) acc[j] = 0.0;
      for (int mu0 = 0; mu0 < nact; mu0 += kDMu) {
        __syncthreads();
        for (int e = threadIdx.x; e < kDMu * kDNu; e += blockDim.x) {
          const int i = e / kDNu, j = e % kDNu;
          const int mu = mu0 + i, nu = nu0 + j;
          Ps[i][j] = (mu < nact && nu < nact) ? Pmat[(long)fn[nu] * nbf + fn[mu]] : 0.0;
        }
        __syncthreads();
        const int mlim = min(kDMu, nact - mu0);
        for (int i = 0; i < mlim; ++i) {
          const double ph = slab[(long)(mu0 + i) * kBlockPoints + p];
#pragma unroll
          for (int j = 0; j < kDNu; ++j) acc[j] = fma(ph, Ps[i][j], acc[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < kDNu; ++j) {
        const int nu = nu0 + j;
        if (nu < nact) {
          r = fma(acc[j], slab[(long)nu * kBlockPoints + p], r);
          g0 = fma(acc[j], slab[(long)(nact + nu) * kBlockPoints + p], g0);
          g1 = fma(acc[j], slab[(long)(2 * nact + nu) * kBlockPoints + p], g1);
          g2 = fma(acc[j], slab[(long)(3 * nact + nu) * kBlockPoints + p], g2);
        }
      }
    }
    if (p < n) {
      rho[(long)s * P.npoints + first + p] = r;
      if (grad) {
        grad[((long)s * 3 + 0) * P.npoints + first + p] = 2.0 * g0;
        grad[((long)s * 3 + 1) * P.npoints + first + p] = 2.0 * g1;
        grad[((long)s * 3 + 2) * P.npoints + first + p] = 2.0 * g2;
      }
    }
  }
}

xcgpu_status fp64_density_chunk(Ctx* c, const DevPlan& P, int b0, int b1, const long* slab_off, const double* scratch,
                                int nspin, const double* Pm, double* rho, double* grad) {
  if (b1 <= b0) return XCGPU_OK;
  KernelTimer kt(c, kDensity);
  fp64_density_kernel<<<b1 - b0, kBlockPoints, 0, c->stream>>>(P, b0, slab_off, scratch, nspin, Pm, rho, grad);
  return c->check_launch("fp64_density_kernel");
}

// ------------------------------------------------------------------------------------
// XC contribution to the nuclear gradient (FuncPotential<M>::getGeomGradients,
// FuncPotential.cpp:113-241).  The reference's pair loop
//   G[atom(nu)][k] -= 2 P_mu,nu sum_p w [ v phi_mu d_k phi_nu
//                       + sum_j g_j (phi_mu d_j d_k phi_nu + d_j phi_mu d_k phi_nu) ]
// is regrouped around two contractions with the block's density matrix,
//   X_p,nu = sum_mu phi_mu(p) P_mu,nu,   Y_p,nu = sum_mu (w g . grad phi_mu)(p) P_mu,nu,
// so that  G[atom(nu)][k] -= 2 sum_p [ X (w v d_k phi_nu + w g_j d_j d_k phi_nu) + Y d_k phi_nu ].
// Slabs hold [value, x, y, z (, xx, xy, xz, yy, yz, zz)][function][128 points].

// Values, gradients and Hessians of the active functions of blocks [b0, b1) (10 planes).
__global__ void __launch_bounds__(128) fp64_eval_hess_kernel(DevBasis B, DevPlan P, int b0,
                                                             const long* __restrict__ slab_off,
                                                             double* __restrict__ scratch) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  double* slab = scratch + slab_off[blockIdx.x];
  const int p = threadIdx.x;
  if (p < n) {
    const double* q = P.xyz + 3 * (first + p);
    eval_point<double, 2>(B, P, b, q[0], q[1], q[2], [&](int f, double v, double gx, double gy, double gz, const double* h) {
      slab[(long)f * kBlockPoints + p] = v;
      slab[(long)(nact + f) * kBlockPoints + p] = gx;
      slab[(long)(2 * nact + f) * kBlockPoints + p] = gy;
      slab[(long)(3 * nact + f) * kBlockPoints + p] = gz;
      for (int c = 0; c < 6; ++c) slab[(long)((4 + c) * nact + f) * kBlockPoints + p] = h[c];
    });
  } else {
    for (int f = 0; f < 10 * nact; ++f) slab[(long)f * kBlockPoints + p] = 0.0;
  }
}

template <bool GGA>
__global__ void __launch_bounds__(128) fp64_xc_gradient_kernel(DevPlan P, int b0, const long* __restrict__ slab_off,
                                                               const double* __restrict__ scratch, int nspin,
                                                               const double* __restrict__ Pm,
                                                               const double* __restrict__ v,
                                                               const double* __restrict__ g,
                                                               const int* __restrict__ fatom, int natoms,
                                                               double* __restrict__ G) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  const int* fn = P.fn_list + P.fn_off[b];
  const double* slab = scratch + slab_off[blockIdx.x];
  const int p = threadIdx.x, lane = p & 31, warp = p >> 5;
  const int nbf = P.nbf;
  const bool live = p < n;
  __shared__ double Ps[kDMu][kDNu];
  __shared__ double red[4][kDNu][3];
  // Hessian plane of the pair (j, k): xx xy xz yy yz zz
  constexpr int hc[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  const double w = live ? P.w[first + p] : 0.0;
  for (int s = 0; s < nspin; ++s) {
    const double* Pmat = Pm + (long)s * nbf * nbf;
    const double wv = live ? w * v[(long)s * P.npoints + first + p] : 0.0;
    double wg[3] = {0.0, 0.0, 0.0};
    if (GGA && live)
      for (int j = 0; j < 3; ++j) wg[j] = w * g[((long)s * 3 + j) * P.npoints + first + p];
    for (int nu0 = 0; nu0 < nact; nu0 += kDNu) {
      double ax[kDNu], ay[kDNu];
#pragma unroll
      for (int j = 0; j < kDNu; ++j) ax[j] = ay[j] = 0.0;
      for (int mu0 = 0; mu0 < nact; mu0 += kDMu) {
        __syncthreads();
        for (int e = threadIdx.x; e < kDMu * kDNu; e += blockDim.x) {
          const int i = e / kDNu, j = e % kDNu;
          const int mu = mu0 + i, nu = nu0 + j;
          Ps[i][j] = (mu < nact && nu < nact) ? Pmat[(long)fn[nu] * nbf + fn[mu]] : 0.0;
        }
        __syncthreads();
        const int mlim = min(kDMu, nact - mu0);
        for (int i = 0; i < mlim; ++i) {
          const int mu = mu0 + i;
          const double ph = slab[(long)mu * kBlockPoints + p];
          double psi = 0.0;
          if (GGA)
            psi = wg[0] * slab[(long)(nact + mu) * kBlockPoints + p] + wg[1] * slab[(long)(2 * nact + mu) * kBlockPoints + p] +
                  wg[2] * slab[(long)(3 * nact + mu) * kBlockPoints + p];
#pragma unroll
          for (int j = 0; j < kDNu; ++j) {
            ax[j] = fma(ph, Ps[i][j], ax[j]);
            if (GGA) ay[j] = fma(psi, Ps[i][j], ay[j]);
          }
        }
      }
      // per-function contributions of this point, summed over the warp's 32 points
#pragma unroll
      for (int j = 0; j < kDNu; ++j) {
        const int nu = nu0 + j;
        double c[3] = {0.0, 0.0, 0.0};
        if (nu < nact && live) {
          double d[3];
          for (int k = 0; k < 3; ++k) d[k] = slab[(long)((1 + k) * nact + nu) * kBlockPoints + p];
          for (int k = 0; k < 3; ++k) c[k] = ax[j] * wv * d[k];
          if (GGA) {
            for (int k = 0; k < 3; ++k) {
              double t = 0.0;
              for (int jj = 0; jj < 3; ++jj) t += wg[jj] * slab[(long)((4 + hc[jj][k]) * nact + nu) * kBlockPoints + p];
              c[k] += ax[j] * t + ay[j] * d[k];
            }
          }
        }
        for (int k = 0; k < 3; ++k) {
          double x = c[k];
          for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
          if (lane == 0) red[warp][j][k] = x;
        }
      }
      __syncthreads();
      if (threadIdx.x < 3 * kDNu) {
        const int j = threadIdx.x / 3, k = threadIdx.x % 3, nu = nu0 + j;
        if (nu < nact) {
          const double t = red[0][j][k] + red[1][j][k] + red[2][j][k] + red[3][j][k];
          atomicAdd(&G[fatom[fn[nu]] + (long)natoms * k], -2.0 * t);
        }
      }
    }
  }
}

xcgpu_status fp64_xc_gradient_chunk(Ctx* c, const DevBasis& B, const DevPlan& P, int b0, int b1, const long* slab_off,
                                    double* scratch, bool gga, int nspin, const double* Pm, const double* v,
                                    const double* g, const int* fatom, int natoms, double* G) {
  if (b1 <= b0) return XCGPU_OK;
  xcgpu_status st;
  {
    KernelTimer kt(c, kEval);
    if (gga) fp64_eval_hess_kernel<<<b1 - b0, kBlockPoints, 0, c->stream>>>(B, P, b0, slab_off, scratch);
    else fp64_eval_kernel<<<b1 - b0, kBlockPoints, 0, c->stream>>>(B, P, b0, slab_off, scratch);
    if ((st = c->check_launch("gradient basis kernel"))) return st;
  }
  KernelTimer kt(c, kOther);
  if (gga)
    fp64_xc_gradient_kernel<true><<<b1 - b0, kBlockPoints, 0, c->stream>>>(P, b0, slab_off, scratch, nspin, Pm, v, g,
                                                                             fatom, natoms, G);
  else
    fp64_xc_gradient_kernel<false><<<b1 - b0, kBlockPoints, 0, c->stream>>>(P, b0, slab_off, scratch, nspin, Pm, v, g,
                                                                              fatom, natoms, G);
  return c->check_launch("fp64_xc_gradient_kernel");
}

// ------------------------------------------------------------------------------------
// Functional on points.  Block skip (XCFun.cpp:136-140): a block of skip_block points
// whose sum |rho_s| < n * 1e-12 for every spin gives zero outputs.
__global__ void __launch_bounds__(128) skip_flags_kernel(long n, int skip_block, int nspin,
                                                         const double* __restrict__ rho,
                                                         unsigned char* __restrict__ skip, long sk0) {
  const long sb = sk0 + blockIdx.x;  // skip block of this CTA
  const long first = sb * skip_block;
  const int m = (int)min((long)skip_block, n - first);
  __shared__ double red[128];
  bool sk = true;
  for (int s = 0; s < nspin; ++s) {
    double a = 0.0;
    for (int p = threadIdx.x; p < m; p += blockDim.x) a += fabs(rho[(long)s * n + first + p]);
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    sk = sk && (red[0] < m * 1e-12);
    __syncthreads();
  }
  if (threadIdx.x == 0) skip[sb] = sk ? 1 : 0;
}

// points [p0, p1) of n (p0 a multiple of 128); partials[k] and partials[nparts + k] get
// the E_xc and N_el sums of the 128 points from 128 k
__global__ void __launch_bounds__(128) functional_kernel(int func, int nspin, long n, int skip_block,
                                                         const unsigned char* __restrict__ skip,
                                                         const double* __restrict__ rho,
                                                         const double* __restrict__ grad, double* __restrict__ epuv,
                                                         double* __restrict__ dfdrho, double* __restrict__ dfdgrad,
                                                         const double* __restrict__ w, double* __restrict__ partials,
                                                         long p0, long p1, int nparts, int pair) {
  const long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool gga = xc::is_gga(func);
  double e = 0.0, rtot = 0.0;
  if (p < p1) {
    const bool sk = skip[p / skip_block] != 0;
    if (nspin == 1) {
      const double r = rho[p];
      double gx = 0, gy = 0, gz = 0;
      if (gga) {
        gx = grad[p];
        gy = grad[n + p];
        gz = grad[2 * n + p];
      }
      double vn = 0.0, vs = 0.0;
      if (!sk) {
        if (pair && func == XCGPU_FUNC_PBE) xc::pbe_restricted_pair(r, gx * gx + gy * gy + gz * gz, e, vn, vs);
        else xc::eval_restricted<double>(func, r, gx * gx + gy * gy + gz * gz, e, vn, vs);
      }
      epuv[p] = e;
      dfdrho[p] = vn;
      if (gga) {
        dfdgrad[p] = 2.0 * vs * gx;
        dfdgrad[n + p] = 2.0 * vs * gy;
        dfdgrad[2 * n + p] = 2.0 * vs * gz;
      }
      rtot = r;
    } else {
      const double ra = rho[p], rb = rho[n + p];
      double ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0};
      if (gga)
        for (int k = 0; k < 3; ++k) {
          ga[k] = grad[k * n + p];
          gb[k] = grad[(3 + k) * n + p];
        }
      double va = 0, vb = 0, vaa = 0, vab = 0, vbb = 0;
      if (!sk) {
        const double saa = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
        const double sab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
        const double sbb = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
        xc::eval_unrestricted<double>(func, ra, rb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
      }
      epuv[p] = e;
      dfdrho[p] = va;
      dfdrho[n + p] = vb;
      if (gga)
        for (int k = 0; k < 3; ++k) {
          dfdgrad[k * n + p] = 2.0 * vaa * ga[k] + vab * gb[k];
          dfdgrad[(3 + k) * n + p] = 2.0 * vbb * gb[k] + vab * ga[k];
        }
      rtot = ra + rb;
    }
  }
  if (partials) {
    __shared__ double red[2][128];
    const double wp = (p < p1) ? w[p] : 0.0;
    red[0][threadIdx.x] = wp * e;
    red[1][threadIdx.x] = wp * rtot;
    __syncthreads();
    for (int s = 64; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        red[0][threadIdx.x] += red[0][threadIdx.x + s];
        red[1][threadIdx.x] += red[1][threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const long k = p0 / 128 + blockIdx.x;
      partials[k] = red[0][0];
      partials[nparts + k] = red[1][0];
    }
  }
}

// the functional at points [p0, p1) of an n-point grid (arrays strided by n); p0 a
// multiple of 128 and, with the block skip, of skip_block.  partials: 2 x nparts sums of
// 128-point groups (nparts = ceil(n / 128)), the groups of the range written.
xcgpu_status launch_functional_range(Ctx* c, int func, int nspin, long n, int skip_block, long p0, long p1,
                                     const double* rho, const double* grad, double* epuv, double* dfdrho,
                                     double* dfdgrad, const double* w, double* partials, unsigned char* skipbuf,
                                     bool pair) {
  if (p1 <= p0) return XCGPU_OK;
  const int sb = skip_block > 0 ? skip_block : 1 << 30;
  const long nsk = (n + sb - 1) / sb;
  xcgpu_status st = XCGPU_OK;
  unsigned char* skip = skipbuf;
  if (!skip) {
    if ((st = c->skip.alloc(c, nsk))) return st;
    skip = c->skip.as<unsigned char>();
  }
  KernelTimer kt(c, kFunctional);
  if (skip_block > 0) {
    const long sk0 = p0 / sb, sk1 = (p1 + sb - 1) / sb;
    skip_flags_kernel<<<(unsigned)(sk1 - sk0), 128, 0, c->stream>>>(n, sb, nspin, rho, skip, sk0);
    if ((st = c->check_launch("skip_flags_kernel"))) return st;
  } else {
    if ((st = c->cuda(cudaMemsetAsync(skip, 0, nsk, c->stream), "memset skip"))) return st;
  }
  const unsigned grid = (unsigned)((p1 - p0 + 127) / 128);
  functional_kernel<<<grid, 128, 0, c->stream>>>(func, nspin, n, sb, skip, rho, grad, epuv, dfdrho, dfdgrad, w,
                                                 partials, p0, p1, (int)((n + 127) / 128), pair ? 1 : 0);
  return c->check_launch("functional_kernel");
}

xcgpu_status launch_functional(Ctx* c, int func, int nspin, long n, int skip_block, const double* rho,
                               const double* grad, double* epuv, double* dfdrho, double* dfdgrad, const double* w,
                               double* partials, int* nparts, unsigned char* skipbuf, bool pair) {
  if (nparts) *nparts = (int)((n + 127) / 128);
  return launch_functional_range(c, func, nspin, n, skip_block, 0, n, rho, grad, epuv, dfdrho, dfdgrad, w, partials,
                                 skipbuf, pair);
}

// ------------------------------------------------------------------------------------
// Adder block skip (ScalarOperatorToMatrixAdder.cpp:200-203, 248-256):
// sum_p (|w v| + |w g_x| + |w g_y| + |w g_z|) / n < threshold.
__global__ void __launch_bounds__(128) adder_skip_kernel(DevPlan P, int nspin, const double* __restrict__ v,
                                                         const double* __restrict__ g, double thr,
                                                         unsigned char* __restrict__ skip, int b0) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  __shared__ double red[128];
  for (int s = 0; s < nspin; ++s) {
    double a = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      const long p = first + q;
      const double w = P.w[p];
      a += fabs(w * v[(long)s * P.npoints + p]);
      if (g)
        for (int k = 0; k < 3; ++k) a += fabs(w * g[((long)s * 3 + k) * P.npoints + p]);
    }
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w2 = 64; w2 > 0; w2 >>= 1) {
      if (threadIdx.x < w2) red[threadIdx.x] += red[threadIdx.x + w2];
      __syncthreads();
    }
    if (threadIdx.x == 0) skip[(long)s * P.nblocks + b] = (red[0] / n < thr) ? 1 : 0;
    __syncthreads();
  }
}

xcgpu_status launch_block_skip_flags_range(Ctx* c, const DevPlan& P, int nspin, const double* v, const double* g,
                                           double thr, unsigned char* skip, int b0, int b1) {
  if (b1 <= b0) return XCGPU_OK;
  KernelTimer kt(c, kOther);
  adder_skip_kernel<<<b1 - b0, 128, 0, c->stream>>>(P, nspin, v, g, thr, skip, b0);
  return c->check_launch("adder_skip_kernel");
}

xcgpu_status launch_block_skip_flags(Ctx* c, const DevPlan& P, int nspin, const double* v, const double* g,
                                     double thr, unsigned char* skip) {
  return launch_block_skip_flags_range(c, P, nspin, v, g, thr, skip, 0, P.nblocks);
}

// ------------------------------------------------------------------------------------
// F_b = T + T^T with T = phi^T G, G = w (v/2 phi + g . grad phi)
// (ScalarOperatorToMatrixAdder.cpp:178-303: tmp = phi_b^T grad_A, F_b = tmp + tmp^T; the
// LDA form phi^T diag(w v) phi is the same with g = 0).  One CTA per (block, 64-row tile
// i, 64-column tile j) over all tile pairs, one product per output (a tile pair of the
// upper triangle with both products would pad the diagonal tiles with their mirror
// halves); 256 threads with 4x4 outputs each; T(a, b) is added into F at (a, b) and
// (b, a) with FP64 atomics.
constexpr int kAT = 64, kAK = 32, kAPad = kAK + 1;
__global__ void __launch_bounds__(256) fp64_adder_kernel(DevPlan P, const int* __restrict__ work, long w0,
                                                         const long* __restrict__ slab_off, int chunk_b0,
                                                         const double* __restrict__ scratch, int nspin,
                                                         const double* __restrict__ v, const double* __restrict__ g,
                                                         const unsigned char* __restrict__ skip,
                                                         double* __restrict__ F) {
  extern __shared__ double sm[];
  double* Pi = sm;                // phi rows of tile i   [64][33]
  double* Gj = Pi + kAT * kAPad;  // G rows of tile j
  const long item = w0 + blockIdx.x;
  const int b = work[3 * item], ti = work[3 * item + 1], tj = work[3 * item + 2];
  const int s = blockIdx.y;
  if (skip[(long)s * P.nblocks + b]) return;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  const int* fn = P.fn_list + P.fn_off[b];
  const double* slab = scratch + slab_off[b - chunk_b0];
  const int ci = min(kAT, nact - ti * kAT), cj = min(kAT, nact - tj * kAT);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = 0.0;
  for (int k0 = 0; k0 < n; k0 += kAK) {
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * kAT * kAK; e += blockDim.x) {
      const int which = e / (kAT * kAK);  // 0: phi of tile i, 1: G of tile j
      const int r = (e % (kAT * kAK)) / kAK, q = e % kAK;
      const int pk = k0 + q;
      double val = 0.0;
      if (which == 0) {
        if (r < ci && pk < n) val = slab[(long)(ti * kAT + r) * kBlockPoints + pk];
        Pi[r * kAPad + q] = val;
      } else {  // G of spin s, formed once per block into the slab's plane 1 + s
        if (r < cj && pk < n) val = slab[(long)((1 + s) * nact + tj * kAT + r) * kBlockPoints + pk];
        Gj[r * kAPad + q] = val;
      }
    }
    __syncthreads();
    const int kl = min(kAK, n - k0);
    for (int q = 0; q < kl; ++q) {
      double pa[4], gb[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        pa[a] = Pi[(ty + 16 * a) * kAPad + q];
        gb[a] = Gj[(tx + 16 * a) * kAPad + q];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = fma(pa[a], gb[c], acc[a][c]);
    }
  }
  const int nbf = P.nbf;
  double* Fs = F + (long)s * nbf * nbf;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int r = ty + 16 * a;
    if (r >= ci) continue;
    const int mu = fn[ti * kAT + r];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int q = tx + 16 * c;
      if (q >= cj) continue;
      const int nu = fn[tj * kAT + q];
      atomicAdd(&Fs[(long)nu * nbf + mu], acc[a][c]);
      atomicAdd(&Fs[(long)mu * nbf + nu], acc[a][c]);
    }
  }
}

// G = w (v/2 phi + g . grad phi) of every active function of the blocks [b0, b0 + grid)
// at their points, per spin, written over the slab's gradient planes (plane 1 + s; the
// density is done with them): formed once per block instead of once per tile pair
__global__ void __launch_bounds__(128) fp64_form_g_kernel(DevPlan P, int b0, const long* __restrict__ slab_off,
                                                          double* __restrict__ scratch, int nspin,
                                                          const double* __restrict__ v, const double* __restrict__ g) {
  const int b = b0 + blockIdx.x;
  const long first = (long)b * P.max_block;
  const int n = (int)min((long)P.max_block, P.npoints - first);
  const int nact = P.fn_off[b + 1] - P.fn_off[b];
  double* slab = scratch + slab_off[blockIdx.x];
  const int p = threadIdx.x;
  if (p >= n) return;
  const double w = P.w[first + p];
  double a[2] = {0.0, 0.0}, gx[2] = {0.0, 0.0}, gy[2] = {0.0, 0.0}, gz[2] = {0.0, 0.0};
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    if (s >= nspin) break;
    a[s] = 0.5 * v[(long)s * P.npoints + first + p];
    if (g) {
      gx[s] = g[((long)s * 3 + 0) * P.npoints + first + p];
      gy[s] = g[((long)s * 3 + 1) * P.npoints + first + p];
      gz[s] = g[((long)s * 3 + 2) * P.npoints + first + p];
    }
  }
  for (int f = 0; f < nact; ++f) {
    const double phi = slab[(long)f * kBlockPoints + p];
    const double dx = slab[(long)(nact + f) * kBlockPoints + p];
    const double dy = slab[(long)(2 * nact + f) * kBlockPoints + p];
    const double dz = slab[(long)(3 * nact + f) * kBlockPoints + p];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (s >= nspin) break;
      double gg = a[s] * phi;
      if (g) gg += gx[s] * dx + gy[s] * dy + gz[s] * dz;
      slab[(long)((1 + s) * nact + f) * kBlockPoints + p] = gg * w;
    }
  }
}

xcgpu_status fp64_adder_chunk(Ctx* c, const DevPlan& P, const int* work, long w0, long w1, int chunk_b0,
                              int chunk_b1, const long* slab_off, double* scratch, int nspin, const double* v,
                              const double* g, const unsigned char* skip, double* F) {
  if (chunk_b1 > chunk_b0) {
    KernelTimer kt(c, kAdder);
    fp64_form_g_kernel<<<chunk_b1 - chunk_b0, kBlockPoints, 0, c->stream>>>(P, chunk_b0, slab_off, scratch, nspin, v, g);
    xcgpu_status st = c->check_launch("fp64_form_g_kernel");
    if (st) return st;
  }
  if (w1 <= w0) return XCGPU_OK;
  const size_t smem = 2 * kAT * kAPad * sizeof(double);
  xcgpu_status st = c->cuda(cudaFuncSetAttribute(fp64_adder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem), "adder smem attribute");
  if (st) return st;
  dim3 grid((unsigned)(w1 - w0), (unsigned)nspin);
  KernelTimer kt(c, kAdder);
  fp64_adder_kernel<<<grid, 256, smem, c->stream>>>(P, work, w0, slab_off, chunk_b0, scratch, nspin, v, g, skip, F);
  return c->check_launch("fp64_adder_kernel");
}

// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) sum_partials_kernel(const double* __restrict__ partials, int nparts, int ncomp,
                                                           double* __restrict__ out) {
  __shared__ double red[256];
  for (int c = 0; c < ncomp; ++c) {
    double a = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) a += partials[(long)c * nparts + i];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
    __syncthreads();
  }
}

__global__ void axpy_kernel(long n, const double* __restrict__ x, double* __restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

xcgpu_status launch_axpy(Ctx* c, long n, const double* x, double* y) {
  if (n == 0) return XCGPU_OK;
  KernelTimer kt(c, kOther);
  axpy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, x, y);
  return c->check_launch("axpy_kernel");
}

__global__ void scale_add_kernel(long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

xcgpu_status launch_scale_add(Ctx* c, long n, double a, const double* x, double* y) {
  if (n == 0) return XCGPU_OK;
  KernelTimer kt(c, kOther);
  scale_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, a, x, y);
  return c->check_launch("scale_add_kernel");
}

xcgpu_status launch_sum_partials(Ctx* c, const double* partials, int nparts, int ncomp, double* out) {
  KernelTimer kt(c, kOther);
  sum_partials_kernel<<<1, 256, 0, c->stream>>>(partials, nparts, ncomp, out);
  return c->check_launch("sum_partials_kernel");
}

}  // namespace xcgpu
