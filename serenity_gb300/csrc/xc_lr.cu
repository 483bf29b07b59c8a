// Linear-response XC kernel (the XC part of a TDDFT / TDA sigma vector,
// KernelSigmavector<RESTRICTED>::calcF, KernelSigmavector.cpp:128-392, singlet).
//
// With the ground-state density n, sigma = |grad n|^2 and a perturbed density rho1 (the
// density of the symmetrised trial matrix), the reference contracts the second
// functional derivatives pp, pg, gg with (rho1, grad rho1) and integrates the result
// like a potential.  The contracted kernel is the directional derivative of the first
// derivatives along the perturbation,
//   v1 = d/de [dF/dn](n + e rho1, sigma + e sigma1),  sigma1 = 2 grad n . grad rho1,
//   g1 = d/de [dF/d grad n] = 2 (d/de dF/dsigma) grad n + 2 dF/dsigma grad rho1,
// so one evaluation of the analytic first-derivative functionals in dual numbers
// (value + one directional derivative) per point gives it exactly, with no second
// derivative formulas of their own.
#include <cuda_runtime.h>

#include "functionals.cuh"
#include "internal.h"

namespace xcgpu {
namespace xc {

// value and one directional derivative
struct Dual {
  double v, d;
  __device__ Dual() : v(0.0), d(0.0) {}
  __device__ Dual(double x) : v(x), d(0.0) {}
  __device__ Dual(double x, double y) : v(x), d(y) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { return a = a * b; }
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(Dual a, Dual b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(Dual a, Dual b) { return a.v != b.v; }

template <> __device__ __forceinline__ bool zeta_is_zero<Dual>(Dual z) { return z.v == 0.0 && z.d == 0.0; }
template <> __device__ __forceinline__ Dual cbrt_<Dual>(Dual x) {
  const double c = cbrt(x.v);
  return Dual(c, x.d == 0.0 ? 0.0 : x.d * c / (3.0 * x.v));
}
template <> __device__ __forceinline__ Dual log_<Dual>(Dual x) { return Dual(log(x.v), x.d / x.v); }
template <> __device__ __forceinline__ Dual exp_<Dual>(Dual x) {
  const double e = exp(x.v);
  return Dual(e, x.d * e);
}
template <> __device__ __forceinline__ Dual atan_<Dual>(Dual x) { return Dual(atan(x.v), x.d / (1.0 + x.v * x.v)); }
template <> __device__ __forceinline__ Dual asinh_<Dual>(Dual x) {
  return Dual(asinh(x.v), x.d / sqrt(1.0 + x.v * x.v));
}
// at 0 only a zero direction is meaningful (sigma = 0 has sigma1 = 0)
template <> __device__ __forceinline__ Dual sqrt_<Dual>(Dual x) {
  const double s = sqrt(x.v);
  return Dual(s, x.d == 0.0 ? 0.0 : x.d / (2.0 * s));
}
// constant exponent
template <> __device__ __forceinline__ Dual pow_<Dual>(Dual x, Dual p) {
  const double y = pow(x.v, p.v);
  return Dual(y, x.d == 0.0 ? 0.0 : x.d * p.v * y / x.v);
}

}  // namespace xc

// Per point: v1 and g1 of the restricted kernel contracted with (rho1, grad rho1);
// blocks of skip_block points whose ground-state density sums below n * 1e-12 give zero
// (the functional data's block skip, XCFun.cpp:136-140).
__global__ void __launch_bounds__(128) lr_kernel_kernel(int func, long n, int skip_block,
                                                        const double* __restrict__ rho0,
                                                        const double* __restrict__ grad0,
                                                        const double* __restrict__ rho1,
                                                        const double* __restrict__ grad1, double* __restrict__ v1,
                                                        double* __restrict__ g1) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool gga = xc::is_gga(func);
  // one CUDA block of 128 threads is one skip block of 128 points (the launch uses
  // blockDim == skip_block): its ground-state density sum decides the skip
  __shared__ double red[128];
  const double a = p < n ? fabs(rho0[p]) : 0.0;
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const long first = (long)blockIdx.x * blockDim.x;
  const long cnt = min((long)skip_block, n - first);
  const bool skip = red[0] < cnt * 1e-12;
  if (p >= n) return;
  double out_v = 0.0, out_g[3] = {0.0, 0.0, 0.0};
  if (!skip) {
    double s0 = 0.0, s1 = 0.0, q0[3] = {0, 0, 0}, q1[3] = {0, 0, 0};
    if (gga)
      for (int k = 0; k < 3; ++k) {
        q0[k] = grad0[k * n + p];
        q1[k] = grad1[k * n + p];
        s0 += q0[k] * q0[k];
        s1 += 2.0 * q0[k] * q1[k];
      }
    xc::Dual e, vn, vs;
    xc::eval_restricted<xc::Dual>(func, xc::Dual(rho0[p], rho1[p]), xc::Dual(s0, s1), e, vn, vs);
    out_v = vn.d;
    if (gga)
      for (int k = 0; k < 3; ++k) out_g[k] = 2.0 * vs.d * q0[k] + 2.0 * vs.v * q1[k];
  }
  v1[p] = out_v;
  if (gga)
    for (int k = 0; k < 3; ++k) g1[k * n + p] = out_g[k];
}

// Per point, the spin-resolved kernel contracted with a perturbation of both spin
// densities: with x = (rho_a, rho_b, s_aa, s_ab, s_bb) the dual numbers carry x1 =
// (rho1_a, rho1_b, 2 grad rho_a . grad rho1_a, grad rho_a . grad rho1_b + grad rho1_a .
// grad rho_b, 2 grad rho_b . grad rho1_b), so one evaluation of the first derivatives gives
//   v1_a = d(dF/drho_a)                 (KernelSigmavector.cpp:422-499, pp and pg terms)
//   g1_a = d(2 F_saa grad rho_a + F_sab grad rho_b)   (the pg and gg terms), alike for b.
// kind 2 (unrestricted): rho0 [2][n], grad0 [2][3][n], rho1 [2][n], grad1 [2][3][n], both
//   spins out (v1 [2][n], g1 [2][3][n]).
// kind 1 (triplet, KernelSigmavector<RESTRICTED> with the spin kernel, :367-391): rho0,
//   grad0 the restricted total density (each spin half of it), the perturbation (+rho1,
//   -rho1); the alpha outputs (f_aa - f_ab contracted with rho1) are written.
// The block skip is the unrestricted functional data's: every spin's |rho| sums below
// n 1e-12 over the block (XCFun.cpp:136-140).
__global__ void __launch_bounds__(128) lr_kernel_spin_kernel(int func, int kind, long n, int skip_block,
                                                             const double* __restrict__ rho0,
                                                             const double* __restrict__ grad0,
                                                             const double* __restrict__ rho1,
                                                             const double* __restrict__ grad1,
                                                             double* __restrict__ v1, double* __restrict__ g1) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool gga = xc::is_gga(func), trip = kind == 1;
  __shared__ double red[2][128];
  double ra = 0.0, rb = 0.0;
  if (p < n) {
    ra = trip ? 0.5 * rho0[p] : rho0[p];
    rb = trip ? ra : rho0[n + p];
  }
  red[0][threadIdx.x] = fabs(ra);
  red[1][threadIdx.x] = fabs(rb);
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  const long first = (long)blockIdx.x * blockDim.x;
  const long cnt = min((long)skip_block, n - first);
  const bool skip = red[0][0] < cnt * 1e-12 && red[1][0] < cnt * 1e-12;
  if (p >= n) return;
  double ov[2] = {0.0, 0.0}, og[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  if (!skip) {
    double a0[3] = {0, 0, 0}, b0[3] = {0, 0, 0}, a1[3] = {0, 0, 0}, b1[3] = {0, 0, 0};
    double ra1, rb1;
    if (trip) {
      ra1 = rho1[p];
      rb1 = -ra1;
    } else {
      ra1 = rho1[p];
      rb1 = rho1[n + p];
    }
    if (gga)
      for (int k = 0; k < 3; ++k) {
        if (trip) {
          a0[k] = b0[k] = 0.5 * grad0[k * n + p];
          a1[k] = grad1[k * n + p];
          b1[k] = -a1[k];
        } else {
          a0[k] = grad0[k * n + p];
          b0[k] = grad0[(3 + k) * n + p];
          a1[k] = grad1[k * n + p];
          b1[k] = grad1[(3 + k) * n + p];
        }
      }
    double saa = 0, sab = 0, sbb = 0, daa = 0, dab = 0, dbb = 0;
    for (int k = 0; k < 3; ++k) {
      saa += a0[k] * a0[k];
      sab += a0[k] * b0[k];
      sbb += b0[k] * b0[k];
      daa += 2.0 * a0[k] * a1[k];
      dab += a0[k] * b1[k] + a1[k] * b0[k];
      dbb += 2.0 * b0[k] * b1[k];
    }
    xc::Dual e, va, vb, vaa, vab, vbb;
    xc::eval_unrestricted<xc::Dual>(func, xc::Dual(ra, ra1), xc::Dual(rb, rb1), xc::Dual(saa, daa),
                                    xc::Dual(sab, dab), xc::Dual(sbb, dbb), e, va, vb, vaa, vab, vbb);
    ov[0] = va.d;
    ov[1] = vb.d;
    if (gga)
      for (int k = 0; k < 3; ++k) {
        og[0][k] = 2.0 * vaa.d * a0[k] + 2.0 * vaa.v * a1[k] + vab.d * b0[k] + vab.v * b1[k];
        og[1][k] = 2.0 * vbb.d * b0[k] + 2.0 * vbb.v * b1[k] + vab.d * a0[k] + vab.v * a1[k];
      }
  }
  const int nout = trip ? 1 : 2;
  for (int s = 0; s < nout; ++s) {
    v1[(long)s * n + p] = ov[s];
    if (gga)
      for (int k = 0; k < 3; ++k) g1[((long)s * 3 + k) * n + p] = og[s][k];
  }
}

// D -> (D + D^T) / 2, column-major n x n
__global__ void symmetrise_half_kernel(const double* __restrict__ D, double* __restrict__ S, int n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * n) return;
  const int r = (int)(i % n), c = (int)(i / n);
  S[i] = 0.5 * (D[i] + D[(long)r * n + c]);
}

xcgpu_status launch_lr_kernel(Ctx* c, int func, long n, const double* rho0, const double* grad0, const double* rho1,
                              const double* grad1, double* v1, double* g1) {
  if (n == 0) return XCGPU_OK;
  KernelTimer kt(c, kFunctional);
  lr_kernel_kernel<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(func, n, kSkipBlock, rho0, grad0, rho1, grad1,
                                                                       v1, g1);
  return c->check_launch("lr_kernel_kernel");
}

xcgpu_status launch_lr_kernel_spin(Ctx* c, int func, int kind, long n, const double* rho0, const double* grad0,
                                   const double* rho1, const double* grad1, double* v1, double* g1) {
  if (n == 0) return XCGPU_OK;
  KernelTimer kt(c, kFunctional);
  lr_kernel_spin_kernel<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(func, kind, n, kSkipBlock, rho0, grad0,
                                                                            rho1, grad1, v1, g1);
  return c->check_launch("lr_kernel_spin_kernel");
}

xcgpu_status launch_symmetrise_half(Ctx* c, const double* D, double* S, int n) {
  KernelTimer kt(c, kOther);
  const long m = (long)n * n;
  symmetrise_half_kernel<<<(unsigned)((m + 255) / 256), 256, 0, c->stream>>>(D, S, n);
  return c->check_launch("symmetrise_half_kernel");
}

}  // namespace xcgpu
