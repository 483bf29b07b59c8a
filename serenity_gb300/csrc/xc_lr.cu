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

xcgpu_status launch_symmetrise_half(Ctx* c, const double* D, double* S, int n) {
  KernelTimer kt(c, kOther);
  const long m = (long)n * n;
  symmetrise_half_kernel<<<(unsigned)((m + 255) / 256), 256, 0, c->stream>>>(D, S, n);
  return c->check_launch("symmetrise_half_kernel");
}

}  // namespace xcgpu
