// Mixed-precision XC build on the sm_103a tensor cores: host side (launch of the
// persistent kernels of xc_mixed_kernel.cuh, the density-matrix split, the mirror of V).
// The kernels for bases up to f functions are instantiated here; those for g..i
// functions in xc_mixed_hl.cu (compiled in parallel).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "xc_mixed_kernel.cuh"

namespace xcgpu {

// Fixed-point slices of the density matrices, once per build: one CTA per (spin,
// column j) finds the column's largest |P_ij|, its power-of-two scale (the largest
// scaled element below 256) and the three FP16 slices of density_slices of every scaled
// element, taken from the FP64 value, so P enters to 2^-27 of its column maximum.
// one column: its largest |P_ij| (block reduction through red[8]), the scale, the slices
__device__ __forceinline__ void split_column(const double* __restrict__ col, uint2* __restrict__ o,
                                             float* __restrict__ colscale, int nbf, double* red) {
  double m = 0.0;
  for (int i = threadIdx.x; i < nbf; i += blockDim.x) m = fmax(m, fabs(col[i]));
  for (int d = 16; d > 0; d >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, d));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
  int e = 0;
  frexp(m, &e);
  const bool zero = !(m > 0.0) || e < -100;
  const double inv = zero ? 0.0 : ldexp(1.0, 8 - e);
  if (threadIdx.x == 0) *colscale = zero ? 0.f : ldexpf(1.f, e - 8);
  for (int i = threadIdx.x; i < nbf; i += blockDim.x) {
    const double v = col[i] * inv;  // |v| < 256, exact
    const double s0 = rint(v);
    const double r1 = (v - s0) * 512.0;
    const double s1 = rint(r1);
    const double s2 = rint((r1 - s1) * 512.0);
    const uint32_t h0 = __half_as_ushort(__float2half_rn((float)s0));
    const uint32_t h1 = __half_as_ushort(__float2half_rn((float)(s1 * (1.0 / 512.0))));
    const uint32_t h2 = __half_as_ushort(__float2half_rn((float)(s2 * (1.0 / 512.0))));
    o[i] = make_uint2(h0 | (h1 << 16), h2);
  }
}

__global__ void __launch_bounds__(256) split_p_kernel(const double* __restrict__ P, uint2* __restrict__ out,
                                                      float* __restrict__ colscale, int nbf) {
  __shared__ double red[8];
  const long c = blockIdx.x;  // spin * nbf + j
  split_column(P + c * nbf, out + c * nbf, colscale + c, nbf, red);
}

// The small per-build steps of a batch of whole builds, one launch each over all its
// builds (launched per build they would be most of a batch of small builds): the split
// of P with the zeroing of V, the mirror of V, the E_xc and N_el sums.  The builds'
// columns (spin, j) form one index space, build i owning [col0[i], col0[i + 1]).
struct SmallItem {
  const double* P;
  uint2* psl;
  float* pcs;
  double* V;
  const double* partials;
  double* exc_nel;
  int nspin, nbf, nparts;
};
struct SmallBatch {
  SmallItem it[kMaxItems];
  long col0[kMaxItems + 1];
  int n;
};

__device__ __forceinline__ int small_locate(const SmallBatch& sb, long c) {
  int lo = 0, hi = sb.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sb.col0[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// one CTA per (build, spin, column j): split column j of P, zero column j of V
__global__ void __launch_bounds__(256) split_zero_batch_kernel(const __grid_constant__ SmallBatch sb) {
  __shared__ double red[8];
  const long c = blockIdx.x;
  const SmallItem& I = sb.it[small_locate(sb, c)];
  const long cl = c - sb.col0[&I - sb.it];  // spin * nbf + j within the build
  split_column(I.P + cl * I.nbf, I.psl + cl * I.nbf, I.pcs + cl, I.nbf, red);
  double* v = I.V + cl * I.nbf;
  for (int i = threadIdx.x; i < I.nbf; i += blockDim.x) v[i] = 0.0;
}

// one CTA per (build, spin, column j): rows below the diagonal from the upper triangle
__global__ void __launch_bounds__(256) mirror_batch_kernel(const __grid_constant__ SmallBatch sb) {
  const long c = blockIdx.x;
  const SmallItem& I = sb.it[small_locate(sb, c)];
  const long cl = c - sb.col0[&I - sb.it];
  const int n = I.nbf, s = (int)(cl / n), j = (int)(cl % n);
  double* M = I.V + (long)s * n * n;
  for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) M[(long)j * n + i] = M[(long)i * n + j];
}

// one CTA of 1024 threads per build: E_xc and N_el from the per-block partial sums (both
// components at once, eight loads in flight per thread, then a tree over the threads)
__global__ void __launch_bounds__(1024) sums_batch_kernel(const __grid_constant__ SmallBatch sb) {
  __shared__ double red[2][1024];
  const SmallItem& I = sb.it[blockIdx.x];
  const int n = I.nparts, t = threadIdx.x;
  double a[2][8];
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int u = 0; u < 8; ++u) a[c][u] = 0.0;
  for (int i0 = 0; i0 < n; i0 += 8 * 1024) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = i0 + u * 1024 + t;
      if (i < n) {
        a[0][u] += I.partials[i];
        a[1][u] += I.partials[(long)n + i];
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 2; ++c)
    red[c][t] = ((a[c][0] + a[c][1]) + (a[c][2] + a[c][3])) + ((a[c][4] + a[c][5]) + (a[c][6] + a[c][7]));
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (t < w) {
      red[0][t] += red[0][t + w];
      red[1][t] += red[1][t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
    I.exc_nel[0] = red[0][0];
    I.exc_nel[1] = red[1][0];
  }
}

// V holds sum_b F_b on and above the diagonal (row <= column): copy it below
__global__ void mirror_upper_kernel(double* V, int nbf, int nspin) {
  const long n2 = (long)nbf * nbf;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * nspin) return;
  const int s = (int)(idx / n2);
  const long e = idx % n2;
  const int i = (int)(e % nbf), j = (int)(e / nbf);  // row i, column j (column-major)
  if (i <= j) return;
  double* M = V + (long)s * n2;
  M[e] = M[(long)i * nbf + j];
}

xcgpu_status mixed_init(Ctx* c) {
  const void* k[] = {(const void*)mx_kernel<kModeDensity, 0, false, 3>, (const void*)mx_kernel<kModeDensity, 1, false, 3>,
                     (const void*)mx_kernel<kModeAdder, 0, false, 3>,   (const void*)mx_kernel<kModeAdder, 1, false, 3>,
                     (const void*)mx_kernel<kModeAdder, 0, true, 3>,    (const void*)mx_kernel<kModeAdder, 1, true, 3>,
                     (const void*)mx_kernel<kModeBuild, 0, false, 3>,   (const void*)mx_kernel<kModeBuild, 1, false, 3>,
                     (const void*)mx_kernel<kModeBuild, 0, true, 3>,    (const void*)mx_kernel<kModeBuild, 1, true, 3>};
  for (const void* fn : k) {
    xcgpu_status st = c->cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx_smem()),
                              "mixed kernel smem attribute");
    if (st) return st;
  }
  return mixed_init_hl(c);
}

static void fill_item(MxItem& it, const MixedWork& w) {
  it.B = *w.B;
  it.P = *w.P;
  it.nspin = w.nspin;
  it.Psl = reinterpret_cast<const uint2*>(w.Psplit);
  it.Pcs = w.Psplit ? reinterpret_cast<const float*>(it.Psl + (long)w.P->nbf * w.P->nbf * w.nspin) : nullptr;
  it.rho = w.rho;
  it.grad = w.grad;
  it.v = w.v;
  it.g = w.g;
  it.skip = w.skip;
  it.V = w.V;
  it.func = w.func;
  it.thr = w.thr;
  it.partials = w.partials;
}

// Scratch floats per CTA for the items [i0, i1): the density's [5][n_b][128] values,
// per adder operand (Phi, G per spin) the FP32 rows with their low parts, the slice
// tiles and the row scales of ft_max 128-function tiles, and for a whole build the
// density's planes followed by the tiles and scales.
static long cta_floats_for(const std::vector<MixedWork>& work, size_t i0, size_t i1, int* ft_max) {
  int amax = 0, smax = 1;
  for (size_t i = i0; i < i1; ++i) {
    amax = std::max(amax, work[i].P->max_active);
    smax = std::max(smax, work[i].nspin);
  }
  const int ft = std::max(1, (amax + 127) / 128);
  *ft_max = ft;
  const long dens = 5L * amax * 128;
  const long add = (long)(1 + smax) * ft * (2 * 128L * 128 + kOpTileFloats + 128);
  const long build = 5L * ft * 128 * 128 + (long)(1 + smax) * ft * (kOpTileFloats + 128);
  return (std::max(std::max(dens, add), build) + 63) & ~63L;
}

// parameter blocks for the items [i0, i1) of a batch
static void make_batch(const std::vector<MixedWork>& work, size_t i0, size_t i1, MxBatch& bt) {
  bt.nitems = (int)(i1 - i0);
  bt.bstart[0] = 0;
  for (size_t i = i0; i < i1; ++i) {
    fill_item(bt.items[i - i0], work[i]);
    bt.bstart[i - i0 + 1] = bt.bstart[i - i0] + work[i].P->nblocks;
  }
  bt.nblocks = bt.bstart[bt.nitems];
}

// the calling stream's scratch, grown to the batch's need (allocation happens only on
// growth, so graph capture works after one uncaptured run of the same batch)
static xcgpu_status batch_scratch(Ctx* c, const std::vector<MixedWork>& work, size_t i0, size_t i1, MxBatch& bt) {
  bt.cta_floats = cta_floats_for(work, i0, i1, &bt.ft_max);
  const size_t bytes = (size_t)bt.cta_floats * c->sm_count * sizeof(float);
  auto& buf = c->mixed_by_stream[c->stream];
  if (!buf) buf.reset(new DevBuf());
  if (buf->bytes < bytes || !buf->p) {
    xcgpu_status st = buf->alloc(c, bytes);
    if (st) return st;
    if ((st = c->cuda(cudaMemsetAsync(buf->p, 0, bytes, c->stream), "memset mixed scratch"))) return st;
  }
  bt.scratch = buf->as<float>();
  return XCGPU_OK;
}

xcgpu_status mixed_split(Ctx* c, const double* Pm, int nspin, int nbf, float* Psplit) {
  KernelTimer kt(c, kOther);
  uint2* sl = reinterpret_cast<uint2*>(Psplit);
  float* cs = reinterpret_cast<float*>(sl + (long)nspin * nbf * nbf);
  split_p_kernel<<<(unsigned)(nspin * nbf), 256, 0, c->stream>>>(Pm, sl, cs, nbf);
  return c->check_launch("split_p_kernel");
}

// one persistent launch per kMaxItems items of the mode's kernel
template <int MODE>
static xcgpu_status mixed_launch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err, int cls,
                                 const char* what) {
  static thread_local MxBatch bt;  // host-side parameter block (the launch copies it)
  for (size_t i0 = 0; i0 < work.size(); i0 += kMaxItems) {
    const size_t i1 = std::min(work.size(), i0 + kMaxItems);
    make_batch(work, i0, i1, bt);
    if (bt.nblocks == 0) continue;
    xcgpu_status st = batch_scratch(c, work, i0, i1, bt);
    if (st) return st;
    if ((st = c->cuda(cudaMemsetAsync(counter, 0, sizeof(int), c->stream), "counter"))) return st;
    bool two = false, gga = false, high_l = false;
    for (size_t i = i0; i < i1; ++i) {
      two = two || work[i].nspin == 2;
      high_l = high_l || work[i].B->maxl > 3;
      gga = gga || (MODE == kModeDensity ? work[i].grad != nullptr
                    : MODE == kModeAdder ? work[i].g != nullptr
                                         : xc::is_gga(work[i].func));
    }
    KernelTimer kt(c, cls);
    if (high_l) {
      mixed_launch_hl(MODE, gga, two, (unsigned)c->sm_count, c->stream, bt, counter, err);
    } else {
      auto* kern = MODE == kModeDensity ? (gga ? mx_kernel<MODE, 1, false, 3> : mx_kernel<MODE, 0, false, 3>)
                   : gga ? (two ? mx_kernel<MODE, 1, true, 3> : mx_kernel<MODE, 1, false, 3>)
                         : (two ? mx_kernel<MODE, 0, true, 3> : mx_kernel<MODE, 0, false, 3>);
      kern<<<c->sm_count, kT, mx_smem(), c->stream>>>(bt, counter, err);
    }
    if ((st = c->check_launch(what))) return st;
  }
  return XCGPU_OK;
}

static xcgpu_status mirror_all(Ctx* c, const std::vector<MixedWork>& work) {
  KernelTimer kt(c, kOther);
  for (const auto& w : work) {
    const long n = (long)w.P->nbf * w.P->nbf * w.nspin;
    mirror_upper_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(w.V, w.P->nbf, w.nspin);
    xcgpu_status st = c->check_launch("mirror_upper_kernel");
    if (st) return st;
  }
  return XCGPU_OK;
}

xcgpu_status mixed_density_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err) {
  return mixed_launch<kModeDensity>(c, work, counter, err, kDensity, "mx_kernel (density)");
}

xcgpu_status mixed_adder_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err) {
  xcgpu_status st = mixed_launch<kModeAdder>(c, work, counter, err, kAdder, "mx_kernel (adder)");
  return st ? st : mirror_all(c, work);
}

// the batched small steps of whole builds: before (split P, zero V) or after (mirror V,
// E_xc and N_el) the build kernel
static xcgpu_status small_launches(Ctx* c, const std::vector<MixedWork>& work, bool before) {
  static thread_local SmallBatch sb;  // host-side parameter block (the launch copies it)
  KernelTimer kt(c, kOther);
  for (size_t i0 = 0; i0 < work.size(); i0 += kMaxItems) {
    const size_t i1 = std::min(work.size(), i0 + kMaxItems);
    sb.n = (int)(i1 - i0);
    sb.col0[0] = 0;
    for (size_t i = i0; i < i1; ++i) {
      const MixedWork& w = work[i];
      const int nbf = w.P->nbf;
      SmallItem& it = sb.it[i - i0];
      it.P = w.Pm;
      it.psl = reinterpret_cast<uint2*>(w.Psplit);
      it.pcs = reinterpret_cast<float*>(it.psl + (long)w.nspin * nbf * nbf);
      it.V = w.V;
      it.partials = w.partials;
      it.exc_nel = w.exc_nel;
      it.nspin = w.nspin;
      it.nbf = nbf;
      it.nparts = w.P->nblocks;
      sb.col0[i - i0 + 1] = sb.col0[i - i0] + (long)w.nspin * nbf;
    }
    const long ncol = sb.col0[sb.n];
    if (before) {
      if (ncol > 0) split_zero_batch_kernel<<<(unsigned)ncol, 256, 0, c->stream>>>(sb);
    } else {
      if (ncol > 0) mirror_batch_kernel<<<(unsigned)ncol, 256, 0, c->stream>>>(sb);
      sums_batch_kernel<<<(unsigned)sb.n, 1024, 0, c->stream>>>(sb);
    }
    xcgpu_status st = c->check_launch(before ? "split_zero_batch_kernel" : "mirror_batch_kernel / sums_batch_kernel");
    if (st) return st;
  }
  return XCGPU_OK;
}

xcgpu_status mixed_build_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err) {
  xcgpu_status st = small_launches(c, work, true);
  if (!st) st = mixed_launch<kModeBuild>(c, work, counter, err, kBuild, "mx_kernel (build)");
  return st ? st : small_launches(c, work, false);
}

}  // namespace xcgpu
