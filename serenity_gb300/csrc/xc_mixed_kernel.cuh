// Mixed-precision XC build on the sm_103a tensor cores.
//
// Basis values and gradients are evaluated in FP32 (with an exponential whose errors
// average to zero); the two dense contractions run as tcgen05 MMAs on fixed-point
// operands: every row (or column) of an operand is scaled by a power of two and cut
// into three 8-bit slices held exactly in FP16, so the products of leading slices are
// integers that the FP32 accumulation in tensor memory (TMEM) sums without rounding,
// whatever the rounding of the tensor core's adder tree:
//   density : X = Phi P_b            (M = 128 points, N = active functions, K = functions)
//             rho = rowsum(X o Phi), grad rho = 2 rowsum(X o grad Phi), summed in FP64
//   adder   : F_b = Phi^T G + G^T Phi (M, N = active functions, K = points)
//             with G = w (v/2 Phi + g . grad Phi); F_b goes to V in FP64 (red.add)
//             (ScalarOperatorToMatrixAdder.cpp:224-303).
// The functional, E_xc, N_el and the cross-block Vxc accumulation stay in FP64.
//
// Both kernels are persistent (one CTA of 512 threads per SM, blocks taken from a
// global counter); one elected thread issues the MMAs; completion is tracked with
// mbarriers through tcgen05.commit; every wait is bounded in time and reports a
// timeout through the error word instead of hanging.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "basis_eval.cuh"
#include "exp_tang.cuh"
#include "functionals.cuh"
#include "internal.h"
#include "tcgen05.cuh"

namespace xcgpu {

constexpr uint32_t kTileA = 128 * 128;  // bytes of a 128-row x 128-byte operand tile
constexpr uint64_t kWaitLimitNs = 2000000000ull;
constexpr int kErrTimeout = 1;  // error word values (read by the host after a build)
constexpr int kErrScratch = 2;

// Point coordinates as FP32 high part + remainder; with the shell records' split
// centres, x = (p_hi - A_hi) + (p_lo - A_lo) carries FP32 relative accuracy of p - A.
struct Pt {
  float h[3], l[3];
};
__device__ __forceinline__ Pt make_pt(const double* xyz) {
  Pt q;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    q.h[i] = (float)xyz[i];
    q.l[i] = (float)(xyz[i] - (double)q.h[i]);
  }
  return q;
}
__device__ __forceinline__ int rec_l(int info) { return info & 7; }
__device__ __forceinline__ bool rec_pure(int info) { return (info >> 3) & 1; }
__device__ __forceinline__ int rec_nprim(int info) { return (info >> 4) & 31; }
__device__ __forceinline__ int rec_nf(int info) { return (info >> 9) & 31; }
__device__ __forceinline__ int rec_f0(int info) { return info >> 14; }

// Evaluate one shell record at a point in FP32; Emit(f, value, value_lo, dx, dy, dz)
// (value_lo: the angular part's and the coefficients' rounding, shell_functions_px).
// Negligible shells (|R| below the radial threshold) emit zeros.  The radial factor and
// its derivative are summed as FP32 pairs (exp_tang2, products and sums with their
// rounding errors) and *rlo receives R_lo / R_hi: all grid points of one radial shell of
// an atom share the atom's functions' R, so its FP32 rounding would be the same error at
// all of them (and at every atom of the element) instead of averaging out; value * (1 +
// *rlo) carries R to ~2^-30, and the gradients take both pairs' low parts
// (shell_functions_px).  The point-centre offset is a pair too: x = (p_hi - A_hi) + (p_lo - A_lo)
// with the first difference's rounding kept (two-sum), so r^2 and the angular factors
// see p - A to ~2^-48 instead of one FP32 rounding per coordinate.
template <int DERIV, int MAXL, class Emit>
__device__ __forceinline__ void shell_rec_at(const ShellRec& r, const float4* __restrict__ prim4, const Pt& q,
                                             float expthr, float thr, float* rlo, Emit&& emit) {
  F2 d[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float s = __fsub_rn(q.h[i], r.ah[i]), bp = __fsub_rn(s, q.h[i]);
    const float e = __fadd_rn(__fsub_rn(q.h[i], __fsub_rn(s, bp)), __fsub_rn(-r.ah[i], bp));
    const float dl = __fadd_rn(__fsub_rn(q.l[i], r.al[i]), e);
    const float h = __fadd_rn(s, dl);
    d[i] = F2{h, __fsub_rn(dl, __fsub_rn(h, s))};
  }
  const float x = d[0].h, y = d[1].h, z = d[2].h;
  // r^2 = r2 + r2l (products by FMA, sums by two-sum, the offsets' low parts to first
  // order): on a radial shell of the function's own atom r^2 is one number, so a
  // rounding of it (or of alpha r^2) would be one relative error t 2^-25 of exp(-t) at
  // every point of the shell
  float r2 = __fmul_rn(x, x), r2l = fmaf(x, x, -r2);
  {
    const float yy = __fmul_rn(y, y), zz = __fmul_rn(z, z);
    const float s1 = __fadd_rn(r2, yy), b1 = __fsub_rn(s1, r2);
    const float e1 = __fadd_rn(__fsub_rn(r2, __fsub_rn(s1, b1)), __fsub_rn(yy, b1));
    const float s2 = __fadd_rn(s1, zz), b2 = __fsub_rn(s2, s1);
    const float e2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b2)), __fsub_rn(zz, b2));
    r2l = __fadd_rn(__fadd_rn(r2l, __fadd_rn(e1, e2)), __fadd_rn(fmaf(y, y, -yy), fmaf(z, z, -zz)));
    r2l = fmaf(2.f, fmaf(x, d[0].l, fmaf(y, d[1].l, __fmul_rn(z, d[2].l))), r2l);
    r2 = s2;
  }
  const int np = rec_nprim(r.info);
  float Rv = 0.f, Rl = 0.f, D = 0.f, Dl = 0.f;  // R and D = sum alpha c exp(-alpha r^2) = -R'/2
  for (int i = 0; i < np; ++i) {
    const float4 ac = __ldg(prim4 + r.prim0 + i);  // alpha = x + z, coef = y + w
    const float t = __fmul_rn(ac.x, r2);           // alpha r^2 = t + tl
    const float tl = fmaf(ac.x, r2l, fmaf(ac.z, r2, fmaf(ac.x, r2, -t)));
    if (t < expthr) {
      // explicit roundings: R comes out bit-identical whether or not dR is formed
      float Eh, El;
      exp_tang2(-t, Eh, El);
      El = fmaf(-Eh, tl, El);  // exp(-t - tl) = (Eh + El)(1 - tl)
      const float eh = __fmul_rn(ac.y, Eh);
      const float el = fmaf(ac.y, El, fmaf(ac.w, Eh, fmaf(ac.y, Eh, -eh)));  // c E - eh
      const float s = __fadd_rn(Rv, eh);                                       // two-sum
      const float bp = __fsub_rn(s, Rv);
      const float err = __fadd_rn(__fsub_rn(Rv, __fsub_rn(s, bp)), __fsub_rn(eh, bp));
      Rl = __fadd_rn(Rl, __fadd_rn(err, el));
      Rv = s;
      if (DERIV >= 1) {  // D += alpha (eh + el), a pair like R
        const float ph = __fmul_rn(ac.x, eh);
        const float pl = fmaf(ac.x, el, fmaf(ac.z, eh, fmaf(ac.x, eh, -ph)));
        const float sd = __fadd_rn(D, ph), bd = __fsub_rn(sd, D);
        Dl = __fadd_rn(Dl, __fadd_rn(__fadd_rn(__fsub_rn(D, __fsub_rn(sd, bd)), __fsub_rn(ph, bd)), pl));
        D = sd;
      }
    }
  }
  const int l = rec_l(r.info);
  if (!(fabsf(Rv) >= thr)) {
    const int nf = rec_nf(r.info);
    for (int f = 0; f < nf; ++f) emit(f, 0.f, 0.f, 0.f, 0.f, 0.f);
    return;
  }
  *rlo = Rv != 0.f ? __fdividef(Rl, Rv) : 0.f;  // a correction of ~2^-24 relative: a few ulp of it suffice
  shell_functions_px_l<DERIV, MAXL>(l, d[0], d[1], d[2], Rv, Rl, -2.f * D, -2.f * Dl, rec_pure(r.info), emit);
}

__device__ __forceinline__ ShellRec load_rec(const ShellRec* p) {
  ShellRec r;
  const float4 a = __ldg(reinterpret_cast<const float4*>(p));
  const float4 b = __ldg(reinterpret_cast<const float4*>(p) + 1);
  r.ah[0] = a.x;
  r.ah[1] = a.y;
  r.ah[2] = a.z;
  r.al[0] = a.w;
  r.al[1] = b.x;
  r.al[2] = b.y;
  r.info = __float_as_int(b.z);
  r.prim0 = __float_as_int(b.w);
  return r;
}

// FP32 -> FP64 by the IEEE 754 bit layouts on the integer pipe (exact; zeros, subnormals,
// infinities and NaNs take the conversion instruction): GB300 converts on its FP64 pipe,
// at 1/64 of the FP32 rate, and every Vxc element of a block passes through here
__device__ __forceinline__ double f32_to_f64(float f) {
  const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  return __longlong_as_double((long long)(((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                                          ((uint64_t)(u & 0x7fffffu) << 29)));
}

// s += x for an FP32-pair running sum (two-sum; the pair keeps ~44 bits over a few dozen
// terms, where an FP64 sum would cost FP64 instructions)
__device__ __forceinline__ void f2_add1(F2& s, float x) {
  const float t = __fadd_rn(s.h, x), bp = __fsub_rn(t, s.h);
  s.l = __fadd_rn(s.l, __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bp)), __fsub_rn(x, bp)));
  s.h = t;
}

__device__ __forceinline__ bool wait_or_abort(uint64_t* mbar, uint32_t parity, int* err) {
  const bool ok = tc::mbar_wait_bounded(mbar, parity, kWaitLimitNs);
  if (!ok) atomicExch(err, kErrTimeout);
  return ok;
}

constexpr int kT = 512;               // threads per CTA (one CTA per SM)
constexpr int kWarps = kT / 32;
constexpr int kQ = kT / 128;          // threads per point of a 128-point block
constexpr int kNT = 128;              // rows of an operand tile (M, and N at most)
constexpr int kTileFloats = 128 * 32;  // one 16 KB operand tile (128 rows x 128 bytes) in floats

// One XC build inside a batched launch: its basis, plan, spin count and buffers.
struct MxItem {
  DevBasis B;
  DevPlan P;
  int nspin;
  const uint2* Psl;  // density kernel: FP16 slices (s0 | s1 << 16, s2) of P, per column scaled
  const float* Pcs;  // by the column's power-of-two scale Pcs[j] (fixed_slices)
  double* rho;  // outputs of the density kernel
  double* grad;
  const double* v;  // inputs of the adder kernel
  const double* g;
  const unsigned char* skip;
  double* V;
  int func;           // build: functional,
  double thr;         // adder block-skip threshold,
  double* partials;   // and the per-block E_xc, N_el partial sums [2][nblocks]
};
// Up to kMaxItems builds per launch, passed by value as the kernel parameter (no
// host staging buffer, so launches can be issued back to back and captured in a
// graph); the blocks of all items form one index space, item i owning
// [bstart[i], bstart[i+1]).  Each CTA owns `cta_floats` floats of `scratch` for the
// basis values of the block it works on.
constexpr int kMaxItems = 64;
struct MxBatch {
  MxItem items[kMaxItems];
  int bstart[kMaxItems + 1];
  int nitems;
  int nblocks;
  float* scratch;
  long cta_floats;
  int ft_max;  // 128-function tiles of the largest block (adder scratch layout)
};
static_assert(sizeof(MxBatch) <= 32764, "kernel parameter block too large");

__device__ __forceinline__ const MxItem& locate(const MxBatch& bt, int gb, int& b) {
  int lo = 0, hi = bt.nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bt.bstart[mid] <= gb) lo = mid;
    else hi = mid - 1;
  }
  b = gb - bt.bstart[lo];
  return bt.items[lo];
}

// =====================================================================================
// density, with the leading products accumulated exactly
//   The tensor core's FP32 accumulation truncates: summing positive products it loses
//   up to an ulp per accumulation step, always towards zero, which shows as a systematic
//   density deficit (about -6e-8 relative with 3xTF32 operands).  Here both operands are
//   fixed point: each row of A = Phi (one point) and each column of B = P (one function
//   nu) is scaled by a power of two that brings its largest element below 256 and cut
//   into three 9-bit slices (density_slices, 27 bits).  Per window of two 64-wide K
//   chunks the products go to four accumulators by order, s0 t0 (integers, sum below
//   2^23), s0 t1 + s1 t0 (sum below 2^24 units of 2^-9), s1 t1 (below 2^23 units of
//   2^-18) and s0 t2 + s2 t0 (below 2^24 units of 2^-18, with s2 stored as a multiple of
//   2^-9 so that every FP16 operand is a normal number): the first three sums are exact
//   in FP32 whatever the rounding of the tensor core's adder tree.  The fourth also takes
//   s1 t2 + s2 t1, which round there at 2^-35 of the leading products; left out, these
//   (2^-27) were the largest noise term of the density.  Only s2 t2 (2^-36) is dropped.
//   The slices are stored pre-scaled as FP16 (exact) and multiplied with kind::f16 MMAs.
//   1. every active shell of the block is evaluated once (value with its low part and,
//      for GGA, gradient) into the CTA's scratch, FP32, [plane][function][128 points],
//      with the largest |phi| of each point;
//   2. per pass of <= 128 functions nu: X = Phi P_b over K chunks of 64 functions mu,
//      A sliced from the scratch, B gathered from the pre-sliced density matrix; the
//      accumulators are read after every window of kWinChunks chunks;
//   3. rho_p += sum_nu X_p,nu phi_nu(p), grad rho_p += 2 sum_nu X_p,nu grad phi_nu(p).
// =====================================================================================
constexpr uint32_t kDStageBytes = 6 * kTileA;  // A slices 0-2, B slices 0-2 (64 FP16 wide)
constexpr int kWinChunks = 2;                  // density: chunks per exact window (128 functions)

// Fixed-point slices of a value v = vh + vl (|vl| at most about an ulp of vh) scaled into
// (-2^R, 2^R): v = s0 + s1 / 2^B + s2 / 2^(2B) + r with integers s0 in [-2^R, 2^R], s1, s2
// in [-2^(B-1), 2^(B-1)], |r| <= 2^-(2B+1); every step is exact (each remainder is a
// multiple of the unit of v; the remainder after s0 takes vl in) except the rounding of s2.
// Returned pre-scaled, (s0, s1 / 2^B, s2 / 2^(2B)), as FP32 values that FP16 holds exactly
// (the smallest in its subnormal range), packed two to a word by pack_h2.
//   adder   R = 7, B = 8: 24 bits; leading products below 2^14, exact sums over 1024
//   (the density uses density_slices below)
//
// Density slices of v = vh + vl (|vl| at most about an ulp of vh) scaled into (-256, 256):
// v = s0 + s1 / 2^9 + s2 / 2^18 + r, s0 in [-256, 256], s1, s2 in [-256, 256], |r| <
// 2^-18; stored as FP16 (s0, s1 / 2^9, s2 / 2^9), all exact and (but zero) normal
// numbers: the s2 products are accumulated apart and scaled by 2^-9 when read.  The last
// digit is rounded stochastically, s2 = floor(r2 + u) with a dither u in [0, 1)
// (Connolly, Higham & Mary, SIAM J. Sci. Comput. 43 (2021) A1508): an s function has the
// same value at every point of a radial shell of its atom (and at every atom of the
// element), where round-to-nearest would repeat one error; the dither makes it zero-mean.
__device__ __forceinline__ void density_slices(float vh, float vl, float u, float& f0, float& f1, float& f2) {
  f0 = rintf(vh);
  const float r1 = __fmul_rn(__fadd_rn(__fsub_rn(vh, f0), vl), 512.f);
  const float s1 = rintf(r1);
  f2 = __fmul_rn(floorf(__fadd_rn(__fmul_rn(__fsub_rn(r1, s1), 512.f), u)), 1.f / 512.f);
  f1 = __fmul_rn(s1, 1.f / 512.f);
}

template <int R, int B>
__device__ __forceinline__ void fixed_slices2(float vh, float vl, float& f0, float& f1, float& f2) {
  constexpr float up = (float)(1 << B), down = 1.f / (float)(1 << B), down2 = down * down;
  f0 = rintf(vh);
  const float r1 = __fmul_rn(__fadd_rn(__fsub_rn(vh, f0), vl), up);
  const float s1 = rintf(r1);
  f2 = __fmul_rn(rintf(__fmul_rn(__fsub_rn(r1, s1), up)), down2);
  f1 = __fmul_rn(s1, down);
}
// two FP16-exact values as one 32-bit word (a in the low half): one packing conversion
__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// dither of point g (global index): a hash to [0, 1); a function mu adds mu times the
// golden ratio (mod 1), so the dithers of one point are spread evenly
__device__ __forceinline__ float point_dither(uint32_t g) {
  g ^= g >> 16;
  g *= 0x7feb352dU;
  g ^= g >> 15;
  g *= 0x846ca68bU;
  g ^= g >> 16;
  return (float)(g >> 8) * (1.f / 16777216.f);
}
__device__ __forceinline__ float function_dither(float up, int mu) {
  const float x = fmaf((float)mu, 0.6180339887f, up);
  return __fsub_rn(x, floorf(x));
}

// power-of-two scale of a row or column with largest magnitude m >= 0: with m = f 2^e,
// 0.5 <= f < 1 (e = biased exponent - 126), scale = 2^(e - R) and inv = 2^(R - e), so
// m * inv < 2^R; rows below 2^-100 (and subnormal ones) count as zero
template <int R>
__device__ __forceinline__ void fixed_scale(float m, float& scale, float& inv) {
  const int be = (__float_as_int(m) >> 23) & 0xff;
  if (!(m > 0.f) || be < 26) {
    scale = inv = 0.f;
    return;
  }
  scale = __int_as_float((be - 126 - R + 127) << 23);
  inv = __int_as_float((R - (be - 126) + 127) << 23);
}

// the six slice products of one 64-wide K chunk: leading x leading into the accumulator
// at column acc0, the five others into the one at accR (first0 / firstR: start them);
// the three A slice tiles at abase, the three B slice tiles at bbase (shared memory)
__device__ __forceinline__ void issue_fixed_chunk2(uint32_t tmem, uint32_t acc0, uint32_t accR, uint32_t abase,
                                                   uint32_t bbase, int N, bool first0, bool firstR) {
  const uint32_t idesc = tc::idesc_f16(128, N);
  uint64_t a[3], b[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = tc::smem_desc_sw128(abase + i * kTileA);
    b[i] = tc::smem_desc_sw128(bbase + i * kTileA);
  }
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {  // 16 FP16 (32 bytes) per MMA
    const uint64_t o = 2u * ks;
    tc::mma_f16(tmem + acc0, a[0] + o, b[0] + o, idesc, (first0 && ks == 0) ? 0u : 1u);
    tc::mma_f16(tmem + accR, a[0] + o, b[1] + o, idesc, (firstR && ks == 0) ? 0u : 1u);
    tc::mma_f16(tmem + accR, a[1] + o, b[0] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[0] + o, b[2] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[1] + o, b[1] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[2] + o, b[0] + o, idesc, 1u);
  }
}

// the same with the slice tiles of A and B `astride` / `bstride` bytes apart (a B operand
// of N rows: N x 128 bytes per slice)
__device__ __forceinline__ void issue_fixed_chunk3(uint32_t tmem, uint32_t acc0, uint32_t accR, uint32_t abase,
                                                   uint32_t astride, uint32_t bbase, uint32_t bstride, int N,
                                                   bool first) {
  const uint32_t idesc = tc::idesc_f16(128, N);
  uint64_t a[3], b[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = tc::smem_desc_sw128(abase + i * astride);
    b[i] = tc::smem_desc_sw128(bbase + i * bstride);
  }
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint64_t o = 2u * ks;
    tc::mma_f16(tmem + acc0, a[0] + o, b[0] + o, idesc, (first && ks == 0) ? 0u : 1u);
    tc::mma_f16(tmem + accR, a[0] + o, b[1] + o, idesc, (first && ks == 0) ? 0u : 1u);
    tc::mma_f16(tmem + accR, a[1] + o, b[0] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[0] + o, b[2] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[1] + o, b[1] + o, idesc, 1u);
    tc::mma_f16(tmem + accR, a[2] + o, b[0] + o, idesc, 1u);
  }
}

// the same with the stage layout of a streamed step: A slices, then B slices
__device__ __forceinline__ void issue_fixed_chunk(uint32_t tmem, uint32_t acc0, uint32_t accR, uint32_t stage, int N,
                                                  bool first0, bool firstR) {
  issue_fixed_chunk2(tmem, acc0, accR, stage, stage + 3 * kTileA, N, first0, firstR);
}

// density: the six slice products of one 64-wide K chunk into four accumulators: s0 t0
// (column 0), s0 t1 + s1 t0 (128), s1 t1 (256), s0 t2 + s2 t0 (384, in units of 2^9);
// first starts them
__device__ __forceinline__ void issue_density_chunk(uint32_t tmem, uint32_t stage, int N, bool first) {
  const uint32_t idesc = tc::idesc_f16(128, N);
  uint64_t a[3], b[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = tc::smem_desc_sw128(stage + i * kTileA);
    b[i] = tc::smem_desc_sw128(stage + (3 + i) * kTileA);
  }
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {  // 16 FP16 (32 bytes) per MMA
    const uint64_t o = 2u * ks;
    const uint32_t acc = (first && ks == 0) ? 0u : 1u;
    tc::mma_f16(tmem + 0, a[0] + o, b[0] + o, idesc, acc);
    tc::mma_f16(tmem + 128, a[0] + o, b[1] + o, idesc, acc);
    tc::mma_f16(tmem + 128, a[1] + o, b[0] + o, idesc, 1u);
    tc::mma_f16(tmem + 256, a[1] + o, b[1] + o, idesc, acc);
    tc::mma_f16(tmem + 384, a[0] + o, b[2] + o, idesc, acc);
    tc::mma_f16(tmem + 384, a[2] + o, b[0] + o, idesc, 1u);
    // the third-order products s1 t2 + s2 t1 carry the same 2^-9 weight as the stored
    // third slices: added here they round in this accumulator (2^-35 of the leading
    // products) instead of being left out (2^-27)
    tc::mma_f16(tmem + 384, a[1] + o, b[2] + o, idesc, 1u);
    tc::mma_f16(tmem + 384, a[2] + o, b[1] + o, idesc, 1u);
  }
}

// =====================================================================================
// adder: F_b = Phi^T G + G^T Phi per block, G = w (v/2 Phi + g . grad Phi); V += F_b with
// FP64 red.add on and above the diagonal (ScalarOperatorToMatrixAdder.cpp:224-303).  The
// leading slice products are accumulated exactly, as in the density:
//   1a. every active shell of the block is evaluated once; Phi and G (per spin) go to
//       the CTA's scratch in FP32 with their low parts, [part][operand][function][128
//       points];
//   1b. one warp per (operand, function) row: the row's largest |value| over the block's
//       points sets its power-of-two scale (kept in the scratch), and the three FP16
//       slices of the scaled row go to the scratch as operand tiles (128 functions x 64
//       points, 128-byte swizzled K-major: the shared-memory image of the tile);
//   2. per spin and function tile pair a <= b: P1 = Phi_a^T G_b and P2 = G_a^T Phi_b
//      (= (Phi_b^T G_a)^T, so F(a, b) = P1 + P2 needs no transposition), each over
//      64-point chunks.  Thread 0 streams the six slice tiles of a step into one of two
//      shared-memory stages with bulk copies (TMA) and issues the MMAs: leading x leading
//      into one accumulator, the five other slice products into a second, per product
//      (all 512 TMEM columns).  After a pair every thread reads its row's 32 columns of
//      the four accumulators, applies the row and column scales and adds F to V.
//   Steps are numbered per CTA (J); step J uses stage J & 1 and completes phase
//   (J >> 1) & 1 of that stage's barriers, so every waiter knows its parity.
// =====================================================================================
constexpr int kOpTileFloats = 2 * 3 * kTileFloats;  // one 128-function tile: 2 chunks x 3 slices
// restricted build blocks of 129..kMidMax functions keep their G slice tiles (all
// functions, both chunks: at most 2 x 3 x 192 x 128 bytes) in shared memory behind one
// 48 KB slot for the Phi tile being multiplied
constexpr int kMidMax = 192;
constexpr uint32_t kMidB = 3 * kTileA;  // offset of the G tiles

// =====================================================================================
// The mixed kernels, one template in three modes:
//   kModeDensity  rho, grad rho of every block (1. + 2. below)
//   kModeAdder    V from given v, g (3. below, with its own shell evaluation)
//   kModeBuild    per block 1., 2., the functional at the block's points, and 3. with G
//                 formed from the stored basis values: a whole build
//                 (FuncPotential::getMatrix) whose basis values are evaluated once and
//                 whose rho, v and g never leave the SM
// =====================================================================================
enum MxMode { kModeDensity = 0, kModeAdder = 1, kModeBuild = 2 };

// MAXL: the largest angular momentum the kernel evaluates (3 for bases up to f
// functions, 6 for the rest): the l = 4..6 code raises the register pressure of the
// whole kernel, so it is only in the kernels that bases with g..i functions select.
template <int MODE, int DERIV, bool TWO_SPINS, int MAXL>
__global__ void __launch_bounds__(kT, 1)
    mx_kernel(const __grid_constant__ MxBatch bt, int* __restrict__ counter, int* __restrict__ err) {
  constexpr bool HAS_D = MODE != kModeAdder, HAS_A = MODE != kModeDensity;
  constexpr int NOPS = TWO_SPINS ? 3 : 2;  // adder operands: Phi, G per spin
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar[2], full[2], mdone[2], fdone, mfull, mmma, afull[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_block, s_abort, s_smask;
  __shared__ int s_next[4];  // basis phase: next shell of the block, per 32-point group
  __shared__ Pt s_pt[HAS_D ? 128 : 1];  // basis phase: the block's points as FP32 pairs (FP64 split once per point)
  __shared__ double s_part[4][kQ - 1][128];  // density: partial sums of a point's threads
  __shared__ unsigned s_amax[128];           // per point: largest |phi| (FP32 bits)
  __shared__ float s_bscale[kNT];            // per function nu of the pass: scale of its column of P
  __shared__ long s_rowoff[kNT];             // and the offset of that column
  __shared__ __align__(16) float s_w[2][4][128];  // adder: per spin and point w v / 2, w g_x, w g_y, w g_z
  __shared__ double s_rg[MODE == kModeBuild ? 2 * 4 * 128 : 1];  // build: rho, grad rho per spin
  const uint32_t base_s = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base_s & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p = tid & 127, quarter = tid >> 7;  // point (TMEM lane), and which of its kQ threads
  const int c0 = 32 * quarter;                  // this thread's 32 accumulator columns
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 512);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&mbar[i], 1);
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&mdone[i], 1);
    }
    tc::mbar_init(&fdone, 1);
    tc::mbar_init(&mfull, 1);
    tc::mbar_init(&mmma, 1);
    tc::mbar_init(&afull[0], 1);
    tc::mbar_init(&afull[1], 1);
    tc::fence_mbar_init();
    s_abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t trow = (uint32_t)(32 * (warp & 3)) << 16;
  uint32_t phase = 0, pend = 0;       // density: per stage (bit) barrier parity; a commit not yet waited for
  int gc = 0;                         // density: chunks issued by this CTA (stage = gc & 1)
  int J0 = 0;                         // adder: steps of earlier blocks (uniform)
  int last_copy = -1, last_mma = -1;  // adder, thread 0: highest step copied / issued
  uint32_t fphase = 0;                // parity of the shared-memory tile pair's barrier
  uint32_t mphase = 0;                // parities of mfull (bit 0) and mmma (bit 1)
  uint32_t aphase = 0;                // density: per stage (bit) parity of afull
  float* const my = bt.scratch + (long)blockIdx.x * bt.cta_floats;
  const long rows_pad = (long)bt.ft_max * 128;
  // adder scratch: (adder mode) FP32 operand rows [2][NOPS][rows_pad][128]: values, low
  // parts; (build) the density phase's planes come first; then the slice tiles
  // [NOPS][ft_max][2 chunks][3 slices][4096] and the row scales [NOPS][rows_pad]
  float* const stg = my;
  float* const tiles = my + (MODE == kModeBuild ? 5 : 2 * NOPS) * rows_pad * 128;
  float* const scl = tiles + NOPS * bt.ft_max * kOpTileFloats;

  // a tile pair's four accumulators -> V of item It (its block's active functions fnb,
  // nact_b of them), on and above the diagonal, FP64 red.add
  auto pair_to_V = [&](const MxItem& It, const int* fnb, int nact_b, int spin, int a, int bb) {
    const int nbf_b = It.P.nbf;
    const int row = 32 * (warp & 3) + lane, c0 = 32 * (warp >> 2);
    const int ma = min(128, nact_b - 128 * a), nb = min(128, nact_b - 128 * bb);
    const int N = (nb + 15) & ~15;
    const bool rok = row < ma;
    const int m = 128 * a + row;
    const float sPm = rok ? scl[m] : 0.f, sGm = rok ? scl[(1 + spin) * rows_pad + m] : 0.f;
    double* Vrow = It.V + (long)spin * nbf_b * nbf_b + (rok ? __ldg(fnb + m) : 0);
    const float* sPn = scl + 128 * bb;
    const float* sGn = scl + (1 + spin) * rows_pad + 128 * bb;
    if (c0 < N) {  // warp-uniform
#pragma unroll 1
      for (int cb = c0; cb < c0 + 32; cb += 8) {
        float p0[8], pr[8], q0[8], qr[8];
        tc::tmem_ld8x4(tmem + trow + 0 + cb, tmem + trow + 128 + cb, tmem + trow + 256 + cb, tmem + trow + 384 + cb, p0,
                       pr, q0, qr);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int n = cb + c;
          if (rok && n < nb && (a < bb || n >= row)) {
            const float f1 = __fmul_rn(__fadd_rn(p0[c], pr[c]), __fmul_rn(sPm, sGn[n]));
            const float f2 = __fmul_rn(__fadd_rn(q0[c], qr[c]), __fmul_rn(sGm, sPn[n]));
            atomicAdd(Vrow + (long)__ldg(fnb + 128 * bb + n) * nbf_b, f32_to_f64(__fadd_rn(f1, f2)));
          }
        }
      }
    }
  };

  // the one tile pair of a restricted block of at most 128 functions: only T = Phi^T G is
  // formed, since F = T + T^T (the other product, G^T Phi, is T transposed: the same slice
  // products summed in another order); T goes through shared memory (the operand tiles,
  // consumed by then) so that each thread pairs T(m, n) with T(n, m)
  auto diag_to_V = [&](const MxItem& It, const int* fnb, int nact_b) {
    const int nbf_b = It.P.nbf;
    const int row = 32 * (warp & 3) + lane, c0 = 32 * (warp >> 2);
    const int N = (nact_b + 15) & ~15;
    float* const T = reinterpret_cast<float*>(sm);  // [128][129]
    if (c0 < N) {  // warp-uniform
      const float sPm = row < nact_b ? scl[row] : 0.f;
      const float* sGn = scl + rows_pad;
#pragma unroll 1
      for (int cb = c0; cb < c0 + 32; cb += 8) {
        float p0[8], pr[8];
        tc::tmem_ld8x2(tmem + trow + cb, tmem + trow + 128 + cb, p0, pr);
#pragma unroll
        for (int c = 0; c < 8; ++c)
          T[row * 129 + cb + c] = __fmul_rn(__fadd_rn(p0[c], pr[c]), __fmul_rn(sPm, sGn[cb + c]));
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (c0 < N && row < nact_b) {
      double* Vrow = It.V + __ldg(fnb + row);
#pragma unroll 4
      for (int c = 0; c < 32; ++c) {
        const int n = c0 + c;
        if (n < nact_b && n >= row)
          atomicAdd(Vrow + (long)__ldg(fnb + n) * nbf_b, f32_to_f64(__fadd_rn(T[row * 129 + n], T[n * 129 + row])));
      }
    }
  };

  for (;;) {
    if (HAS_D && tid < 128) s_amax[tid] = 0u;
    if (tid < 4) s_next[tid] = 0;
    __syncthreads();
    if (tid == 0) s_block = atomicAdd(counter, 1);
    __syncthreads();
    const int gb = s_block;
    if (gb >= bt.nblocks || s_abort) break;
    int b;
    const MxItem& I = locate(bt, gb, b);
    const DevBasis& B = I.B;
    const DevPlan& P = I.P;
    const int nspin = I.nspin, nbf = P.nbf;
    const long first = (long)b * P.max_block;
    const int npts = (int)min((long)P.max_block, P.npoints - first);
    const int nact = P.fn_off[b + 1] - P.fn_off[b];
    const int* __restrict__ fn = P.fn_list + P.fn_off[b];
    const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
    const long cs = (long)nact * 128;  // plane stride of the density scratch: value, its low part, gradient
    const int nft = (nact + 127) >> 7;
    // a restricted build block of at most 128 functions: its Phi and G slice tiles (2 x 96
    // KB) take the place of the two MMA stages, so the slicing writes them straight to
    // shared memory and the one tile pair's MMAs read them there (no round trip through
    // the global scratch and no bulk copies)
    const bool tiles_in_smem = MODE == kModeBuild && !TWO_SPINS && nft == 1;
    // 129..kMidMax functions: G tiles in shared memory, T = Phi^T G one Phi tile at a time
    const bool tiles_mid = MODE == kModeBuild && !TWO_SPINS && nft == 2 && nact <= kMidMax;
    const int npad = (nact + 15) & ~15;
    int smask = 0;
    if constexpr (MODE == kModeAdder) {
      for (int s = 0; s < nspin; ++s)
        if (!I.skip[(long)s * P.nblocks + b]) smask |= 1 << s;
      if (smask == 0 || nact == 0) continue;
    }
    if (HAS_A && (nft > bt.ft_max || nspin > NOPS - 1 ||
                  (tiles - my) + (long)NOPS * (bt.ft_max * kOpTileFloats + rows_pad) > bt.cta_floats)) {
      if (tid == 0) atomicExch(err, kErrScratch);  // scratch sized for a smaller block: report, skip
      continue;
    }
    if constexpr (HAS_D) {
      if (5L * rows_pad * 128 + (long)nft * kOpTileFloats > bt.cta_floats) {  // scratch sized for a smaller block
        if (tid == 0) atomicExch(err, kErrScratch);
        continue;
      }
      const bool live = p < npts;
      if (quarter == 0) s_pt[p] = make_pt(P.xyz + 3 * (first + (live ? p : 0)));
      __syncthreads();
    // ---- 1. basis values (and gradients) of the block, largest |phi| per point ----
    {
      const Pt pt = s_pt[p];
      const float expthr = (float)P.exponent_threshold, thr = (float)P.radial_threshold;
      float* const col = my + p;
      float vmax = 0.f;
      // the kQ warps of a 32-point group take the block's shells from a shared counter
      // (shells differ in cost: a fixed split leaves warps waiting at the barrier)
      const int nsh = s1 - s0;
      auto grab = [&]() {
        int v = 0;
        if (lane == 0) v = atomicAdd(&s_next[warp & 3], 1);
        return __shfl_sync(0xffffffffu, v, 0);
      };
      int cur = grab();
      ShellRec next;
      if (cur < nsh) next = load_rec(P.rec + s0 + cur);
      while (cur < nsh) {  // warp-uniform
        const ShellRec r = next;
        const int nx = grab();
        if (nx < nsh) next = load_rec(P.rec + s0 + nx);  // in flight while r is evaluated
        cur = nx;
        float* const t0 = col + (long)rec_f0(r.info) * 128;
        float rlo = 0.f;
        auto put = [&](int f, float v, float vl, float dx, float dy, float dz) {
          float* t = t0 + f * 128;
          t[0] = v;
          t[cs] = fmaf(v, rlo, vl);  // the value's low part: radial factor's and coefficients'
          vmax = fmaxf(vmax, fabsf(v));
          if (DERIV) {
            t[2 * cs] = dx;
            t[3 * cs] = dy;
            t[4 * cs] = dz;
          }
        };
        if (live) {
          shell_rec_at<DERIV, MAXL>(r, B.prim4, pt, expthr, thr, &rlo, put);
        } else {
          const int nf = rec_nf(r.info);
          for (int f = 0; f < nf; ++f) put(f, 0.f, 0.f, 0.f, 0.f, 0.f);
        }
      }
      atomicMax(&s_amax[p], __float_as_uint(vmax));  // non-negative floats order as integers
    }
    __syncthreads();
      {
    float sa, inva;  // this point's row scale
    fixed_scale<8>(__uint_as_float(s_amax[p]), sa, inva);
    const float up = point_dither((uint32_t)(first + p));
    const int nkc = (nact + 63) / 64;
    for (int s = 0; s < nspin; ++s) {
      const uint2* __restrict__ Psl = I.Psl + (long)s * nbf * nbf;
      const float* __restrict__ Pcs = I.Pcs + (long)s * nbf;
      // this thread's share of rho and grad rho over its columns, summed in FP32 pairs
      F2 r2{0.f, 0.f}, g2[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      // the basis values' low parts enter through their own FP32 sum: added into rr, each
      // (about an ulp of rr) would mostly round away, a systematic loss of the corrections
      float r_lo = 0.f;
      for (int nu0 = 0; nu0 < nact; nu0 += kNT) {
        const int nnu = min(kNT, nact - nu0);
        const int N = (nnu + 15) & ~15;
        if (tid < nnu) {
          const int f = __ldg(fn + nu0 + tid);
          s_bscale[tid] = __ldg(Pcs + f);
          s_rowoff[tid] = (long)f * nbf;
        }
        __syncthreads();  // the B fill of the pass's first chunk reads s_rowoff
        for (int kc = 0; kc < nkc; ++kc) {
          const int st = gc & 1;
          if ((pend >> st) & 1u) {  // the MMAs of two chunks ago still read this stage
            const bool ok = wait_or_abort(&mbar[st], (phase >> st) & 1u, err);
            phase ^= 1u << st;
            pend &= ~(1u << st);
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
          }
          uint8_t* const stage = sm + st * kDStageBytes;
          const int mu0 = kc * 64;
          // A of chunk kc is the same in every pass and for every spin: in the two-spin
          // kernels it is sliced in the first pass of the first spin, kept in the scratch
          // after the planes and copied back into the stage by the later passes (in the
          // one-spin kernels the extra code cost more in the rest of the kernel, measured,
          // than it saved in their few multi-pass blocks)
          const bool reuseA = TWO_SPINS && (nu0 > 0 || s > 0);
          const bool saveA = TWO_SPINS && !reuseA && (nact > kNT || nspin > 1);
          uint8_t* const agl = reinterpret_cast<uint8_t*>(my + 5 * rows_pad * 128) + kc * 3 * kTileA;
          if (reuseA) {
            if (tid == 0) {
              tc::mbar_arrive_expect_tx(&afull[st], 3 * kTileA);
#pragma unroll
              for (int q = 0; q < 3; ++q) tc::bulk_g2s(stage + q * kTileA, agl + q * kTileA, kTileA, &afull[st]);
            }
          } else {
          // ---- A: row p, 16-byte chunks j = 2 quarter, 2 quarter + 1 (8 functions each) ----
            float av[16], al[16];  // all loads in flight before any is used
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const int mu = mu0 + 16 * quarter + e;
              av[e] = mu < nact ? my[(long)mu * 128 + p] : 0.f;
              al[e] = mu < nact ? my[cs + (long)mu * 128 + p] : 0.f;
            }
#pragma unroll
            for (int jj = 0; jj < 2; ++jj) {
              const int j = 2 * quarter + jj;
              uint32_t w0[4], w1[4], w2[4];
#pragma unroll
              for (int e = 0; e < 8; e += 2) {
                float a0, a1, a2, b0, b1, b2;
                const int k = 8 * jj + e, mu = mu0 + 16 * quarter + k;
                density_slices(__fmul_rn(av[k], inva), __fmul_rn(al[k], inva), function_dither(up, mu), a0, a1, a2);
                density_slices(__fmul_rn(av[k + 1], inva), __fmul_rn(al[k + 1], inva), function_dither(up, mu + 1),
                                 b0, b1, b2);
                w0[e >> 1] = pack_h2(a0, b0);
                w1[e >> 1] = pack_h2(a1, b1);
                w2[e >> 1] = pack_h2(a2, b2);
              }
              const uint32_t off = (uint32_t)(p * 128 + ((j ^ (p & 7)) << 4));
              const uint4 q0 = make_uint4(w0[0], w0[1], w0[2], w0[3]), q1 = make_uint4(w1[0], w1[1], w1[2], w1[3]),
                          q2 = make_uint4(w2[0], w2[1], w2[2], w2[3]);
              *reinterpret_cast<uint4*>(stage + off) = q0;
              *reinterpret_cast<uint4*>(stage + kTileA + off) = q1;
              *reinterpret_cast<uint4*>(stage + 2 * kTileA + off) = q2;
              if (saveA) {
                *reinterpret_cast<uint4*>(agl + off) = q0;
                *reinterpret_cast<uint4*>(agl + kTileA + off) = q1;
                *reinterpret_cast<uint4*>(agl + 2 * kTileA + off) = q2;
              }
            }
            if (saveA) tc::fence_async_global();  // read back by the later passes' bulk copies
          }
          // ---- B: row nu, elements mu0 + 2 lane, + 1: P[fn[mu]][fn[nu]] (symmetric P); a
          //      warp's rows (at most 8) loaded together, row offsets from shared memory ----
          {
            const int k0 = 2 * lane;
            const int muA = mu0 + k0, muB = muA + 1;
            const long cA = muA < nact ? (long)__ldg(fn + muA) : -1;
            const long cB = muB < nact ? (long)__ldg(fn + muB) : -1;
            uint2 ea[kNT / kWarps], eb[kNT / kWarps];
#pragma unroll
            for (int k = 0; k < kNT / kWarps; ++k) {
              const int row = warp + k * kWarps;
              ea[k] = eb[k] = make_uint2(0u, 0u);
              if (row < nnu) {
                const uint2* prow = Psl + s_rowoff[row];
                if (cA >= 0) ea[k] = __ldg(prow + cA);
                if (cB >= 0) eb[k] = __ldg(prow + cB);
              }
            }
#pragma unroll
            for (int k = 0; k < kNT / kWarps; ++k) {
              const int row = warp + k * kWarps;
              if (row < N) {
                const uint32_t off = tc::swz_offset_h(row, k0);
                *reinterpret_cast<uint32_t*>(stage + 3 * kTileA + off) = (ea[k].x & 0xFFFFu) | (eb[k].x << 16);
                *reinterpret_cast<uint32_t*>(stage + 4 * kTileA + off) = (ea[k].x >> 16) | (eb[k].x & 0xFFFF0000u);
                *reinterpret_cast<uint32_t*>(stage + 5 * kTileA + off) = (ea[k].y & 0xFFFFu) | (eb[k].y << 16);
              }
            }
          }
          tc::fence_async_smem();
          __syncthreads();
          const int kw = kc % kWinChunks;  // chunk within the window
          if (tid == 0) {
            tc::fence_after_sync();
            bool aok = true;
            if (reuseA) {
              aok = tc::mbar_wait_bounded(&afull[st], (aphase >> st) & 1u, kWaitLimitNs);
              if (!aok) {  // report and leave after this block; the copy lands before the CTA exits
                atomicExch(err, kErrTimeout);
                s_abort = 1;
                tc::mbar_wait_bounded(&afull[st], (aphase >> st) & 1u, kWaitLimitNs);
              }
            }
            if (aok) issue_density_chunk(tmem, tc::smem_u32(stage), N, kw == 0);
            tc::mma_commit(&mbar[st]);  // (with no MMAs issued it arrives at once)
          }
          if (reuseA) aphase ^= 1u << st;
          pend |= 1u << st;
          ++gc;
          if ((kc % kWinChunks) != kWinChunks - 1 && kc != nkc - 1) continue;
          // ---- end of a window: wait for its MMAs (older stage first), read X ----
          bool ok = true;
#pragma unroll
          for (int q = 1; q >= 0; --q) {
            const int sq = (st + q) & 1;  // q = 1: the other (older) stage
            if ((pend >> sq) & 1u) {
              ok = wait_or_abort(&mbar[sq], (phase >> sq) & 1u, err) && ok;
              phase ^= 1u << sq;
              pend &= ~(1u << sq);
            }
          }
          if (__syncthreads_or(!ok)) {
            if (tid == 0) s_abort = 1;
            goto done;
          }
          tc::fence_after_sync();
          if (c0 < N) {  // warp-uniform
            const float* t = my + (long)nu0 * 128 + p;
#pragma unroll 1
            for (int cb = c0; cb < c0 + 32; cb += 8) {
              float a0[8], a1[8], ar[8], a3[8];
              tc::tmem_ld8x4(tmem + trow + cb, tmem + trow + 128 + cb, tmem + trow + 256 + cb, tmem + trow + 384 + cb,
                             a0, a1, ar, a3);
#pragma unroll
              for (int c = 0; c < 8; ++c)
                ar[c] = __fadd_rn(__fadd_rn(a0[c], a1[c]), fmaf(a3[c], 1.f / 512.f, ar[c]));
              if (live) {
                float rr = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                  const int col = cb + c;
                  if (col < nnu) {
                    const float xv = __fmul_rn(ar[c], __fmul_rn(sa, s_bscale[col]));
                    const float* tc_ = t + (long)col * 128;
                    rr = fmaf(xv, tc_[0], rr);
                    r_lo = fmaf(xv, tc_[cs], r_lo);
                    if (DERIV) {
                      gx = fmaf(xv, tc_[2 * cs], gx);
                      gy = fmaf(xv, tc_[3 * cs], gy);
                      gz = fmaf(xv, tc_[4 * cs], gz);
                    }
                  }
                }
                f2_add1(r2, rr);
                if (DERIV) {
                  f2_add1(g2[0], gx);
                  f2_add1(g2[1], gy);
                  f2_add1(g2[2], gz);
                }
              }
            }
          }
          tc::fence_before_sync();
          __syncthreads();  // the accumulators and s_bscale are reused
        }
      }
      double r_acc = ((double)r2.h + (double)r2.l) + (double)r_lo;
      double g_acc[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) g_acc[k] = (double)g2[k].h + (double)g2[k].l;
      // combine the kQ partial sums of each point
      if (quarter > 0) {
        s_part[0][quarter - 1][p] = r_acc;
        s_part[1][quarter - 1][p] = g_acc[0];
        s_part[2][quarter - 1][p] = g_acc[1];
        s_part[3][quarter - 1][p] = g_acc[2];
      }
      __syncthreads();
      if (quarter == 0) {
        if (live) {
#pragma unroll
          for (int k = 0; k < kQ - 1; ++k) {
            r_acc += s_part[0][k][p];
            g_acc[0] += s_part[1][k][p];
            g_acc[1] += s_part[2][k][p];
            g_acc[2] += s_part[3][k][p];
          }
        }
        if constexpr (MODE == kModeDensity) {
          if (live) {
            I.rho[(long)s * P.npoints + first + p] = r_acc;
            if (DERIV && I.grad) {
              I.grad[((long)s * 3 + 0) * P.npoints + first + p] = 2.0 * g_acc[0];
              I.grad[((long)s * 3 + 1) * P.npoints + first + p] = 2.0 * g_acc[1];
              I.grad[((long)s * 3 + 2) * P.npoints + first + p] = 2.0 * g_acc[2];
            }
          }
        } else {  // kept on the SM for the functional
          s_rg[(s * 4 + 0) * 128 + p] = live ? r_acc : 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k) s_rg[(s * 4 + 1 + k) * 128 + p] = live ? 2.0 * g_acc[k] : 0.0;
        }
      }
      __syncthreads();
    }
      }
    }
    // ---- 1b. row scales and FP16 slice tiles, one warp per (operand, function) row;
    //      rows r = oi * nact + m of operand oi (0: Phi, then G of the active spins),
    //      [rbeg, rend) by warp wi of a group of nw ----
    auto slice_rows = [&](int rbeg, int rend, int wi, int nw) {
      if (rbeg + wi >= rend) return;
      const int k4 = 4 * lane;  // this lane's 4 points
      // U rows per pass, their loads issued together (the rows were just written: L2
      // latency, not bandwidth, bounds this loop)
      constexpr int U = (TWO_SPINS || MODE == kModeBuild) ? 2 : 4;  // rows per pass (registers)
      int oi0 = (rbeg + wi) / nact, m0 = rbeg + wi - oi0 * nact;  // row r0 = oi0 * nact + m0
      for (int r0 = rbeg + wi; r0 < rend; r0 += U * nw) {
        float4 v[U], vl[U];
        int ou[U], mu[U];
        {
          int oi = oi0, m = m0;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            ou[u] = oi == 0 ? 0 : (smask == 2 ? 2 : oi);
            mu[u] = m;
            v[u] = vl[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r0 + u * nw < rend) {
              if constexpr (MODE == kModeAdder) {
                v[u] = *reinterpret_cast<const float4*>(stg + ((long)ou[u] * rows_pad + m) * 128 + k4);
                vl[u] = *reinterpret_cast<const float4*>(stg + ((long)(NOPS + ou[u]) * rows_pad + m) * 128 + k4);
              } else {
                // the density phase's planes (value, low part, gradient) of function m: Phi
                // itself, or G = w v/2 phi + w g . grad phi formed here as the adder's
                // shell evaluation forms it
                const float* ph = my + (long)m * 128 + k4;
                const float4 f = *reinterpret_cast<const float4*>(ph);
                const float4 fl = *reinterpret_cast<const float4*>(ph + cs);
                if (ou[u] == 0) {
                  v[u] = f;
                  vl[u] = fl;
                } else {
                  const int sp = ou[u] - 1;
                  const float4 w0 = *reinterpret_cast<const float4*>(&s_w[sp][0][k4]);
                  float4 g = make_float4(__fmul_rn(w0.x, f.x), __fmul_rn(w0.y, f.y), __fmul_rn(w0.z, f.z),
                                         __fmul_rn(w0.w, f.w));
                  if (DERIV) {
                    const float4 dx = *reinterpret_cast<const float4*>(ph + 2 * cs);
                    const float4 dy = *reinterpret_cast<const float4*>(ph + 3 * cs);
                    const float4 dz = *reinterpret_cast<const float4*>(ph + 4 * cs);
                    const float4 w1 = *reinterpret_cast<const float4*>(&s_w[sp][1][k4]);
                    const float4 w2 = *reinterpret_cast<const float4*>(&s_w[sp][2][k4]);
                    const float4 w3 = *reinterpret_cast<const float4*>(&s_w[sp][3][k4]);
                    g.x = fmaf(w3.x, dz.x, fmaf(w2.x, dy.x, fmaf(w1.x, dx.x, g.x)));
                    g.y = fmaf(w3.y, dz.y, fmaf(w2.y, dy.y, fmaf(w1.y, dx.y, g.y)));
                    g.z = fmaf(w3.z, dz.z, fmaf(w2.z, dy.z, fmaf(w1.z, dx.z, g.z)));
                    g.w = fmaf(w3.w, dz.w, fmaf(w2.w, dy.w, fmaf(w1.w, dx.w, g.w)));
                  }
                  v[u] = g;
                  vl[u] = make_float4(__fmul_rn(w0.x, fl.x), __fmul_rn(w0.y, fl.y), __fmul_rn(w0.z, fl.z),
                                      __fmul_rn(w0.w, fl.w));
                }
              }
            }
            m += nw;
            while (m >= nact) {
              m -= nact;
              ++oi;
            }
          }
          oi0 = oi;
          m0 = m;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (r0 + u * nw >= rend) break;  // warp-uniform
          const int o = ou[u], m = mu[u];
          float4 x = v[u], xl = vl[u];
          if (k4 + 0 >= npts) x.x = xl.x = 0.f;
          if (k4 + 1 >= npts) x.y = xl.y = 0.f;
          if (k4 + 2 >= npts) x.z = xl.z = 0.f;
          if (k4 + 3 >= npts) x.w = xl.w = 0.f;
          float mx = fmaxf(fmaxf(fabsf(x.x), fabsf(x.y)), fmaxf(fabsf(x.z), fabsf(x.w)));
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
          float scale, inv;
          fixed_scale<7>(mx, scale, inv);
          if (lane == 0) scl[o * rows_pad + m] = scale;
          float h[3][4];
          fixed_slices2<7, 8>(__fmul_rn(x.x, inv), __fmul_rn(xl.x, inv), h[0][0], h[1][0], h[2][0]);
          fixed_slices2<7, 8>(__fmul_rn(x.y, inv), __fmul_rn(xl.y, inv), h[0][1], h[1][1], h[2][1]);
          fixed_slices2<7, 8>(__fmul_rn(x.z, inv), __fmul_rn(xl.z, inv), h[0][2], h[1][2], h[2][2]);
          fixed_slices2<7, 8>(__fmul_rn(x.w, inv), __fmul_rn(xl.w, inv), h[0][3], h[1][3], h[2][3]);
          uint8_t* tb;
          uint32_t sstride = kTileA, off = tc::swz_offset_h(m & 127, k4 & 63);
          if (tiles_in_smem) {
            tb = sm + ((o == 0 ? 0 : 2) + (k4 >> 6)) * 3 * kTileA;
          } else if (tiles_mid && o != 0) {  // G rows of all functions, one tile per chunk
            sstride = (uint32_t)npad * 128u;
            tb = sm + kMidB + (k4 >> 6) * 3 * sstride;
            off = tc::swz_offset_h(m, k4 & 63);
          } else {
            tb = reinterpret_cast<uint8_t*>(tiles + (((long)o * bt.ft_max + (m >> 7)) * 2 + (k4 >> 6)) * 3 * kTileFloats);
          }
#pragma unroll
          for (int i = 0; i < 3; ++i)
            *reinterpret_cast<uint2*>(tb + i * sstride + off) = make_uint2(pack_h2(h[i][0], h[i][1]), pack_h2(h[i][2], h[i][3]));
        }
      }
      if (tiles_in_smem || tiles_mid) tc::fence_async_smem();  // these generic writes are read by the MMAs below
      if (!tiles_in_smem) tc::fence_async_global();            // ... by the bulk copies below
    };
    if constexpr (MODE == kModeBuild) {
    // ---- the functional at the block's points (build): the reference's steps, with the
    //      reductions in the same order as the separate kernels (functional skip of the
    //      block, E_xc and N_el partials, the adder's block skip per spin, the weights) ----
    // warps 0-3 evaluate the functional (group barrier 1) while warps 4-15 slice the
    // adder's Phi rows, which do not depend on it
    if (warp < 4) {
      auto group_sync = [] { asm volatile("bar.sync 1, 128;" ::: "memory"); };
      double* red = &s_part[0][0][0];  // 2 x 128 doubles (the density's partial sums are done)
      const bool pt = tid < 128;
      const int q = tid;
      const bool gga = xc::is_gga(I.func);
      bool fsk = true;  // XCFun's block skip (functional data): sum |rho| < n 1e-12 for every spin
      for (int s = 0; s < nspin; ++s) {
        if (pt) red[q] = q < npts ? fabs(s_rg[(s * 4) * 128 + q]) : 0.0;
        group_sync();
        for (int w2 = 64; w2 > 0; w2 >>= 1) {
          if (tid < w2) red[tid] += red[tid + w2];
          group_sync();
        }
        fsk = fsk && (red[0] < npts * 1e-12);
        group_sync();
      }
      double e = 0.0, rtot = 0.0, vv[2] = {0.0, 0.0}, gg[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
      if (pt && q < npts) {
        if (nspin == 1) {
          const double r = s_rg[0 * 128 + q];
          const double gx = s_rg[1 * 128 + q], gy = s_rg[2 * 128 + q], gz = s_rg[3 * 128 + q];
          double vn = 0.0, vs = 0.0;
          // restricted PBE in FP32 pairs (~1e-13 relative): FP64 at 1/64 of the FP32 rate
          // would make it the longest step of the block
          if (!fsk) {
            if (I.func == XCGPU_FUNC_PBE) xc::pbe_restricted_pair(r, gx * gx + gy * gy + gz * gz, e, vn, vs);
            else xc::eval_restricted<double>(I.func, r, gga ? gx * gx + gy * gy + gz * gz : 0.0, e, vn, vs);
          }
          vv[0] = vn;
          if (gga) {
            gg[0][0] = 2.0 * vs * gx;
            gg[0][1] = 2.0 * vs * gy;
            gg[0][2] = 2.0 * vs * gz;
          }
          rtot = r;
        } else {
          const double ra = s_rg[0 * 128 + q], rb = s_rg[4 * 128 + q];
          double ga[3], gb[3];
          for (int k = 0; k < 3; ++k) {
            ga[k] = gga ? s_rg[(1 + k) * 128 + q] : 0.0;
            gb[k] = gga ? s_rg[(5 + k) * 128 + q] : 0.0;
          }
          double va = 0, vb = 0, vaa = 0, vab = 0, vbb = 0;
          if (!fsk) {
            const double saa = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
            const double sab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
            const double sbb = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
            xc::eval_unrestricted<double>(I.func, ra, rb, saa, sab, sbb, e, va, vb, vaa, vab, vbb);
          }
          vv[0] = va;
          vv[1] = vb;
          if (gga)
            for (int k = 0; k < 3; ++k) {
              gg[0][k] = 2.0 * vaa * ga[k] + vab * gb[k];
              gg[1][k] = 2.0 * vbb * gb[k] + vab * ga[k];
            }
          rtot = ra + rb;
        }
      }
      const double wp = (pt && q < npts) ? P.w[first + q] : 0.0;
      if (pt) {
        red[q] = wp * e;
        red[128 + q] = wp * rtot;
      }
      group_sync();
      for (int w2 = 64; w2 > 0; w2 >>= 1) {
        if (tid < w2) {
          red[tid] += red[tid + w2];
          red[128 + tid] += red[128 + tid + w2];
        }
        group_sync();
      }
      if (tid == 0) {
        I.partials[b] = red[0];
        I.partials[P.nblocks + b] = red[128];
      }
      group_sync();
      for (int s = 0; s < nspin; ++s) {  // ScalarOperatorToMatrixAdder's block skip
        double a = 0.0;
        if (pt && q < npts) {
          a += fabs(wp * vv[s]);
          if (gga)
            for (int k = 0; k < 3; ++k) a += fabs(wp * gg[s][k]);
        }
        if (pt) red[q] = a;
        group_sync();
        for (int w2 = 64; w2 > 0; w2 >>= 1) {
          if (tid < w2) red[tid] += red[tid + w2];
          group_sync();
        }
        if (!(red[0] / npts < I.thr)) smask |= 1 << s;
        group_sync();
      }
      if (pt)
        for (int s = 0; s < 2; ++s) {
          float w4[4] = {0.f, 0.f, 0.f, 0.f};
          if (((smask >> s) & 1) && q < npts) {
            w4[0] = (float)(0.5 * wp * vv[s]);
            if (DERIV && gga)
              for (int c = 0; c < 3; ++c) w4[1 + c] = (float)(wp * gg[s][c]);
          }
          for (int c = 0; c < 4; ++c) s_w[s][c][q] = w4[c];
        }
      if (tid == 0) s_smask = smask;
    } else if (nact > 0) {
      slice_rows(0, nact, warp - 4, kWarps - 4);
    }
    __syncthreads();
    smask = s_smask;
      if (smask == 0 || nact == 0) continue;
    }
    if constexpr (HAS_A) {
      const int nkc = (npts + 63) >> 6;
      if constexpr (MODE == kModeAdder) {
    // ---- weights ----
    if (tid < 256) {
      const int s = tid >> 7, q = tid & 127;
      float w4[4] = {0.f, 0.f, 0.f, 0.f};
      if (((smask >> s) & 1) && q < npts) {
        const double w = P.w[first + q];
        w4[0] = (float)(0.5 * w * I.v[(long)s * P.npoints + first + q]);
        if (DERIV && I.g) {
#pragma unroll
          for (int c = 0; c < 3; ++c) w4[1 + c] = (float)(w * I.g[((long)s * 3 + c) * P.npoints + first + q]);
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) s_w[s][c][q] = w4[c];
    }
    __syncthreads();
    const bool sp0 = smask & 1, sp1 = TWO_SPINS && ((smask >> 1) & 1);
    // ---- 1a. Phi and G of the block's points in FP32 (points past npts are masked in 1b) ----
    {
      const int p = tid & 127, quarter = tid >> 7;
      if (p < npts) {
        const Pt pt = make_pt(P.xyz + 3 * (first + p));
        const float expthr = (float)P.exponent_threshold, thr = (float)P.radial_threshold;
        constexpr int NS = TWO_SPINS ? 2 : 1;
        float wsp[NS][4];
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
          for (int c = 0; c < 4; ++c) wsp[s][c] = s_w[s][c][p];
        float* const col = stg + p;
        ShellRec next;
        if (s0 + quarter < s1) next = load_rec(P.rec + s0 + quarter);
        for (int si = s0 + quarter; si < s1; si += kQ) {
          const ShellRec r = next;
          if (si + kQ < s1) next = load_rec(P.rec + si + kQ);  // in flight while r is evaluated
          float* const t0 = col + (long)rec_f0(r.info) * 128;
          float rlo = 0.f;
          const long lo = (long)NOPS * rows_pad * 128;  // plane offset of the low parts
          // Phi and G with the low part of the value (radial factor's and coefficients',
          // the same at every point of a radial shell); the gradient terms stay FP32
          auto put = [&](int f, float val, float vl, float dx, float dy, float dz) {
            float* t = t0 + f * 128;
            const float vlo = fmaf(val, rlo, vl);
            t[0] = val;
            t[lo] = vlo;
            if (sp0) {
              float gv = __fmul_rn(wsp[0][0], val);
              if (DERIV) gv = fmaf(wsp[0][3], dz, fmaf(wsp[0][2], dy, fmaf(wsp[0][1], dx, gv)));
              t[rows_pad * 128] = gv;
              t[lo + rows_pad * 128] = __fmul_rn(wsp[0][0], vlo);
            }
            if (TWO_SPINS && sp1) {
              float gv = __fmul_rn(wsp[NS - 1][0], val);
              if (DERIV) gv = fmaf(wsp[NS - 1][3], dz, fmaf(wsp[NS - 1][2], dy, fmaf(wsp[NS - 1][1], dx, gv)));
              t[2 * rows_pad * 128] = gv;
              t[lo + 2 * rows_pad * 128] = __fmul_rn(wsp[NS - 1][0], vlo);
            }
          };
          shell_rec_at<DERIV, MAXL>(r, B.prim4, pt, expthr, thr, &rlo, put);
        }
      }
    }
    __syncthreads();
      }
    if constexpr (MODE == kModeAdder) {
      slice_rows(0, (1 + __popc(smask)) * nact, warp, kWarps);
    } else {  // the Phi rows were sliced beside the functional
      slice_rows(nact, (1 + __popc(smask)) * nact, warp, kWarps);
    }
    __syncthreads();
    if (tiles_mid) {
      // ---- 2. T = Phi^T G over all functions, one 128-row tile of Phi at a time (the Phi
      //      tile's chunks streamed from the scratch into the slot, G's from shared
      //      memory; N = npad <= 192: accumulators at columns 0 and 256); T's first tile
      //      goes to the scratch (the planes are consumed), its second and then the first
      //      to shared memory as T[m][n] (row stride nact | 1), and F = T + T^T is paired
      //      there ----
      const float* const sGn = scl + rows_pad;
      float* const Tg = my;  // first tile, column-major [npad][128]
      const int ldT = nact | 1;
      float* const Ts = reinterpret_cast<float*>(sm);
      for (int a = 0; a < 2; ++a) {
        const int ma = min(128, nact - 128 * a);
        bool ok = true;
        if (tid == 0) {
          tc::fence_after_sync();
          const uint32_t ab = (uint32_t)((ma + 7) & ~7) * 128u;
          int stuck = 0;  // 1: a copy, 2: MMAs still in flight after a wait gave up
          for (int kc = 0; kc < nkc; ++kc) {
            const float* ta = tiles + ((long)a * 2 + kc) * 3 * kTileFloats;  // operand 0 (Phi), tile a
            tc::mbar_arrive_expect_tx(&mfull, 3 * ab);
#pragma unroll
            for (int q = 0; q < 3; ++q) tc::bulk_g2s(sm + q * kTileA, ta + q * kTileFloats, ab, &mfull);
            if (!tc::mbar_wait_bounded(&mfull, mphase & 1u, kWaitLimitNs)) {
              stuck = 1;
              break;
            }
            mphase ^= 1u;
            tc::fence_after_sync();
            issue_fixed_chunk3(tmem, 0u, 256u, tc::smem_u32(sm), kTileA,
                               tc::smem_u32(sm + kMidB + kc * 3 * npad * 128), (uint32_t)npad * 128u, npad, kc == 0);
            tc::mma_commit(&mmma);
            if (!tc::mbar_wait_bounded(&mmma, (mphase >> 1) & 1u, kWaitLimitNs)) {  // the slot is free again
              stuck = 2;
              break;
            }
            mphase ^= 2u;
          }
          if (stuck) {
            ok = false;
            atomicExch(err, kErrTimeout);
            s_abort = 1;
            // what was issued lands before the CTA gives up its memory
            if (stuck == 1) tc::mbar_wait_bounded(&mfull, mphase & 1u, kWaitLimitNs);
            else tc::mbar_wait_bounded(&mmma, (mphase >> 1) & 1u, kWaitLimitNs);
          }
        }
        if (__syncthreads_or(!ok)) goto done;
        tc::fence_after_sync();
        // drain: row (lane) r of the tile, 8 columns at a time
        const int r = 32 * (warp & 3) + lane;
        const float sPm = r < ma ? scl[128 * a + r] : 0.f;
#pragma unroll 1
        for (int cb = 32 * (warp >> 2); cb < npad; cb += 128) {
#pragma unroll 1
          for (int c8 = cb; c8 < cb + 32 && c8 < npad; c8 += 8) {
            float p0[8], pr[8];
            tc::tmem_ld8x2(tmem + trow + c8, tmem + trow + 256 + c8, p0, pr);
            if (r < ma) {
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                const int n = c8 + c;
                if (n < nact) {
                  const float t = __fmul_rn(__fadd_rn(p0[c], pr[c]), __fmul_rn(sPm, sGn[n]));
                  if (a == 0) Tg[n * 128 + r] = t;
                  else Ts[(128 + r) * ldT + n] = t;
                }
              }
            }
          }
        }
        tc::fence_before_sync();
        __syncthreads();  // the accumulators are reused by the second tile
      }
      // the first tile from the scratch into shared memory
      for (int e = tid; e < 128 * nact; e += kT) {
        const int n = e >> 7, r = e & 127;
        Ts[r * ldT + n] = Tg[e];
      }
      __syncthreads();
      {
        const int nbf_b = I.P.nbf;
#pragma unroll 1
        for (int n = warp; n < nact; n += kWarps) {
          double* const Vc = I.V + (long)__ldg(fn + n) * nbf_b;
#pragma unroll 1
          for (int m = lane; m <= n; m += 32)
            atomicAdd(Vc + __ldg(fn + m), f32_to_f64(__fadd_rn(Ts[m * ldT + n], Ts[n * ldT + m])));
        }
      }
      __syncthreads();  // the shared memory is reused by the next block
      continue;
    }
    if (tiles_in_smem) {
      // ---- 2. the one tile pair from shared memory: Phi tiles at the first stage, G at
      //      the second; T = Phi^T G over every chunk ----
      if (tid == 0) {
        tc::fence_after_sync();
        const int N = (nact + 15) & ~15;
        for (int kc = 0; kc < nkc; ++kc) {
          const uint32_t tp = tc::smem_u32(sm + kc * 3 * kTileA), tg = tc::smem_u32(sm + (2 + kc) * 3 * kTileA);
          issue_fixed_chunk2(tmem, 0u, 128u, tp, tg, N, kc == 0, kc == 0);
        }
        tc::mma_commit(&fdone);
      }
      const bool fok = tc::mbar_wait_bounded(&fdone, fphase, kWaitLimitNs);
      fphase ^= 1u;
      if (__syncthreads_or(!fok)) {
        if (tid == 0) {
          atomicExch(err, kErrTimeout);
          s_abort = 1;
          tc::mbar_wait_bounded(&fdone, fphase ^ 1u, kWaitLimitNs);  // let the MMAs land
        }
        goto done;
      }
      tc::fence_after_sync();
      diag_to_V(I, fn, nact);
      tc::fence_before_sync();
      __syncthreads();  // the accumulators and the stages are reused by the next block
      continue;
    }
    // ---- 2. tile pairs ----
    const int spp = 2 * nkc;                              // steps per pair: 2 products x chunks
    const int npairs = __popc(smask) * (nft * (nft + 1) / 2);
    const int nsteps = npairs * spp;
    // step i of this block -> (spin, a, b, product, chunk); pairs ordered (spin, a, b >= a)
    auto decode = [&](int i, int& spin, int& a, int& bb, int& ph, int& kc) {
      kc = i % nkc;
      ph = (i / nkc) & 1;
      int q = i / spp;
      const int per = nft * (nft + 1) / 2;
      const int si = q / per;
      q -= si * per;
      a = 0;
      while (q >= nft - a) {
        q -= nft - a;
        ++a;
      }
      bb = a + q;
      spin = (smask == 2) ? 1 : si;
    };
    auto issue_copy = [&](int i) {
      int spin, a, bb, ph, kc;
      decode(i, spin, a, bb, ph, kc);
      const int J = J0 + i, st = J & 1;
      uint8_t* dst = sm + st * kDStageBytes;
      const int oA = ph ? 1 + spin : 0, oB = ph ? 0 : 1 + spin;
      const int nM = min(128, nact - 128 * a), nN = min(128, nact - 128 * bb);
      const uint32_t ab = (uint32_t)((nM + 7) & ~7) * 128u, bbytes = (uint32_t)((nN + 7) & ~7) * 128u;
      const float* ta = tiles + (((long)oA * bt.ft_max + a) * 2 + kc) * 3 * kTileFloats;
      const float* tb = tiles + (((long)oB * bt.ft_max + bb) * 2 + kc) * 3 * kTileFloats;
      tc::mbar_arrive_expect_tx(&full[st], 3 * ab + 3 * bbytes);
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        tc::bulk_g2s(dst + s * kTileA, ta + s * kTileFloats, ab, &full[st]);
        tc::bulk_g2s(dst + (3 + s) * kTileA, tb + s * kTileFloats, bbytes, &full[st]);
      }
      last_copy = J;
    };
    bool ok = true;
    if (tid == 0)
      for (int i = 0; i < min(2, nsteps); ++i) issue_copy(i);
    for (int q = 0; q < npairs; ++q) {
      const int iL = q * spp + spp - 1;  // the pair's last step
      if (tid == 0 && ok) {
        for (int i = q * spp; i <= iL; ++i) {
          const int J = J0 + i, st = J & 1;
          if (!tc::mbar_wait_bounded(&full[st], (J >> 1) & 1u, kWaitLimitNs)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          int spin, a, bb, ph, kc;
          decode(i, spin, a, bb, ph, kc);
          const int N = (min(128, nact - 128 * bb) + 15) & ~15;
          issue_fixed_chunk(tmem, ph ? 256u : 0u, ph ? 384u : 128u, tc::smem_u32(sm + st * kDStageBytes), N, kc == 0,
                            kc == 0);
          tc::mma_commit(&mdone[st]);
          last_mma = J;
          // the stage of step i - 1 (same pair) is free once its MMAs are done: refill it
          if (i > q * spp && i + 1 < nsteps) {
            if (!tc::mbar_wait_bounded(&mdone[(J - 1) & 1], ((J - 1) >> 1) & 1u, kWaitLimitNs)) {
              ok = false;
              break;
            }
            issue_copy(i + 1);
          }
        }
      }
      // ---- the pair's accumulators -> V ----
      const int JL = J0 + iL;
      const bool done_ok = tc::mbar_wait_bounded(&mdone[JL & 1], (JL >> 1) & 1u, kWaitLimitNs);
      if (tid == 0 && done_ok && ok && iL + 2 < nsteps) issue_copy(iL + 2);  // prefetch during the drain
      if (__syncthreads_or(!(done_ok && ok))) {
        if (tid == 0) atomicExch(err, kErrTimeout);
        goto abort;
      }
      tc::fence_after_sync();
      {
        int spin, a, bb, ph, kc;
        decode(iL, spin, a, bb, ph, kc);
        pair_to_V(I, fn, nact, spin, a, bb);
      }
      tc::fence_before_sync();
      __syncthreads();  // the accumulators are reused by the next pair
    }
      J0 += nsteps;
    }
  }
  goto done;
abort:
  if (tid == 0) {
    s_abort = 1;
    // let every copy and MMA still in flight land before the CTA gives up its memory
    for (int J = last_mma + 1; J <= last_copy; ++J) tc::mbar_wait_bounded(&full[J & 1], (J >> 1) & 1u, kWaitLimitNs);
    if (last_mma >= 0) tc::mbar_wait_bounded(&mdone[last_mma & 1], (last_mma >> 1) & 1u, kWaitLimitNs);
  }
done:
#pragma unroll
  for (int q = 0; q < 2; ++q)
    if ((pend >> q) & 1u) wait_or_abort(&mbar[q], (phase >> q) & 1u, err);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// threads per CTA and dynamic shared memory of every mixed kernel launch
inline size_t mx_smem() { return 2 * kDStageBytes + 1024; }  // two stages, 1024-byte aligned

// the kernels for bases with g..i functions (MAXL 6), instantiated in xc_mixed_hl.cu
xcgpu_status mixed_init_hl(Ctx* c);
void mixed_launch_hl(int mode, bool gga, bool two, unsigned grid, cudaStream_t s, const MxBatch& bt, int* counter,
                     int* err);

}  // namespace xcgpu
