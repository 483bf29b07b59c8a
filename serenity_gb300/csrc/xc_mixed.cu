// Mixed-precision XC build on the sm_103a tensor cores.
//
// Basis values and gradients are evaluated in FP32 on the fly (never stored in
// global memory); the two dense contractions run as 3xTF32 tcgen05 MMAs with FP32
// accumulation in tensor memory (TMEM):
//   density : X = Phi P_b            (M = 128 points, N = active functions, K = functions)
//             rho = rowsum(X o Phi), grad rho = 2 rowsum(X o grad Phi), summed in FP64
//   adder   : D = Phi^T G            (M = active functions, N = active functions, K = points)
//             with G = w (v/2 Phi + g . grad Phi); D goes to V in FP64 (red.add), and
//             V + V^T at the end gives sum_b (D_b + D_b^T) = sum_b F_b
//             (ScalarOperatorToMatrixAdder.cpp:224-303).
// The functional, E_xc, N_el and the cross-block Vxc accumulation stay in FP64.
//
// Both kernels are persistent (one CTA of 128 threads per SM, blocks taken from a
// global counter); one elected thread issues the MMAs; completion is tracked with
// mbarriers through tcgen05.commit; every wait is bounded in time and reports a
// timeout through the error word instead of hanging.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "basis_eval.cuh"
#include "internal.h"
#include "tcgen05.cuh"

namespace xcgpu {

constexpr uint32_t kTileA = 128 * 128;  // bytes of a 128-row x 32-element operand tile
constexpr uint64_t kWaitLimitNs = 2000000000ull;
constexpr int kErrTimeout = 1;

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

// Evaluate one shell record at a point in FP32; Emit(f, value, dx, dy, dz).
// Negligible shells (|R| below the radial threshold) emit zeros.
template <int DERIV, class Emit>
__device__ __forceinline__ void shell_rec_at(const ShellRec& r, const float2* __restrict__ prim2, const Pt& q,
                                             float expthr, float thr, Emit&& emit) {
  const float x = (q.h[0] - r.ah[0]) + (q.l[0] - r.al[0]);
  const float y = (q.h[1] - r.ah[1]) + (q.l[1] - r.al[1]);
  const float z = (q.h[2] - r.ah[2]) + (q.l[2] - r.al[2]);
  const float r2 = x * x + y * y + z * z;
  const int np = rec_nprim(r.info);
  float Rv = 0.f, dR = 0.f;
  for (int i = 0; i < np; ++i) {
    const float2 ac = __ldg(prim2 + r.prim0 + i);
    const float t = ac.x * r2;
    if (t < expthr) {
      const float e = ac.y * expf(-t);
      Rv += e;
      if (DERIV >= 1) dR -= 2.f * ac.x * e;
    }
  }
  const int l = rec_l(r.info);
  if (!(fabsf(Rv) >= thr)) {
    const int nf = rec_nf(r.info);
    for (int f = 0; f < nf; ++f) emit(f, 0.f, 0.f, 0.f, 0.f);
    return;
  }
  shell_functions_cx_l<float, DERIV>(l, x, y, z, Rv, dR, rec_pure(r.info), emit);
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

__device__ __forceinline__ void st_tf32_pair(uint8_t* hi, uint8_t* lo, uint32_t off, float v) {
  uint32_t h, l;
  tc::split_tf32(v, h, l);
  *reinterpret_cast<uint32_t*>(hi + off) = h;
  *reinterpret_cast<uint32_t*>(lo + off) = l;
}

__device__ __forceinline__ bool wait_or_abort(uint64_t* mbar, uint32_t parity, int* err) {
  const bool ok = tc::mbar_wait_bounded(mbar, parity, kWaitLimitNs);
  if (!ok) atomicExch(err, kErrTimeout);
  return ok;
}

// Pipeline shared by both kernels (256 threads, 8 warps, one CTA per SM):
//   per K-chunk of 32: fill operand stage (kc & 1) -> wait for the MMAs of chunk kc-1
//   -> drain its hi*hi accumulator into an FP32 (round-to-nearest) sum in shared
//   memory -> issue chunk kc: hi*hi into a fresh TMEM accumulator (kc & 1), the two
//   cross products into one accumulator for the whole pass.
// Keeping every hi*hi accumulation chain to 4 MMAs (and the small cross terms in
// their own accumulator) bounds the bias of the tensor core's truncating FP32
// accumulation; long chains over all K gave a relative density bias of -6e-7.
// TMEM columns: hh0 [0,128), hh1 [128,256), cross [256,384).
constexpr int kT = 256;
constexpr int kNT = 128;  // functions per pass / tile (N), and rows of an M tile
constexpr uint32_t kStageBytes = 4 * kTileA;  // A_hi, A_lo, B_hi, B_lo (128 rows each)
constexpr uint32_t kColsHH0 = 0, kColsHH1 = 128, kColsX = 256;

// hi*hi (fresh per chunk) + cross terms for one 32-wide K chunk
__device__ __forceinline__ void issue_chunk(uint32_t tmem, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, int N,
                                            int hh_cols, bool first_chunk) {
  const uint32_t idesc = tc::idesc_tf32(128, N);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint32_t o = ks * 32;
    tc::mma_tf32(tmem + hh_cols, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bh + o), idesc, ks > 0 ? 1u : 0u);
    tc::mma_tf32(tmem + kColsX, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bl + o), idesc,
                 (!first_chunk || ks > 0) ? 1u : 0u);
    tc::mma_tf32(tmem + kColsX, tc::smem_desc_sw128(al + o), tc::smem_desc_sw128(bh + o), idesc, 1u);
  }
}

// add (or store) TMEM columns [col, col + 64) of this warp's 32 lanes into S rows
__device__ __forceinline__ void drain64(uint32_t tmem_cols, int warp, int lane, float* S, int ld, int c0, int N,
                                        bool store) {
  const int row = 32 * (warp & 3) + lane;
  for (int c = c0; c < c0 + 64 && c < N; c += 32) {
    float v[32];
    tc::tmem_ld32(tmem_cols + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)c, v);
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (c + i < N) {
        float* d = S + row * ld + c + i;
        *d = store ? v[i] : *d + v[i];
      }
  }
}

// One XC build inside a batched launch: its basis, plan, spin count and buffers.
struct MxItem {
  DevBasis B;
  DevPlan P;
  int nspin;
  const float* Phi;  // TF32 split of the density matrices (density kernel)
  const float* Plo;
  double* rho;  // outputs of the density kernel
  double* grad;
  const double* v;  // inputs of the adder kernel
  const double* g;
  const unsigned char* skip;
  double* V;
};
// Up to kMaxItems builds per launch, passed by value as the kernel parameter (no
// host staging buffer, so launches can be issued back to back and captured in a
// graph); the blocks of all items form one index space, item i owning
// [bstart[i], bstart[i+1]).
constexpr int kMaxItems = 64;
struct MxBatch {
  MxItem items[kMaxItems];
  int bstart[kMaxItems + 1];
  int nitems;
  int nblocks;
};

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
// density
// =====================================================================================
__global__ void __launch_bounds__(kT, 1)
    mx_density_kernel(const __grid_constant__ MxBatch bt, int* __restrict__ counter, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_block, s_abort;
  __shared__ double s_part[4][128];
  const uint32_t base_s = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base_s & 1023)) & 1023);
  float* Xs = reinterpret_cast<float*>(sm + 2 * kStageBytes);  // [128][kNT + 1]
  const int ld = kNT + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p = tid & 127, half = tid >> 7;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
    s_abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  uint32_t phase[2] = {0, 0};
  int outstanding = -1;  // stage whose commit has not been waited for (-1: none)

  for (;;) {
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
    const float* __restrict__ Phi = I.Phi;
    const float* __restrict__ Plo = I.Plo;
    double* __restrict__ rho = I.rho;
    double* __restrict__ grad = I.grad;
    const long first = (long)b * P.max_block;
    const int npts = (int)min((long)P.max_block, P.npoints - first);
    const int nact = P.fn_off[b + 1] - P.fn_off[b];
    const int* fn = P.fn_list + P.fn_off[b];
    const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
    const bool live = p < npts;
    const Pt pt = make_pt(P.xyz + 3 * (first + (live ? p : 0)));
    const ShellRec* recs = P.rec;
    const float expthr = (float)P.exponent_threshold, thr = (float)P.radial_threshold;
    for (int s = 0; s < nspin; ++s) {
      const float* Ph = Phi + (long)s * nbf * nbf;
      const float* Pl = Plo + (long)s * nbf * nbf;
      double r_acc = 0.0, g_acc[3] = {0.0, 0.0, 0.0};
      for (int nu0 = 0; nu0 < nact; nu0 += kNT) {
        const int nnu = min(kNT, nact - nu0);
        const int N = (nnu + 15) & ~15;
        const int nkc = (nact + 31) / 32;
        int sh_cursor = s0;
        for (int kc = 0; kc < nkc; ++kc) {
          const int st = kc & 1;
          uint8_t* Ahi = sm + st * kStageBytes;
          uint8_t* Alo = Ahi + kTileA;
          uint8_t* Bhi = Alo + kTileA;
          uint8_t* Blo = Bhi + kTileA;
          const int mu0 = kc * 32;
          // ---- A: Phi[p][mu0 + 16 half .. + 16) ----
          {
            const int k0 = 16 * half;
#pragma unroll
            for (int k = k0; k < k0 + 16; ++k) {
              *reinterpret_cast<uint32_t*>(Ahi + tc::swz_offset(p, k)) = 0u;
              *reinterpret_cast<uint32_t*>(Alo + tc::swz_offset(p, k)) = 0u;
            }
            const int lo = mu0 + k0;
            while (sh_cursor < s1) {
              const int info = __ldg(&recs[sh_cursor].info);
              if (rec_f0(info) + rec_nf(info) > lo) break;
              ++sh_cursor;
            }
            if (live) {
              for (int si = sh_cursor; si < s1; ++si) {
                const ShellRec r = load_rec(recs + si);
                const int f0 = rec_f0(r.info);
                if (f0 >= lo + 16) break;
                shell_rec_at<0>(r, B.prim2, pt, expthr, thr, [&](int f, float v, float, float, float) {
                  const int k = f0 + f - mu0;
                  if (k >= k0 && k < k0 + 16) st_tf32_pair(Ahi, Alo, tc::swz_offset(p, k), v);
                });
              }
            }
          }
          // ---- B: P_b[nu][mu0 .. mu0 + 32), pre-split TF32 parts ----
          {
            const int nu = tid & 127;
            if (nu < N) {
              const bool nuok = nu < nnu;
              const long colnu = nuok ? fn[nu0 + nu] : 0;
#pragma unroll 4
              for (int k = half; k < 32; k += 2) {
                const int mu = mu0 + k;
                float h = 0.f, l = 0.f;
                if (nuok && mu < nact) {
                  const long o = (long)fn[mu] * nbf + colnu;
                  h = __ldg(Ph + o);
                  l = __ldg(Pl + o);
                }
                const uint32_t off = tc::swz_offset(nu, k);
                *reinterpret_cast<float*>(Bhi + off) = h;
                *reinterpret_cast<float*>(Blo + off) = l;
              }
            }
          }
          tc::fence_async_smem();
          // ---- drain the previous chunk's hi*hi accumulator ----
          if (kc > 0) {
            const int pst = (kc - 1) & 1;
            const bool ok = wait_or_abort(&mbar[pst], phase[pst], err);
            phase[pst] ^= 1;
            outstanding = -1;
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
            tc::fence_after_sync();
            drain64(tmem + (pst ? kColsHH1 : kColsHH0), warp, lane, Xs, ld, 64 * (warp >> 2), N, kc == 1);
            tc::fence_before_sync();
          }
          __syncthreads();
          if (tid == 0) {
            tc::fence_after_sync();
            issue_chunk(tmem, tc::smem_u32(Ahi), tc::smem_u32(Alo), tc::smem_u32(Bhi), tc::smem_u32(Blo), N,
                        st ? kColsHH1 : kColsHH0, kc == 0);
            tc::mma_commit(&mbar[st]);
          }
          outstanding = st;
        }
        // ---- last chunk: drain hh, add the cross accumulator ----
        {
          const int pst = (nkc - 1) & 1;
          const bool ok = wait_or_abort(&mbar[pst], phase[pst], err);
          phase[pst] ^= 1;
          outstanding = -1;
          if (__syncthreads_or(!ok)) {
            if (tid == 0) s_abort = 1;
            goto done;
          }
          tc::fence_after_sync();
          drain64(tmem + (pst ? kColsHH1 : kColsHH0), warp, lane, Xs, ld, 64 * (warp >> 2), N, nkc == 1);
          drain64(tmem + kColsX, warp, lane, Xs, ld, 64 * (warp >> 2), N, false);
          tc::fence_before_sync();
          __syncthreads();
        }
        // ---- row dots: rho_p += sum_nu X_p,nu phi_p,nu (shells split between the two halves) ----
        if (live) {
          int j = 0;
          for (int si = s0; si < s1; ++si) {
            const int info = __ldg(&recs[si].info);
            const int f0 = rec_f0(info), nf = rec_nf(info);
            if (f0 + nf > nu0 && f0 < nu0 + nnu && ((j++ & 1) == half)) {
              const ShellRec r = load_rec(recs + si);
              float rr = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
              shell_rec_at<1>(r, B.prim2, pt, expthr, thr, [&](int f, float v, float dx, float dy, float dz) {
                const int c = f0 + f - nu0;
                if (c >= 0 && c < nnu) {
                  const float xv = Xs[p * ld + c];
                  rr = fmaf(xv, v, rr);
                  gx = fmaf(xv, dx, gx);
                  gy = fmaf(xv, dy, gy);
                  gz = fmaf(xv, dz, gz);
                }
              });
              r_acc += (double)rr;
              g_acc[0] += (double)gx;
              g_acc[1] += (double)gy;
              g_acc[2] += (double)gz;
            }
          }
        }
        __syncthreads();  // Xs and the stages are reused by the next pass
      }
      // combine the two halves of each point
      if (half == 1) {
        s_part[0][p] = r_acc;
        s_part[1][p] = g_acc[0];
        s_part[2][p] = g_acc[1];
        s_part[3][p] = g_acc[2];
      }
      __syncthreads();
      if (half == 0 && live) {
        rho[(long)s * P.npoints + first + p] = r_acc + s_part[0][p];
        if (grad) {
          grad[((long)s * 3 + 0) * P.npoints + first + p] = 2.0 * (g_acc[0] + s_part[1][p]);
          grad[((long)s * 3 + 1) * P.npoints + first + p] = 2.0 * (g_acc[1] + s_part[2][p]);
          grad[((long)s * 3 + 2) * P.npoints + first + p] = 2.0 * (g_acc[2] + s_part[3][p]);
        }
      }
      __syncthreads();
    }
  }
done:
  if (outstanding >= 0) wait_or_abort(&mbar[outstanding], phase[outstanding], err);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// =====================================================================================
// adder
// =====================================================================================
__global__ void __launch_bounds__(kT, 1)
    mx_adder_kernel(const __grid_constant__ MxBatch bt, int* __restrict__ counter, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_block, s_abort;
  __shared__ float s_wv[128], s_wg[3][128];
  const uint32_t base_s = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base_s & 1023)) & 1023);
  float* Ds = reinterpret_cast<float*>(sm + 2 * kStageBytes);  // [128][kNT + 1]
  const int ld = kNT + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
    s_abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  uint32_t phase[2] = {0, 0};
  int outstanding = -1;

  for (;;) {
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
    const double* __restrict__ v = I.v;
    const double* __restrict__ g = I.g;
    const unsigned char* __restrict__ skip = I.skip;
    double* __restrict__ V = I.V;
    const long first = (long)b * P.max_block;
    const int npts = (int)min((long)P.max_block, P.npoints - first);
    const int nact = P.fn_off[b + 1] - P.fn_off[b];
    const int* fn = P.fn_list + P.fn_off[b];
    const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
    for (int s = 0; s < nspin; ++s) {
      if (skip[(long)s * P.nblocks + b]) continue;
      if (tid < 128) {
        const int q = tid;
        float wv = 0.f, wg0 = 0.f, wg1 = 0.f, wg2 = 0.f;
        if (q < npts) {
          const double w = P.w[first + q];
          wv = (float)(0.5 * w * v[(long)s * P.npoints + first + q]);
          if (g) {
            wg0 = (float)(w * g[((long)s * 3 + 0) * P.npoints + first + q]);
            wg1 = (float)(w * g[((long)s * 3 + 1) * P.npoints + first + q]);
            wg2 = (float)(w * g[((long)s * 3 + 2) * P.npoints + first + q]);
          }
        }
        s_wv[q] = wv;
        s_wg[0][q] = wg0;
        s_wg[1][q] = wg1;
        s_wg[2][q] = wg2;
      }
      __syncthreads();
      double* Vs = V + (long)s * nbf * nbf;
      for (int nt0 = 0; nt0 < nact; nt0 += kNT) {
        const int nN = min(kNT, nact - nt0);
        const int N = (nN + 15) & ~15;
        for (int mt0 = 0; mt0 < nact; mt0 += kNT) {
          const int nM = min(kNT, nact - mt0);
          // zero the padding rows of both stages (A rows >= nM, B rows in [nN, N))
          for (int e = tid; e < 2 * ((128 - nM) + (N - nN)) * 32; e += kT) {
            const int stg = e / (((128 - nM) + (N - nN)) * 32);
            const int r0 = (e / 32) % ((128 - nM) + (N - nN)), k = e % 32;
            uint8_t* base = sm + stg * kStageBytes;
            if (r0 < 128 - nM) {
              const uint32_t off = tc::swz_offset(nM + r0, k);
              *reinterpret_cast<uint32_t*>(base + off) = 0u;
              *reinterpret_cast<uint32_t*>(base + kTileA + off) = 0u;
            } else {
              const uint32_t off = tc::swz_offset(nN + r0 - (128 - nM), k);
              *reinterpret_cast<uint32_t*>(base + 2 * kTileA + off) = 0u;
              *reinterpret_cast<uint32_t*>(base + 3 * kTileA + off) = 0u;
            }
          }
          __syncthreads();
          const int nkp = (npts + 31) / 32;  // 32-point chunks holding live points
          for (int kc = 0; kc < nkp; ++kc) {
            const int st = kc & 1;
            uint8_t* Ahi = sm + st * kStageBytes;
            uint8_t* Alo = Ahi + kTileA;
            uint8_t* Bhi = Alo + kTileA;
            uint8_t* Blo = Bhi + kTileA;
            // fill: lane <-> point of the chunk, warps split the shells
            {
              const int q = kc * 32 + lane;
              const bool qlive = q < npts;
              const Pt pt = make_pt(P.xyz + 3 * (first + (qlive ? q : 0)));
              float wv = 0.f, wx = 0.f, wy = 0.f, wz = 0.f;
              if (qlive) {
                wv = s_wv[q];
                wx = s_wg[0][q];
                wy = s_wg[1][q];
                wz = s_wg[2][q];
              }
              int j = 0;
              for (int si = s0; si < s1; ++si) {
                const int info = __ldg(&P.rec[si].info);
                const int f0 = rec_f0(info), nf = rec_nf(info);
                const bool inM = (f0 + nf > mt0) && (f0 < mt0 + nM);
                const bool inN = (f0 + nf > nt0) && (f0 < nt0 + nN);
                if ((inM || inN) && ((j++ & 7) == warp)) {
                  auto put = [&](int f, float val, float dx, float dy, float dz) {
                    const int mu = f0 + f;
                    if (mu >= mt0 && mu < mt0 + nM) st_tf32_pair(Ahi, Alo, tc::swz_offset(mu - mt0, lane), val);
                    if (mu >= nt0 && mu < nt0 + nN)
                      st_tf32_pair(Bhi, Blo, tc::swz_offset(mu - nt0, lane), wv * val + wx * dx + wy * dy + wz * dz);
                  };
                  if (qlive) {
                    shell_rec_at<1>(load_rec(P.rec + si), B.prim2, pt, (float)P.exponent_threshold,
                                    (float)P.radial_threshold, put);
                  } else {
                    for (int f = 0; f < nf; ++f) put(f, 0.f, 0.f, 0.f, 0.f);
                  }
                }
              }
            }
            tc::fence_async_smem();
            if (kc > 0) {
              const int pst = (kc - 1) & 1;
              const bool ok = wait_or_abort(&mbar[pst], phase[pst], err);
              phase[pst] ^= 1;
              outstanding = -1;
              if (__syncthreads_or(!ok)) {
                if (tid == 0) s_abort = 1;
                goto done;
              }
              tc::fence_after_sync();
              drain64(tmem + (pst ? kColsHH1 : kColsHH0), warp, lane, Ds, ld, 64 * (warp >> 2), N, kc == 1);
              tc::fence_before_sync();
            }
            __syncthreads();
            if (tid == 0) {
              tc::fence_after_sync();
              issue_chunk(tmem, tc::smem_u32(Ahi), tc::smem_u32(Alo), tc::smem_u32(Bhi), tc::smem_u32(Blo), N,
                          st ? kColsHH1 : kColsHH0, kc == 0);
              tc::mma_commit(&mbar[st]);
            }
            outstanding = st;
          }
          // last chunk: drain, add the cross terms, scatter into V
          {
            const int pst = (nkp - 1) & 1;
            const bool ok = wait_or_abort(&mbar[pst], phase[pst], err);
            phase[pst] ^= 1;
            outstanding = -1;
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
            tc::fence_after_sync();
            drain64(tmem + (pst ? kColsHH1 : kColsHH0), warp, lane, Ds, ld, 64 * (warp >> 2), N, nkp == 1);
            drain64(tmem + kColsX, warp, lane, Ds, ld, 64 * (warp >> 2), N, false);
            tc::fence_before_sync();
            const int row = 32 * (warp & 3) + lane;
            if (row < nM) {
              const long colmu = fn[mt0 + row];
              const int c0 = 64 * (warp >> 2);
              for (int c = c0; c < c0 + 64 && c < nN; ++c)
                atomicAdd(&Vs[(long)fn[nt0 + c] * nbf + colmu], (double)Ds[row * ld + c]);
            }
            __syncthreads();
          }
        }
      }
    }
  }
done:
  if (outstanding >= 0) wait_or_abort(&mbar[outstanding], phase[outstanding], err);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// TF32 split of the density matrices (hi = TF32(P), lo = TF32(P - hi)), once per build
__global__ void split_p_kernel(const double* __restrict__ P, float* __restrict__ hi, float* __restrict__ lo, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t h, l;
  tc::split_tf32(P[i], h, l);
  hi[i] = __uint_as_float(h);
  lo[i] = __uint_as_float(l);
}

// V <- V + V^T (per spin), turning sum_b D_b into sum_b (D_b + D_b^T)
__global__ void symmetrize_kernel(double* V, int nbf, int nspin) {
  const long n2 = (long)nbf * nbf;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * nspin) return;
  const int s = (int)(idx / n2);
  const long e = idx % n2;
  const int i = (int)(e % nbf), j = (int)(e / nbf);
  if (i > j) return;
  double* M = V + (long)s * n2;
  if (i == j) {
    M[e] *= 2.0;
  } else {
    const double t = M[(long)j * nbf + i] + M[(long)i * nbf + j];
    M[(long)j * nbf + i] = t;
    M[(long)i * nbf + j] = t;
  }
}

static size_t mixed_smem() { return 2 * kStageBytes + 128 * (kNT + 1) * sizeof(float) + 1024; }

xcgpu_status mixed_init(Ctx* c) {
  xcgpu_status st = c->cuda(cudaFuncSetAttribute(mx_density_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)mixed_smem()), "density smem attribute");
  if (st) return st;
  return c->cuda(cudaFuncSetAttribute(mx_adder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mixed_smem()),
                 "adder smem attribute");
}

static void fill_item(MxItem& it, const MixedWork& w) {
  it.B = *w.B;
  it.P = *w.P;
  it.nspin = w.nspin;
  const long n = (long)w.P->nbf * w.P->nbf * w.nspin;
  it.Phi = w.Psplit;
  it.Plo = w.Psplit ? w.Psplit + n : nullptr;
  it.rho = w.rho;
  it.grad = w.grad;
  it.v = w.v;
  it.g = w.g;
  it.skip = w.skip;
  it.V = w.V;
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

xcgpu_status mixed_split(Ctx* c, const double* Pm, float* Psplit, long n) {
  KernelTimer kt(c, kOther);
  split_p_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(Pm, Psplit, Psplit + n, n);
  return c->check_launch("split_p_kernel");
}

xcgpu_status mixed_density_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err) {
  static thread_local MxBatch bt;  // host-side parameter block (the launch copies it)
  for (size_t i0 = 0; i0 < work.size(); i0 += kMaxItems) {
    make_batch(work, i0, std::min(work.size(), i0 + kMaxItems), bt);
    if (bt.nblocks == 0) continue;
    xcgpu_status st = c->cuda(cudaMemsetAsync(counter, 0, sizeof(int), c->stream), "counter");
    if (st) return st;
    KernelTimer kt(c, kDensity);
    mx_density_kernel<<<c->sm_count, kT, mixed_smem(), c->stream>>>(bt, counter, err);
    if ((st = c->check_launch("mx_density_kernel"))) return st;
  }
  return XCGPU_OK;
}

xcgpu_status mixed_adder_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err) {
  static thread_local MxBatch bt;
  xcgpu_status st = XCGPU_OK;
  for (size_t i0 = 0; i0 < work.size(); i0 += kMaxItems) {
    make_batch(work, i0, std::min(work.size(), i0 + kMaxItems), bt);
    if (bt.nblocks == 0) continue;
    if ((st = c->cuda(cudaMemsetAsync(counter, 0, sizeof(int), c->stream), "counter"))) return st;
    KernelTimer kt(c, kAdder);
    mx_adder_kernel<<<c->sm_count, kT, mixed_smem(), c->stream>>>(bt, counter, err);
    if ((st = c->check_launch("mx_adder_kernel"))) return st;
  }
  KernelTimer kt2(c, kOther);
  for (const auto& w : work) {
    const long n = (long)w.P->nbf * w.P->nbf * w.nspin;
    symmetrize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(w.V, w.P->nbf, w.nspin);
    if ((st = c->check_launch("symmetrize_kernel"))) return st;
  }
  return XCGPU_OK;
}

}  // namespace xcgpu
