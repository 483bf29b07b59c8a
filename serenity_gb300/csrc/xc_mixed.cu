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

#include "basis_eval.cuh"
#include "internal.h"
#include "tcgen05.cuh"

namespace xcgpu {

constexpr int kMxThreads = 128;
constexpr int kDNPass = 256;            // functions per density pass (TMEM columns)
constexpr uint32_t kTileA = 128 * 128;  // bytes of a 128-row x 32-element operand tile
constexpr uint64_t kWaitLimitNs = 2000000000ull;
constexpr int kErrTimeout = 1;

// active shell list of block b with the local index of each shell's first function
struct BlockShells {
  int s0, s1;  // range in P.sh_list
};

__device__ __forceinline__ int shell_nf(const DevBasis& B, int sh) {
  return B.pure[sh] ? 2 * B.l[sh] + 1 : ncart_d(B.l[sh]);
}

// Evaluate one shell (FP32) at a point given in FP64; returns false if negligible
// there (all functions zero).  DERIV 0: values, 1: values + gradients.
template <int DERIV, class Emit>
__device__ __forceinline__ void shell_at(const DevBasis& B, const DevPlan& P, int sh, double px, double py, double pz,
                                         Emit&& emit) {
  const int l = B.l[sh];
  const bool pure = B.pure[sh] != 0;
  const float x = (float)(px - B.center[3 * sh]), y = (float)(py - B.center[3 * sh + 1]),
              z = (float)(pz - B.center[3 * sh + 2]);
  const float r2 = x * x + y * y + z * z;
  float Rv, dR, ddR;
  const int o = B.prim_off[sh];
  const bool sig = shell_radial<float, DERIV>(B.alpha + o, B.coef + o, B.nprim[sh], r2, (float)P.exponent_threshold,
                                              (float)P.radial_threshold, Rv, dR, ddR);
  if (!sig) {
    const int nf = pure ? 2 * l + 1 : ncart_d(l);
    float hz[6] = {0, 0, 0, 0, 0, 0};
    for (int f = 0; f < nf; ++f) emit(f, 0.f, 0.f, 0.f, 0.f, hz);
    return;
  }
  shell_functions_l<float, DERIV>(l, x, y, z, Rv, dR, ddR, pure, B.trans + B.trans_off[l], B.cnorm + B.cnorm_off[l],
                                  emit);
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

// =====================================================================================
// density
// =====================================================================================
__global__ void __launch_bounds__(kMxThreads, 1)
    mx_density_kernel(DevBasis B, DevPlan P, int nspin, const double* __restrict__ Pm, double* __restrict__ rho,
                      double* __restrict__ grad, int* __restrict__ counter, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_block;
  __shared__ int s_abort;
  // 1024-byte aligned operand area: 2 stages x (A_hi, A_lo: 16 KB; B_hi, B_lo: 32 KB)
  const uint32_t base_s = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base_s & 1023)) & 1023);
  const uint32_t kStage = 2 * kTileA + 2 * 2 * kTileA;  // 96 KB
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, kDNPass);
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
  bool pending[2] = {false, false};
  uint32_t chunk_seq = 0;
  const int nbf = P.nbf;

  for (;;) {
    __syncthreads();  // every thread is done with the previous s_block
    if (tid == 0) s_block = atomicAdd(counter, 1);
    __syncthreads();
    const int b = s_block;
    if (b >= P.nblocks || s_abort) break;
    const long first = (long)b * P.max_block;
    const int npts = (int)min((long)P.max_block, P.npoints - first);
    const int nact = P.fn_off[b + 1] - P.fn_off[b];
    const int* fn = P.fn_list + P.fn_off[b];
    const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
    const int p = tid;
    const bool live = p < npts;
    double px = 0, py = 0, pz = 0;
    if (live) {
      px = P.xyz[3 * (first + p)];
      py = P.xyz[3 * (first + p) + 1];
      pz = P.xyz[3 * (first + p) + 2];
    }
    for (int s = 0; s < nspin; ++s) {
      const double* Pmat = Pm + (long)s * nbf * nbf;
      double r_acc = 0.0, g_acc[3] = {0.0, 0.0, 0.0};
      for (int nu0 = 0; nu0 < nact; nu0 += kDNPass) {
        const int nnu = min(kDNPass, nact - nu0);
        const int N = (nnu + 15) & ~15;
        const int nkc = (nact + 31) / 32;
        int sh_cursor = s0, f_cursor = 0;  // first shell that may overlap the next chunk
        for (int kc = 0; kc < nkc; ++kc) {
          const int st = chunk_seq & 1;
          if (pending[st]) {
            const bool ok = wait_or_abort(&mbar[st], phase[st], err);
            phase[st] ^= 1;
            pending[st] = false;
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
          }
          uint8_t* Ahi = sm + st * kStage;
          uint8_t* Alo = Ahi + kTileA;
          uint8_t* Bhi = Alo + kTileA;
          uint8_t* Blo = Bhi + 2 * kTileA;
          const int mu0 = kc * 32;
          // ---- A: Phi[p][mu0 .. mu0+32) ----
          {
            // zero this thread's row first (covers padding and negligible shells)
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
              *reinterpret_cast<uint32_t*>(Ahi + tc::swz_offset(p, k)) = 0u;
              *reinterpret_cast<uint32_t*>(Alo + tc::swz_offset(p, k)) = 0u;
            }
            while (sh_cursor < s1 && f_cursor + shell_nf(B, P.sh_list[sh_cursor]) <= mu0) {
              f_cursor += shell_nf(B, P.sh_list[sh_cursor]);
              ++sh_cursor;
            }
            if (live) {
              int si = sh_cursor, f0 = f_cursor;
              while (si < s1 && f0 < mu0 + 32) {
                const int sh = P.sh_list[si];
                const int nf = shell_nf(B, sh);
                shell_at<0>(B, P, sh, px, py, pz, [&](int f, float v, float, float, float, const float*) {
                  const int k = f0 + f - mu0;
                  if (k >= 0 && k < 32) st_tf32_pair(Ahi, Alo, tc::swz_offset(p, k), v);
                });
                f0 += nf;
                ++si;
              }
            }
          }
          // ---- B: P_b[nu][mu0 .. mu0+32) for nu in [nu0, nu0 + N) ----
          for (int e = tid; e < N * 32; e += kMxThreads) {
            const int nu = e % N, k = e / N;
            const int mu = mu0 + k;
            double val = 0.0;
            if (nu < nnu && mu < nact) val = Pmat[(long)fn[mu] * nbf + fn[nu0 + nu]];
            uint32_t h, l;
            tc::split_tf32(val, h, l);
            const uint32_t off = tc::swz_offset(nu, k);
            *reinterpret_cast<uint32_t*>(Bhi + off) = h;
            *reinterpret_cast<uint32_t*>(Blo + off) = l;
          }
          tc::fence_async_smem();
          __syncthreads();
          if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t idesc = tc::idesc_tf32(128, N);
            const uint32_t ah = tc::smem_u32(Ahi), al = tc::smem_u32(Alo), bh = tc::smem_u32(Bhi),
                           bl = tc::smem_u32(Blo);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint32_t o = ks * 32;
              const uint32_t acc0 = (kc > 0 || ks > 0) ? 1u : 0u;
              tc::mma_tf32(tmem, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bh + o), idesc, acc0);
              tc::mma_tf32(tmem, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bl + o), idesc, 1u);
              tc::mma_tf32(tmem, tc::smem_desc_sw128(al + o), tc::smem_desc_sw128(bh + o), idesc, 1u);
            }
            tc::mma_commit(&mbar[st]);
          }
          pending[st] = true;
          ++chunk_seq;
        }
        // drain both stages
        for (int st = 0; st < 2; ++st)
          if (pending[st]) {
            const bool ok = wait_or_abort(&mbar[st], phase[st], err);
            phase[st] ^= 1;
            pending[st] = false;
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
          }
        tc::fence_after_sync();
        // ---- epilogue: X (TMEM) -> shared memory rows, then the row dots ----
        float* Xs = reinterpret_cast<float*>(sm);
        const int ld = N + 1;
        for (int c0 = 0; c0 < N; c0 += 32) {
          float v[32];
          tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (c0 + i < N) Xs[(32 * warp + lane) * ld + c0 + i] = v[i];
        }
        tc::fence_before_sync();
        __syncthreads();
        if (live) {
          int f0 = 0;
          for (int si = s0; si < s1; ++si) {
            const int sh = P.sh_list[si];
            const int nf = shell_nf(B, sh);
            if (f0 + nf > nu0 && f0 < nu0 + nnu) {
              float r = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
              shell_at<1>(B, P, sh, px, py, pz, [&](int f, float v, float dx, float dy, float dz, const float*) {
                const int c = f0 + f - nu0;
                if (c >= 0 && c < nnu) {
                  const float xv = Xs[p * ld + c];
                  r = fmaf(xv, v, r);
                  gx = fmaf(xv, dx, gx);
                  gy = fmaf(xv, dy, gy);
                  gz = fmaf(xv, dz, gz);
                }
              });
              r_acc += (double)r;
              g_acc[0] += (double)gx;
              g_acc[1] += (double)gy;
              g_acc[2] += (double)gz;
            }
            f0 += nf;
          }
        }
        __syncthreads();  // X staging area is reused by the next chunk fill
      }
      if (live) {
        rho[(long)s * P.npoints + first + p] = r_acc;
        if (grad) {
          grad[((long)s * 3 + 0) * P.npoints + first + p] = 2.0 * g_acc[0];
          grad[((long)s * 3 + 1) * P.npoints + first + p] = 2.0 * g_acc[1];
          grad[((long)s * 3 + 2) * P.npoints + first + p] = 2.0 * g_acc[2];
        }
      }
    }
  }
done:
  // leave only after every committed MMA has finished with TMEM and shared memory
  for (int st = 0; st < 2; ++st)
    if (pending[st]) wait_or_abort(&mbar[st], phase[st], err);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kDNPass);
}

// =====================================================================================
// adder
// =====================================================================================
constexpr int kANTile = 256;  // functions per N tile
constexpr int kAMRows = 256;  // functions per M pass (two 128-row MMAs)

__global__ void __launch_bounds__(kMxThreads, 1)
    mx_adder_kernel(DevBasis B, DevPlan P, int nspin, const double* __restrict__ v, const double* __restrict__ g,
                    const unsigned char* __restrict__ skip, double* __restrict__ V, int* __restrict__ counter,
                    int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_block;
  __shared__ int s_abort;
  __shared__ float s_wv[128], s_wg[3][128];
  const uint32_t base_s = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base_s & 1023)) & 1023);
  // A_hi, A_lo: 2 x 16 KB each (two 128-row M tiles); B_hi, B_lo: 32 KB each
  uint8_t* Ahi = sm;
  uint8_t* Alo = Ahi + 2 * kTileA;
  uint8_t* Bhi = Alo + 2 * kTileA;
  uint8_t* Blo = Bhi + 2 * kTileA;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
    s_abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  uint32_t phase = 0;
  bool pending = false;
  const int nbf = P.nbf;

  for (;;) {
    __syncthreads();  // every thread is done with the previous s_block
    if (tid == 0) s_block = atomicAdd(counter, 1);
    __syncthreads();
    const int b = s_block;
    if (b >= P.nblocks || s_abort) break;
    const long first = (long)b * P.max_block;
    const int npts = (int)min((long)P.max_block, P.npoints - first);
    const int nact = P.fn_off[b + 1] - P.fn_off[b];
    const int* fn = P.fn_list + P.fn_off[b];
    const int s0 = P.sh_off[b], s1 = P.sh_off[b + 1];
    for (int s = 0; s < nspin; ++s) {
      if (skip[(long)s * P.nblocks + b]) continue;
      // weighted potentials of the block's points (FP64 -> FP32)
      {
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
      for (int nt0 = 0; nt0 < nact; nt0 += kANTile) {
        const int nN = min(kANTile, nact - nt0);
        const int N = (nN + 15) & ~15;
        for (int mt0 = 0; mt0 < nact; mt0 += kAMRows) {
          const int nM = min(kAMRows, nact - mt0);
          const int mtiles = (nM + 127) / 128;
          for (int kc = 0; kc < 4; ++kc) {
            if (pending) {
              const bool ok = wait_or_abort(&mbar, phase, err);
              phase ^= 1;
              pending = false;
              if (__syncthreads_or(!ok)) {
                if (tid == 0) s_abort = 1;
                goto done;
              }
            }
            // zero the operand rows this chunk uses (padding rows and negligible shells stay 0)
            {
              const int rowsA = mtiles * 128;
              for (int e = tid; e < (rowsA + N) * 32; e += kMxThreads) {
                const int r = e / 32, k = e % 32;
                if (r < rowsA) {
                  const uint32_t off = (uint32_t)(r / 128) * kTileA + tc::swz_offset(r % 128, k);
                  *reinterpret_cast<uint32_t*>(Ahi + off) = 0u;
                  *reinterpret_cast<uint32_t*>(Alo + off) = 0u;
                } else {
                  const uint32_t off = tc::swz_offset(r - rowsA, k);
                  *reinterpret_cast<uint32_t*>(Bhi + off) = 0u;
                  *reinterpret_cast<uint32_t*>(Blo + off) = 0u;
                }
              }
            }
            __syncthreads();
            // fill: lane <-> point (32 points of this chunk), warps split the shells
            const int q = kc * 32 + lane;
            if (q < npts) {
              const double px = P.xyz[3 * (first + q)], py = P.xyz[3 * (first + q) + 1],
                           pz = P.xyz[3 * (first + q) + 2];
              const float wv = s_wv[q], wx = s_wg[0][q], wy = s_wg[1][q], wz = s_wg[2][q];
              int f0 = 0, j = 0;
              for (int si = s0; si < s1; ++si) {
                const int sh = P.sh_list[si];
                const int nf = shell_nf(B, sh);
                const bool inM = (f0 + nf > mt0) && (f0 < mt0 + nM);
                const bool inN = (f0 + nf > nt0) && (f0 < nt0 + nN);
                if ((inM || inN) && ((j++ & 3) == warp)) {
                  shell_at<1>(B, P, sh, px, py, pz, [&](int f, float val, float dx, float dy, float dz, const float*) {
                    const int mu = f0 + f;
                    if (mu >= mt0 && mu < mt0 + nM) {
                      const int r = mu - mt0;
                      st_tf32_pair(Ahi, Alo, (uint32_t)(r / 128) * kTileA + tc::swz_offset(r % 128, lane), val);
                    }
                    if (mu >= nt0 && mu < nt0 + nN) {
                      const float gval = wv * val + wx * dx + wy * dy + wz * dz;
                      st_tf32_pair(Bhi, Blo, tc::swz_offset(mu - nt0, lane), gval);
                    }
                  });
                }
                f0 += nf;
              }
            }
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
              tc::fence_after_sync();
              const uint32_t idesc = tc::idesc_tf32(128, N);
              const uint32_t bh = tc::smem_u32(Bhi), bl = tc::smem_u32(Blo);
              for (int mt = 0; mt < mtiles; ++mt) {
                const uint32_t ah = tc::smem_u32(Ahi) + mt * kTileA, al = tc::smem_u32(Alo) + mt * kTileA;
                const uint32_t d = tmem + (uint32_t)(mt * 256);
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                  const uint32_t o = ks * 32;
                  const uint32_t acc0 = (kc > 0 || ks > 0) ? 1u : 0u;
                  tc::mma_tf32(d, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bh + o), idesc, acc0);
                  tc::mma_tf32(d, tc::smem_desc_sw128(ah + o), tc::smem_desc_sw128(bl + o), idesc, 1u);
                  tc::mma_tf32(d, tc::smem_desc_sw128(al + o), tc::smem_desc_sw128(bh + o), idesc, 1u);
                }
              }
              tc::mma_commit(&mbar);
            }
            pending = true;
          }
          // wait for the tile's MMAs, then scatter D into V (FP64)
          {
            const bool ok = wait_or_abort(&mbar, phase, err);
            phase ^= 1;
            pending = false;
            if (__syncthreads_or(!ok)) {
              if (tid == 0) s_abort = 1;
              goto done;
            }
          }
          tc::fence_after_sync();
          double* Vs = V + (long)s * nbf * nbf;
          for (int mt = 0; mt < mtiles; ++mt) {
            const int r = mt * 128 + 32 * warp + lane;  // row of D = function mt0 + r
            const int mu = mt0 + r;
            const long col_mu = (mu < mt0 + nM) ? fn[mu] : 0;
            for (int c0 = 0; c0 < N; c0 += 32) {
              float dv[32];
              tc::tmem_ld32(tmem + (uint32_t)(mt * 256) + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, dv);
              if (mu < mt0 + nM) {
#pragma unroll 4
                for (int i = 0; i < 32; ++i) {
                  const int nu = nt0 + c0 + i;
                  if (c0 + i < nN) atomicAdd(&Vs[(long)fn[nu] * nbf + col_mu], (double)dv[i]);
                }
              }
            }
          }
          tc::fence_before_sync();
          __syncthreads();
        }
      }
    }
  }
done:
  if (pending) wait_or_abort(&mbar, phase, err);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
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

static size_t density_smem() { return 2 * (2 * kTileA + 4 * kTileA) + 1024; }
static size_t adder_smem() { return 8 * kTileA + 1024; }

xcgpu_status mixed_density(Ctx* c, const DevBasis& B, const DevPlan& P, int nspin, const double* Pm, double* rho,
                           double* grad, int* counter, int* err) {
  if (P.nblocks == 0) return XCGPU_OK;
  xcgpu_status st = c->cuda(cudaFuncSetAttribute(mx_density_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)density_smem()), "density smem attribute");
  if (st) return st;
  if ((st = c->cuda(cudaMemsetAsync(counter, 0, sizeof(int), c->stream), "counter"))) return st;
  KernelTimer kt(c, kDensity);
  mx_density_kernel<<<c->sm_count, kMxThreads, density_smem(), c->stream>>>(B, P, nspin, Pm, rho, grad, counter, err);
  return c->check_launch("mx_density_kernel");
}

xcgpu_status mixed_adder(Ctx* c, const DevBasis& B, const DevPlan& P, int nspin, const double* v, const double* g,
                         const unsigned char* skip, double* V, int* counter, int* err) {
  if (P.nblocks == 0) return XCGPU_OK;
  xcgpu_status st = c->cuda(cudaFuncSetAttribute(mx_adder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)adder_smem()), "adder smem attribute");
  if (st) return st;
  if ((st = c->cuda(cudaMemsetAsync(counter, 0, sizeof(int), c->stream), "counter"))) return st;
  {
    KernelTimer kt(c, kAdder);
    mx_adder_kernel<<<c->sm_count, kMxThreads, adder_smem(), c->stream>>>(B, P, nspin, v, g, skip, V, counter, err);
    if ((st = c->check_launch("mx_adder_kernel"))) return st;
  }
  KernelTimer kt2(c, kOther);
  const long n = (long)P.nbf * P.nbf * nspin;
  symmetrize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(V, P.nbf, nspin);
  return c->check_launch("symmetrize_kernel");
}

}  // namespace xcgpu
