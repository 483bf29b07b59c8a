// Thin inline-PTX layer for the sm_100-family tensor cores (tcgen05 / TMEM),
// shared-memory matrix descriptors, mbarriers and bulk copies.
//
// Operand layout used everywhere: K-major, 128-byte swizzle.  A tile of R rows
// (R % 8 == 0) and 128 bytes per row (64 FP16, or 32 FP32/TF32 elements) starts on a
// 1024-byte boundary; byte b of row r lives at
//     r * 128 + (((b >> 4) ^ (r & 7)) << 4) + (b & 15)
// (16-byte chunks XOR-permuted by the row index within each 8-row, 1024-byte atom).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace xcgpu {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start >> 4 in bits [0,14), leading byte
// offset >> 4 in [16,30), stride byte offset >> 4 in [32,46), version 1 in [46,48),
// swizzle mode in [61,64) (2 = 128-byte swizzle).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = FP16 (bits 7-9,
// 10-12 = 0), both K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ __forceinline__ uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

// warp-wide TMEM allocation; the base address is written to *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase: gives up after `limit_ns` of wall time and
// returns false (the caller records an error and leaves without hanging the GPU).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(mbar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(mbar, parity)) return true;
    if ((it & 255) == 255 && globaltimer() - t0 > limit_ns) return false;
  }
}

// mbarrier arrival that also announces `bytes` of bulk-copy transactions
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
}
// bulk copy (TMA, non-tensor) global -> shared, completing on an mbarrier; both
// addresses 16-byte aligned, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}
// order this thread's generic-proxy global writes before later async-proxy (TMA) reads
__device__ __forceinline__ void fence_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// TMEM loads: thread i of the warp gets row (lane base + i); the columns of each load
// follow the address.
// n loads of 32 lanes x 8 columns each (columns taddr[i] .. + 8), then one wait: the
// destination registers pass through the wait so no use of them is scheduled before it
#define XCGPU_TMEM_LD8(T, R)                                                                          \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"               \
               : "=r"((R)[0]), "=r"((R)[1]), "=r"((R)[2]), "=r"((R)[3]), "=r"((R)[4]), "=r"((R)[5]), \
                 "=r"((R)[6]), "=r"((R)[7])                                                           \
               : "r"(T))
#define XCGPU_TMEM_PASS8(R)                                                                             \
  "+r"((R)[0]), "+r"((R)[1]), "+r"((R)[2]), "+r"((R)[3]), "+r"((R)[4]), "+r"((R)[5]), "+r"((R)[6]), \
      "+r"((R)[7])
__device__ __forceinline__ void tmem_ld8x2(uint32_t t0, uint32_t t1, float* a, float* b) {
  uint32_t r0[8], r1[8];
  XCGPU_TMEM_LD8(t0, r0);
  XCGPU_TMEM_LD8(t1, r1);
  asm volatile("tcgen05.wait::ld.sync.aligned;" : XCGPU_TMEM_PASS8(r0), XCGPU_TMEM_PASS8(r1)::"memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = __uint_as_float(r0[i]);
    b[i] = __uint_as_float(r1[i]);
  }
}
__device__ __forceinline__ void tmem_ld8x4(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t t3, float* a, float* b,
                                           float* c, float* d) {
  uint32_t r0[8], r1[8], r2[8], r3[8];
  XCGPU_TMEM_LD8(t0, r0);
  XCGPU_TMEM_LD8(t1, r1);
  XCGPU_TMEM_LD8(t2, r2);
  XCGPU_TMEM_LD8(t3, r3);
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : XCGPU_TMEM_PASS8(r0), XCGPU_TMEM_PASS8(r1), XCGPU_TMEM_PASS8(r2), XCGPU_TMEM_PASS8(r3)::"memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = __uint_as_float(r0[i]);
    b[i] = __uint_as_float(r1[i]);
    c[i] = __uint_as_float(r2[i]);
    d[i] = __uint_as_float(r3[i]);
  }
}
#undef XCGPU_TMEM_LD8
#undef XCGPU_TMEM_PASS8

// byte offset of FP16 element (r, k), k < 64, in a 128-byte-swizzled K-major tile
// (64 FP16 per 128-byte row; the same 16-byte chunk permutation as above)
__device__ __forceinline__ uint32_t swz_offset_h(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + (k & 7) * 2);
}

}  // namespace tc
}  // namespace xcgpu
