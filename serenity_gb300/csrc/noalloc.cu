// FP64 density on the grid for callers that cannot allocate device memory.
//
// Some hosts of this library may not call cudaMalloc at the point where they need
// rho: an SCF driver embedded in a program that owns all device memory through its
// own fixed pool, or a real-time loop whose memory was reserved up front.  For them,
// xcgpu_density_fp64_noalloc computes rho and grad rho with the same FP64 kernels as
// xcgpu_density, but keeps the per-block basis slabs in a fixed, file-scope device
// array instead of allocating scratch.  It calls no cudaMalloc, cudaFree or other
// allocating routine; the plan, P and the outputs are the caller's.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "internal.h"

namespace xcgpu {

// 64 MiB of FP64 scratch, held by every GPU that loads the library until the process
// exits.  Shared by all calls: it keeps the last call's contents, so calls that
// overlap on the GPU (other host threads, other streams) race on it.
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
constexpr long kNoAllocDoubles = (long)(kNoAllocScratchBytes / sizeof(double));
constexpr long kNoAllocMaxBlocks = 4096;  // slab offsets kept at the front of the array
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

// Device address of the static scratch in the current context.  The host-side name of
// the array is only a stand-in, not a device address, and the array's address belongs
// to the context that loaded the module, so it is looked up on every call (which
// allocates nothing) rather than remembered per device ordinal.
static xcgpu_status scratch_address(Ctx* c, double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return c->cuda(e, "cudaGetSymbolAddress(no-allocation scratch)");
  *out = static_cast<double*>(p);
  return XCGPU_OK;
}

// slab offsets of blocks [b0, b0 + nb): 4 components x 128 points per active function
__global__ void noalloc_offsets_kernel(const int* __restrict__ fn_off, int b0, int nb, long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) out[i] = 4L * kBlockPoints * (long)(fn_off[b0 + i] - fn_off[b0]);
}

}  // namespace xcgpu

using namespace xcgpu;

extern "C" xcgpu_status xcgpu_density_fp64_noalloc(xcgpu_plan* P, int nspin, const double* Pm, double* rho,
                                                    double* grad) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if ((nspin != 1 && nspin != 2) || !Pm || !rho) return c->fail(XCGPU_ERR_INVALID, "density_noalloc: bad arguments");
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return c->cuda(e, "cudaSetDevice");
  double* base = nullptr;
  xcgpu_status st = scratch_address(c, &base);
  if (st) return st;
  long* offsets = reinterpret_cast<long*>(base);
  double* slabs = base + kNoAllocMaxBlocks;  // sizeof(long) == sizeof(double)
  const long cap = kNoAllocDoubles - kNoAllocMaxBlocks;
  // chunks of consecutive blocks whose slabs fit the fixed scratch
  int b0 = 0;
  while (b0 < P->nblocks) {
    long need = 0;
    int b1 = b0;
    while (b1 < P->nblocks && b1 - b0 < kNoAllocMaxBlocks) {
      const long nb = 4L * kBlockPoints * (P->fn_off[b1 + 1] - P->fn_off[b1]);
      if (need + nb > cap) break;
      need += nb;
      ++b1;
    }
    if (b1 == b0) {
      const long nb = 4L * kBlockPoints * (P->fn_off[b0 + 1] - P->fn_off[b0]);
      return c->fail(XCGPU_ERR_BUDGET, "density_noalloc: block " + std::to_string(b0) + " needs " +
                                           std::to_string(nb * sizeof(double)) +
                                           " bytes of scratch, more than the fixed " +
                                           std::to_string(cap * sizeof(double)) + " bytes of this entry point");
    }
    noalloc_offsets_kernel<<<(b1 - b0 + 127) / 128, 128, 0, c->stream>>>(P->dev.fn_off, b0, b1 - b0, offsets);
    if ((st = c->check_launch("noalloc_offsets_kernel"))) return st;
    if ((st = fp64_eval_chunk(c, P->basis->dev, P->dev, b0, b1, offsets, slabs, 1))) return st;
    if ((st = fp64_density_chunk(c, P->dev, b0, b1, offsets, slabs, nspin, Pm, rho, grad))) return st;
    b0 = b1;
  }
  return c->cuda(cudaStreamSynchronize(c->stream), "density_noalloc");
}
