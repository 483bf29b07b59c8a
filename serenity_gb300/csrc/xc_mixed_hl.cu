// The mixed-precision kernels of xc_mixed_kernel.cuh for bases with g, h or i functions
// (MAXL 6): a translation unit of their own, so that they compile in parallel with the
// l <= 3 kernels the SVP/TZVP builds use.
#include "xc_mixed_kernel.cuh"

namespace xcgpu {

xcgpu_status mixed_init_hl(Ctx* c) {
  const void* k[] = {(const void*)mx_kernel<kModeDensity, 0, false, 6>, (const void*)mx_kernel<kModeDensity, 1, false, 6>,
                     (const void*)mx_kernel<kModeAdder, 0, false, 6>,   (const void*)mx_kernel<kModeAdder, 1, false, 6>,
                     (const void*)mx_kernel<kModeAdder, 0, true, 6>,    (const void*)mx_kernel<kModeAdder, 1, true, 6>,
                     (const void*)mx_kernel<kModeBuild, 0, false, 6>,   (const void*)mx_kernel<kModeBuild, 1, false, 6>,
                     (const void*)mx_kernel<kModeBuild, 0, true, 6>,    (const void*)mx_kernel<kModeBuild, 1, true, 6>};
  for (const void* fn : k) {
    xcgpu_status st = c->cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx_smem()),
                              "mixed kernel smem attribute");
    if (st) return st;
  }
  return XCGPU_OK;
}

void mixed_launch_hl(int mode, bool gga, bool two, unsigned grid, cudaStream_t s, const MxBatch& bt, int* counter,
                     int* err) {
  void (*kern)(MxBatch, int*, int*);
  if (mode == kModeDensity) kern = gga ? mx_kernel<kModeDensity, 1, false, 6> : mx_kernel<kModeDensity, 0, false, 6>;
  else if (mode == kModeAdder)
    kern = gga ? (two ? mx_kernel<kModeAdder, 1, true, 6> : mx_kernel<kModeAdder, 1, false, 6>)
               : (two ? mx_kernel<kModeAdder, 0, true, 6> : mx_kernel<kModeAdder, 0, false, 6>);
  else
    kern = gga ? (two ? mx_kernel<kModeBuild, 1, true, 6> : mx_kernel<kModeBuild, 1, false, 6>)
               : (two ? mx_kernel<kModeBuild, 0, true, 6> : mx_kernel<kModeBuild, 0, false, 6>);
  kern<<<grid, kT, mx_smem(), s>>>(bt, counter, err);
}

}  // namespace xcgpu
