// Internal declarations of the xcgpu library (GB300 / sm_103a XC integration).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/xcgpu.h"

namespace xcgpu {

constexpr int kMaxL = 6;              // AM_MAX (Constants.h:31)
constexpr int kBlockPoints = 128;     // points per block handled by one CTA
constexpr int kSkipBlock = 128;       // FunctionalLibrary(128) block (FuncPotential.cpp:86)
constexpr double kDensTiny = 1e-14;   // point cut-off of the functional

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Device-side basis description (struct of arrays, all device pointers).
struct DevBasis {
  int nshell = 0, nbf = 0, maxl = 0;
  const int* l = nullptr;          // [nshell]
  const int* pure = nullptr;       // [nshell]
  const int* nprim = nullptr;      // [nshell]
  const int* prim_off = nullptr;   // [nshell]
  const int* first = nullptr;      // [nshell] first function index
  const double* center = nullptr;  // [3*nshell]
  const double* alpha = nullptr;   // [nprim total]
  const double* coef = nullptr;    // [nprim total] normalised
  const double* trans = nullptr;   // transform tables: per l, (2l+1) x ncart(l) solid harmonics
  const double* cnorm = nullptr;   // per l, ncart(l) Cartesian factors
  const int* trans_off = nullptr;  // [kMaxL+1] offsets into trans
  const int* cnorm_off = nullptr;  // [kMaxL+1] offsets into cnorm
  const float4* prim4 = nullptr;   // FP32 kernels: (alpha_hi, coef_hi, alpha_lo, coef_lo), x = x_hi + x_lo
};

// Per (block, active shell) record used by the FP32 kernels (32 bytes).  The centre
// is split into an FP32 high part and FP32 remainder so that p - A keeps FP32
// relative accuracy; info packs l (bits 0-2), pure (3), nprim (4-8), nfunc (9-13)
// and the shell's first function within the block's active list (14-31).
struct __align__(16) ShellRec {
  float ah[3];
  float al[3];
  int info;
  int prim0;  // offset of the shell's primitives in DevBasis::prim4
};

// Device-side block table of a plan.
struct DevPlan {
  int nblocks = 0, max_block = 0, nbf = 0;
  int max_active = 0;              // largest active-function count of the blocks
  long npoints = 0;
  const double* xyz = nullptr;     // [3*npoints]
  const double* w = nullptr;       // [npoints]
  const int* sh_off = nullptr;     // [nblocks+1] active shells of block b: sh_list[sh_off[b] .. sh_off[b+1])
  const int* sh_list = nullptr;
  const int* fn_off = nullptr;     // [nblocks+1] active functions of block b
  const int* fn_list = nullptr;
  const ShellRec* rec = nullptr;   // parallel to sh_list
  double radial_threshold = 1e-9, exponent_threshold = 0.0;
};

struct Ctx;

// Simple owning device buffer that books its size against the context budget.
struct DevBuf {
  Ctx* ctx = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf();
  void* h = nullptr;  // pinned host buffer (alloc_host)
  size_t hbytes = 0;
  xcgpu_status alloc(Ctx* c, size_t n);       // device; no-op if already >= n
  xcgpu_status alloc_host(Ctx* c, size_t n);  // pinned host; no-op if already >= n
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

enum KernelClass { kEval = 0, kDensity = 1, kFunctional = 2, kAdder = 3, kOther = 4, kBuild = 5, kClasses = 6 };

struct Ctx {
  int device = 0;
  // per-kernel timing (xcgpu_set_timing)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  double t_ms[kClasses] = {0, 0, 0, 0, 0, 0};
  uint64_t t_count[kClasses] = {0, 0, 0, 0, 0, 0};
  cudaEvent_t take_event() {
    if (ev_pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = ev_pool.back();
    ev_pool.pop_back();
    return e;
  }
  uint64_t budget = 0, in_use = 0, scratch_cap = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  uint64_t launches = 0;
  std::string err;
  int sm_count = 0;
  // reusable scratch
  DevBuf scratch, scratch2, partials, skip, batch_items, host_items;
  // block counters and the error word of the builds issued on each stream (builds on
  // different streams may be in flight together)
  std::map<cudaStream_t, std::unique_ptr<DevBuf>> aux_by_stream;
  // per-CTA basis scratch of the mixed-precision kernels, per stream
  std::map<cudaStream_t, std::unique_ptr<DevBuf>> mixed_by_stream;
  // per stream: the work buffers of the whole builds in flight on it (one arena carved
  // per request, so plans stay read-only and any number of requests may share one) and
  // the FP64 basis-value slabs
  std::map<cudaStream_t, std::unique_ptr<DevBuf>> arena_by_stream, fp64_by_stream;
  DevBuf& on_stream(std::map<cudaStream_t, std::unique_ptr<DevBuf>>& m) {
    auto& b = m[stream];
    if (!b) b.reset(new DevBuf());
    return *b;
  }
  xcgpu_status aux(int** out) {
    auto& b = aux_by_stream[stream];
    if (!b) b.reset(new DevBuf());
    xcgpu_status st = b->alloc(this, 4 * sizeof(int));
    if (st) return st;
    *out = b->as<int>();
    return XCGPU_OK;
  }
  xcgpu_status fail(xcgpu_status s, const std::string& msg) {
    err = msg;
    return s;
  }
  xcgpu_status cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return XCGPU_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return XCGPU_ERR_CUDA;
  }
  xcgpu_status check_launch(const char* what) {
    ++launches;
    return cuda(cudaGetLastError(), what);
  }
};

// Brackets the kernel launches of one class with events when timing is enabled.
struct KernelTimer {
  Ctx* c;
  int cls;
  cudaEvent_t a = nullptr;
  KernelTimer(Ctx* ctx, int k) : c(ctx), cls(k) {
    if (c->timing) {
      a = c->take_event();
      cudaEventRecord(a, c->stream);
    }
  }
  ~KernelTimer() {
    if (c->timing) {
      cudaEvent_t b = c->take_event();
      cudaEventRecord(b, c->stream);
      c->ev_pending.push_back({cls, {a, b}});
    }
  }
};

}  // namespace xcgpu

struct xcgpu_ctx : xcgpu::Ctx {};

struct xcgpu_grid {
  xcgpu::Ctx* ctx = nullptr;
  long n = 0;
  xcgpu::DevBuf xyz, w;
};

struct xcgpu_basis {
  xcgpu::Ctx* ctx = nullptr;
  int nshell = 0, nbf = 0, maxl = 0;
  std::vector<int> l, pure, nprim, prim_off, first;
  std::vector<double> center, alpha, coef;
  xcgpu::DevBuf d_l, d_pure, d_nprim, d_prim_off, d_first, d_center, d_alpha, d_coef, d_trans, d_cnorm, d_toff, d_coff,
      d_prim4;
  xcgpu::DevBasis dev;
};

struct xcgpu_plan {
  xcgpu::Ctx* ctx = nullptr;
  xcgpu_grid* grid = nullptr;
  xcgpu_basis* basis = nullptr;
  int max_block = 128, nblocks = 0;
  double radial_threshold = 1e-9;
  std::vector<int> sh_off, sh_list, fn_off, fn_list;  // host copies
  int max_active = 0;
  double flops = 0.0;
  xcgpu::DevBuf d_sh_off, d_sh_list, d_fn_off, d_fn_list, d_rec;
  // adder tile work list (block, tile_i, tile_j) for 64-wide tiles, all pairs
  std::vector<int> work;  // 3 ints per item, sorted by block
  std::vector<long> work_off;  // [nblocks+1]
  xcgpu::DevBuf d_work;
  xcgpu::DevPlan dev;
  // resident work buffers of the build (kept across calls: no allocation per build)
  bool chunks_ready = false;
  std::vector<int> chunk_bounds;
  long chunk_max_doubles = 0;
  xcgpu::DevBuf w_fskip, w_psplit, w_slab, w_P, w_V, w_rho, w_grad, w_epuv, w_dfdrho, w_dfdgrad, w_partials, w_sums, w_skip, w_aux;
  // supersystem quantities of a non-additive build whose active subsystem is this plan
  xcgpu::DevBuf n_rho, n_grad, n_epuv, n_dfdrho, n_dfdgrad, n_partials, n_fskip, n_sums;
};

namespace xcgpu {

// host helpers implemented in the .cu files
std::vector<double> solid_harmonic_matrix(int l);
std::vector<double> cartesian_norms(int l);

// kernels (launchers); all return a status and record errors on ctx
xcgpu_status launch_screen(Ctx* c, const DevBasis& B, const double* xyz, long npoints, int max_block, int nblocks,
                           double thr, unsigned char* flags /*nblocks*nshell*/, int* nfn /*nblocks*/);
xcgpu_status launch_block_values(Ctx* c, const DevBasis& B, const DevPlan& P, int block, int deriv, double* out,
                                 int ld /*npts per function*/);
xcgpu_status fp64_eval_chunk(Ctx* c, const DevBasis& B, const DevPlan& P, int b0, int b1, const long* slab_off,
                             double* scratch, int deriv);
xcgpu_status fp64_density_chunk(Ctx* c, const DevPlan& P, int b0, int b1, const long* slab_off, const double* scratch,
                                int nspin, const double* Pm, double* rho, double* grad);
xcgpu_status launch_functional_range(Ctx* c, int func, int nspin, long n, int skip_block, long p0, long p1,
                                     const double* rho, const double* grad, double* epuv, double* dfdrho,
                                     double* dfdgrad, const double* w, double* partials, unsigned char* skipbuf,
                                     bool pair = false);
xcgpu_status launch_block_skip_flags_range(Ctx* c, const DevPlan& P, int nspin, const double* v, const double* g,
                                           double thr, unsigned char* skip, int b0, int b1);
xcgpu_status launch_functional(Ctx* c, int func, int nspin, long n, int skip_block, const double* rho,
                               const double* grad, double* epuv, double* dfdrho, double* dfdgrad, const double* w,
                               double* partials /*2*nparts or null*/, int* nparts,
                               unsigned char* skipbuf /*(n+skip_block-1)/skip_block, or null: context buffer*/,
                               bool pair = false /*restricted PBE in FP32 pairs, as the mixed build*/);
xcgpu_status launch_block_skip_flags(Ctx* c, const DevPlan& P, int nspin, const double* v, const double* g,
                                     double thr, unsigned char* skip /*nspin*nblocks*/);
// forms G over the chunk's gradient planes, then adds every tile pair of [w0, w1)
xcgpu_status fp64_adder_chunk(Ctx* c, const DevPlan& P, const int* work, long w0, long w1, int chunk_b0,
                              int chunk_b1, const long* slab_off, double* scratch, int nspin, const double* v,
                              const double* g, const unsigned char* skip, double* F);
xcgpu_status launch_axpy(Ctx* c, long n, const double* x, double* y);  // y += x
xcgpu_status fp64_xc_gradient_chunk(Ctx* c, const DevBasis& B, const DevPlan& P, int b0, int b1, const long* slab_off,
                                    double* scratch, bool gga, int nspin, const double* Pm, const double* v,
                                    const double* g, const int* fatom, int natoms, double* G);
xcgpu_status launch_lr_kernel(Ctx* c, int func, long n, const double* rho0, const double* grad0, const double* rho1,
                              const double* grad1, double* v1, double* g1);
xcgpu_status launch_lr_kernel_spin(Ctx* c, int func, int kind, long n, const double* rho0, const double* grad0,
                                   const double* rho1, const double* grad1, double* v1, double* g1);
xcgpu_status launch_symmetrise_half(Ctx* c, const double* D, double* S, int n);
xcgpu_status launch_scale_add(Ctx* c, long n, double a, const double* x, double* y);  // y += a x
xcgpu_status launch_sum_partials(Ctx* c, const double* partials, int nparts, int ncomp, double* out /*device*/);
// mixed precision (tcgen05 over fixed-point FP16 slices): one persistent launch over the
// blocks of every build in `work`; the density writes rho / grad rho (FP64), the adder
// accumulates F_b on and above the diagonal of V and mirrors it, a whole build does both
// with the functional in between.
struct MixedWork {
  const DevBasis* B;
  const DevPlan* P;
  int nspin;
  float* Psplit;  // psplit_bytes(nspin, nbf): the density matrices' fixed-point slices and column scales
  double* rho;
  double* grad;
  const double* v;
  const double* g;
  const unsigned char* skip;
  double* V;
  int func = 0;               // whole builds: functional,
  double thr = 0.0;           // adder block-skip threshold,
  double* partials = nullptr;  // per-block E_xc, N_el sums [2][nblocks],
  const double* Pm = nullptr;  // the FP64 density matrices (split into Psplit by the build)
  double* exc_nel = nullptr;   // and where E_xc, N_el go
};
xcgpu_status mixed_init(Ctx* c);
// bytes of the density kernel's form of nspin density matrices: 8 bytes of FP16
// slices per element, then one FP32 scale per column
inline size_t psplit_bytes(int nspin, int nbf) { return (size_t)nspin * nbf * nbf * 8 + (size_t)nspin * nbf * 4; }
xcgpu_status mixed_split(Ctx* c, const double* Pm, int nspin, int nbf, float* Psplit);
// whole builds (density, functional, Vxc per block) of the MixedWork items with func,
// thr, partials, Pm and exc_nel set (plans of 128-point blocks): one launch splits every
// item's P and zeroes its V, the persistent build kernel runs over all blocks, one launch
// mirrors every V and one sums every item's partials into its E_xc and N_el
xcgpu_status mixed_build_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err);
xcgpu_status mixed_density_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err);
xcgpu_status mixed_adder_batch(Ctx* c, const std::vector<MixedWork>& work, int* counter, int* err);

}  // namespace xcgpu
