/*
 * xcgpu -- GB300 (sm_103a) exchange-correlation numerical integration.
 *
 * C ABI of the drop-in for Serenity's XC grid path.  Every entry point takes
 * plain pointers and sizes; handles are opaque; errors are status codes with a
 * message from xcgpu_last_error() (the C++ facade in serenity_xc.hpp turns them
 * back into exceptions, as the reference throws SerenityError).  One context
 * drives one GPU; a context is not thread-safe (one context per host thread).
 *
 * Conventions (the reference's):
 *   points      xyz interleaved (x0,y0,z0,x1,...), bohr; weights alongside
 *   matrices    n_bf x n_bf FP64, column-major (Eigen default); spin-resolved
 *               inputs/outputs are nspin consecutive matrices (alpha, beta)
 *   grid data   nspin consecutive vectors of length n; gradients as x, y, z
 *               vectors of length n per spin
 *   blocks      consecutive runs of max_block points, the last one ragged
 *   mem         XCGPU_MEM_HOST: arguments are host pointers (copied inside);
 *               XCGPU_MEM_DEVICE: arguments are device pointers on the
 *               context's GPU (no copies)
 */
#ifndef XCGPU_H
#define XCGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  XCGPU_OK = 0,
  XCGPU_ERR_INVALID = 1,     /* bad argument: sizes, mismatched grid/basis, unknown functional */
  XCGPU_ERR_CUDA = 2,        /* a CUDA call failed; message holds cudaGetErrorString */
  XCGPU_ERR_NO_MEMORY = 3,   /* device allocation failed */
  XCGPU_ERR_BUDGET = 4,      /* request exceeds the context's HBM budget */
  XCGPU_ERR_UNSUPPORTED = 5, /* e.g. angular momentum > 6, derivative order > 2 */
  XCGPU_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  XCGPU_ERR_IO = 7           /* a data file could not be read */
} xcgpu_status;

enum { XCGPU_MEM_HOST = 0, XCGPU_MEM_DEVICE = 1 };

/* precision of a whole build */
enum {
  XCGPU_PREC_FP64 = 0, /* every stage in FP64: the drop-in */
  XCGPU_PREC_MIXED = 1 /* FP32 basis values with FP32-pair corrections, tensor-core
                          contractions over fixed-point FP16 slices whose leading products
                          sum exactly; FP64 functional, grid sums and cross-block Vxc */
};

/* functionals (CompositeFunctionals.cpp:233-246; basic_functionals.dat) */
enum {
  XCGPU_FUNC_LDA = 1,  /* Slater + VWN5 */
  XCGPU_FUNC_PBE = 2,  /* PBE exchange + PBE correlation */
  XCGPU_FUNC_BLYP = 3, /* Becke 88 + LYP */
  XCGPU_FUNC_BP86 = 4, /* Becke 88 + P86 (PZ81 + Perdew 86 gradient correction) */
  XCGPU_FUNC_SLATER = 16,
  XCGPU_FUNC_VWN5 = 17,
  XCGPU_FUNC_PBEX = 18,
  XCGPU_FUNC_PBEC = 19,
  XCGPU_FUNC_B88 = 20,
  XCGPU_FUNC_LYP = 21,
  XCGPU_FUNC_PW92 = 22,
  XCGPU_FUNC_P86 = 23, /* PZ81 + the Perdew 86 gradient correction (C_P86) */
  XCGPU_FUNC_PZ81 = 24 /* Perdew-Zunger 1981 local correlation */
};

typedef struct xcgpu_ctx xcgpu_ctx;
typedef struct xcgpu_grid xcgpu_grid;
typedef struct xcgpu_basis xcgpu_basis;
typedef struct xcgpu_plan xcgpu_plan;

typedef struct {
  int device;              /* CUDA device ordinal */
  uint64_t hbm_budget;     /* bytes this context may hold; 0 = 90% of free memory at creation */
  uint64_t scratch_bytes;  /* cap on per-build scratch; 0 = automatic */
} xcgpu_config;

/* ---- context ------------------------------------------------------------------------- */
xcgpu_status xcgpu_ctx_create(const xcgpu_config* cfg, xcgpu_ctx** out);
void xcgpu_ctx_destroy(xcgpu_ctx* ctx);
const char* xcgpu_last_error(const xcgpu_ctx* ctx);
/* stream the context launches on (a cudaStream_t); NULL = the context's own stream */
xcgpu_status xcgpu_set_stream(xcgpu_ctx* ctx, void* stream);
xcgpu_status xcgpu_synchronize(xcgpu_ctx* ctx);
/* bytes currently held on the device by this context */
uint64_t xcgpu_bytes_in_use(const xcgpu_ctx* ctx);
/* number of this library's kernels launched by the context so far */
uint64_t xcgpu_kernel_launches(const xcgpu_ctx* ctx);

/* Per-kernel device timing: when enabled, every kernel launch of the context is
 * bracketed by CUDA events on the context's stream; xcgpu_get_timing() synchronises
 * and returns the summed milliseconds and launch counts per kernel class
 * (XCGPU_KERNEL_* below), then resets them. */
enum {
  XCGPU_KERNEL_EVAL = 0,       /* basis functions on the grid (FP64 path) */
  XCGPU_KERNEL_DENSITY = 1,    /* rho / grad rho */
  XCGPU_KERNEL_FUNCTIONAL = 2, /* functional + grid sums */
  XCGPU_KERNEL_ADDER = 3,      /* Vxc accumulation */
  XCGPU_KERNEL_OTHER = 4,      /* screening, skip flags, reductions, symmetrisation */
  XCGPU_KERNEL_BUILD = 5,      /* whole mixed-precision builds in one kernel (density,
                                  functional and Vxc per grid block) */
  XCGPU_KERNEL_CLASSES = 6
};
xcgpu_status xcgpu_set_timing(xcgpu_ctx* ctx, int enable);
xcgpu_status xcgpu_get_timing(xcgpu_ctx* ctx, double* ms, uint64_t* launches);

/* ---- grid: replaces GridController/AtomCenteredGridController ------------------------ */
/* Wrap an existing grid (GridController::getGridPoints()/getWeights(),
 * src/grid/GridController.h:58-69). */
xcgpu_status xcgpu_grid_create(xcgpu_ctx* ctx, const double* xyz, const double* w, uint64_t npoints, xcgpu_grid** out);
/* Build an atom-centred Becke grid (GridFactory::produce, GridFactory.cpp:52-320, with
 * AtomGridFactory's Ahlrichs radial rule, AtomGridFactory.cpp:78-290): Becke partition
 * weights on the GPU, Hilbert ordering (HilbertRTreeSorting.cpp:46-216) when sort != 0.
 * accuracy in 1..7 selects the reference's pruned scheme; accuracy 0 uses n_rad x n_ang
 * unpruned.  lebedev_table: path of serenity_gb300/data/lebedev.txt. */
xcgpu_status xcgpu_grid_build(xcgpu_ctx* ctx, int natoms, const int* Z, const double* xyz_bohr, int n_rad, int n_ang,
                              int accuracy, double weight_threshold, int smoothing, int sort,
                              const char* lebedev_table, xcgpu_grid** out);
/* Atom partition of the grid weights (Options::GRID_TYPES, GridFactory.cpp:176-268). */
enum {
  XCGPU_PARTITION_BECKE = 0, /* Becke cells with size adjustment and `smoothing` iterations */
  XCGPU_PARTITION_SSF = 1    /* Stratmann-Scuseria-Frisch (a = 0.64, no size adjustment, smoothing unused) */
};
/* xcgpu_grid_build with the partition chosen (the reference's GRIDTYPE setting). */
xcgpu_status xcgpu_grid_build_partition(xcgpu_ctx* ctx, int natoms, const int* Z, const double* xyz_bohr, int n_rad,
                                        int n_ang, int accuracy, double weight_threshold, int partition, int smoothing,
                                        int sort, const char* lebedev_table, xcgpu_grid** out);
uint64_t xcgpu_grid_npoints(const xcgpu_grid* grid);
xcgpu_status xcgpu_grid_copy(const xcgpu_grid* grid, double* xyz, double* w); /* to host */
void xcgpu_grid_destroy(xcgpu_grid* grid);

/* ---- basis: replaces BasisController (src/basis/BasisController.h:157-175) ----------- */
typedef struct {
  int32_t l;      /* angular momentum, 0..6 */
  int32_t pure;   /* 1 = real solid harmonics (m = -l..l), 0 = Cartesian (x^l ... z^l) */
  int32_t nprim;
  double center[3];
  const double* alpha; /* nprim exponents */
  const double* coef;  /* nprim raw contraction coefficients (normalised inside, Shell.cpp:30-47) */
} xcgpu_shell;
xcgpu_status xcgpu_basis_create(xcgpu_ctx* ctx, const xcgpu_shell* shells, uint32_t nshell, xcgpu_basis** out);
uint32_t xcgpu_basis_nbf(const xcgpu_basis* basis);
/* normalised coefficients of shell s (nprim values) */
xcgpu_status xcgpu_basis_coefs(const xcgpu_basis* basis, uint32_t s, double* out);
void xcgpu_basis_destroy(xcgpu_basis* basis);

/* ---- plan: replaces BasisFunctionOnGridController -------------------------------------
 * (BasisFunctionOnGridController.h:105-287; ctor .cpp:75-101).  Partitions the grid into
 * blocks of max_block (<= 128) points and screens every shell against every block
 * (.cpp:192-255), storing the compacted active-function list per block. */
xcgpu_status xcgpu_plan_create(xcgpu_ctx* ctx, xcgpu_grid* grid, xcgpu_basis* basis, uint32_t max_block,
                               double radial_threshold, xcgpu_plan** out);
typedef struct {
  uint32_t nblocks, max_block, nbf, max_active;
  uint64_t npoints;
  uint64_t sum_active;      /* sum over blocks of the active-function count */
  double flops_per_spin;    /* sum over blocks of 4 * npts_b * n_b^2 */
} xcgpu_plan_stats;
xcgpu_status xcgpu_plan_get_stats(const xcgpu_plan* plan, xcgpu_plan_stats* out);
/* getBlockOnGridData(b) (.cpp:122-131): dense npts_b x nbf column-major values, 3 such
 * gradient matrices (x,y,z) when deriv >= 1, 6 Hessian matrices (xx,xy,xz,yy,yz,zz) when
 * deriv == 2, and negligible[nbf]; host outputs.  deriv > 2 -> XCGPU_ERR_UNSUPPORTED. */
xcgpu_status xcgpu_block_on_grid(xcgpu_plan* plan, uint32_t block, int deriv, double* values, double* grad,
                                 double* hess, int32_t* negligible);
/* active-function list of a block (ascending function indices), returns the count */
int32_t xcgpu_block_active(const xcgpu_plan* plan, uint32_t block, int32_t* idx);
void xcgpu_plan_destroy(xcgpu_plan* plan);

/* ---- stages ----------------------------------------------------------------------------
 * DensityOnGridCalculator::calcDensityAndGradientOnGrid (DensityOnGridCalculator.h:53-128,
 * MatrixOperatorToGridTransformer.cpp:37-198): rho = rowsum((phi P_b) o phi),
 * grad rho = 2 rowsum((phi P_b) o grad phi).  grad may be NULL (density only).
 * precision: XCGPU_PREC_FP64 (the drop-in) or XCGPU_PREC_MIXED (tensor cores). */
xcgpu_status xcgpu_density(xcgpu_plan* plan, int nspin, const double* P, double* rho, double* grad, int precision,
                           int mem);
/* FP64 rho and grad rho without any device allocation.  No counterpart in the reference:
 * it serves hosts that cannot call cudaMalloc when they need the density (a program that
 * owns all device memory through its own fixed pool, or a loop whose memory was reserved
 * up front).  Same kernels and results as xcgpu_density at XCGPU_PREC_FP64; the per-block
 * scratch lives in a fixed 64 MiB static device array that every GPU loading the library
 * holds until exit, so a block needing more (more than ~16 000 active functions) is
 * rejected with XCGPU_ERR_BUDGET.  P, rho, grad (may be NULL) are device pointers; the call
 * synchronises the context stream.  Every call looks up the array's device address
 * (cudaGetSymbolAddress, which allocates nothing), so a reset device or another context gets
 * the right address; make the first call on a device before any stream capture (it may load
 * the module).  All calls share the array, so calls that overlap on the GPU race. */
xcgpu_status xcgpu_density_fp64_noalloc(xcgpu_plan* plan, int nspin, const double* P, double* rho, double* grad);
/* FunctionalLibrary::calcData(GRADIENTS, f, ., order 1) (FunctionalLibrary.cpp:40-71,
 * XCFun.cpp:39-158): epuv (energy per volume), dF/drho and, for GGAs, dF/d(grad rho).
 * skip_block > 0 applies the reference's block skip (sum |rho| < n * 1e-12 on blocks of
 * skip_block points, XCFun.cpp:136-140). */
xcgpu_status xcgpu_functional(xcgpu_ctx* ctx, int func, int nspin, uint64_t npoints, uint32_t skip_block,
                              const double* rho, const double* grad, double* epuv, double* dfdrho, double* dfdgrad,
                              int mem);
/* The same with the functional arithmetic of a precision: XCGPU_PREC_FP64 as above,
 * XCGPU_PREC_MIXED as the mixed build evaluates it (restricted PBE in FP32 pairs, ~1e-13
 * relative to FP64; every other functional and spin case in FP64). */
xcgpu_status xcgpu_functional_prec(xcgpu_ctx* ctx, int func, int nspin, uint64_t npoints, uint32_t skip_block,
                                   const double* rho, const double* grad, double* epuv, double* dfdrho,
                                   double* dfdgrad, int precision, int mem);
int xcgpu_functional_is_gga(int func);
/* ScalarOperatorToMatrixAdder::addScalarOperatorToMatrix (ScalarOperatorToMatrixAdder.h:56-93,
 * .cpp:51-113,178-303): F += sum_p w (v phi phi^T) (+ the GGA term with g = dF/d grad rho
 * when g != NULL).  Adds into F; blocks below block_ave_threshold are skipped. */
xcgpu_status xcgpu_add_scalar(xcgpu_plan* plan, double block_ave_threshold, int nspin, const double* v,
                              const double* g, double* F, int precision, int mem);

/* ---- whole build: FuncPotential::getMatrix + getEnergy (FuncPotential.cpp:74-110) -----
 * V (nspin matrices) is overwritten with the XC potential matrix; Exc = sum_p w_p epuv_p;
 * Nel = sum_p w_p rho_p (total density).  P, V in `mem` space; Exc, Nel host scalars. */
xcgpu_status xcgpu_vxc(xcgpu_plan* plan, int func, int nspin, int precision, double block_ave_threshold,
                       const double* P, double* V, double* Exc, double* Nel, int mem);

/* ---- linear-response XC kernel (TDDFT / TDA sigma vectors) --------------------------
 * KernelSigmavector<RESTRICTED>::calcF (KernelSigmavector.cpp:128-392), singlet: for each
 * trial matrix D[t] (column-major n_bf x n_bf), the density of (D + D^T)/2 and its
 * gradient are contracted with the second functional derivatives at the ground-state
 * density of P0 (total), v1 = F_nn rho1 + F_n,sigma sigma1, g1 = 2 (F_sigma,n rho1 +
 * F_sigma,sigma sigma1) grad n + 2 F_sigma grad rho1, and integrated like a potential:
 * F[t] = phi^T w (v1/2 phi + g1 . grad phi) + transpose, overwritten.  The reference's
 * per-element screening of D and of the integration (at 1e-11) is replaced by the
 * adder's block skip.  All matrices in `mem` space. */
xcgpu_status xcgpu_lr_kernel(xcgpu_plan* plan, int func, const double* P0, uint32_t ntrial, const double* const* D,
                             double* const* F, int precision, double block_ave_threshold, int mem);
/* The kinds of xcgpu_lr_kernel_spin */
enum { XCGPU_LR_SINGLET = 0, XCGPU_LR_TRIPLET = 1, XCGPU_LR_UNRESTRICTED = 2 };
/* KernelSigmavector<M>::calcF with the spin kernels (KernelSigmavector.cpp:127-253 with
 * contractBlock :363-499): XCGPU_LR_SINGLET is xcgpu_lr_kernel; XCGPU_LR_TRIPLET contracts
 * (f_aa - f_ab) of the restricted ground state P0 (total density, nbf x nbf) with each
 * symmetrised trial matrix D[t] (nbf x nbf) into F[t] (nbf x nbf); XCGPU_LR_UNRESTRICTED
 * takes P0 = (P_alpha, P_beta), D[t] = (D_alpha, D_beta) and returns F[t] = (F_alpha,
 * F_beta), each 2 x nbf x nbf, the spin blocks consecutive.  Each F is the directional
 * derivative of the XC matrix: F_s(D) = d/de Vxc_s[P_a + e D_a, P_b + e D_b] with the
 * triplet's perturbation (+D, -D) about (P0/2, P0/2).  F is overwritten. */
xcgpu_status xcgpu_lr_kernel_spin(xcgpu_plan* plan, int func, int kind, const double* P0, uint32_t ntrial,
                                  const double* const* D, double* const* F, int precision,
                                  double block_ave_threshold, int mem);

/* ---- XC part of the nuclear gradient ------------------------------------------------
 * FuncPotential<M>::getGeomGradients (FuncPotential.cpp:113-241): for every pair of active
 * functions of a block, the atom of nu collects -2 P_mu,nu sum_p w [v phi_mu d_k phi_nu +
 * sum_j g_j (phi_mu d_j d_k phi_nu + d_j phi_mu d_k phi_nu)] (second basis derivatives for
 * GGA), summed over spins; no grid-weight derivatives, as in the reference.  FP64.
 * shell_atom[s] = atom index of shell s (BasisController::getAtomIndicesOfBasis); G is
 * natoms x 3 column-major (the reference's Eigen::MatrixXd), overwritten; P and G in
 * `mem` space. */
xcgpu_status xcgpu_xc_gradient(xcgpu_plan* plan, int func, int nspin, const double* P, const int* shell_atom,
                               int natoms, double* G, int mem);

/* ---- non-additive XC potential of subsystem DFT (frozen-density embedding) -----------
 * NAddFuncPotential<M>::getMatrix / getEnergy (NAddFuncPotential.cpp:189-243, 297-318) with
 * the supersystem density of SupersystemDensityOnGridController.cpp:101-187: every
 * subsystem's density is formed from its own basis and density matrix on the active
 * system's grid (all plans share one grid; one batched launch in mixed precision), then
 *   rho_tot = rho_active + sum_i rho_env_i,
 *   V       = adder_active(dF/drho[rho_tot] - dF/drho[rho_active], same for dF/d grad rho),
 *   E_nadd  = E_xc[rho_tot] - E_xc[rho_active] - sum_i E_xc[rho_env_i].
 * P_active: nspin column-major matrices of the active basis; P_env[i] those of env[i]'s
 * basis; V (nspin, active basis) is overwritten; all in `mem` space; E_nadd a host scalar.
 * The exact-exchange part of hybrid functionals (integrals) is not part of this path. */
xcgpu_status xcgpu_nadd_vxc(xcgpu_plan* active, xcgpu_plan* const* env, uint32_t n_env, int func, int nspin,
                            int precision, double block_ave_threshold, const double* P_active,
                            const double* const* P_env, double* V, double* E_nadd, int mem);

/* Every subsystem's non-additive potential at once (a Jacobi freeze-and-thaw cycle, or
 * the final energy evaluation of FreezeAndThawTask.cpp:151-411): with one set of
 * subsystem densities on the supersystem grid, V[i] = adder_i(dF[rho_tot] - dF[rho_i])
 * for every i, E_nadd = E_xc[rho_tot] - sum_i E_xc[rho_i] (the same for all i).  Equals
 * n_sub calls of xcgpu_nadd_vxc, each with the others as environment, with each density
 * formed once instead of n_sub times; the densities and the adders of all subsystems run
 * as one batched launch each in mixed precision.  P[i], V[i] as in xcgpu_nadd_vxc. */
xcgpu_status xcgpu_nadd_vxc_all(xcgpu_plan* const* plans, uint32_t n_sub, int func, int nspin, int precision,
                                double block_ave_threshold, const double* const* P, double* const* V, double* E_nadd,
                                int mem);

/* ---- batched builds (many subsystems, e.g. a freeze-and-thaw step) -------------------
 * All requests run as one persistent launch per heavy stage (mixed precision) on the
 * context stream, without host synchronisation unless XCGPU_BATCH_SYNC is set; P, V and
 * exc_nel are device pointers.  Results are valid once the stream has reached this
 * point (xcgpu_check_async synchronises and reports a device-side timeout).  The call
 * can be captured in a CUDA graph (xcgpu_graph_begin/end) once every request's plan has
 * run one build of the same spin count and functional class (work buffers are allocated
 * on first use). */
typedef struct {
  xcgpu_plan* plan;
  int func;
  int nspin;
  double block_ave_threshold;
  const double* P; /* device, nspin column-major n_bf x n_bf */
  double* V;       /* device, overwritten */
  double* exc_nel; /* device, 2 doubles: E_xc, N_el */
} xcgpu_request;
enum { XCGPU_BATCH_SYNC = 1 };
xcgpu_status xcgpu_vxc_batch(xcgpu_ctx* ctx, const xcgpu_request* reqs, uint32_t n, int precision, int flags);
xcgpu_status xcgpu_check_async(xcgpu_ctx* ctx);
/* CUDA graph capture of the work issued on the context stream between begin and end */
xcgpu_status xcgpu_graph_begin(xcgpu_ctx* ctx);
xcgpu_status xcgpu_graph_end(xcgpu_ctx* ctx, void** graph_exec);
xcgpu_status xcgpu_graph_launch(xcgpu_ctx* ctx, void* graph_exec);
void xcgpu_graph_destroy(void* graph_exec);

#ifdef __cplusplus
}
#endif
#endif /* XCGPU_H */
