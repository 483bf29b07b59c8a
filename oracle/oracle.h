/*
 * ORACLE -- test infrastructure only.
 *
 * CPU (FP64, OpenMP) restatement of the reference's exchange-correlation grid
 * path (Serenity 1.6.2).  It exists to check the GPU product against, and to be
 * timed as the CPU baseline.  Nothing in the product links, loads or calls it;
 * only tests/, the smoke check and bench.py's CPU-baseline leg do.
 *
 * Parity status: pinned against the reference's own golden vectors (basis
 * values/gradients/Hessians, rho/grad rho, adder matrix, H2 LDA Fock matrices)
 * in tests/golden/.  PBE, B88 and LYP have no absolute golden value at this
 * boundary in the reference (its libxc test only compares two libraries):
 * for those functionals parity is unpinned and rests on literature formulas,
 * limiting cases and finite-difference checks.
 *
 * Conventions (all follow the reference):
 *   points  : xyz interleaved (x0,y0,z0,x1,...), bohr
 *   matrices: n_bf x n_bf, column-major (symmetric inputs)
 *   blocks  : consecutive runs of max_block_size points
 *     (BasisFunctionOnGridController.cpp:75-148)
 */
#ifndef SERENITY_XC_ORACLE_H
#define SERENITY_XC_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* functional identifiers (shared numbering with the product's C ABI) */
enum {
  ORC_FUNC_LDA = 1,  /* Slater + VWN5          (CompositeFunctionals.cpp:233-235) */
  ORC_FUNC_PBE = 2,  /* PBE x + PBE c          (CompositeFunctionals.cpp:242-244) */
  ORC_FUNC_BLYP = 3, /* B88 + LYP              (CompositeFunctionals.cpp:239-241) */
  ORC_FUNC_BP86 = 4, /* B88 + P86              (CompositeFunctionals.cpp:244-246) */
  ORC_FUNC_SLATER = 16,
  ORC_FUNC_VWN5 = 17,
  ORC_FUNC_PBEX = 18,
  ORC_FUNC_PBEC = 19,
  ORC_FUNC_B88 = 20,
  ORC_FUNC_LYP = 21,
  ORC_FUNC_PW92 = 22,
  ORC_FUNC_P86 = 23, /* PZ81 + the P86 gradient correction (xcfun "p86c") */
  ORC_FUNC_PZ81 = 24
};

/* Basis: shells with raw (file) contraction coefficients; the oracle applies the
 * libint2 normalisation convention itself (Shell.cpp:30-47). */
void* orc_basis_create(int nshell, const int* l, const int* pure, const int* nprim, const double* centers,
                       const double* alpha, const double* coef);
void orc_basis_free(void* basis);
int orc_basis_nbf(const void* basis);
/* normalised primitive coefficients of shell s into out (nprim values) */
void orc_basis_shell_coefs(const void* basis, int s, double* out);

/* One block of points: values/gradients/Hessians (deriv 0,1,2) for all functions,
 * column-major npts x nbf each; negligible[nbf] (1 = skipped for this block). */
int orc_block_on_grid(const void* basis, const double* xyz, int npts, double radial_threshold, int deriv,
                      double* values, double* grad /*3*npts*nbf or NULL*/, double* hess /*6*npts*nbf or NULL*/,
                      int* negligible);

/* rho (and grad rho) of nspin density matrices, block-wise with screening. */
int orc_density(const void* basis, const double* xyz, long npts, int max_block, double radial_threshold, int nspin,
                const double* P, double* rho /*nspin*npts*/, double* grad /*nspin*3*npts or NULL*/);

/* Functional evaluation at points (GRADIENTS data type, order 1).
 * rho: nspin*npts, grad: nspin*3*npts (GGA), outputs epuv[npts], dfdrho[nspin*npts],
 * dfdgrad[nspin*3*npts] (GGA).  Blocks with sum|rho| < n*1e-12 are skipped as in
 * XCFun.cpp:136-140 when max_block > 0. */
int orc_functional(int func, int nspin, long npts, int max_block, const double* rho, const double* grad,
                   double* epuv, double* dfdrho, double* dfdgrad);
/* is the functional a GGA (needs gradients)? */
int orc_functional_is_gga(int func);
/* sum over blocks of the non-negligible function count (the screening of the block data) */
long orc_active_functions(const void* basis, const double* xyz, long npts, int max_block, double thr);

/* F += sum_p w v phi phi (+ GGA term), ScalarOperatorToMatrixAdder.cpp:178-303. */
int orc_add_scalar(const void* basis, const double* xyz, const double* w, long npts, int max_block,
                   double radial_threshold, double block_ave_threshold, int nspin, const double* v,
                   const double* g /*nspin*3*npts or NULL*/, double* F /*nspin*nbf*nbf, added into*/);

/* Whole XC build (FuncPotential.cpp:74-110 with FunctionalLibrary(128)).
 * V (nspin*nbf*nbf) is overwritten; Exc = sum w*epuv; Nel = sum w*rho_total.
 * threads <= 0 uses every core. */
int orc_vxc(const void* basis, const double* xyz, const double* w, long npts, int max_block, double radial_threshold,
            double block_ave_threshold, int func, int nspin, const double* P, double* V, double* Exc, double* Nel,
            int threads);

/* Atom-centred Becke grid (GridFactory.cpp:52-320, AtomGridFactory.cpp:78-290).
 * Z[natoms], xyz[3*natoms] (bohr).  If accuracy > 0 the reference's pruned
 * accuracy scheme is used, else n_rad x n_ang (unpruned).  lebedev_path points to
 * the node table.  Returns the number of points written (<= capacity), or -1. */
long orc_becke_grid(int natoms, const int* Z, const double* xyz, int n_rad, int n_ang, int accuracy,
                    double weight_threshold, int smoothing, int sort, const char* lebedev_path, double* out_xyz,
                    double* out_w, long capacity, int partition /* 0 Becke, 1 SSF */);

/* Ahlrichs M3 radial rule (AtomGridFactory.cpp:238-260). */
void orc_ahlrichs_radial(double alpha, int n, double* r, double* w);
/* Real solid harmonic values at a point, m = -l..l (the reference's order). */
void orc_solid_harmonics(int l, double x, double y, double z, double* out);

/* XC part of the nuclear gradient (FuncPotential<M>::getGeomGradients,
 * FuncPotential.cpp:113-241): shell_atom[s] = atom index of shell s; P column-major per
 * spin (restricted: total); out natoms x 3 column-major.  No grid-weight derivatives. */
int orc_xc_gradient(const void* basis, const int* shell_atom, int natoms, const double* xyz, const double* w,
                    long npts, int max_block, double thr, int func, int nspin, const double* P, double* out);

/* Restricted (singlet) linear-response XC kernel contracted with a perturbed density:
 * v1 = F_nn rho1 + F_n,sigma sigma1, g1 = 2 (F_sigma,n rho1 + F_sigma,sigma sigma1) grad n +
 * 2 F_sigma grad rho1 (sigma1 = 2 grad n . grad rho1), second derivatives by second-order
 * forward-mode differentiation of the energy expressions; block skip of 128 points on
 * rho0 as the functional data.  grad arrays [3][npts] (GGA). */
int orc_lr_kernel(int func, long npts, const double* rho0, const double* grad0, const double* rho1,
                  const double* grad1, double* v1, double* g1);
/* The spin-resolved contraction: kind 2 unrestricted (per-spin inputs and outputs), kind 1
 * triplet (restricted ground state, perturbation (+rho1, -rho1), alpha outputs). */
int orc_lr_kernel_spin(int func, int kind, long npts, const double* rho0, const double* grad0, const double* rho1,
                       const double* grad1, double* v1, double* g1);

#ifdef __cplusplus
}
#endif
#endif
