/* ORACLE -- test infrastructure only (see oracle.h).  Internal declarations. */
#ifndef SERENITY_XC_ORACLE_INTERNAL_H
#define SERENITY_XC_ORACLE_INTERNAL_H
#include <vector>

#include "oracle.h"

namespace orc {

struct Shell {
  int l = 0;
  bool pure = false;
  double O[3] = {0, 0, 0};
  std::vector<double> alpha, coef;  // coef: normalised
  int nfunc = 0, first = 0;
  std::vector<int> ax, ay, az;
  std::vector<double> cartnorm;
  std::vector<double> sph;  // (2l+1) x ncart(l)
};

struct Basis {
  std::vector<Shell> shells;
  int nbf = 0;
  Basis(int nshell, const int* l, const int* pure, const int* nprim, const double* centers, const double* alpha,
        const double* coef);
};

int ncart(int l);
void block_on_grid(const Basis& B, const double* xyz, int npts, double thr, int deriv, double* val, double* grad,
                   double* hess, int* negligible);
int block_active(const Basis& B, const double* xyz, int npts, double thr, int deriv, int* act, double* val,
                 double* grad);

/* per-point functional evaluation (GRADIENTS data, order 1).
 * restricted: in = {n, gx, gy, gz}; out = {e, dF/dn, dF/dgx, dF/dgy, dF/dgz}
 * unrestricted: in = {na, nb, gax, gay, gaz, gbx, gby, gbz};
 *               out = {e, dF/dna, dF/dnb, dF/dga(3), dF/dgb(3)} */
void functional_point(int func, int nspin, const double* in, double* out);
bool functional_is_gga(int func);
/* restricted linear-response kernel contracted with (rho1, grad rho1): v1, g1[3] */
void lr_kernel_point(int func, double n0, const double* g0, double n1, const double* g1, double* v1, double* gg1);
void lr_kernel_spin_point(int func, const double* n0, const double* g0, const double* n1, const double* g1,
                          double* v1, double* gg1);

}  // namespace orc
#endif
