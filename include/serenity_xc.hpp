/*
 * C++ facade of the GB300 XC integration with the class names, constructor
 * arguments and methods of Serenity's XC grid path, on top of the C ABI (xcgpu.h):
 *
 *   BasisFunctionOnGridController     src/data/grid/BasisFunctionOnGridController.h:44-308
 *   DensityOnGridCalculator<M>        src/data/grid/DensityOnGridCalculator.h:45-135
 *   DensityMatrixController<M>        src/data/matrices/DensityMatrixController.h (the density
 *                                     matrix and its notification of dependent objects)
 *   DensityOnGridController<M>        src/data/grid/DensityOnGridController.h:40-140
 *   DensityMatrixDensityOnGridController<M>  src/data/grid/DensityMatrixDensityOnGridController.h:37-136
 *   Functional, CompositeFunctionals  src/dft/Functional.h, src/dft/functionals/CompositeFunctionals.h
 *   FunctionalLibrary<M>              src/dft/functionals/FunctionalLibrary.h:51-64
 *   ScalarOperatorToMatrixAdder<M>    src/data/grid/ScalarOperatorToMatrixAdder.h:56-93
 *   FuncPotential<M> (getMatrix, getEnergy)  src/potentials/FuncPotential.h
 *   NAddFuncPotential<M> (getMatrix, getEnergy)  src/potentials/NAddFuncPotential.h
 *   FuncPotential<M>::getGeomGradients           src/potentials/FuncPotential.cpp:113-241
 *   KernelSigmavector<M>::calcF (singlet, triplet, unrestricted)  src/postHF/LRSCF/Sigmavectors/KernelSigmavector.h
 *
 * Errors are thrown as SerenityError, as in the reference.  Matrices and grid data are
 * plain column-major containers with the memory layout of Eigen's defaults
 * (Eigen::MatrixXd, Eigen::Matrix3Xd, Eigen::VectorXd), so a build with Eigen can map
 * them without copies.  Header-only; link with libxcgpu.so.
 */
#ifndef SERENITY_XC_HPP
#define SERENITY_XC_HPP

#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "xcgpu.h"

namespace Serenity {

class SerenityError : public std::runtime_error {
 public:
  explicit SerenityError(const std::string& what) : std::runtime_error(what) {}
};

namespace Options {
enum class SCF_MODES { RESTRICTED, UNRESTRICTED };
}

/* The reference's IO switches that this path reads (src/settings/IOOptions.h):
 * gridAccuracyCheck prints the electron count integrated over the grid whenever a
 * DensityMatrixDensityOnGridController forms a density. */
struct IOOptions {
  bool gridAccuracyCheck = false;
};
inline IOOptions iOOptions;

/* Notification (src/notification/ObjectSensitiveClass.h, NotifyingClass.h): an object
 * whose data depends on another registers with it and is told when that data changes.
 * _self is a non-owning handle to the object itself, expiring with it. */
class ObjectSensitiveClass {
 public:
  ObjectSensitiveClass() : _self(this, [](ObjectSensitiveClass*) {}) {}
  virtual ~ObjectSensitiveClass() = default;
  virtual void notify() = 0;

 protected:
  std::shared_ptr<ObjectSensitiveClass> _self;
};
class NotifyingClass {
 public:
  virtual ~NotifyingClass() = default;
  void addSensitiveObject(std::weak_ptr<ObjectSensitiveClass> object) { sensitive_.push_back(std::move(object)); }

 protected:
  void notifyObjects() {
    for (size_t i = 0; i < sensitive_.size();) {
      if (auto o = sensitive_[i].lock()) {
        o->notify();
        ++i;
      } else {
        sensitive_.erase(sensitive_.begin() + (long)i);
      }
    }
  }

 private:
  std::vector<std::weak_ptr<ObjectSensitiveClass>> sensitive_;
};

/* Eigen::SparseVector<int> as returned by getNonNegligibleBlocks: rows() entries, the
 * non-zero ones listed in increasing index order */
struct SparseVectorInt {
  long size = 0;
  std::vector<int> indices, values;
  long rows() const { return size; }
  long nonZeros() const { return (long)indices.size(); }
  int coeff(long i) const {
    for (size_t k = 0; k < indices.size(); ++k)
      if (indices[k] == i) return values[k];
    return 0;
  }
};
constexpr Options::SCF_MODES RESTRICTED = Options::SCF_MODES::RESTRICTED;
constexpr Options::SCF_MODES UNRESTRICTED = Options::SCF_MODES::UNRESTRICTED;

/* column-major dense matrix (Eigen::MatrixXd layout) */
class Matrix {
 public:
  Matrix(long rows = 0, long cols = 0) : r_(rows), c_(cols), d_((size_t)(rows * cols), 0.0) {}
  double& operator()(long i, long j) { return d_[(size_t)(i + j * r_)]; }
  double operator()(long i, long j) const { return d_[(size_t)(i + j * r_)]; }
  long rows() const { return r_; }
  long cols() const { return c_; }
  double* data() { return d_.data(); }
  const double* data() const { return d_.data(); }
  void setZero() { std::fill(d_.begin(), d_.end(), 0.0); }
  void resize(long rows, long cols) {
    r_ = rows;
    c_ = cols;
    d_.assign((size_t)(rows * cols), 0.0);
  }

 private:
  long r_, c_;
  std::vector<double> d_;
};
using Vector = std::vector<double>;

template <class T>
struct Gradient {
  T x, y, z;
};
template <class T>
struct Hessian {
  T xx, xy, xz, yy, yz, zz;
};
template <class T>
struct SpinPair {
  T alpha, beta;
};
template <Options::SCF_MODES M, class T>
struct Spin {
  using type = T;
};
template <class T>
struct Spin<Options::SCF_MODES::UNRESTRICTED, T> {
  using type = SpinPair<T>;
};
/* SPMatrix<M>, DensityOnGrid<M>, GridPotential<M> as in SpinPolarizedData.h */
template <Options::SCF_MODES M>
using SPMatrix = typename Spin<M, Matrix>::type;
template <Options::SCF_MODES M>
using DensityMatrix = SPMatrix<M>;
template <Options::SCF_MODES M>
using FockMatrix = SPMatrix<M>;
template <Options::SCF_MODES M>
using GridPotential = typename Spin<M, Vector>::type;
template <Options::SCF_MODES M>
using DensityOnGrid = typename Spin<M, Vector>::type;

namespace detail {
inline void check(xcgpu_ctx* ctx, xcgpu_status st) {
  if (st != XCGPU_OK) throw SerenityError(std::string("xcgpu: ") + xcgpu_last_error(ctx));
}
template <Options::SCF_MODES M>
constexpr int nspin() {
  return M == Options::SCF_MODES::RESTRICTED ? 1 : 2;
}
// spin-resolved containers <-> consecutive buffers
inline void pack(const Matrix& m, std::vector<double>& out) { out.assign(m.data(), m.data() + m.rows() * m.cols()); }
inline void pack(const SpinPair<Matrix>& m, std::vector<double>& out) {
  out.assign(m.alpha.data(), m.alpha.data() + m.alpha.rows() * m.alpha.cols());
  out.insert(out.end(), m.beta.data(), m.beta.data() + m.beta.rows() * m.beta.cols());
}
inline void pack(const Vector& v, std::vector<double>& out) { out = v; }
inline void pack(const SpinPair<Vector>& v, std::vector<double>& out) {
  out = v.alpha;
  out.insert(out.end(), v.beta.begin(), v.beta.end());
}
inline void unpack(const double* src, Matrix& m) { std::copy(src, src + m.rows() * m.cols(), m.data()); }
inline void unpack(const double* src, SpinPair<Matrix>& m) {
  const long n = m.alpha.rows() * m.alpha.cols();
  std::copy(src, src + n, m.alpha.data());
  std::copy(src + n, src + 2 * n, m.beta.data());
}
inline void unpack(const double* src, long n, Vector& v) { v.assign(src, src + n); }
inline void unpack(const double* src, long n, SpinPair<Vector>& v) {
  v.alpha.assign(src, src + n);
  v.beta.assign(src + n, src + 2 * n);
}
inline long nbf_of(const Matrix& m) { return m.rows(); }
inline long nbf_of(const SpinPair<Matrix>& m) { return m.alpha.rows(); }
}  // namespace detail

/* one GPU context shared by the controllers that use it */
class XcContext {
 public:
  explicit XcContext(int device = 0, uint64_t hbm_budget = 0) {
    xcgpu_config cfg{device, hbm_budget, 0};
    if (xcgpu_ctx_create(&cfg, &ctx_) != XCGPU_OK) throw SerenityError("xcgpu: no usable CUDA device");
  }
  ~XcContext() { xcgpu_ctx_destroy(ctx_); }
  XcContext(const XcContext&) = delete;
  XcContext& operator=(const XcContext&) = delete;
  xcgpu_ctx* get() const { return ctx_; }

 private:
  xcgpu_ctx* ctx_ = nullptr;
};

/* GridController: points (3 x N, column-major like Eigen::Matrix3Xd) and weights */
class GridController {
 public:
  GridController(std::shared_ptr<XcContext> ctx, const std::vector<double>& xyz, const std::vector<double>& w)
      : ctx_(ctx) {
    if (xyz.size() != 3 * w.size()) throw SerenityError("GridController: points and weights do not match");
    detail::check(ctx->get(), xcgpu_grid_create(ctx->get(), xyz.data(), w.data(), w.size(), &grid_));
    points_ = xyz;
    weights_ = w;
  }
  ~GridController() { xcgpu_grid_destroy(grid_); }
  unsigned int getNGridPoints() const { return (unsigned int)weights_.size(); }
  const std::vector<double>& getGridPoints() const { return points_; }
  const std::vector<double>& getWeights() const { return weights_; }
  xcgpu_grid* handle() const { return grid_; }
  std::shared_ptr<XcContext> context() const { return ctx_; }

 private:
  std::shared_ptr<XcContext> ctx_;
  xcgpu_grid* grid_ = nullptr;
  std::vector<double> points_, weights_;
};

/* BasisController: shells with raw contraction coefficients (normalised inside) */
struct ShellData {
  int l;
  bool spherical;
  double center[3];
  std::vector<double> exponents, contractions;
};
class BasisController {
 public:
  BasisController(std::shared_ptr<XcContext> ctx, const std::vector<ShellData>& shells) : ctx_(ctx) {
    std::vector<xcgpu_shell> s;
    for (const auto& sh : shells)
      s.push_back(xcgpu_shell{sh.l, sh.spherical ? 1 : 0, (int)sh.exponents.size(),
                              {sh.center[0], sh.center[1], sh.center[2]}, sh.exponents.data(),
                              sh.contractions.data()});
    detail::check(ctx->get(), xcgpu_basis_create(ctx->get(), s.data(), (uint32_t)s.size(), &basis_));
  }
  ~BasisController() { xcgpu_basis_destroy(basis_); }
  unsigned int getNBasisFunctions() const { return xcgpu_basis_nbf(basis_); }
  xcgpu_basis* handle() const { return basis_; }

 private:
  std::shared_ptr<XcContext> ctx_;
  xcgpu_basis* basis_ = nullptr;
};

class BasisFunctionOnGridController {
 public:
  struct BasisFunctionBlockOnGridData {
    std::vector<int> negligible;
    Matrix functionValues;  // blockSize x nBasisFunctions
    std::shared_ptr<Gradient<Matrix>> derivativeValues;
    std::shared_ptr<Hessian<Matrix>> secondDerivativeValues;
  };

  BasisFunctionOnGridController(std::shared_ptr<BasisController> basisController,
                                std::shared_ptr<GridController> gridController, unsigned int maxBlockSize,
                                double radialThreshold, unsigned int highestDerivative)
      : basis_(basisController), grid_(gridController), maxBlockSize_(maxBlockSize), highest_(highestDerivative) {
    if (highestDerivative > 2) throw SerenityError("Third derivatives of basis functions on the grid are not implemented!");
    ctx_ = gridController->context();
    detail::check(ctx_->get(), xcgpu_plan_create(ctx_->get(), gridController->handle(), basisController->handle(),
                                                 maxBlockSize, radialThreshold, &plan_));
  }
  ~BasisFunctionOnGridController() { xcgpu_plan_destroy(plan_); }
  unsigned int getNBlocks() const {
    xcgpu_plan_stats s;
    xcgpu_plan_get_stats(plan_, &s);
    return s.nblocks;
  }
  unsigned int getFirstIndexOfBlock(unsigned int blockIndex) const { return blockIndex * maxBlockSize_; }
  unsigned int getNGridPoints() const { return grid_->getNGridPoints(); }
  unsigned int getNBasisFunctions() const { return basis_->getNBasisFunctions(); }
  unsigned int getMaxBlockSize() const { return maxBlockSize_; }
  unsigned int getHighestDerivative() const { return highest_; }
  void setHighestDerivative(unsigned int d) {
    if (d > 2) throw SerenityError("Third derivatives of basis functions on the grid are not implemented!");
    highest_ = d;
  }
  std::shared_ptr<BasisFunctionBlockOnGridData> getBlockOnGridData(unsigned int blockIndex) {
    const unsigned int nbf = getNBasisFunctions();
    const unsigned int first = getFirstIndexOfBlock(blockIndex);
    const unsigned int n = std::min(maxBlockSize_, getNGridPoints() - first);
    auto out = std::make_shared<BasisFunctionBlockOnGridData>();
    out->functionValues.resize(n, nbf);
    out->negligible.assign(nbf, 0);
    std::vector<double> g(highest_ >= 1 ? 3 * (size_t)n * nbf : 0), h(highest_ >= 2 ? 6 * (size_t)n * nbf : 0);
    detail::check(ctx_->get(), xcgpu_block_on_grid(plan_, blockIndex, (int)highest_, out->functionValues.data(),
                                                   g.empty() ? nullptr : g.data(), h.empty() ? nullptr : h.data(),
                                                   out->negligible.data()));
    const size_t plane = (size_t)n * nbf;
    if (highest_ >= 1) {
      out->derivativeValues = std::make_shared<Gradient<Matrix>>();
      Matrix* comp[3] = {&out->derivativeValues->x, &out->derivativeValues->y, &out->derivativeValues->z};
      for (int k = 0; k < 3; ++k) {
        comp[k]->resize(n, nbf);
        std::copy(g.data() + k * plane, g.data() + (k + 1) * plane, comp[k]->data());
      }
    }
    if (highest_ >= 2) {
      out->secondDerivativeValues = std::make_shared<Hessian<Matrix>>();
      auto& H = *out->secondDerivativeValues;
      Matrix* comp[6] = {&H.xx, &H.xy, &H.xz, &H.yy, &H.yz, &H.zz};
      for (int k = 0; k < 6; ++k) {
        comp[k]->resize(n, nbf);
        std::copy(h.data() + k * plane, h.data() + (k + 1) * plane, comp[k]->data());
      }
    }
    return out;
  }
  std::shared_ptr<BasisController> getBasisController() const { return basis_; }
  std::shared_ptr<GridController> getGridController() const { return grid_; }
  xcgpu_plan* handle() const { return plan_; }
  xcgpu_ctx* ctx() const { return ctx_->get(); }

 private:
  std::shared_ptr<BasisController> basis_;
  std::shared_ptr<GridController> grid_;
  std::shared_ptr<XcContext> ctx_;
  unsigned int maxBlockSize_, highest_;
  xcgpu_plan* plan_ = nullptr;
};

template <Options::SCF_MODES M>
class DensityOnGridCalculator {
 public:
  DensityOnGridCalculator(std::shared_ptr<BasisFunctionOnGridController> bfog, double blockAverageThreshold,
                          int precision = XCGPU_PREC_FP64)
      : bfog_(bfog), thr_(blockAverageThreshold), precision_(precision) {}
  /* calcDensityOnGrid(P, densityOnGrid) (DensityOnGridCalculator.cpp:38-44) */
  void calcDensityOnGrid(const DensityMatrix<M>& P, DensityOnGrid<M>& rho) { run(P, rho, nullptr); }
  DensityOnGrid<M> calcDensityOnGrid(const DensityMatrix<M>& P) {
    DensityOnGrid<M> rho;
    run(P, rho, nullptr);
    return rho;
  }
  void calcDensityAndGradientOnGrid(const DensityMatrix<M>& P, DensityOnGrid<M>& rho,
                                    Gradient<DensityOnGrid<M>>& grad) {
    run(P, rho, &grad);
  }
  std::shared_ptr<BasisFunctionOnGridController> getBasisFunctionOnGridController() const { return bfog_; }
  std::shared_ptr<GridController> getGridController() const { return bfog_->getGridController(); }
  /* the blocks with at least one non-negligible basis function in the last transform
   * (MatrixOperatorToGridTransformer.cpp:102-124, DensityOnGridCalculator.h:126-128) */
  SparseVectorInt getNonNegligibleBlocks() { return nonNegligible_; }

 private:
  void run(const DensityMatrix<M>& P, DensityOnGrid<M>& rho, Gradient<DensityOnGrid<M>>* grad) {
    const int ns = detail::nspin<M>();
    if (detail::nbf_of(P) != (long)bfog_->getNBasisFunctions())
      throw SerenityError("MatrixOperatorToGridTransformer: Mismatch of data field sizes.");
    std::vector<double> Pv;
    detail::pack(P, Pv);
    const long n = bfog_->getNGridPoints();
    std::vector<double> r((size_t)ns * n), g(grad ? (size_t)ns * 3 * n : 0);
    detail::check(bfog_->ctx(), xcgpu_density(bfog_->handle(), ns, Pv.data(), r.data(), grad ? g.data() : nullptr,
                                              precision_, XCGPU_MEM_HOST));
    detail::unpack(r.data(), n, rho);
    if (grad) {
      // per spin x, y, z consecutive vectors
      std::vector<double> gx, gy, gz;
      for (int s = 0; s < ns; ++s) {
        gx.insert(gx.end(), g.begin() + (s * 3 + 0) * n, g.begin() + (s * 3 + 1) * n);
        gy.insert(gy.end(), g.begin() + (s * 3 + 1) * n, g.begin() + (s * 3 + 2) * n);
        gz.insert(gz.end(), g.begin() + (s * 3 + 2) * n, g.begin() + (s * 3 + 3) * n);
      }
      detail::unpack(gx.data(), n, grad->x);
      detail::unpack(gy.data(), n, grad->y);
      detail::unpack(gz.data(), n, grad->z);
    }
    const unsigned nb = bfog_->getNBlocks();
    nonNegligible_ = SparseVectorInt{};
    nonNegligible_.size = nb;
    for (unsigned b = 0; b < nb; ++b)
      if (xcgpu_block_active(bfog_->handle(), b, nullptr) > 0) {
        nonNegligible_.indices.push_back((int)b);
        nonNegligible_.values.push_back(1);
      }
  }
  std::shared_ptr<BasisFunctionOnGridController> bfog_;
  double thr_;
  int precision_;
  SparseVectorInt nonNegligible_;
};

/* DensityMatrixController<M>: holds the density matrix; setting a new one notifies the
 * objects built on it (a DensityMatrixDensityOnGridController, say) */
template <Options::SCF_MODES M>
class DensityMatrixController : public NotifyingClass {
 public:
  explicit DensityMatrixController(const DensityMatrix<M>& P) : P_(P) {}
  const DensityMatrix<M>& getDensityMatrix() const { return P_; }
  void setDensityMatrix(const DensityMatrix<M>& P) {
    P_ = P;
    this->notifyObjects();
  }

 private:
  DensityMatrix<M> P_;
};

/* DensityOnGridController<M> (DensityOnGridController.h:40-140): a density on a grid,
 * formed lazily, invalidated through notify() */
template <Options::SCF_MODES M>
class DensityOnGridController : public NotifyingClass, public ObjectSensitiveClass {
 public:
  DensityOnGridController(std::shared_ptr<GridController> grid, unsigned int highestDerivative)
      : _gridController(grid), _highestDerivative(highestDerivative), _nGridPoints(grid->getNGridPoints()) {}
  virtual const DensityOnGrid<M>& getDensityOnGrid() = 0;
  virtual const Gradient<DensityOnGrid<M>>& getDensityGradientOnGrid() = 0;
  virtual const Hessian<DensityOnGrid<M>>& getDensityHessianOnGrid() {
    throw SerenityError("Density Hessians on the grid are not part of this XC path.");
  }
  unsigned int getNGridPoints() const { return _nGridPoints; }
  unsigned int getHighestDerivative() const { return _highestDerivative; }
  virtual void setHighestDerivative(unsigned int newHighestDerivative) = 0;
  std::shared_ptr<GridController> getGridController() const { return _gridController; }
  void notify() override {
    _upToDate = false;
    this->notifyObjects();
  }
  virtual SparseVectorInt getNonNegligibleBlocks() {
    throw SerenityError("Overwrite this function in the specific realizations, please!");
  }
  virtual unsigned int getNBlocks() { throw SerenityError("Overwrite this function in the specific realizations, please!"); }
  virtual unsigned int getMaxBlockSize() {
    throw SerenityError("Overwrite this function in the specific realizations, please!");
  }

 protected:
  const std::shared_ptr<GridController> _gridController;
  unsigned int _highestDerivative;
  unsigned int _nGridPoints;
  bool _upToDate = false;
  DensityOnGrid<M> _densityOnGrid;
  Gradient<DensityOnGrid<M>> _densityGradientOnGrid;
};

/* DensityMatrixDensityOnGridController<M> (DensityMatrixDensityOnGridController.cpp:28-187):
 * the density of a DensityMatrixController's matrix on the grid, formed on first use after
 * every change of the matrix (it registers with the controller); with
 * iOOptions.gridAccuracyCheck it prints the electrons integrated over the grid per spin. */
template <Options::SCF_MODES M>
class DensityMatrixDensityOnGridController : public DensityOnGridController<M> {
 public:
  DensityMatrixDensityOnGridController(std::shared_ptr<DensityOnGridCalculator<M>> calc,
                                       std::shared_ptr<DensityMatrixController<M>> dmat)
      : DensityMatrixDensityOnGridController(calc, dmat,
                                             calc->getBasisFunctionOnGridController()->getHighestDerivative()) {}
  DensityMatrixDensityOnGridController(std::shared_ptr<DensityOnGridCalculator<M>> calc,
                                       std::shared_ptr<DensityMatrixController<M>> dmat, unsigned int highestDerivative)
      : DensityOnGridController<M>(calc->getGridController(), highestDerivative), calc_(calc), dmat_(dmat) {
    if (highestDerivative > calc->getBasisFunctionOnGridController()->getHighestDerivative())
      throw SerenityError("DensityMatrixDensityOnGridController: derivative beyond the basis data's");
    dmat_->addSensitiveObject(this->_self);
  }
  const DensityOnGrid<M>& getDensityOnGrid() override {
    if (!this->_upToDate) calculateData();
    return this->_densityOnGrid;
  }
  const Gradient<DensityOnGrid<M>>& getDensityGradientOnGrid() override {
    if (this->_highestDerivative < 1) setHighestDerivative(1);
    if (!this->_upToDate) calculateData();
    return this->_densityGradientOnGrid;
  }
  void setHighestDerivative(unsigned int d) override {
    if (d > 1) throw SerenityError("Density Hessians on the grid are not part of this XC path.");
    if (d != this->_highestDerivative) this->notify();
    this->_highestDerivative = d;
  }
  SparseVectorInt getNonNegligibleBlocks() override { return calc_->getNonNegligibleBlocks(); }
  unsigned int getNBlocks() override { return calc_->getBasisFunctionOnGridController()->getNBlocks(); }
  unsigned int getMaxBlockSize() override { return calc_->getBasisFunctionOnGridController()->getMaxBlockSize(); }
  std::shared_ptr<DensityOnGridCalculator<M>> getDensityOnGridCalculator() const { return calc_; }
  /* electrons integrated over the grid per spin at the last evaluation (what
   * gridAccuracyCheck prints) */
  const std::vector<double>& getLastElectronCount() const { return nel_; }

 private:
  void calculateData() {
    const auto& P = dmat_->getDensityMatrix();
    if (this->_highestDerivative == 0)
      calc_->calcDensityOnGrid(P, this->_densityOnGrid);
    else
      calc_->calcDensityAndGradientOnGrid(P, this->_densityOnGrid, this->_densityGradientOnGrid);
    const auto& w = this->_gridController->getWeights();
    std::vector<double> r;
    detail::pack(this->_densityOnGrid, r);
    const int ns = detail::nspin<M>();
    nel_.assign(ns, 0.0);
    for (int s = 0; s < ns; ++s)
      for (size_t p = 0; p < w.size(); ++p) nel_[s] += r[s * w.size() + p] * w[p];
    if (iOOptions.gridAccuracyCheck)
      for (int s = 0; s < ns; ++s) std::printf("nElectrons from integration over grid: %.10f\n", nel_[s]);
    this->_upToDate = true;
  }
  std::shared_ptr<DensityOnGridCalculator<M>> calc_;
  std::shared_ptr<DensityMatrixController<M>> dmat_;
  std::vector<double> nel_;
};

enum class FUNCTIONAL_DATA_TYPE { GRADIENTS };

namespace CompositeFunctionals {
/* the composite functionals of this path (CompositeFunctionals.cpp:233-246) */
enum class FUNCTIONALS { LDA, PBE, BLYP, BP86 };
enum class CLASSES { NONE, LDA, GGA, MODELL };
}  // namespace CompositeFunctionals

/* A resolved functional (src/dft/Functional.h): its library identifier and class */
class Functional {
 public:
  explicit constexpr Functional(int id = XCGPU_FUNC_LDA) : id_(id) {}
  int id() const { return id_; }
  bool isGGA() const { return xcgpu_functional_is_gga(id_) != 0; }
  CompositeFunctionals::CLASSES getFunctionalClass() const {
    return isGGA() ? CompositeFunctionals::CLASSES::GGA : CompositeFunctionals::CLASSES::LDA;
  }
  explicit operator int() const { return id_; }
  bool operator==(const Functional& o) const { return id_ == o.id_; }
  static const Functional LDA, PBE, BLYP, BP86;

 private:
  int id_;
};
inline const Functional Functional::LDA{XCGPU_FUNC_LDA};
inline const Functional Functional::PBE{XCGPU_FUNC_PBE};
inline const Functional Functional::BLYP{XCGPU_FUNC_BLYP};
inline const Functional Functional::BP86{XCGPU_FUNC_BP86};

namespace CompositeFunctionals {
/* CompositeFunctionals::resolveFunctional (CompositeFunctionals.cpp:42-73) */
inline Functional resolveFunctional(FUNCTIONALS f) {
  switch (f) {
    case FUNCTIONALS::LDA: return Functional::LDA;
    case FUNCTIONALS::PBE: return Functional::PBE;
    case FUNCTIONALS::BLYP: return Functional::BLYP;
    case FUNCTIONALS::BP86: return Functional::BP86;
  }
  throw SerenityError("You have requested a functional that this path cannot provide.");
}
}  // namespace CompositeFunctionals

/* FunctionalData<M> (PartialDerivatives.h:931-1090): the energy, the energy per volume and
 * the first derivatives, held by shared pointers as in the reference */
template <Options::SCF_MODES M>
struct FunctionalData {
  double energy = 0.0;
  std::shared_ptr<Vector> epuv;
  std::shared_ptr<GridPotential<M>> dFdRho;
  std::shared_ptr<Gradient<GridPotential<M>>> dFdGradRho;
};

template <Options::SCF_MODES M>
class FunctionalLibrary {
 public:
  explicit FunctionalLibrary(unsigned int maxBlockSize) : block_(maxBlockSize) {}
  /* FunctionalLibrary<M>::calcData (FunctionalLibrary.h:60-62): the density (and, for a
   * GGA, its gradient) comes from the controller, formed there on demand */
  FunctionalData<M> calcData(FUNCTIONAL_DATA_TYPE type, const Functional& f,
                             std::shared_ptr<DensityOnGridController<M>> densityOnGridController,
                             unsigned int order = 1) {
    const bool gga = f.isGGA();
    if (gga && densityOnGridController->getHighestDerivative() < 1)
      throw SerenityError("XCFun: Density gradient required for GGA functional, but DensityOnGridController does not have it.");
    const auto& rho = densityOnGridController->getDensityOnGrid();
    const Gradient<DensityOnGrid<M>>* grad = gga ? &densityOnGridController->getDensityGradientOnGrid() : nullptr;
    return calcData(type, f, *densityOnGridController->getGridController(), rho, grad, order);
  }
  /* the same from a density already on the grid */
  FunctionalData<M> calcData(FUNCTIONAL_DATA_TYPE, const Functional& f, const GridController& grid,
                             const DensityOnGrid<M>& rho, const Gradient<DensityOnGrid<M>>* grad,
                             unsigned int order = 1) {
    if (order != 1) throw SerenityError("only first functional derivatives are available on this path");
    const int ns = detail::nspin<M>();
    const long n = grid.getNGridPoints();
    const int func = f.id();
    const bool gga = f.isGGA();
    if (gga && !grad)
      throw SerenityError("XCFun: Density gradient required for GGA functional, but DensityOnGridController does not have it.");
    std::vector<double> r, g;
    detail::pack(rho, r);
    if (r.size() != (size_t)ns * n) throw SerenityError("FunctionalLibrary: density and grid do not match");
    if (gga) {
      for (int s = 0; s < ns; ++s)
        for (const auto* comp : {&grad->x, &grad->y, &grad->z}) {
          std::vector<double> c;
          detail::pack(*comp, c);
          g.insert(g.end(), c.begin() + s * n, c.begin() + (s + 1) * n);
        }
    }
    FunctionalData<M> out;
    out.epuv = std::make_shared<Vector>(n, 0.0);
    out.dFdRho = std::make_shared<GridPotential<M>>();
    std::vector<double> dr((size_t)ns * n), dg(gga ? (size_t)ns * 3 * n : 0);
    auto ctx = grid.context();
    detail::check(ctx->get(), xcgpu_functional(ctx->get(), func, ns, n, block_, r.data(), gga ? g.data() : nullptr,
                                               out.epuv->data(), dr.data(), gga ? dg.data() : nullptr, XCGPU_MEM_HOST));
    detail::unpack(dr.data(), n, *out.dFdRho);
    const auto& w = grid.getWeights();
    for (long p = 0; p < n; ++p) out.energy += (*out.epuv)[p] * w[p];
    if (gga) {
      out.dFdGradRho = std::make_shared<Gradient<GridPotential<M>>>();
      std::vector<double> cx, cy, cz;
      for (int s = 0; s < ns; ++s) {
        cx.insert(cx.end(), dg.begin() + (s * 3 + 0) * n, dg.begin() + (s * 3 + 1) * n);
        cy.insert(cy.end(), dg.begin() + (s * 3 + 1) * n, dg.begin() + (s * 3 + 2) * n);
        cz.insert(cz.end(), dg.begin() + (s * 3 + 2) * n, dg.begin() + (s * 3 + 3) * n);
      }
      detail::unpack(cx.data(), n, out.dFdGradRho->x);
      detail::unpack(cy.data(), n, out.dFdGradRho->y);
      detail::unpack(cz.data(), n, out.dFdGradRho->z);
    }
    return out;
  }

 private:
  unsigned int block_;
};

template <Options::SCF_MODES M>
class ScalarOperatorToMatrixAdder {
 public:
  ScalarOperatorToMatrixAdder(std::shared_ptr<BasisFunctionOnGridController> bfog, double blockAveThreshold,
                              int precision = XCGPU_PREC_FP64)
      : bfog_(bfog), thr_(blockAveThreshold), precision_(precision) {}
  void addScalarOperatorToMatrix(SPMatrix<M>& matrix, const GridPotential<M>& scalarOperator) {
    add(matrix, scalarOperator, nullptr);
  }
  void addScalarOperatorToMatrix(SPMatrix<M>& matrix, const GridPotential<M>& scalarOperator,
                                 const Gradient<GridPotential<M>>& gradientOperator) {
    add(matrix, scalarOperator, &gradientOperator);
  }

 private:
  void add(SPMatrix<M>& F, const GridPotential<M>& v, const Gradient<GridPotential<M>>* g) {
    const int ns = detail::nspin<M>();
    const long n = bfog_->getNGridPoints();
    std::vector<double> vv, gg, Fv;
    detail::pack(v, vv);
    if (vv.size() != (size_t)ns * n)
      throw SerenityError("The scalar operator and the BasisFunctionOnGridController passed to addScalarOperatorToMatrix "
                          "are not defined on the same grid!");
    if (g)
      for (int s = 0; s < ns; ++s)
        for (const auto* comp : {&g->x, &g->y, &g->z}) {
          std::vector<double> c;
          detail::pack(*comp, c);
          gg.insert(gg.end(), c.begin() + s * n, c.begin() + (s + 1) * n);
        }
    detail::pack(F, Fv);
    detail::check(bfog_->ctx(), xcgpu_add_scalar(bfog_->handle(), thr_, ns, vv.data(), g ? gg.data() : nullptr,
                                                 Fv.data(), precision_, XCGPU_MEM_HOST));
    detail::unpack(Fv.data(), F);
  }
  std::shared_ptr<BasisFunctionOnGridController> bfog_;
  double thr_;
  int precision_;
};

/* FuncPotential<M>::getMatrix / getEnergy for an LDA or GGA functional (FuncPotential.cpp:74-110) */
template <Options::SCF_MODES M>
class FuncPotential {
 public:
  FuncPotential(std::shared_ptr<BasisFunctionOnGridController> bfog, Functional f, double blockAveThreshold = 1e-11,
                int precision = XCGPU_PREC_FP64)
      : bfog_(bfog), f_(f), thr_(blockAveThreshold), precision_(precision) {}
  FockMatrix<M> getMatrix(const DensityMatrix<M>& P) {
    const int ns = detail::nspin<M>();
    const long nbf = bfog_->getNBasisFunctions();
    std::vector<double> Pv, Vv((size_t)ns * nbf * nbf);
    detail::pack(P, Pv);
    detail::check(bfog_->ctx(), xcgpu_vxc(bfog_->handle(), f_.id(), ns, precision_, thr_, Pv.data(), Vv.data(),
                                          &energy_, &nel_, XCGPU_MEM_HOST));
    FockMatrix<M> F = P;
    detail::unpack(Vv.data(), F);
    return F;
  }
  double getEnergy() const { return energy_; }
  double getNumberOfElectrons() const { return nel_; }
  // getGeomGradients (FuncPotential.cpp:113-241): natoms x 3; shellAtoms[s] = atom of shell s
  // (BasisController::getAtomIndicesOfBasis).  FP64.
  Matrix getGeomGradients(const DensityMatrix<M>& P, const std::vector<int>& shellAtoms, int natoms) {
    const int ns = detail::nspin<M>();
    std::vector<double> Pv;
    detail::pack(P, Pv);
    Matrix G(natoms, 3);
    detail::check(bfog_->ctx(), xcgpu_xc_gradient(bfog_->handle(), f_.id(), ns, Pv.data(), shellAtoms.data(), natoms,
                                                  G.data(), XCGPU_MEM_HOST));
    return G;
  }

 private:
  std::shared_ptr<BasisFunctionOnGridController> bfog_;
  Functional f_;
  double thr_;
  int precision_;
  double energy_ = 0.0, nel_ = 0.0;
};

// The XC kernel part of linear-response sigma vectors (KernelSigmavector<M>::calcF,
// src/postHF/LRSCF/Sigmavectors/KernelSigmavector.cpp:127-253, contractBlock :363-499):
// calcF(P0, trials) returns one matrix per trial matrix.  Restricted: the singlet kernel,
// or with triplet = true the triplet's f_aa - f_ab; unrestricted: alpha and beta trial
// and result matrices.
template <Options::SCF_MODES M>
class KernelSigmavector {
 public:
  KernelSigmavector(std::shared_ptr<BasisFunctionOnGridController> bfog, Functional f,
                    double blockAveThreshold = 1e-11, int precision = XCGPU_PREC_FP64, bool triplet = false)
      : bfog_(bfog), f_(f), thr_(blockAveThreshold), precision_(precision), triplet_(triplet) {
    if (triplet && M == Options::SCF_MODES::UNRESTRICTED)
      throw SerenityError("KernelSigmavector: the triplet kernel belongs to a restricted ground state");
  }
  std::vector<SPMatrix<M>> calcF(const SPMatrix<M>& P0, const std::vector<SPMatrix<M>>& trials) {
    const long nbf = bfog_->getNBasisFunctions();
    const int ns = detail::nspin<M>();
    std::vector<double> P0v;
    detail::pack(P0, P0v);
    if (P0v.size() != (size_t)ns * nbf * nbf) throw SerenityError("KernelSigmavector: size mismatch");
    std::vector<std::vector<double>> Dv(trials.size()), Fv(trials.size(), std::vector<double>((size_t)ns * nbf * nbf));
    std::vector<const double*> d;
    std::vector<double*> f;
    for (size_t t = 0; t < trials.size(); ++t) {
      detail::pack(trials[t], Dv[t]);
      if (Dv[t].size() != (size_t)ns * nbf * nbf) throw SerenityError("KernelSigmavector: size mismatch");
      d.push_back(Dv[t].data());
      f.push_back(Fv[t].data());
    }
    const int kind = M == Options::SCF_MODES::UNRESTRICTED ? XCGPU_LR_UNRESTRICTED
                     : triplet_                             ? XCGPU_LR_TRIPLET
                                                            : XCGPU_LR_SINGLET;
    detail::check(bfog_->ctx(), xcgpu_lr_kernel_spin(bfog_->handle(), f_.id(), kind, P0v.data(), (uint32_t)trials.size(),
                                                     d.data(), f.data(), precision_, thr_, XCGPU_MEM_HOST));
    std::vector<SPMatrix<M>> F(trials.begin(), trials.end());
    for (size_t t = 0; t < trials.size(); ++t) detail::unpack(Fv[t].data(), F[t]);
    return F;
  }

 private:
  std::shared_ptr<BasisFunctionOnGridController> bfog_;
  Functional f_;
  double thr_;
  int precision_;
  bool triplet_;
};

// NAddFuncPotential<M> (src/potentials/NAddFuncPotential.h:93-200): the non-additive XC
// potential of an active subsystem in the field of environment subsystems, all densities
// on the active system's grid.  getMatrix(P_active, P_env) returns the potential in the
// active basis (NAddFuncPotential.cpp:189-243); getEnergy() the non-additive energy
// E_xc[sum] - E_xc[active] - sum E_xc[env] of that call.  Environment controllers must be
// built on the same grid controller as the active one.
template <Options::SCF_MODES M>
class NAddFuncPotential {
 public:
  NAddFuncPotential(std::shared_ptr<BasisFunctionOnGridController> active,
                    std::vector<std::shared_ptr<BasisFunctionOnGridController>> env, Functional f,
                    double blockAveThreshold = 1e-11, int precision = XCGPU_PREC_FP64)
      : active_(active), env_(std::move(env)), f_(f), thr_(blockAveThreshold), precision_(precision) {}
  FockMatrix<M> getMatrix(const DensityMatrix<M>& P, const std::vector<DensityMatrix<M>>& Penv) {
    if (Penv.size() != env_.size()) throw SerenityError("NAddFuncPotential: one density matrix per environment system");
    const int ns = detail::nspin<M>();
    const long nbf = active_->getNBasisFunctions();
    std::vector<double> Pv, Vv((size_t)ns * nbf * nbf);
    detail::pack(P, Pv);
    std::vector<std::vector<double>> Pe(env_.size());
    std::vector<xcgpu_plan*> plans;
    std::vector<const double*> ptrs;
    for (size_t i = 0; i < env_.size(); ++i) {
      detail::pack(Penv[i], Pe[i]);
      plans.push_back(env_[i]->handle());
      ptrs.push_back(Pe[i].data());
    }
    detail::check(active_->ctx(), xcgpu_nadd_vxc(active_->handle(), plans.data(), (uint32_t)plans.size(), f_.id(), ns,
                                                 precision_, thr_, Pv.data(), ptrs.data(), Vv.data(), &energy_,
                                                 XCGPU_MEM_HOST));
    FockMatrix<M> F = P;
    detail::unpack(Vv.data(), F);
    return F;
  }
  double getEnergy() const { return energy_; }

 private:
  std::shared_ptr<BasisFunctionOnGridController> active_;
  std::vector<std::shared_ptr<BasisFunctionOnGridController>> env_;
  Functional f_;
  double thr_;
  int precision_;
  double energy_ = 0.0;
};

}  // namespace Serenity
#endif /* SERENITY_XC_HPP */
