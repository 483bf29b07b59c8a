// Drives the C++ facade (include/serenity_xc.hpp) the way Serenity's own tests drive
// its classes: SMALL_MIXED basis on the TINY / VERY_SMALL grids
// (testsupply/BasisController__TEST_SUPPLY.cpp:59-84, GridController__TEST_SUPPLY.cpp:31-46).
// Prints the results as JSON; tests/test_facade.py compares them with the golden
// vectors of the reference tests.
#include <cmath>
#include <cstdio>
#include <memory>

#include "serenity_xc.hpp"

using namespace Serenity;

// every member of the class templates compiles against the C ABI
template class Serenity::DensityMatrixDensityOnGridController<RESTRICTED>;
template class Serenity::DensityMatrixDensityOnGridController<UNRESTRICTED>;
template class Serenity::FunctionalLibrary<RESTRICTED>;
template class Serenity::FunctionalLibrary<UNRESTRICTED>;
template class Serenity::KernelSigmavector<RESTRICTED>;
template class Serenity::KernelSigmavector<UNRESTRICTED>;
template class Serenity::NAddFuncPotential<RESTRICTED>;
template class Serenity::NAddFuncPotential<UNRESTRICTED>;
template class Serenity::FuncPotential<RESTRICTED>;
template class Serenity::FuncPotential<UNRESTRICTED>;

static std::vector<ShellData> small_mixed() {
  return {{0, false, {0.0, 0.0, 0.0}, {1.0, 2.0}, {1.0, 0.1}},
          {1, false, {1.0, 0.0, 0.0}, {1.0, 2.0}, {1.0, 0.1}},
          {2, false, {-1.0, 2.5, 1.0}, {0.5, 1.2}, {0.8, 0.4}}};
}

static void print_vec(const char* name, const std::vector<double>& v, bool last = false) {
  std::printf("\"%s\": [", name);
  for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
  std::printf("]%s\n", last ? "" : ",");
}

int main() {
  auto ctx = std::make_shared<XcContext>(0);
  auto basis = std::make_shared<BasisController>(ctx, small_mixed());
  // The reference's FuncPotential::getMatrix chain (FuncPotential.cpp:57-105) on the facade,
  // call for call: a DensityMatrixController, a DensityOnGridCalculator and the lazy
  // DensityMatrixDensityOnGridController, FunctionalLibrary(128).calcData(GRADIENTS, f,
  // controller) and the adder; against the fused build (FuncPotential::getMatrix here).
  // gridAccuracyCheck prints its electron counts before the JSON below.
  std::vector<double> staged_F, fused_F, rho_before, rho_after;
  double staged_E = 0.0, fused_E = 0.0, nel_grid = 0.0, nel_sum = 0.0;
  long nonneg = 0, nblocks_lazy = 0;
  {
    std::vector<double> xyz, w;
    for (int i = 0; i < 200; ++i) {  // 200 points around the SMALL_MIXED centres
      const double t = 0.37 * i;
      xyz.insert(xyz.end(), {-1.5 + 0.02 * i, 2.0 * std::sin(t), 1.5 * std::cos(1.3 * t)});
      w.push_back(0.05 + 0.001 * (i % 7));
    }
    auto grid = std::make_shared<GridController>(ctx, xyz, w);
    auto bfog = std::make_shared<BasisFunctionOnGridController>(basis, grid, 128, 1e-9, 1);
    Matrix P(10, 10);
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) P(i, j) = (i == j ? 0.6 : 0.0) + 0.05 / (1.0 + i + j);
    auto dmat = std::make_shared<DensityMatrixController<RESTRICTED>>(P);
    auto calc = std::make_shared<DensityOnGridCalculator<RESTRICTED>>(bfog, 1e-11);
    auto dens = std::make_shared<DensityMatrixDensityOnGridController<RESTRICTED>>(calc, dmat);
    auto adder = std::make_shared<ScalarOperatorToMatrixAdder<RESTRICTED>>(bfog, 1e-11);
    const Functional f = CompositeFunctionals::resolveFunctional(CompositeFunctionals::FUNCTIONALS::PBE);
    iOOptions.gridAccuracyCheck = true;
    FunctionalLibrary<RESTRICTED> flib(128);
    auto funcData = flib.calcData(FUNCTIONAL_DATA_TYPE::GRADIENTS, f, dens);
    iOOptions.gridAccuracyCheck = false;
    FockMatrix<RESTRICTED> pot(10, 10);
    if (f.getFunctionalClass() == CompositeFunctionals::CLASSES::GGA)
      adder->addScalarOperatorToMatrix(pot, *funcData.dFdRho, *funcData.dFdGradRho);
    else
      adder->addScalarOperatorToMatrix(pot, *funcData.dFdRho);
    staged_E = funcData.energy;
    staged_F.assign(pot.data(), pot.data() + 100);
    FuncPotential<RESTRICTED> fused(bfog, f);
    auto F = fused.getMatrix(P);
    fused_E = fused.getEnergy();
    fused_F.assign(F.data(), F.data() + 100);
    nel_grid = dens->getLastElectronCount()[0];
    for (size_t p = 0; p < w.size(); ++p) nel_sum += dens->getDensityOnGrid()[p] * w[p];
    rho_before = dens->getDensityOnGrid();
    Matrix P2 = P;
    for (int i = 0; i < 10; ++i) P2(i, i) *= 2.0;
    dmat->setDensityMatrix(P2);  // notifies the controller: the next read recomputes
    rho_after = dens->getDensityOnGrid();
    nonneg = dens->getNonNegligibleBlocks().nonZeros();
    nblocks_lazy = dens->getNBlocks();
  }
  std::printf("{\n");
  print_vec("staged_F", staged_F);
  print_vec("fused_F", fused_F);
  print_vec("rho_before", rho_before);
  print_vec("rho_after", rho_after);
  std::printf("\"staged_E\": %.17g, \"fused_E\": %.17g, \"nel_grid\": %.17g, \"nel_sum\": %.17g,\n", staged_E,
              fused_E, nel_grid, nel_sum);
  std::printf("\"nonnegligible_blocks\": %ld, \"nblocks_lazy\": %ld,\n", nonneg, nblocks_lazy);
  {  // density on TINY, blocks of 3, no radial cut-off (DensityOnGridCalculator_test.cpp:43-256)
    std::vector<double> xyz = {0.0, 0.0, 0.0, 1.0, 0.0, 0.0, -2.0, 1.0, 1.0, 3.0, 0.5, -1.0};
    auto grid = std::make_shared<GridController>(ctx, xyz, std::vector<double>(4, 1.0));
    auto bfog = std::make_shared<BasisFunctionOnGridController>(basis, grid, 3, 0.0, 1);
    DensityOnGridCalculator<RESTRICTED> calc(bfog, 0.0);
    Matrix P(10, 10);
    std::FILE* f = std::fopen(std::getenv("FACADE_P"), "r");
    for (int i = 0; i < 100; ++i)
      if (std::fscanf(f, "%lf", P.data() + i) != 1) return 2;
    std::fclose(f);
    DensityOnGrid<RESTRICTED> rho;
    Gradient<DensityOnGrid<RESTRICTED>> grad;
    calc.calcDensityAndGradientOnGrid(P, rho, grad);
    print_vec("rho", rho);
    print_vec("grad_x", grad.x);
    std::printf("\"nblocks\": %u,\n", bfog->getNBlocks());
    auto blk = bfog->getBlockOnGridData(1);
    print_vec("block1_negligible", std::vector<double>(blk->negligible.begin(), blk->negligible.end()));
  }
  {  // adder on VERY_SMALL (ScalarOperatorToMatrixAdder_test.cpp:41-148)
    std::vector<double> xyz = {-1.0, 0.0, 0.0, 0.0, 0.5, 0.4, 0.0, -0.4, -0.5, 0.8, 0.1, -0.1, 0.1, -0.1, 0.1};
    std::vector<double> w = {0.1, 0.2, 0.15, 0.15, 0.4};
    auto grid = std::make_shared<GridController>(ctx, xyz, w);
    auto bfog = std::make_shared<BasisFunctionOnGridController>(basis, grid, 3, 1e-11, 1);
    ScalarOperatorToMatrixAdder<RESTRICTED> adder(bfog, 1e-11);
    GridPotential<RESTRICTED> pot = {1.3, -0.7, 5.4, 0.0003, -0.3};
    Gradient<GridPotential<RESTRICTED>> g;
    g.x = {0.0002, -0.02, 1.3, 0.004, -0.001};
    g.y = {-0.01, 0.1, -2.2, -0.03, 0.0025};
    g.z = {1.03, -0.007, 0.4, -0.0000007, -0.00004};
    FockMatrix<RESTRICTED> F(10, 10);
    adder.addScalarOperatorToMatrix(F, pot, g);
    print_vec("F", std::vector<double>(F.data(), F.data() + 100));
    bool threw = false;
    try {
      GridPotential<RESTRICTED> bad(3, 1.0);
      adder.addScalarOperatorToMatrix(F, bad);
    } catch (const SerenityError&) {
      threw = true;
    }
    std::printf("\"grid_mismatch_throws\": %s\n", threw ? "true" : "false");
  }
  std::printf("}\n");
  return 0;
}
