// Drives the C++ facade (include/serenity_xc.hpp) the way Serenity's own tests drive
// its classes: SMALL_MIXED basis on the TINY / VERY_SMALL grids
// (testsupply/BasisController__TEST_SUPPLY.cpp:59-84, GridController__TEST_SUPPLY.cpp:31-46).
// Prints the results as JSON; tests/test_facade.py compares them with the golden
// vectors of the reference tests.
#include <cstdio>
#include <memory>

#include "serenity_xc.hpp"

using namespace Serenity;

// every member of the class templates compiles against the C ABI
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
  std::printf("{\n");
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
