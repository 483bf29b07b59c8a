// Test-infrastructure helper (oracle side, never shipped in the product path).
// Links against the reference's own Lebedev routines, compiled in place from
// src/grid/construction/sphere_lebedev_rule.cpp, and prints every rule that the
// reference's AtomGridFactory can select (AtomGridFactory.cpp:150-190 and
// 292-466: orders 6 ... 770, the largest that accuracy 7 selects) as plain text: "order n" followed by n lines "x y z w".
// The output is the node/weight table the grid builders read at run time.
#include <cstdio>
#include <vector>
#include "grid/construction/sphere_lebedev_rule.h"

typedef void (*rule_fn)(double*, double*, double*, double*);

int main() {
  struct R { int n; rule_fn f; };
  const R rules[] = {{6, Serenity::ld0006},   {14, Serenity::ld0014},   {26, Serenity::ld0026},
                     {38, Serenity::ld0038},  {50, Serenity::ld0050},   {74, Serenity::ld0074},
                     {86, Serenity::ld0086},  {110, Serenity::ld0110},  {146, Serenity::ld0146},
                     {170, Serenity::ld0170}, {194, Serenity::ld0194},  {230, Serenity::ld0230},
                     {266, Serenity::ld0266}, {302, Serenity::ld0302},  {350, Serenity::ld0350},
                     {434, Serenity::ld0434}, {590, Serenity::ld0590},  {770, Serenity::ld0770}};
  for (const R& r : rules) {
    std::vector<double> x(r.n), y(r.n), z(r.n), w(r.n);
    r.f(x.data(), y.data(), z.data(), w.data());
    std::printf("order %d\n", r.n);
    for (int i = 0; i < r.n; ++i) std::printf("%.17g %.17g %.17g %.17g\n", x[i], y[i], z[i], w[i]);
  }
  return 0;
}
