// Atom-centred integration grid: Ahlrichs radial x Lebedev angular atom grids
// (AtomGridFactory.cpp:78-290), Becke fuzzy-cell partition weights with atomic
// size adjustment and smoothing (GridFactory.cpp:52-346) computed on the GPU,
// weight cut-off, and Hilbert-curve ordering of the points
// (HilbertRTreeSorting.cpp:29-216).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "internal.h"

namespace xcgpu {

// Treutler-Ahlrichs radial scaling per element (AtomGridFactory.cpp:39-52), Z = 1..36.
static const double kAlpha[37] = {1.1, 0.8, 0.9, 1.8, 1.4, 1.3, 1.1, 0.9, 0.9, 0.9, 0.9, 1.4, 1.3,
                                  1.3, 1.2, 1.1, 1.0, 1.0, 1.0, 1.5, 1.4, 1.3, 1.2, 1.2, 1.2, 1.2,
                                  1.2, 1.2, 1.1, 1.1, 1.1, 1.1, 1.0, 0.9, 0.9, 0.9, 0.9};
// Clementi radii (pruning zones, AtomGridFactory.cpp:53-62).
static const double kClementiR[37] = {1.00, 1.00, 0.59, 3.16, 2.12, 1.64, 1.27, 1.06, 0.91, 0.79, 0.72, 3.59, 2.74,
                                      2.23, 2.10, 1.85, 1.66, 1.49, 1.34, 4.59, 3.67, 3.48, 3.33, 3.23, 3.14, 3.04,
                                      2.95, 2.87, 2.82, 2.74, 2.68, 2.57, 2.36, 2.15, 1.95, 1.78, 1.66};
// Bragg-Slater radii / Angstrom (AtomicParameters.h:454-462; H = 0.25, AtomTypeFactory.cpp:105-108).
static const double kBraggSlaterR[37] = {-1.0, 0.25, 1.20, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50, 0.38, 1.80, 1.50,
                                         1.25, 1.10, 1.00, 1.00, 1.00, 0.71, 2.20, 1.80, 1.60, 1.40, 1.35, 1.40, 1.40,
                                         1.40, 1.35, 1.35, 1.35, 1.35, 1.30, 1.25, 1.15, 1.15, 1.15, 0.88};
static const int kOrders[18] = {6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302, 350, 434, 590, 770};

static int element_row(int Z) { return Z <= 2 ? 1 : Z <= 10 ? 2 : Z <= 18 ? 3 : Z <= 36 ? 4 : 5; }

static bool read_lebedev(const char* path, std::map<int, std::vector<double>>& rules) {
  std::ifstream f(path);
  if (!f) return false;
  std::string tok;
  while (f >> tok) {
    if (tok != "order") continue;
    int n = 0;
    f >> n;
    auto& v = rules[n];
    v.resize(4 * n);
    for (int i = 0; i < 4 * n; ++i) f >> v[i];
  }
  return !rules.empty();
}

// Ahlrichs M3 mapping with m = 0.6 and Chebyshev (second kind) nodes
// (J. Chem. Phys. 102, 346 (1995); AtomGridFactory.cpp:238-260); ascending radii.
static void radial(double alpha, int n, std::vector<double>& r, std::vector<double>& w) {
  r.assign(n, 0.0);
  w.assign(n, 0.0);
  const double s = alpha / std::log(2.0);
  for (int i = 1; i <= n; ++i) {
    const double x = std::cos(i * M_PI / (n + 1.0));
    const double ln = std::log((1.0 - x) / 2.0);
    const double q = std::sqrt((1.0 + x) / (1.0 - x));
    r[n - i] = s * std::pow(x + 1.0, 0.6) * std::log(2.0 / (1.0 - x));
    w[n - i] = (M_PI / (n + 1.0)) * std::pow(1.0 + x, 1.8) * s * s * s * (q * ln * ln - 0.6 * ln * ln * ln / q);
  }
}

// Becke cell weight of candidate point i (one thread per point).
__global__ void becke_kernel(int natoms, const double* __restrict__ A, const double* __restrict__ rdist,
                             const double* __restrict__ adj, const int* __restrict__ sig_off,
                             const int* __restrict__ sig_list, long npts, const double* __restrict__ pts,
                             const int* __restrict__ owner, const double* __restrict__ wref, int smoothing,
                             double* __restrict__ wout) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const double gx = pts[3 * i], gy = pts[3 * i + 1], gz = pts[3 * i + 2];
  const int k = owner[i];
  const int s0 = sig_off[k], s1 = sig_off[k + 1];
  double weight = wref[i], sum = 0.0;
  const double dxk = A[3 * k] - gx, dyk = A[3 * k + 1] - gy, dzk = A[3 * k + 2] - gz;
  const double rk = sqrt(dxk * dxk + dyk * dyk + dzk * dzk);
  for (int li = s0; li < s1; ++li) {
    const int l = sig_list[li];
    const double dxl = A[3 * l] - gx, dyl = A[3 * l + 1] - gy, dzl = A[3 * l + 2] - gz;
    const double rl = sqrt(dxl * dxl + dyl * dyl + dzl * dzl);
    if (l != k) {
      // the owner atom's factor first: for atoms far from the point it is exactly zero,
      // and a zero factor makes the cell zero in any order of the product
      const double mu = (rl - rk) * rdist[l + (long)natoms * k];
      double nu = mu + adj[k + (long)natoms * l] * (1.0 - mu * mu);
      for (int s = 0; s < smoothing; ++s) nu = (3.0 - nu * nu) * nu / 2.0;
      if (0.5 * (1.0 - nu) == 0.0) continue;
    }
    double cell = 1.0;
    for (int ji = s0; ji < s1 && cell != 0.0; ++ji) {
      const int j = sig_list[ji];
      if (j == l) continue;
      const double dxj = A[3 * j] - gx, dyj = A[3 * j + 1] - gy, dzj = A[3 * j + 2] - gz;
      const double rj = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
      const double mu = (rl - rj) * rdist[l + (long)natoms * j];
      double nu = mu + adj[j + (long)natoms * l] * (1.0 - mu * mu);
      for (int s = 0; s < smoothing; ++s) nu = (3.0 - nu * nu) * nu / 2.0;
      cell *= 0.5 * (1.0 - nu);
    }
    if (l == k) weight *= cell;
    sum += cell;
  }
  wout[i] = weight / sum;
}

// Stratmann-Scuseria-Frisch weight of candidate point i (GridFactory.cpp:209-268): the
// reference weight stays inside 0.5 (1 - a) of the owner's nearest-neighbour distance;
// a point with some nu_kj >= a is dropped (NaN marker, removed by the weight cut);
// otherwise the cell products with the SSF polynomial, a = 0.64, over all atoms.
__global__ void ssf_kernel(int natoms, const double* __restrict__ A, const double* __restrict__ dist,
                           const double* __restrict__ min_dist, long npts, const double* __restrict__ pts,
                           const int* __restrict__ owner, const double* __restrict__ wref, double* __restrict__ wout) {
  constexpr double a = 0.64;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const double gx = pts[3 * i], gy = pts[3 * i + 1], gz = pts[3 * i + 2];
  const int k = owner[i];
  auto r = [&](int l) {
    const double dx = A[3 * l] - gx, dy = A[3 * l + 1] - gy, dz = A[3 * l + 2] - gz;
    return sqrt(dx * dx + dy * dy + dz * dz);
  };
  double weight = wref[i];
  const double rk = r(k);
  if (!(rk >= 0.5 * (1.0 - a) * min_dist[k])) {
    wout[i] = weight;
    return;
  }
  for (int j = 0; j < natoms; ++j) {
    if ((rk - r(j)) / dist[k + (long)natoms * j] >= a) {  // j == k: 0/0 compares false
      wout[i] = nan("");
      return;
    }
  }
  double sum = 0.0;
  for (int l = 0; l < natoms; ++l) {
    const double rl = r(l);
    double cell = 1.0;
    for (int j = 0; j < natoms; ++j) {
      if (j == l) continue;
      double nu = (rl - r(j)) / dist[l + (long)natoms * j];
      if (nu <= -a) continue;
      if (nu >= a) {
        cell = 0.0;
        break;
      }
      nu /= a;
      const double n3 = nu * nu * nu;
      const double poly = (-5.0 * n3 * n3 * nu + 21.0 * n3 * nu * nu - 35.0 * n3 + 35.0 * nu) / 16.0;
      cell *= 0.5 * (1 - poly);
    }
    if (l == k) weight *= cell;
    sum += cell;
  }
  wout[i] = weight / sum;
}

static void hilbert_order(const std::vector<double>& pts, std::vector<long>& order) {
  const long n = (long)pts.size() / 3;
  long length = 2, nvert = 8;
  while (n * 8 > nvert) {
    length *= 2;
    nvert *= 8;
  }
  double mn[3], sp[3];
  for (int k = 0; k < 3; ++k) {
    double lo = 1e300, hi = -1e300;
    for (long i = 0; i < n; ++i) {
      lo = std::min(lo, pts[3 * i + k]);
      hi = std::max(hi, pts[3 * i + k]);
    }
    mn[k] = lo;
    sp[k] = double(length) / (hi - lo);
  }
  static const int trans[8][8] = {{0, 7, 6, 1, 2, 5, 4, 3}, {0, 3, 4, 6, 7, 5, 2, 1}, {0, 3, 4, 6, 7, 5, 2, 1},
                                  {2, 3, 0, 1, 6, 7, 4, 5}, {2, 3, 0, 1, 6, 7, 4, 5}, {6, 5, 2, 1, 0, 3, 4, 7},
                                  {6, 5, 2, 1, 0, 3, 4, 7}, {4, 3, 2, 5, 6, 1, 0, 7}};
  static const int first[2][2][2] = {{{5, 6}, {4, 7}}, {{2, 1}, {3, 0}}};
  std::vector<long> key(n);
#pragma omp parallel for
  for (long i = 0; i < n; ++i) {
    int q[3];
    for (int k = 0; k < 3; ++k) q[k] = int((pts[3 * i + k] - mn[k]) * sp[k]);
    int h = (int)(length / 2);
    int ux = q[0] > h, uy = q[1] > h, uz = q[2] > h;
    int cell = first[ux][uy][uz];
    long idx = cell;
    while (h > 1) {
      idx *= 8;
      if (ux) q[0] -= h;
      if (uy) q[1] -= h;
      if (uz) q[2] -= h;
      h /= 2;
      ux = q[0] > h;
      uy = q[1] > h;
      uz = q[2] > h;
      cell = trans[cell][first[ux][uy][uz]];
      idx += cell;
    }
    key[i] = idx;
  }
  order.resize(n);
  for (long i = 0; i < n; ++i) order[i] = i;
  // descending index, ties in input order
  std::stable_sort(order.begin(), order.end(), [&](long a, long b) { return key[a] > key[b]; });
}

}  // namespace xcgpu

using namespace xcgpu;

extern "C" xcgpu_status xcgpu_grid_build(xcgpu_ctx* c, int natoms, const int* Z, const double* xyz, int n_rad,
                                         int n_ang, int acc, double wthr, int smoothing, int sort, const char* table,
                                         xcgpu_grid** out) {
  return xcgpu_grid_build_partition(c, natoms, Z, xyz, n_rad, n_ang, acc, wthr, XCGPU_PARTITION_BECKE, smoothing, sort,
                                    table, out);
}

extern "C" xcgpu_status xcgpu_grid_build_partition(xcgpu_ctx* c, int natoms, const int* Z, const double* xyz,
                                                   int n_rad, int n_ang, int acc, double wthr, int partition,
                                                   int smoothing, int sort, const char* table, xcgpu_grid** out) {
  if (!c || !out || natoms <= 0 || !Z || !xyz || !table) return c ? c->fail(XCGPU_ERR_INVALID, "grid_build: bad arguments") : XCGPU_ERR_INVALID;
  if (partition != XCGPU_PARTITION_BECKE && partition != XCGPU_PARTITION_SSF)
    return c->fail(XCGPU_ERR_INVALID, "grid_build: unknown partition");
  if (acc < 0 || acc > 7) return c->fail(XCGPU_ERR_INVALID, "Invalid accuracy level chosen, must be between [1,7].");
  std::map<int, std::vector<double>> leb;
  if (!read_lebedev(table, leb)) return c->fail(XCGPU_ERR_IO, std::string("cannot read Lebedev table ") + table);
  if (acc == 0 && (n_rad <= 0 || !leb.count(n_ang)))
    return c->fail(XCGPU_ERR_INVALID, "grid_build: unsupported n_rad / n_ang");
  for (int a = 0; a < natoms; ++a)
    if (Z[a] < 1 || Z[a] > 36) return c->fail(XCGPU_ERR_UNSUPPORTED, "grid_build: elements beyond Kr are not tabulated");
  cudaSetDevice(c->device);
  // candidate points (all atoms, reference weights), atom by atom
  std::vector<double> pts, wref;
  std::vector<int> owner;
  for (int k = 0; k < natoms; ++k) {
    const int z = Z[k], row = element_row(z);
    int nr = n_rad;
    if (acc > 0) {
      static const int radAcc[7] = {13, 13, 13, 14, 15, 16, 17};
      nr = (int)(5.0 * (radAcc[acc - 1] + row - 8));
    }
    std::vector<double> r, rw;
    radial(kAlpha[z], nr, r, rw);
    static const int ldval[7][5] = {{4, 4, 4, 4, 4},     {4, 4, 4, 7, 4},      {4, 4, 7, 10, 7},    {4, 7, 10, 13, 10},
                                    {7, 10, 13, 15, 13}, {10, 13, 15, 16, 15}, {13, 15, 16, 17, 16}};
    static const double zones[3][4] = {{0.25, 0.5, 1.0, 4.5}, {0.1667, 0.5, 0.9, 3.5}, {0.1, 0.4, 0.8, 2.5}};
    const int zr = row > 3 ? 2 : row - 1;
    const int red = (row == 1 && acc > 1) ? 2 : 1;
    int sa = 0;
    for (int i = 0; i < nr; ++i) {
      int order = n_ang;
      if (acc > 0) {
        if (sa < 4 && r[i] > zones[zr][sa] * kClementiR[z]) ++sa;
        order = kOrders[ldval[acc - red][sa]];
      }
      const auto& rule = leb.at(order);
      for (int q = 0; q < order; ++q) {
        wref.push_back(rule[4 * q + 3] * rw[i] * 4.0 * M_PI);
        pts.push_back(rule[4 * q] * r[i] + xyz[3 * k]);
        pts.push_back(rule[4 * q + 1] * r[i] + xyz[3 * k + 1]);
        pts.push_back(rule[4 * q + 2] * r[i] + xyz[3 * k + 2]);
        owner.push_back(k);
      }
    }
  }
  // pair data
  std::vector<double> dist((size_t)natoms * natoms), rdist((size_t)natoms * natoms), adj((size_t)natoms * natoms);
  for (int i = 0; i < natoms; ++i)
    for (int j = 0; j < natoms; ++j) {
      double s = 0;
      for (int q = 0; q < 3; ++q) s += (xyz[3 * i + q] - xyz[3 * j + q]) * (xyz[3 * i + q] - xyz[3 * j + q]);
      dist[i + (size_t)natoms * j] = std::sqrt(s);
      rdist[i + (size_t)natoms * j] = i == j ? 0.0 : 1.0 / std::sqrt(s);
      const double chi = std::sqrt(kBraggSlaterR[Z[j]] / kBraggSlaterR[Z[i]]);
      const double u = (chi - 1) / (chi + 1);
      adj[j + (size_t)natoms * i] = std::min(0.5, std::max(-0.5, u / (u * u - 1)));
    }
  std::vector<double> min_dist(natoms, 999999999.9);
  for (int k = 0; k < natoms; ++k)
    for (int l = 0; l < natoms; ++l)
      if (l != k) min_dist[k] = std::min(min_dist[k], dist[l + (size_t)natoms * k]);
  std::vector<int> sig_off(1, 0), sig_list;
  for (int k = 0; k < natoms; ++k) {
    for (int l = 0; l < natoms; ++l)
      if (dist[l + (size_t)natoms * k] < 40.0) sig_list.push_back(l);
    sig_off.push_back((int)sig_list.size());
  }
  const long nc = (long)wref.size();
  DevBuf dA, dD, dAdj, dSo, dSl, dP, dO, dW, dWo, dDist, dMin;
  std::vector<double> A(xyz, xyz + 3 * natoms);
  auto up = [&](DevBuf& b, const void* src, size_t bytes) -> xcgpu_status {
    xcgpu_status st = b.alloc(c, bytes);
    if (st) return st;
    return c->cuda(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream), "grid upload");
  };
  xcgpu_status st = up(dA, A.data(), A.size() * 8);
  if (!st) st = up(dD, rdist.data(), rdist.size() * 8);
  if (!st) st = up(dAdj, adj.data(), adj.size() * 8);
  if (!st) st = up(dSo, sig_off.data(), sig_off.size() * 4);
  if (!st) st = up(dSl, sig_list.data(), sig_list.size() * 4);
  if (!st) st = up(dP, pts.data(), pts.size() * 8);
  if (!st) st = up(dO, owner.data(), owner.size() * 4);
  if (!st) st = up(dW, wref.data(), wref.size() * 8);
  if (!st) st = dWo.alloc(c, nc * 8);
  if (st) return st;
  if (partition == XCGPU_PARTITION_SSF) {
    if (!st) st = up(dDist, dist.data(), dist.size() * 8);
    if (!st) st = up(dMin, min_dist.data(), min_dist.size() * 8);
    if (st) return st;
    ssf_kernel<<<(unsigned)((nc + 127) / 128), 128, 0, c->stream>>>(natoms, dA.as<double>(), dDist.as<double>(),
                                                                    dMin.as<double>(), nc, dP.as<double>(),
                                                                    dO.as<int>(), dW.as<double>(), dWo.as<double>());
  } else {
    becke_kernel<<<(unsigned)((nc + 127) / 128), 128, 0, c->stream>>>(
        natoms, dA.as<double>(), dD.as<double>(), dAdj.as<double>(), dSo.as<int>(), dSl.as<int>(), nc, dP.as<double>(),
        dO.as<int>(), dW.as<double>(), smoothing, dWo.as<double>());
  }
  if ((st = c->check_launch("grid partition kernel"))) return st;
  std::vector<double> w(nc);
  if ((st = c->cuda(cudaMemcpyAsync(w.data(), dWo.p, nc * 8, cudaMemcpyDeviceToHost, c->stream), "grid weights")))
    return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "becke"))) return st;
  std::vector<double> fp, fw;
  fp.reserve(pts.size());
  fw.reserve(nc);
  for (long i = 0; i < nc; ++i)
    if (w[i] > wthr) {
      fw.push_back(w[i]);
      fp.insert(fp.end(), &pts[3 * i], &pts[3 * i] + 3);
    }
  if (sort && !fw.empty()) {
    std::vector<long> order;
    hilbert_order(fp, order);
    std::vector<double> p2(fp.size()), w2(fw.size());
    for (size_t i = 0; i < order.size(); ++i) {
      for (int q = 0; q < 3; ++q) p2[3 * i + q] = fp[3 * order[i] + q];
      w2[i] = fw[order[i]];
    }
    fp.swap(p2);
    fw.swap(w2);
  }
  return xcgpu_grid_create(c, fp.data(), fw.data(), fw.size(), out);
}
