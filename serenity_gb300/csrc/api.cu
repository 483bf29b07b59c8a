// C ABI of the xcgpu library: contexts, device memory under an HBM budget, grids,
// bases, plans (block partition + screening) and the XC stages / whole build.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "functionals.cuh"
#include "internal.h"

namespace xcgpu {

DevBuf::~DevBuf() { release(); }

void DevBuf::release() {
  if (p) {
    cudaFree(p);
    if (ctx) ctx->in_use -= bytes;
  }
  p = nullptr;
  bytes = 0;
  if (h) cudaFreeHost(h);
  h = nullptr;
  hbytes = 0;
}

xcgpu_status DevBuf::alloc_host(Ctx* c, size_t n) {
  if (n <= hbytes && h) return XCGPU_OK;
  if (h) {
    // the previous contents may still be read by an in-flight copy
    cudaStreamSynchronize(c->stream);
    cudaFreeHost(h);
  }
  h = nullptr;
  hbytes = 0;
  cudaError_t e = cudaMallocHost(&h, n);
  if (e != cudaSuccess) {
    h = nullptr;
    cudaGetLastError();
    return c->fail(XCGPU_ERR_NO_MEMORY, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
  }
  hbytes = n;
  return XCGPU_OK;
}

xcgpu_status DevBuf::alloc(Ctx* c, size_t n) {
  if (n <= bytes && p) return XCGPU_OK;
  release();
  ctx = c;
  if (n == 0) n = 16;
  if (c->in_use + n > c->budget)
    return c->fail(XCGPU_ERR_BUDGET, "device allocation of " + std::to_string(n) + " bytes exceeds the HBM budget (" +
                                         std::to_string(c->in_use) + " of " + std::to_string(c->budget) + " in use)");
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    return c->fail(XCGPU_ERR_NO_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  bytes = n;
  c->in_use += n;
  return XCGPU_OK;
}

template <class T>
static xcgpu_status upload(Ctx* c, DevBuf& b, const T* src, size_t count) {
  xcgpu_status st = b.alloc(c, count * sizeof(T));
  if (st) return st;
  if (count == 0) return XCGPU_OK;
  return c->cuda(cudaMemcpyAsync(b.p, src, count * sizeof(T), cudaMemcpyHostToDevice, c->stream), "upload");
}

static double dfact(int n) {
  double r = 1.0;
  for (int k = n; k > 1; k -= 2) r *= k;
  return r;
}
static double factorial(int n) {
  double r = 1.0;
  for (int k = 2; k <= n; ++k) r *= k;
  return r;
}
static double choose(int n, int k) {
  return (k < 0 || k > n) ? 0.0 : factorial(n) / (factorial(k) * factorial(n - k));
}

// Real solid harmonics as polynomials in the Cartesian monomials x^a y^b z^c (order
// a = l..0, b = l-a..0), m = -l..l; closed form of Helgaker, Joergensen & Olsen,
// "Molecular Electronic-Structure Theory", section 6.4.
std::vector<double> solid_harmonic_matrix(int l) {
  const int nc = ncart(l);
  std::vector<double> T((2 * l + 1) * nc, 0.0);
  auto col = [l](int a, int b) {  // index of (a, b, l-a-b)
    int k = 0;
    for (int aa = l; aa > a; --aa) k += l - aa + 1;
    return k + (l - a - b);
  };
  for (int m = -l; m <= l; ++m) {
    const int am = std::abs(m);
    const int twice_vm = m < 0 ? 1 : 0;
    const double N = std::sqrt(2.0 * factorial(l + am) * factorial(l - am) / (m == 0 ? 2.0 : 1.0)) /
                     (std::pow(2.0, am) * factorial(l));
    for (int t = 0; t <= (l - am) / 2; ++t)
      for (int u = 0; u <= t; ++u)
        for (int tv = twice_vm; tv <= am; tv += 2) {  // 2v runs over vm*2, vm*2+2, ... <= |m|
          const int sign_exp = t + (tv - twice_vm) / 2;
          const double C = (sign_exp % 2 ? -1.0 : 1.0) * std::pow(0.25, t) * choose(l, t) * choose(l - t, am + t) *
                           choose(t, u) * choose(am, tv);
          const int py = 2 * u + tv;
          const int px = 2 * t + am - py;
          T[(m + l) * nc + col(px, py)] += N * C;
        }
  }
  return T;
}

// Cartesian factors sqrt((2l-1)!! / ((2a-1)!! (2b-1)!! (2c-1)!!)) (Normalization.h:82-87).
std::vector<double> cartesian_norms(int l) {
  std::vector<double> out;
  for (int a = l; a >= 0; --a)
    for (int b = l - a; b >= 0; --b) {
      const int c = l - a - b;
      out.push_back(std::sqrt(dfact(2 * l - 1) / (dfact(2 * a - 1) * dfact(2 * b - 1) * dfact(2 * c - 1))));
    }
  return out;
}

}  // namespace xcgpu

using namespace xcgpu;

#define XC_TRY(expr)                 \
  do {                               \
    xcgpu_status _s = (expr);        \
    if (_s != XCGPU_OK) return _s;   \
  } while (0)

extern "C" {

xcgpu_status xcgpu_ctx_create(const xcgpu_config* cfg, xcgpu_ctx** out) {
  if (!out) return XCGPU_ERR_INVALID;
  *out = nullptr;
  xcgpu_ctx* c = new xcgpu_ctx();
  c->device = cfg ? cfg->device : 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= c->device) {
    cudaGetLastError();
    delete c;
    return XCGPU_ERR_CUDA;
  }
  if ((e = cudaSetDevice(c->device)) != cudaSuccess) {
    delete c;
    return XCGPU_ERR_CUDA;
  }
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->budget = (cfg && cfg->hbm_budget) ? cfg->hbm_budget : (uint64_t)(0.9 * fr);
  c->scratch_cap = (cfg && cfg->scratch_bytes) ? cfg->scratch_bytes : std::min<uint64_t>(c->budget / 4, 4ull << 30);
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return XCGPU_ERR_CUDA;
  }
  c->stream = c->own_stream;
  if (mixed_init(c) != XCGPU_OK) {
    cudaStreamDestroy(c->own_stream);
    delete c;
    return XCGPU_ERR_CUDA;
  }
  *out = c;
  return XCGPU_OK;
}

void xcgpu_ctx_destroy(xcgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->scratch.release();
  c->scratch2.release();
  c->partials.release();
  c->skip.release();
  c->batch_items.release();
  c->host_items.release();
  c->aux_by_stream.clear();
  c->arena_by_stream.clear();
  c->fp64_by_stream.clear();
  for (auto& pe : c->ev_pending) {
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  cudaStreamDestroy(c->own_stream);
  delete c;
}

const char* xcgpu_last_error(const xcgpu_ctx* c) { return c ? c->err.c_str() : "no context"; }

xcgpu_status xcgpu_set_stream(xcgpu_ctx* c, void* s) {
  if (!c) return XCGPU_ERR_INVALID;
  c->stream = s ? static_cast<cudaStream_t>(s) : c->own_stream;
  return XCGPU_OK;
}

xcgpu_status xcgpu_synchronize(xcgpu_ctx* c) {
  if (!c) return XCGPU_ERR_INVALID;
  return c->cuda(cudaStreamSynchronize(c->stream), "synchronize");
}

xcgpu_status xcgpu_set_timing(xcgpu_ctx* c, int enable) {
  if (!c) return XCGPU_ERR_INVALID;
  c->timing = enable != 0;
  return XCGPU_OK;
}

xcgpu_status xcgpu_get_timing(xcgpu_ctx* c, double* ms, uint64_t* launches) {
  if (!c) return XCGPU_ERR_INVALID;
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "timing"));
  for (auto& pe : c->ev_pending) {
    float t = 0.f;
    cudaEventElapsedTime(&t, pe.second.first, pe.second.second);
    c->t_ms[pe.first] += t;
    c->t_count[pe.first] += 1;
    c->ev_pool.push_back(pe.second.first);
    c->ev_pool.push_back(pe.second.second);
  }
  c->ev_pending.clear();
  for (int k = 0; k < kClasses; ++k) {
    if (ms) ms[k] = c->t_ms[k];
    if (launches) launches[k] = c->t_count[k];
    c->t_ms[k] = 0;
    c->t_count[k] = 0;
  }
  return XCGPU_OK;
}

uint64_t xcgpu_bytes_in_use(const xcgpu_ctx* c) { return c ? c->in_use : 0; }
uint64_t xcgpu_kernel_launches(const xcgpu_ctx* c) { return c ? c->launches : 0; }

/* ---- grid ---- */
xcgpu_status xcgpu_grid_create(xcgpu_ctx* c, const double* xyz, const double* w, uint64_t n, xcgpu_grid** out) {
  if (!c || !out || (n && (!xyz || !w))) return c ? c->fail(XCGPU_ERR_INVALID, "grid: null argument") : XCGPU_ERR_INVALID;
  cudaSetDevice(c->device);
  auto* g = new xcgpu_grid();
  g->ctx = c;
  g->n = (long)n;
  xcgpu_status st = upload(c, g->xyz, xyz, 3 * n);
  if (!st) st = upload(c, g->w, w, n);
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "grid upload");
  if (st) {
    delete g;
    return st;
  }
  *out = g;
  return XCGPU_OK;
}

uint64_t xcgpu_grid_npoints(const xcgpu_grid* g) { return g ? (uint64_t)g->n : 0; }

xcgpu_status xcgpu_grid_copy(const xcgpu_grid* g, double* xyz, double* w) {
  if (!g) return XCGPU_ERR_INVALID;
  Ctx* c = g->ctx;
  if (xyz) XC_TRY(c->cuda(cudaMemcpy(xyz, g->xyz.p, 3 * g->n * sizeof(double), cudaMemcpyDeviceToHost), "grid copy"));
  if (w) XC_TRY(c->cuda(cudaMemcpy(w, g->w.p, g->n * sizeof(double), cudaMemcpyDeviceToHost), "grid copy"));
  return XCGPU_OK;
}

void xcgpu_grid_destroy(xcgpu_grid* g) { delete g; }

/* ---- basis ---- */
xcgpu_status xcgpu_basis_create(xcgpu_ctx* c, const xcgpu_shell* shells, uint32_t nshell, xcgpu_basis** out) {
  if (!c || !out || (nshell && !shells)) return c ? c->fail(XCGPU_ERR_INVALID, "basis: null argument") : XCGPU_ERR_INVALID;
  cudaSetDevice(c->device);
  auto* B = new xcgpu_basis();
  B->ctx = c;
  B->nshell = (int)nshell;
  const double pi32 = std::pow(M_PI, 1.5);
  for (uint32_t s = 0; s < nshell; ++s) {
    const xcgpu_shell& sh = shells[s];
    if (sh.l < 0 || sh.l > kMaxL) {
      delete B;
      return c->fail(XCGPU_ERR_UNSUPPORTED, "Angular momentum too high for transformation spherical harmonics.");
    }
    if (sh.nprim <= 0 || sh.nprim > 31 || !sh.alpha || !sh.coef) {
      delete B;
      return c->fail(XCGPU_ERR_INVALID, "basis: shell without primitives");
    }
    B->l.push_back(sh.l);
    B->pure.push_back(sh.pure ? 1 : 0);
    B->nprim.push_back(sh.nprim);
    B->prim_off.push_back((int)B->alpha.size());
    B->first.push_back(B->nbf);
    for (int k = 0; k < 3; ++k) B->center.push_back(sh.center[k]);
    // libint2 convention (Shell.cpp:30-47): normalise each primitive for the x^l
    // component, then scale the contraction to unit self-overlap.
    const int L = sh.l;
    std::vector<double> cf(sh.coef, sh.coef + sh.nprim);
    for (int p = 0; p < sh.nprim; ++p) {
      const double ta = 2.0 * sh.alpha[p];
      cf[p] *= std::sqrt(std::pow(2.0, L) * std::pow(ta, L + 1.5) / (pi32 * dfact(2 * L - 1)));
    }
    double ov = 0.0;
    for (int p = 0; p < sh.nprim; ++p)
      for (int q = 0; q < sh.nprim; ++q)
        ov += dfact(2 * L - 1) * pi32 * cf[p] * cf[q] / (std::pow(2.0, L) * std::pow(sh.alpha[p] + sh.alpha[q], L + 1.5));
    for (int p = 0; p < sh.nprim; ++p) {
      B->alpha.push_back(sh.alpha[p]);
      B->coef.push_back(cf[p] / std::sqrt(ov));
    }
    B->nbf += sh.pure ? 2 * L + 1 : ncart(L);
    B->maxl = std::max(B->maxl, L);
  }
  std::vector<double> trans, cnorm;
  std::vector<int> toff, coff;
  for (int l = 0; l <= kMaxL; ++l) {
    toff.push_back((int)trans.size());
    coff.push_back((int)cnorm.size());
    auto T = solid_harmonic_matrix(l);
    auto N = cartesian_norms(l);
    trans.insert(trans.end(), T.begin(), T.end());
    cnorm.insert(cnorm.end(), N.begin(), N.end());
  }
  xcgpu_status st = XCGPU_OK;
  if (!st) st = upload(c, B->d_l, B->l.data(), nshell);
  if (!st) st = upload(c, B->d_pure, B->pure.data(), nshell);
  if (!st) st = upload(c, B->d_nprim, B->nprim.data(), nshell);
  if (!st) st = upload(c, B->d_prim_off, B->prim_off.data(), nshell);
  if (!st) st = upload(c, B->d_first, B->first.data(), nshell);
  if (!st) st = upload(c, B->d_center, B->center.data(), B->center.size());
  if (!st) st = upload(c, B->d_alpha, B->alpha.data(), B->alpha.size());
  if (!st) st = upload(c, B->d_coef, B->coef.data(), B->coef.size());
  if (!st) st = upload(c, B->d_trans, trans.data(), trans.size());
  if (!st) st = upload(c, B->d_cnorm, cnorm.data(), cnorm.size());
  if (!st) st = upload(c, B->d_toff, toff.data(), toff.size());
  if (!st) st = upload(c, B->d_coff, coff.data(), coff.size());
  // FP32 pairs carry the exponents and coefficients to ~2^-48: a single FP32 rounding
  // of them is the same relative error at every grid point (all atoms of an element
  // share it), which would bias the density by a few 1e-8
  std::vector<float> prim4;
  for (size_t i = 0; i < B->alpha.size(); ++i) {
    const float ah = (float)B->alpha[i], ch = (float)B->coef[i];
    prim4.push_back(ah);
    prim4.push_back(ch);
    prim4.push_back((float)(B->alpha[i] - (double)ah));
    prim4.push_back((float)(B->coef[i] - (double)ch));
  }
  if (!st) st = upload(c, B->d_prim4, prim4.data(), prim4.size());
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "basis upload");
  if (st) {
    delete B;
    return st;
  }
  DevBasis& d = B->dev;
  d.nshell = B->nshell;
  d.nbf = B->nbf;
  d.maxl = B->maxl;
  d.l = B->d_l.as<int>();
  d.pure = B->d_pure.as<int>();
  d.nprim = B->d_nprim.as<int>();
  d.prim_off = B->d_prim_off.as<int>();
  d.first = B->d_first.as<int>();
  d.center = B->d_center.as<double>();
  d.alpha = B->d_alpha.as<double>();
  d.coef = B->d_coef.as<double>();
  d.trans = B->d_trans.as<double>();
  d.cnorm = B->d_cnorm.as<double>();
  d.trans_off = B->d_toff.as<int>();
  d.cnorm_off = B->d_coff.as<int>();
  d.prim4 = B->d_prim4.as<float4>();
  *out = B;
  return XCGPU_OK;
}

uint32_t xcgpu_basis_nbf(const xcgpu_basis* b) { return b ? (uint32_t)b->nbf : 0; }

xcgpu_status xcgpu_basis_coefs(const xcgpu_basis* b, uint32_t s, double* out) {
  if (!b || (int)s >= b->nshell || !out) return XCGPU_ERR_INVALID;
  for (int i = 0; i < b->nprim[s]; ++i) out[i] = b->coef[b->prim_off[s] + i];
  return XCGPU_OK;
}

void xcgpu_basis_destroy(xcgpu_basis* b) { delete b; }

/* ---- plan ---- */
xcgpu_status xcgpu_plan_create(xcgpu_ctx* c, xcgpu_grid* g, xcgpu_basis* B, uint32_t max_block, double thr,
                               xcgpu_plan** out) {
  if (!c || !g || !B || !out) return c ? c->fail(XCGPU_ERR_INVALID, "plan: null argument") : XCGPU_ERR_INVALID;
  if (max_block == 0 || max_block > (uint32_t)kBlockPoints)
    return c->fail(XCGPU_ERR_UNSUPPORTED, "plan: max_block must be in 1..128");
  if (g->ctx != c || B->ctx != c) return c->fail(XCGPU_ERR_INVALID, "plan: grid and basis belong to another context");
  cudaSetDevice(c->device);
  auto* P = new xcgpu_plan();
  P->ctx = c;
  P->grid = g;
  P->basis = B;
  P->max_block = (int)max_block;
  P->radial_threshold = thr;
  P->nblocks = (int)((g->n + max_block - 1) / max_block);
  const int nb = P->nblocks, ns = B->nshell;
  DevBuf flags, nfn;
  xcgpu_status st = flags.alloc(c, (size_t)nb * ns + 1);
  if (!st) st = nfn.alloc(c, (size_t)nb * sizeof(int) + 4);
  if (!st) st = launch_screen(c, B->dev, g->xyz.as<double>(), g->n, P->max_block, nb, thr, flags.as<unsigned char>(),
                              nfn.as<int>());
  std::vector<unsigned char> hf((size_t)nb * ns);
  if (!st && nb)
    st = c->cuda(cudaMemcpyAsync(hf.data(), flags.p, hf.size(), cudaMemcpyDeviceToHost, c->stream), "plan flags");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "plan screen");
  if (st) {
    delete P;
    return st;
  }
  P->sh_off.assign(1, 0);
  P->fn_off.assign(1, 0);
  P->work_off.assign(1, 0);
  for (int b = 0; b < nb; ++b) {
    for (int s = 0; s < ns; ++s)
      if (hf[(size_t)b * ns + s]) {
        P->sh_list.push_back(s);
        const int nf = B->pure[s] ? 2 * B->l[s] + 1 : ncart(B->l[s]);
        for (int f = 0; f < nf; ++f) P->fn_list.push_back(B->first[s] + f);
      }
    P->sh_off.push_back((int)P->sh_list.size());
    P->fn_off.push_back((int)P->fn_list.size());
    const int nact = P->fn_off[b + 1] - P->fn_off[b];
    P->max_active = std::max(P->max_active, nact);
    const long npts = std::min<long>(P->max_block, g->n - (long)b * P->max_block);
    P->flops += 4.0 * npts * (double)nact * nact;
    const int nt = (nact + 63) / 64;
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < nt; ++j) {
        P->work.push_back(b);
        P->work.push_back(i);
        P->work.push_back(j);
      }
    P->work_off.push_back((long)P->work.size() / 3);
  }
  std::vector<ShellRec> rec(P->sh_list.size());
  for (int b = 0; b < nb; ++b) {
    int f0 = 0;
    for (int k = P->sh_off[b]; k < P->sh_off[b + 1]; ++k) {
      const int s = P->sh_list[k];
      ShellRec& r = rec[k];
      for (int q = 0; q < 3; ++q) {
        const double a = B->center[3 * s + q];
        r.ah[q] = (float)a;
        r.al[q] = (float)(a - (double)r.ah[q]);
      }
      const int nf = B->pure[s] ? 2 * B->l[s] + 1 : ncart(B->l[s]);
      r.info = B->l[s] | (B->pure[s] << 3) | (B->nprim[s] << 4) | (nf << 9) | (f0 << 14);
      r.prim0 = B->prim_off[s];
      f0 += nf;
    }
  }
  st = upload(c, P->d_rec, rec.data(), rec.size());
  if (!st) st = upload(c, P->d_sh_off, P->sh_off.data(), P->sh_off.size());
  if (!st) st = upload(c, P->d_sh_list, P->sh_list.data(), P->sh_list.size());
  if (!st) st = upload(c, P->d_fn_off, P->fn_off.data(), P->fn_off.size());
  if (!st) st = upload(c, P->d_fn_list, P->fn_list.data(), P->fn_list.size());
  if (!st) st = upload(c, P->d_work, P->work.data(), P->work.size());
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "plan upload");
  if (st) {
    delete P;
    return st;
  }
  DevPlan& d = P->dev;
  d.nblocks = nb;
  d.max_block = P->max_block;
  d.max_active = P->max_active;
  d.nbf = B->nbf;
  d.npoints = g->n;
  d.xyz = g->xyz.as<double>();
  d.w = g->w.as<double>();
  d.sh_off = P->d_sh_off.as<int>();
  d.sh_list = P->d_sh_list.as<int>();
  d.fn_off = P->d_fn_off.as<int>();
  d.fn_list = P->d_fn_list.as<int>();
  d.rec = P->d_rec.as<ShellRec>();
  d.radial_threshold = thr;
  d.exponent_threshold = thr > 0 ? -std::log(thr) : HUGE_VAL;
  *out = P;
  return XCGPU_OK;
}

xcgpu_status xcgpu_plan_get_stats(const xcgpu_plan* P, xcgpu_plan_stats* s) {
  if (!P || !s) return XCGPU_ERR_INVALID;
  s->nblocks = (uint32_t)P->nblocks;
  s->max_block = (uint32_t)P->max_block;
  s->nbf = (uint32_t)P->basis->nbf;
  s->max_active = (uint32_t)P->max_active;
  s->npoints = (uint64_t)P->grid->n;
  s->sum_active = P->fn_list.size();
  s->flops_per_spin = P->flops;
  return XCGPU_OK;
}

int32_t xcgpu_block_active(const xcgpu_plan* P, uint32_t b, int32_t* idx) {
  if (!P || (int)b >= P->nblocks) return -1;
  const int n = P->fn_off[b + 1] - P->fn_off[b];
  if (idx)
    for (int i = 0; i < n; ++i) idx[i] = P->fn_list[P->fn_off[b] + i];
  return n;
}

void xcgpu_plan_destroy(xcgpu_plan* P) { delete P; }

xcgpu_status xcgpu_block_on_grid(xcgpu_plan* P, uint32_t b, int deriv, double* values, double* grad, double* hess,
                                 int32_t* negligible) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if (deriv > 2 || deriv < 0)
    return c->fail(XCGPU_ERR_UNSUPPORTED, "Third derivatives of basis functions on the grid are not implemented!");
  if ((int)b >= P->nblocks) return c->fail(XCGPU_ERR_INVALID, "block index out of range");
  cudaSetDevice(c->device);
  const int nbf = P->basis->nbf;
  const int npts = (int)std::min<long>(P->max_block, P->grid->n - (long)b * P->max_block);
  const int ncomp = deriv == 0 ? 1 : deriv == 1 ? 4 : 10;
  const size_t plane = (size_t)npts * nbf;
  DevBuf buf;
  XC_TRY(buf.alloc(c, ncomp * plane * sizeof(double)));
  XC_TRY(c->cuda(cudaMemsetAsync(buf.p, 0, ncomp * plane * sizeof(double), c->stream), "memset"));
  XC_TRY(launch_block_values(c, P->basis->dev, P->dev, (int)b, deriv, buf.as<double>(), npts));
  std::vector<double> h(ncomp * plane);
  XC_TRY(c->cuda(cudaMemcpyAsync(h.data(), buf.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "copy"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "block_on_grid"));
  if (values) std::memcpy(values, h.data(), plane * sizeof(double));
  if (grad && deriv >= 1) std::memcpy(grad, h.data() + plane, 3 * plane * sizeof(double));
  if (hess && deriv >= 2) std::memcpy(hess, h.data() + 4 * plane, 6 * plane * sizeof(double));
  if (negligible) {
    for (int i = 0; i < nbf; ++i) negligible[i] = 1;
    for (int i = P->fn_off[b]; i < P->fn_off[b + 1]; ++i) negligible[P->fn_list[i]] = 0;
  }
  return XCGPU_OK;
}

int xcgpu_functional_is_gga(int func) { return xc::is_gga(func) ? 1 : 0; }

}  // extern "C"

/* ---- stages and the whole build ------------------------------------------------------ */
namespace xcgpu {

// Chunks of consecutive blocks whose FP64 slabs fit the scratch cap; computed
// once per plan (slab offsets resident on the device).
struct Chunks {
  std::vector<int> bounds;  // chunk k covers blocks [bounds[k], bounds[k+1])
  long max_chunk_doubles = 0;
};

static xcgpu_status prep_chunks(xcgpu_plan* P) {
  if (P->chunks_ready) return XCGPU_OK;
  Ctx* c = P->ctx;
  const long cap = std::max<long>((long)(c->scratch_cap / sizeof(double)), 4L * kBlockPoints * std::max(P->max_active, 1));
  std::vector<long> slab_off;
  P->chunk_bounds.assign(1, 0);
  long cur = 0, mx = 0;
  for (int b = 0; b < P->nblocks; ++b) {
    const long need = 4L * kBlockPoints * (P->fn_off[b + 1] - P->fn_off[b]);
    if (cur + need > cap && cur > 0) {
      P->chunk_bounds.push_back(b);
      mx = std::max(mx, cur);
      cur = 0;
    }
    slab_off.push_back(cur);
    cur += need;
  }
  P->chunk_max_doubles = std::max(mx, cur);
  P->chunk_bounds.push_back(P->nblocks);
  XC_TRY(upload(c, P->w_slab, slab_off.data(), slab_off.size()));
  // plans are shared by builds on several streams: the offsets must be on the device
  // before any stream's kernels can read them (once per plan)
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "plan chunks"));
  P->chunks_ready = true;
  return XCGPU_OK;
}

// the calling stream's FP64 slab scratch, grown to the plan's largest chunk (growth
// waits for the stream: earlier builds on it may still read the old slabs)
static xcgpu_status fp64_scratch(xcgpu_plan* P, double** out) {
  Ctx* c = P->ctx;
  DevBuf& b = c->on_stream(c->fp64_by_stream);
  const size_t need = std::max<long>(P->chunk_max_doubles, 1) * sizeof(double);
  if (b.p && b.bytes < need) XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "fp64 scratch"));
  XC_TRY(b.alloc(c, need));
  *out = b.as<double>();
  return XCGPU_OK;
}

static xcgpu_status stage_density(xcgpu_plan* P, int nspin, const double* dP, double* rho, double* grad) {
  Ctx* c = P->ctx;
  XC_TRY(prep_chunks(P));
  double* scr = nullptr;
  XC_TRY(fp64_scratch(P, &scr));
  for (size_t k = 0; k + 1 < P->chunk_bounds.size(); ++k) {
    const int b0 = P->chunk_bounds[k], b1 = P->chunk_bounds[k + 1];
    const long* so = P->w_slab.as<long>() + b0;
    XC_TRY(fp64_eval_chunk(c, P->basis->dev, P->dev, b0, b1, so, scr, 1));
    XC_TRY(fp64_density_chunk(c, P->dev, b0, b1, so, scr, nspin, dP, rho, grad));
  }
  return XCGPU_OK;
}

// skip: nspin * nblocks + 1 bytes of block skip flags (written here)
static xcgpu_status stage_adder(xcgpu_plan* P, int nspin, const double* v, const double* g, double thr,
                                unsigned char* skip, double* F) {
  Ctx* c = P->ctx;
  XC_TRY(prep_chunks(P));
  XC_TRY(launch_block_skip_flags(c, P->dev, nspin, v, g, thr, skip));
  double* scr = nullptr;
  XC_TRY(fp64_scratch(P, &scr));
  for (size_t k = 0; k + 1 < P->chunk_bounds.size(); ++k) {
    const int b0 = P->chunk_bounds[k], b1 = P->chunk_bounds[k + 1];
    const long* so = P->w_slab.as<long>() + b0;
    XC_TRY(fp64_eval_chunk(c, P->basis->dev, P->dev, b0, b1, so, scr, 1));
    XC_TRY(fp64_adder_chunk(c, P->dev, P->d_work.as<int>(), P->work_off[b0], P->work_off[b1], b0, b1, so, scr, nspin,
                            v, g, skip, F));
  }
  return XCGPU_OK;
}

static xcgpu_status stage_adder(xcgpu_plan* P, int nspin, const double* v, const double* g, double thr, double* F) {
  XC_TRY(P->w_skip.alloc(P->ctx, (size_t)nspin * P->nblocks + 1));
  return stage_adder(P, nspin, v, g, thr, P->w_skip.as<unsigned char>(), F);
}

template <class T>
static xcgpu_status to_device(Ctx* c, DevBuf& tmp, const T* src, size_t count, int mem, const T** dst) {
  if (mem == XCGPU_MEM_DEVICE) {
    *dst = src;
    return XCGPU_OK;
  }
  XC_TRY(upload(c, tmp, src, count));
  *dst = tmp.as<T>();
  return XCGPU_OK;
}

// status for the error word of the mixed-precision kernels (0: none)
static xcgpu_status device_error(Ctx* c, int herr, const char* where) {
  if (herr == 0) return XCGPU_OK;
  if (herr == 2)
    return c->fail(XCGPU_ERR_INVALID, std::string(where) + ": a block needs more basis scratch than was sized for it");
  return c->fail(XCGPU_ERR_TIMEOUT, std::string(where) + ": a bounded device-side wait gave up (tensor-core pipeline)");
}

struct BuildReq {
  xcgpu_plan* plan;
  int func, nspin;
  double thr;
  const double* P;
  double* V;
  double* exc_nel;
};

// work buffers kept in the plan, for the entry points that run one build at a time on
// a plan (non-additive potentials, gradients, response kernels)
static xcgpu_status ensure_work(xcgpu_plan* P, int nspin, bool gga, bool mixed) {
  Ctx* c = P->ctx;
  const long n = P->grid->n;
  const int nbf = P->basis->nbf;
  XC_TRY(P->w_rho.alloc(c, (size_t)nspin * n * sizeof(double)));
  XC_TRY(P->w_epuv.alloc(c, (size_t)n * sizeof(double)));
  XC_TRY(P->w_dfdrho.alloc(c, (size_t)nspin * n * sizeof(double)));
  if (gga) {
    XC_TRY(P->w_grad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
    XC_TRY(P->w_dfdgrad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
  }
  XC_TRY(P->w_partials.alloc(c, 2 * ((n + 127) / 128) * sizeof(double) + 16));
  XC_TRY(P->w_skip.alloc(c, (size_t)nspin * P->nblocks + 1));
  XC_TRY(P->w_fskip.alloc(c, (size_t)(n + kSkipBlock - 1) / kSkipBlock + 1));
  if (mixed) XC_TRY(P->w_psplit.alloc(c, psplit_bytes(nspin, nbf)));
  return XCGPU_OK;
}

// work buffers of one build (FuncPotential::getMatrix), 256-byte aligned slices of
// one allocation; with base == nullptr only the size is computed
struct BuildWork {
  double *rho = nullptr, *grad = nullptr, *epuv = nullptr, *dfdrho = nullptr, *dfdgrad = nullptr, *partials = nullptr;
  unsigned char *skip = nullptr, *fskip = nullptr;
  float* psplit = nullptr;
};

static size_t layout_work(const BuildReq& r, bool mixed, uint8_t* base, BuildWork& w) {
  const long n = r.plan->grid->n;
  const size_t ns = r.nspin, nbf = r.plan->basis->nbf;
  size_t off = 0;
  auto take = [&](size_t bytes) -> void* {
    void* p = base ? base + off : nullptr;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  w = BuildWork();
  w.rho = static_cast<double*>(take(ns * n * sizeof(double)));
  w.epuv = static_cast<double*>(take(n * sizeof(double)));
  w.dfdrho = static_cast<double*>(take(ns * n * sizeof(double)));
  if (xc::is_gga(r.func)) {
    w.grad = static_cast<double*>(take(ns * 3 * n * sizeof(double)));
    w.dfdgrad = static_cast<double*>(take(ns * 3 * n * sizeof(double)));
  }
  w.partials = static_cast<double*>(take(2 * ((n + 127) / 128) * sizeof(double) + 16));
  w.skip = static_cast<unsigned char*>(take(ns * r.plan->nblocks + 1));
  w.fskip = static_cast<unsigned char*>(take((n + kSkipBlock - 1) / kSkipBlock + 1));
  if (mixed) w.psplit = static_cast<float*>(take(psplit_bytes((int)ns, (int)nbf)));
  return off;
}

// the work buffers of every request, carved from the calling stream's arena; the arena
// grows (after the stream's earlier builds have finished with it) and never shrinks, so
// a repeated batch allocates nothing and can be captured in a graph
static xcgpu_status carve_work(Ctx* c, const std::vector<BuildReq>& reqs, bool mixed, std::vector<BuildWork>& out) {
  out.resize(reqs.size());
  size_t total = 0;
  for (size_t i = 0; i < reqs.size(); ++i) total += layout_work(reqs[i], mixed, nullptr, out[i]);
  DevBuf& a = c->on_stream(c->arena_by_stream);
  if (a.p && a.bytes < total) XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "work arena"));
  XC_TRY(a.alloc(c, total));
  uint8_t* base = a.as<uint8_t>();
  for (size_t i = 0; i < reqs.size(); ++i) base += layout_work(reqs[i], mixed, base, out[i]);
  return XCGPU_OK;
}

// Whole builds (FuncPotential::getMatrix) for a list of requests, all on the context
// stream without host synchronisation: mixed precision runs one persistent launch per
// heavy stage over the blocks of every request.  Plans are only read, so requests may
// share a plan (several density matrices of one geometry in one batch).
static xcgpu_status run_builds(Ctx* c, std::vector<BuildReq>& reqs, int precision) {
  const bool mixed = precision == XCGPU_PREC_MIXED;
  std::vector<BuildWork> bw;
  XC_TRY(carve_work(c, reqs, mixed, bw));
  int* counter = nullptr;
  XC_TRY(c->aux(&counter));
  int* err = counter + 2;
  XC_TRY(c->cuda(cudaMemsetAsync(counter, 0, 4 * sizeof(int), c->stream), "memset aux"));
  std::vector<MixedWork> work;
  // mixed precision with 128-point blocks (the functional's block skip then coincides
  // with the plan's blocks): one kernel per launch does density, functional and Vxc of
  // each block, the basis values evaluated once
  bool fused = mixed;
  for (const auto& r : reqs) fused = fused && r.plan->max_block == kSkipBlock;
  if (fused) {
    for (size_t i = 0; i < reqs.size(); ++i) {
      const BuildReq& r = reqs[i];
      xcgpu_plan* P = r.plan;
      MixedWork mw{&P->basis->dev, &P->dev, r.nspin, bw[i].psplit, nullptr, nullptr, nullptr, nullptr, nullptr, r.V};
      mw.func = r.func;
      mw.thr = r.thr;
      mw.partials = bw[i].partials;
      mw.Pm = r.P;
      mw.exc_nel = r.exc_nel;
      work.push_back(mw);
    }
    return mixed_build_batch(c, work, counter, err);  // split, build kernel, mirror and sums
  }
  bool chunked = !mixed;
  for (const auto& r : reqs) chunked = chunked && r.plan->max_block == kSkipBlock;
  if (chunked) {
    // FP64 build chunk by chunk: the basis slabs of a chunk of blocks serve its density,
    // and after the functional at the chunk's points, its Vxc (the basis is evaluated
    // once per build).  Per point and block the same arithmetic as the three separate
    // phases (FuncPotential.cpp:74-110): E_xc and N_el from the same 128-point partial
    // sums in the same order; only the order of the FP64 atomic adds into V differs.
    for (size_t i = 0; i < reqs.size(); ++i) {
      const BuildReq& r = reqs[i];
      const BuildWork& w = bw[i];
      xcgpu_plan* P = r.plan;
      const long n = P->grid->n;
      const int nbf = P->basis->nbf;
      XC_TRY(c->cuda(cudaMemsetAsync(r.V, 0, (size_t)r.nspin * nbf * nbf * sizeof(double), c->stream), "memset V"));
      XC_TRY(prep_chunks(P));
      double* scr = nullptr;
      XC_TRY(fp64_scratch(P, &scr));
      for (size_t k = 0; k + 1 < P->chunk_bounds.size(); ++k) {
        const int b0 = P->chunk_bounds[k], b1 = P->chunk_bounds[k + 1];
        const long* so = P->w_slab.as<long>() + b0;
        const long p0 = (long)b0 * P->max_block, p1 = std::min(n, (long)b1 * P->max_block);
        XC_TRY(fp64_eval_chunk(c, P->basis->dev, P->dev, b0, b1, so, scr, 1));
        XC_TRY(fp64_density_chunk(c, P->dev, b0, b1, so, scr, r.nspin, r.P, w.rho, w.grad));
        XC_TRY(launch_functional_range(c, r.func, r.nspin, n, kSkipBlock, p0, p1, w.rho, w.grad, w.epuv, w.dfdrho,
                                       w.dfdgrad, P->dev.w, w.partials, w.fskip));
        XC_TRY(launch_block_skip_flags_range(c, P->dev, r.nspin, w.dfdrho, w.dfdgrad, r.thr, w.skip, b0, b1));
        XC_TRY(fp64_adder_chunk(c, P->dev, P->d_work.as<int>(), P->work_off[b0], P->work_off[b1], b0, b1, so, scr,
                                r.nspin, w.dfdrho, w.dfdgrad, w.skip, r.V));
      }
      const int nparts = (int)((n + 127) / 128);
      if (nparts) XC_TRY(launch_sum_partials(c, w.partials, nparts, 2, r.exc_nel));
      else XC_TRY(c->cuda(cudaMemsetAsync(r.exc_nel, 0, 2 * sizeof(double), c->stream), "memset sums"));
    }
    return XCGPU_OK;
  }
  // 1. rho, grad rho
  for (size_t i = 0; i < reqs.size(); ++i) {
    const BuildReq& r = reqs[i];
    const BuildWork& w = bw[i];
    xcgpu_plan* P = r.plan;
    if (mixed) {
      XC_TRY(mixed_split(c, r.P, r.nspin, P->basis->nbf, w.psplit));
      work.push_back(MixedWork{&P->basis->dev, &P->dev, r.nspin, w.psplit, w.rho, w.grad, w.dfdrho, w.dfdgrad, w.skip,
                               r.V});
    } else {
      XC_TRY(stage_density(P, r.nspin, r.P, w.rho, w.grad));
    }
  }
  if (mixed) XC_TRY(mixed_density_batch(c, work, counter, err));
  // 2. functional, E_xc and N_el, adder skip flags
  for (size_t i = 0; i < reqs.size(); ++i) {
    const BuildReq& r = reqs[i];
    const BuildWork& w = bw[i];
    xcgpu_plan* P = r.plan;
    const long n = P->grid->n;
    int nparts = 0;
    XC_TRY(launch_functional(c, r.func, r.nspin, n, kSkipBlock, w.rho, w.grad, w.epuv, w.dfdrho, w.dfdgrad, P->dev.w,
                             w.partials, &nparts, w.fskip));
    if (nparts) XC_TRY(launch_sum_partials(c, w.partials, nparts, 2, r.exc_nel));
    else XC_TRY(c->cuda(cudaMemsetAsync(r.exc_nel, 0, 2 * sizeof(double), c->stream), "memset sums"));
    const int nbf = P->basis->nbf;
    XC_TRY(c->cuda(cudaMemsetAsync(r.V, 0, (size_t)r.nspin * nbf * nbf * sizeof(double), c->stream), "memset V"));
    if (mixed)
      XC_TRY(launch_block_skip_flags(c, P->dev, r.nspin, w.dfdrho, w.dfdgrad, r.thr, w.skip));
    else
      XC_TRY(stage_adder(P, r.nspin, w.dfdrho, w.dfdgrad, r.thr, w.skip, r.V));
  }
  // 3. Vxc (mixed: one launch for all requests)
  if (mixed) XC_TRY(mixed_adder_batch(c, work, counter + 1, err));
  return XCGPU_OK;
}

}  // namespace xcgpu

extern "C" {

xcgpu_status xcgpu_density(xcgpu_plan* P, int nspin, const double* Pm, double* rho, double* grad, int precision,
                           int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if ((nspin != 1 && nspin != 2) || !Pm || !rho) return c->fail(XCGPU_ERR_INVALID, "density: bad arguments");
  cudaSetDevice(c->device);
  const long n = P->grid->n;
  const int nbf = P->basis->nbf;
  DevBuf dPm, drho, dgrad;
  const double* Pd = nullptr;
  XC_TRY(to_device(c, dPm, Pm, (size_t)nspin * nbf * nbf, mem, &Pd));
  double* r = rho;
  double* gr = grad;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(drho.alloc(c, (size_t)nspin * n * sizeof(double)));
    r = drho.as<double>();
    if (grad) {
      XC_TRY(dgrad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
      gr = dgrad.as<double>();
    }
  }
  XC_TRY(c->cuda(cudaMemsetAsync(r, 0, (size_t)nspin * n * sizeof(double), c->stream), "memset rho"));
  if (precision == XCGPU_PREC_MIXED) {
    XC_TRY(P->w_aux.alloc(c, 4 * sizeof(int)));
    XC_TRY(c->cuda(cudaMemsetAsync(P->w_aux.p, 0, 4 * sizeof(int), c->stream), "memset aux"));
    XC_TRY(P->w_psplit.alloc(c, psplit_bytes(nspin, nbf)));
    XC_TRY(mixed_split(c, Pd, nspin, nbf, P->w_psplit.as<float>()));
    std::vector<MixedWork> work(1);
    work[0] = MixedWork{&P->basis->dev, &P->dev, nspin, P->w_psplit.as<float>(), r, gr, nullptr, nullptr, nullptr,
                        nullptr};
    XC_TRY(mixed_density_batch(c, work, P->w_aux.as<int>(), P->w_aux.as<int>() + 2));
  } else {
    XC_TRY(stage_density(P, nspin, Pd, r, gr));
  }
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(c->cuda(cudaMemcpyAsync(rho, r, (size_t)nspin * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "rho"));
    if (grad)
      XC_TRY(c->cuda(cudaMemcpyAsync(grad, gr, (size_t)nspin * 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                     "grad"));
  }
  int herr = 0;
  if (precision == XCGPU_PREC_MIXED)
    XC_TRY(c->cuda(cudaMemcpyAsync(&herr, P->w_aux.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream),
                   "error word"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "density"));
  return device_error(c, herr, "density");
}

xcgpu_status xcgpu_functional(xcgpu_ctx* c, int func, int nspin, uint64_t n, uint32_t skip_block, const double* rho,
                              const double* grad, double* epuv, double* dfdrho, double* dfdgrad, int mem) {
  return xcgpu_functional_prec(c, func, nspin, n, skip_block, rho, grad, epuv, dfdrho, dfdgrad, XCGPU_PREC_FP64, mem);
}

xcgpu_status xcgpu_functional_prec(xcgpu_ctx* c, int func, int nspin, uint64_t n, uint32_t skip_block,
                                   const double* rho, const double* grad, double* epuv, double* dfdrho,
                                   double* dfdgrad, int precision, int mem) {
  if (!c) return XCGPU_ERR_INVALID;
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "functional: unknown precision");
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "unknown functional");
  const bool gga = xc::is_gga(func);
  if ((nspin != 1 && nspin != 2) || !rho || !epuv || !dfdrho || (gga && (!grad || !dfdgrad)))
    return c->fail(XCGPU_ERR_INVALID, "functional: bad arguments");
  cudaSetDevice(c->device);
  DevBuf a, b, o1, o2, o3;
  const double *dr = rho, *dg = grad;
  double *e = epuv, *v = dfdrho, *vg = dfdgrad;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, a, rho, (size_t)nspin * n));
    dr = a.as<double>();
    if (gga) {
      XC_TRY(upload(c, b, grad, (size_t)nspin * 3 * n));
      dg = b.as<double>();
    }
    XC_TRY(o1.alloc(c, n * sizeof(double)));
    XC_TRY(o2.alloc(c, (size_t)nspin * n * sizeof(double)));
    e = o1.as<double>();
    v = o2.as<double>();
    if (gga) {
      XC_TRY(o3.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
      vg = o3.as<double>();
    }
  }
  XC_TRY(launch_functional(c, func, nspin, (long)n, (int)skip_block, dr, gga ? dg : nullptr, e, v, gga ? vg : nullptr,
                           nullptr, nullptr, nullptr, nullptr, precision == XCGPU_PREC_MIXED));
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(c->cuda(cudaMemcpyAsync(epuv, e, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "epuv"));
    XC_TRY(c->cuda(cudaMemcpyAsync(dfdrho, v, (size_t)nspin * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                   "dfdrho"));
    if (gga)
      XC_TRY(c->cuda(
          cudaMemcpyAsync(dfdgrad, vg, (size_t)nspin * 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
          "dfdgrad"));
  }
  return c->cuda(cudaStreamSynchronize(c->stream), "functional");
}

xcgpu_status xcgpu_add_scalar(xcgpu_plan* P, double thr, int nspin, const double* v, const double* g, double* F,
                              int precision, int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if ((nspin != 1 && nspin != 2) || !v || !F) return c->fail(XCGPU_ERR_INVALID, "add_scalar: bad arguments");
  cudaSetDevice(c->device);
  const long n = P->grid->n;
  const int nbf = P->basis->nbf;
  DevBuf dv, dg, dF;
  const double *vd = nullptr, *gd = nullptr;
  XC_TRY(to_device(c, dv, v, (size_t)nspin * n, mem, &vd));
  if (g) XC_TRY(to_device(c, dg, g, (size_t)nspin * 3 * n, mem, &gd));
  double* Fd = F;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, dF, F, (size_t)nspin * nbf * nbf));
    Fd = dF.as<double>();
  }
  if (precision == XCGPU_PREC_MIXED) {
    // the mixed adder accumulates into a zeroed matrix and symmetrises it; add that to F
    DevBuf tmpF;
    XC_TRY(tmpF.alloc(c, (size_t)nspin * nbf * nbf * sizeof(double)));
    XC_TRY(c->cuda(cudaMemsetAsync(tmpF.p, 0, (size_t)nspin * nbf * nbf * sizeof(double), c->stream), "memset"));
    XC_TRY(P->w_aux.alloc(c, 4 * sizeof(int)));
    XC_TRY(c->cuda(cudaMemsetAsync(P->w_aux.p, 0, 4 * sizeof(int), c->stream), "memset aux"));
    XC_TRY(P->w_skip.alloc(c, (size_t)nspin * P->nblocks + 1));
    XC_TRY(launch_block_skip_flags(c, P->dev, nspin, vd, gd, thr, P->w_skip.as<unsigned char>()));
    std::vector<MixedWork> work(1);
    work[0] = MixedWork{&P->basis->dev, &P->dev, nspin, nullptr, nullptr, nullptr, vd, gd,
                        P->w_skip.as<unsigned char>(), tmpF.as<double>()};
    XC_TRY(mixed_adder_batch(c, work, P->w_aux.as<int>() + 1, P->w_aux.as<int>() + 2));
    XC_TRY(launch_axpy(c, (long)nspin * nbf * nbf, tmpF.as<double>(), Fd));
  } else {
    XC_TRY(stage_adder(P, nspin, vd, gd, thr, Fd));
  }
  if (mem == XCGPU_MEM_HOST)
    XC_TRY(c->cuda(cudaMemcpyAsync(F, Fd, (size_t)nspin * nbf * nbf * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                   "F"));
  int herr = 0;
  if (precision == XCGPU_PREC_MIXED)
    XC_TRY(c->cuda(cudaMemcpyAsync(&herr, P->w_aux.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream),
                   "error word"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "add_scalar"));
  return device_error(c, herr, "add_scalar");
}

xcgpu_status xcgpu_vxc(xcgpu_plan* P, int func, int nspin, int precision, double thr, const double* Pm, double* V,
                       double* Exc, double* Nel, int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "unknown functional");
  if ((nspin != 1 && nspin != 2) || !Pm || !V) return c->fail(XCGPU_ERR_INVALID, "vxc: bad arguments");
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "vxc: unknown precision");
  cudaSetDevice(c->device);
  const int nbf = P->basis->nbf;
  const double* Pd = Pm;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, P->w_P, Pm, (size_t)nspin * nbf * nbf));
    Pd = P->w_P.as<double>();
  }
  double* Vd = V;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(P->w_V.alloc(c, (size_t)nspin * nbf * nbf * sizeof(double)));
    Vd = P->w_V.as<double>();
  }
  XC_TRY(P->w_sums.alloc(c, 2 * sizeof(double)));
  std::vector<BuildReq> reqs(1);
  reqs[0] = BuildReq{P, func, nspin, thr, Pd, Vd, P->w_sums.as<double>()};
  XC_TRY(run_builds(c, reqs, precision));
  double hs[2] = {0, 0};
  int herr = 0;
  XC_TRY(c->cuda(cudaMemcpyAsync(hs, P->w_sums.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "sums"));
  int* aux = nullptr;
  XC_TRY(c->aux(&aux));
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, aux + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  if (mem == XCGPU_MEM_HOST)
    XC_TRY(c->cuda(cudaMemcpyAsync(V, Vd, (size_t)nspin * nbf * nbf * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                   "V"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "vxc"));
  if (herr) return device_error(c, herr, "vxc");
  if (Exc) *Exc = hs[0];
  if (Nel) *Nel = hs[1];
  return XCGPU_OK;
}

xcgpu_status xcgpu_vxc_batch(xcgpu_ctx* c, const xcgpu_request* reqs, uint32_t n, int precision, int flags) {
  if (!c || (n && !reqs)) return c ? c->fail(XCGPU_ERR_INVALID, "vxc_batch: null argument") : XCGPU_ERR_INVALID;
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "vxc_batch: unknown precision");
  cudaSetDevice(c->device);
  std::vector<BuildReq> rq;
  for (uint32_t i = 0; i < n; ++i) {
    const xcgpu_request& r = reqs[i];
    if (!r.plan || r.plan->ctx != c || !xc::is_known(r.func) || (r.nspin != 1 && r.nspin != 2) || !r.P || !r.V ||
        !r.exc_nel)
      return c->fail(XCGPU_ERR_INVALID, "vxc_batch: bad request " + std::to_string(i));
    rq.push_back(BuildReq{r.plan, r.func, r.nspin, r.block_ave_threshold, r.P, r.V, r.exc_nel});
  }
  XC_TRY(run_builds(c, rq, precision));
  if (flags & XCGPU_BATCH_SYNC) return xcgpu_check_async(c);
  return XCGPU_OK;
}

xcgpu_status xcgpu_nadd_vxc(xcgpu_plan* A, xcgpu_plan* const* env, uint32_t n_env, int func, int nspin,
                            int precision, double thr, const double* P_active, const double* const* P_env, double* V,
                            double* E_nadd, int mem) {
  if (!A) return XCGPU_ERR_INVALID;
  Ctx* c = A->ctx;
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "nadd: unknown functional");
  if ((nspin != 1 && nspin != 2) || !P_active || !V || (n_env > 0 && (!env || !P_env)))
    return c->fail(XCGPU_ERR_INVALID, "nadd: bad arguments");
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "nadd: unknown precision");
  std::vector<xcgpu_plan*> plans(1, A);
  std::vector<const double*> Psrc(1, P_active);
  for (uint32_t i = 0; i < n_env; ++i) {
    if (!env[i] || !P_env[i]) return c->fail(XCGPU_ERR_INVALID, "nadd: null environment plan or density matrix");
    if (env[i]->ctx != c) return c->fail(XCGPU_ERR_INVALID, "nadd: environment plan of another context");
    if (env[i]->grid != A->grid)  // SupersystemDensityOnGridController.cpp:49 (isDefinedOnSameGrid)
      return c->fail(XCGPU_ERR_INVALID, "nadd: all subsystem densities must live on the active system's grid");
    for (auto* q : plans)
      if (q == env[i]) return c->fail(XCGPU_ERR_INVALID, "nadd: one plan per subsystem (a plan appears twice)");
    plans.push_back(env[i]);
    Psrc.push_back(P_env[i]);
  }
  cudaSetDevice(c->device);
  const bool gga = xc::is_gga(func), mixed = precision == XCGPU_PREC_MIXED;
  const long n = A->grid->n;
  const int nbfA = A->basis->nbf;
  for (auto* q : plans) XC_TRY(ensure_work(q, nspin, gga, mixed));
  std::vector<const double*> Pd(plans.size());
  for (size_t i = 0; i < plans.size(); ++i) {
    const size_t cnt = (size_t)nspin * plans[i]->basis->nbf * plans[i]->basis->nbf;
    if (mem == XCGPU_MEM_HOST) {
      XC_TRY(upload(c, plans[i]->w_P, Psrc[i], cnt));
      Pd[i] = plans[i]->w_P.as<double>();
    } else {
      Pd[i] = Psrc[i];
    }
  }
  int* counter = nullptr;
  XC_TRY(c->aux(&counter));
  int* err = counter + 2;
  XC_TRY(c->cuda(cudaMemsetAsync(counter, 0, 4 * sizeof(int), c->stream), "memset aux"));
  // 1. every subsystem's density on the shared grid (one batched launch in mixed precision)
  if (mixed) {
    std::vector<MixedWork> work;
    for (size_t i = 0; i < plans.size(); ++i) {
      xcgpu_plan* q = plans[i];
      XC_TRY(mixed_split(c, Pd[i], nspin, q->basis->nbf, q->w_psplit.as<float>()));
      work.push_back(MixedWork{&q->basis->dev, &q->dev, nspin, q->w_psplit.as<float>(), q->w_rho.as<double>(),
                               gga ? q->w_grad.as<double>() : nullptr, nullptr, nullptr, nullptr, nullptr});
    }
    XC_TRY(mixed_density_batch(c, work, counter, err));
  } else {
    for (size_t i = 0; i < plans.size(); ++i)
      XC_TRY(stage_density(plans[i], nspin, Pd[i], plans[i]->w_rho.as<double>(),
                           gga ? plans[i]->w_grad.as<double>() : nullptr));
  }
  // 2. supersystem density: the sum of the subsystem densities
  //    (SupersystemDensityOnGridController.cpp:101-187)
  XC_TRY(A->n_rho.alloc(c, (size_t)nspin * n * sizeof(double)));
  XC_TRY(A->n_epuv.alloc(c, (size_t)n * sizeof(double)));
  XC_TRY(A->n_dfdrho.alloc(c, (size_t)nspin * n * sizeof(double)));
  if (gga) {
    XC_TRY(A->n_grad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
    XC_TRY(A->n_dfdgrad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
  }
  XC_TRY(A->n_partials.alloc(c, 2 * ((n + 127) / 128) * sizeof(double) + 16));
  XC_TRY(A->n_fskip.alloc(c, (size_t)(n + kSkipBlock - 1) / kSkipBlock + 1));
  XC_TRY(A->n_sums.alloc(c, 2 * (plans.size() + 1) * sizeof(double)));
  XC_TRY(c->cuda(cudaMemcpyAsync(A->n_rho.p, A->w_rho.p, (size_t)nspin * n * sizeof(double), cudaMemcpyDeviceToDevice,
                                 c->stream), "supersystem density"));
  if (gga)
    XC_TRY(c->cuda(cudaMemcpyAsync(A->n_grad.p, A->w_grad.p, (size_t)nspin * 3 * n * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream), "supersystem gradient"));
  for (size_t i = 1; i < plans.size(); ++i) {
    XC_TRY(launch_axpy(c, (long)nspin * n, plans[i]->w_rho.as<double>(), A->n_rho.as<double>()));
    if (gga) XC_TRY(launch_axpy(c, (long)nspin * 3 * n, plans[i]->w_grad.as<double>(), A->n_grad.as<double>()));
  }
  // 3. functional of the supersystem, of the active and of every environment density;
  //    sums: [E, N] of the supersystem, of the active system, of environment i
  double* sums = A->n_sums.as<double>();
  auto functional = [&](const double* rho, const double* grad, double* epuv, double* dfdrho, double* dfdgrad,
                        double* partials, unsigned char* fskip, double* out) -> xcgpu_status {
    int nparts = 0;
    xcgpu_status st = launch_functional(c, func, nspin, n, kSkipBlock, rho, gga ? grad : nullptr, epuv, dfdrho,
                                        gga ? dfdgrad : nullptr, A->dev.w, partials, &nparts, fskip);
    if (st) return st;
    if (nparts) return launch_sum_partials(c, partials, nparts, 2, out);
    return c->cuda(cudaMemsetAsync(out, 0, 2 * sizeof(double), c->stream), "memset sums");
  };
  XC_TRY(functional(A->n_rho.as<double>(), A->n_grad.as<double>(), A->n_epuv.as<double>(), A->n_dfdrho.as<double>(),
                    A->n_dfdgrad.as<double>(), A->n_partials.as<double>(), A->n_fskip.as<unsigned char>(), sums));
  for (size_t i = 0; i < plans.size(); ++i) {
    xcgpu_plan* q = plans[i];
    XC_TRY(functional(q->w_rho.as<double>(), q->w_grad.as<double>(), q->w_epuv.as<double>(), q->w_dfdrho.as<double>(),
                      q->w_dfdgrad.as<double>(), q->w_partials.as<double>(), q->w_fskip.as<unsigned char>(),
                      sums + 2 * (i + 1)));
  }
  // 4. potential difference on the grid (NAddFuncPotential.cpp:213-225)
  XC_TRY(launch_scale_add(c, (long)nspin * n, -1.0, A->w_dfdrho.as<double>(), A->n_dfdrho.as<double>()));
  if (gga) XC_TRY(launch_scale_add(c, (long)nspin * 3 * n, -1.0, A->w_dfdgrad.as<double>(), A->n_dfdgrad.as<double>()));
  // 5. adder on the active basis
  double* Vd = V;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(A->w_V.alloc(c, (size_t)nspin * nbfA * nbfA * sizeof(double)));
    Vd = A->w_V.as<double>();
  }
  XC_TRY(c->cuda(cudaMemsetAsync(Vd, 0, (size_t)nspin * nbfA * nbfA * sizeof(double), c->stream), "memset V"));
  const double* gv = gga ? A->n_dfdgrad.as<double>() : nullptr;
  if (mixed) {
    XC_TRY(launch_block_skip_flags(c, A->dev, nspin, A->n_dfdrho.as<double>(), gv, thr, A->w_skip.as<unsigned char>()));
    std::vector<MixedWork> work(1);
    work[0] = MixedWork{&A->basis->dev, &A->dev, nspin, nullptr, nullptr, nullptr, A->n_dfdrho.as<double>(), gv,
                        A->w_skip.as<unsigned char>(), Vd};
    XC_TRY(mixed_adder_batch(c, work, counter + 1, err));
  } else {
    XC_TRY(stage_adder(A, nspin, A->n_dfdrho.as<double>(), gv, thr, Vd));
  }
  std::vector<double> hs(2 * (plans.size() + 1));
  int herr = 0;
  XC_TRY(c->cuda(cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                 "sums"));
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  if (mem == XCGPU_MEM_HOST)
    XC_TRY(c->cuda(cudaMemcpyAsync(V, Vd, (size_t)nspin * nbfA * nbfA * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->stream), "V"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "nadd"));
  if (herr) return device_error(c, herr, "nadd");
  if (E_nadd) {
    double e = hs[0] - hs[2];  // E_xc[rho_tot] - E_xc[rho_active]
    for (size_t i = 1; i < plans.size(); ++i) e -= hs[2 * (i + 1)];
    *E_nadd = e;
  }
  return XCGPU_OK;
}

xcgpu_status xcgpu_xc_gradient(xcgpu_plan* P, int func, int nspin, const double* Pm, const int* shell_atom, int natoms,
                               double* G, int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "xc_gradient: unknown functional");
  if ((nspin != 1 && nspin != 2) || !Pm || !shell_atom || natoms <= 0 || !G)
    return c->fail(XCGPU_ERR_INVALID, "xc_gradient: bad arguments");
  const xcgpu_basis* B = P->basis;
  std::vector<int> fatom(B->nbf);
  for (int sh = 0; sh < B->nshell; ++sh) {
    if (shell_atom[sh] < 0 || shell_atom[sh] >= natoms)
      return c->fail(XCGPU_ERR_INVALID, "xc_gradient: shell atom index out of range");
    const int nf = B->pure[sh] ? 2 * B->l[sh] + 1 : ncart(B->l[sh]);
    for (int f = 0; f < nf; ++f) fatom[B->first[sh] + f] = shell_atom[sh];
  }
  cudaSetDevice(c->device);
  const bool gga = xc::is_gga(func);
  const long n = P->grid->n;
  const int nbf = B->nbf;
  XC_TRY(ensure_work(P, nspin, gga, false));
  const double* Pd = Pm;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, P->w_P, Pm, (size_t)nspin * nbf * nbf));
    Pd = P->w_P.as<double>();
  }
  // rho, grad rho and the potential of the functional (FuncPotential.cpp:115-116)
  double* grad = gga ? P->w_grad.as<double>() : nullptr;
  XC_TRY(stage_density(P, nspin, Pd, P->w_rho.as<double>(), grad));
  int nparts = 0;
  XC_TRY(launch_functional(c, func, nspin, n, kSkipBlock, P->w_rho.as<double>(), grad, P->w_epuv.as<double>(),
                           P->w_dfdrho.as<double>(), gga ? P->w_dfdgrad.as<double>() : nullptr, P->dev.w,
                           P->w_partials.as<double>(), &nparts, P->w_fskip.as<unsigned char>()));
  // chunks of blocks whose slabs (4 planes, 10 with Hessians) fit the scratch cap
  const int planes = gga ? 10 : 4;
  const long cap = std::max<long>((long)(c->scratch_cap / sizeof(double)),
                                  (long)planes * kBlockPoints * std::max(P->max_active, 1));
  std::vector<long> off(P->nblocks);
  std::vector<int> bounds(1, 0);
  long cur = 0, mx = 0;
  for (int b = 0; b < P->nblocks; ++b) {
    const long need = (long)planes * kBlockPoints * (P->fn_off[b + 1] - P->fn_off[b]);
    if (cur + need > cap && cur > 0) {
      bounds.push_back(b);
      mx = std::max(mx, cur);
      cur = 0;
    }
    off[b] = cur;
    cur += need;
  }
  mx = std::max(mx, cur);
  bounds.push_back(P->nblocks);
  DevBuf d_off, d_fatom, d_G;
  XC_TRY(upload(c, d_off, off.data(), off.size()));
  XC_TRY(upload(c, d_fatom, fatom.data(), fatom.size()));
  XC_TRY(d_G.alloc(c, (size_t)3 * natoms * sizeof(double)));
  XC_TRY(c->cuda(cudaMemsetAsync(d_G.p, 0, (size_t)3 * natoms * sizeof(double), c->stream), "memset G"));
  XC_TRY(c->scratch2.alloc(c, std::max<long>(mx, 1) * sizeof(double)));
  for (size_t k = 0; k + 1 < bounds.size(); ++k) {
    const int b0 = bounds[k], b1 = bounds[k + 1];
    XC_TRY(fp64_xc_gradient_chunk(c, B->dev, P->dev, b0, b1, d_off.as<long>() + b0, c->scratch2.as<double>(), gga,
                                  nspin, Pd, P->w_dfdrho.as<double>(), gga ? P->w_dfdgrad.as<double>() : nullptr,
                                  d_fatom.as<int>(), natoms, d_G.as<double>()));
  }
  XC_TRY(c->cuda(cudaMemcpyAsync(G, d_G.p, (size_t)3 * natoms * sizeof(double),
                                 mem == XCGPU_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, c->stream),
                 "G"));
  return c->cuda(cudaStreamSynchronize(c->stream), "xc_gradient");
}

xcgpu_status xcgpu_lr_kernel(xcgpu_plan* P, int func, const double* P0, uint32_t ntrial, const double* const* D,
                             double* const* F, int precision, double thr, int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "lr_kernel: unknown functional");
  if (!P0 || (ntrial > 0 && (!D || !F))) return c->fail(XCGPU_ERR_INVALID, "lr_kernel: bad arguments");
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "lr_kernel: unknown precision");
  for (uint32_t t = 0; t < ntrial; ++t)
    if (!D[t] || !F[t]) return c->fail(XCGPU_ERR_INVALID, "lr_kernel: null trial or output matrix");
  cudaSetDevice(c->device);
  const bool gga = xc::is_gga(func), mixed = precision == XCGPU_PREC_MIXED;
  const long n = P->grid->n;
  const int nbf = P->basis->nbf;
  const size_t nn = (size_t)nbf * nbf;
  XC_TRY(ensure_work(P, 1, gga, mixed));
  XC_TRY(P->n_rho.alloc(c, (size_t)n * sizeof(double)));
  XC_TRY(P->n_dfdrho.alloc(c, (size_t)n * sizeof(double)));
  if (gga) {
    XC_TRY(P->n_grad.alloc(c, (size_t)3 * n * sizeof(double)));
    XC_TRY(P->n_dfdgrad.alloc(c, (size_t)3 * n * sizeof(double)));
  }
  const double* P0d = P0;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, P->w_P, P0, nn));
    P0d = P->w_P.as<double>();
  }
  DevBuf dD, dS, dF;
  XC_TRY(dS.alloc(c, nn * sizeof(double)));
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(dD.alloc(c, nn * sizeof(double)));
    XC_TRY(dF.alloc(c, nn * sizeof(double)));
  }
  int* counter = nullptr;
  XC_TRY(c->aux(&counter));
  int* err = counter + 2;
  XC_TRY(c->cuda(cudaMemsetAsync(counter, 0, 4 * sizeof(int), c->stream), "memset aux"));
  // density of a symmetric matrix M into (rho, grad)
  auto density = [&](const double* M, double* rho, double* grad) -> xcgpu_status {
    if (!mixed) return stage_density(P, 1, M, rho, grad);
    xcgpu_status st = mixed_split(c, M, 1, P->basis->nbf, P->w_psplit.as<float>());
    if (st) return st;
    std::vector<MixedWork> work(1);
    work[0] = MixedWork{&P->basis->dev, &P->dev, 1, P->w_psplit.as<float>(), rho, grad, nullptr, nullptr, nullptr, nullptr};
    return mixed_density_batch(c, work, counter, err);
  };
  // ground state (the kernel's expansion point)
  XC_TRY(density(P0d, P->w_rho.as<double>(), gga ? P->w_grad.as<double>() : nullptr));
  for (uint32_t t = 0; t < ntrial; ++t) {
    const double* Dd = D[t];
    double* Fd = F[t];
    if (mem == XCGPU_MEM_HOST) {
      XC_TRY(c->cuda(cudaMemcpyAsync(dD.p, D[t], nn * sizeof(double), cudaMemcpyHostToDevice, c->stream), "trial"));
      Dd = dD.as<double>();
      Fd = dF.as<double>();
    }
    // perturbed density of (D + D^T) / 2 (KernelSigmavector.cpp:227-233 symmetrises D)
    XC_TRY(launch_symmetrise_half(c, Dd, dS.as<double>(), nbf));
    XC_TRY(density(dS.as<double>(), P->n_rho.as<double>(), gga ? P->n_grad.as<double>() : nullptr));
    XC_TRY(launch_lr_kernel(c, func, n, P->w_rho.as<double>(), gga ? P->w_grad.as<double>() : nullptr,
                            P->n_rho.as<double>(), gga ? P->n_grad.as<double>() : nullptr, P->n_dfdrho.as<double>(),
                            gga ? P->n_dfdgrad.as<double>() : nullptr));
    XC_TRY(c->cuda(cudaMemsetAsync(Fd, 0, nn * sizeof(double), c->stream), "memset F"));
    const double* gv = gga ? P->n_dfdgrad.as<double>() : nullptr;
    if (mixed) {
      XC_TRY(launch_block_skip_flags(c, P->dev, 1, P->n_dfdrho.as<double>(), gv, thr, P->w_skip.as<unsigned char>()));
      std::vector<MixedWork> work(1);
      work[0] = MixedWork{&P->basis->dev, &P->dev, 1, nullptr, nullptr, nullptr, P->n_dfdrho.as<double>(), gv,
                          P->w_skip.as<unsigned char>(), Fd};
      XC_TRY(mixed_adder_batch(c, work, counter + 1, err));
    } else {
      XC_TRY(stage_adder(P, 1, P->n_dfdrho.as<double>(), gv, thr, Fd));
    }
    if (mem == XCGPU_MEM_HOST)
      XC_TRY(c->cuda(cudaMemcpyAsync(F[t], Fd, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "F"));
  }
  int herr = 0;
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "lr_kernel"));
  return device_error(c, herr, "lr_kernel");
}

xcgpu_status xcgpu_lr_kernel_spin(xcgpu_plan* P, int func, int kind, const double* P0, uint32_t ntrial,
                                  const double* const* D, double* const* F, int precision, double thr, int mem) {
  if (!P) return XCGPU_ERR_INVALID;
  Ctx* c = P->ctx;
  if (kind == XCGPU_LR_SINGLET) return xcgpu_lr_kernel(P, func, P0, ntrial, D, F, precision, thr, mem);
  if (kind != XCGPU_LR_TRIPLET && kind != XCGPU_LR_UNRESTRICTED)
    return c->fail(XCGPU_ERR_INVALID, "lr_kernel_spin: unknown kind");
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "lr_kernel_spin: unknown functional");
  if (!P0 || (ntrial > 0 && (!D || !F))) return c->fail(XCGPU_ERR_INVALID, "lr_kernel_spin: bad arguments");
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "lr_kernel_spin: unknown precision");
  for (uint32_t t = 0; t < ntrial; ++t)
    if (!D[t] || !F[t]) return c->fail(XCGPU_ERR_INVALID, "lr_kernel_spin: null trial or output matrix");
  cudaSetDevice(c->device);
  const bool gga = xc::is_gga(func), mixed = precision == XCGPU_PREC_MIXED;
  const int ns = kind == XCGPU_LR_UNRESTRICTED ? 2 : 1;  // spins of P0, of each trial and of each F
  const long n = P->grid->n;
  const int nbf = P->basis->nbf;
  const size_t nn = (size_t)nbf * nbf;
  XC_TRY(ensure_work(P, ns, gga, mixed));
  XC_TRY(P->n_rho.alloc(c, (size_t)ns * n * sizeof(double)));
  XC_TRY(P->n_dfdrho.alloc(c, (size_t)ns * n * sizeof(double)));
  if (gga) {
    XC_TRY(P->n_grad.alloc(c, (size_t)ns * 3 * n * sizeof(double)));
    XC_TRY(P->n_dfdgrad.alloc(c, (size_t)ns * 3 * n * sizeof(double)));
  }
  const double* P0d = P0;
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(upload(c, P->w_P, P0, ns * nn));
    P0d = P->w_P.as<double>();
  }
  DevBuf dD, dS, dF;
  XC_TRY(dS.alloc(c, ns * nn * sizeof(double)));
  if (mem == XCGPU_MEM_HOST) {
    XC_TRY(dD.alloc(c, ns * nn * sizeof(double)));
    XC_TRY(dF.alloc(c, ns * nn * sizeof(double)));
  }
  int* counter = nullptr;
  XC_TRY(c->aux(&counter));
  int* err = counter + 2;
  XC_TRY(c->cuda(cudaMemsetAsync(counter, 0, 4 * sizeof(int), c->stream), "memset aux"));
  auto density = [&](const double* M, double* rho, double* grad) -> xcgpu_status {
    if (!mixed) return stage_density(P, ns, M, rho, grad);
    xcgpu_status st = mixed_split(c, M, ns, nbf, P->w_psplit.as<float>());
    if (st) return st;
    std::vector<MixedWork> work(1);
    work[0] = MixedWork{&P->basis->dev, &P->dev, ns, P->w_psplit.as<float>(), rho, grad, nullptr, nullptr, nullptr, nullptr};
    return mixed_density_batch(c, work, counter, err);
  };
  // ground state: per spin (unrestricted), or the restricted total density (triplet)
  XC_TRY(density(P0d, P->w_rho.as<double>(), gga ? P->w_grad.as<double>() : nullptr));
  for (uint32_t t = 0; t < ntrial; ++t) {
    const double* Dd = D[t];
    double* Fd = F[t];
    if (mem == XCGPU_MEM_HOST) {
      XC_TRY(c->cuda(cudaMemcpyAsync(dD.p, D[t], ns * nn * sizeof(double), cudaMemcpyHostToDevice, c->stream), "trial"));
      Dd = dD.as<double>();
      Fd = dF.as<double>();
    }
    // every spin's trial matrix symmetrised (KernelSigmavector.cpp:202-208)
    for (int sp = 0; sp < ns; ++sp) XC_TRY(launch_symmetrise_half(c, Dd + sp * nn, dS.as<double>() + sp * nn, nbf));
    XC_TRY(density(dS.as<double>(), P->n_rho.as<double>(), gga ? P->n_grad.as<double>() : nullptr));
    XC_TRY(launch_lr_kernel_spin(c, func, kind, n, P->w_rho.as<double>(), gga ? P->w_grad.as<double>() : nullptr,
                                 P->n_rho.as<double>(), gga ? P->n_grad.as<double>() : nullptr,
                                 P->n_dfdrho.as<double>(), gga ? P->n_dfdgrad.as<double>() : nullptr));
    XC_TRY(c->cuda(cudaMemsetAsync(Fd, 0, ns * nn * sizeof(double), c->stream), "memset F"));
    const double* gv = gga ? P->n_dfdgrad.as<double>() : nullptr;
    if (mixed) {
      XC_TRY(launch_block_skip_flags(c, P->dev, ns, P->n_dfdrho.as<double>(), gv, thr, P->w_skip.as<unsigned char>()));
      std::vector<MixedWork> work(1);
      work[0] = MixedWork{&P->basis->dev, &P->dev, ns, nullptr, nullptr, nullptr, P->n_dfdrho.as<double>(), gv,
                          P->w_skip.as<unsigned char>(), Fd};
      XC_TRY(mixed_adder_batch(c, work, counter + 1, err));
    } else {
      XC_TRY(stage_adder(P, ns, P->n_dfdrho.as<double>(), gv, thr, Fd));
    }
    if (mem == XCGPU_MEM_HOST)
      XC_TRY(c->cuda(cudaMemcpyAsync(F[t], Fd, ns * nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "F"));
  }
  int herr = 0;
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "lr_kernel_spin"));
  return device_error(c, herr, "lr_kernel_spin");
}

xcgpu_status xcgpu_nadd_vxc_all(xcgpu_plan* const* plans, uint32_t n_sub, int func, int nspin, int precision,
                                double thr, const double* const* P, double* const* V, double* E_nadd, int mem) {
  if (!plans || n_sub == 0 || !plans[0]) return XCGPU_ERR_INVALID;
  xcgpu_plan* A = plans[0];
  Ctx* c = A->ctx;
  if (!xc::is_known(func)) return c->fail(XCGPU_ERR_INVALID, "nadd_all: unknown functional");
  if ((nspin != 1 && nspin != 2) || !P || !V) return c->fail(XCGPU_ERR_INVALID, "nadd_all: bad arguments");
  if (precision != XCGPU_PREC_FP64 && precision != XCGPU_PREC_MIXED)
    return c->fail(XCGPU_ERR_INVALID, "nadd_all: unknown precision");
  for (uint32_t i = 0; i < n_sub; ++i) {
    if (!plans[i] || !P[i] || !V[i]) return c->fail(XCGPU_ERR_INVALID, "nadd_all: null plan, density or output");
    if (plans[i]->ctx != c) return c->fail(XCGPU_ERR_INVALID, "nadd_all: plan of another context");
    if (plans[i]->grid != A->grid)
      return c->fail(XCGPU_ERR_INVALID, "nadd_all: all subsystem densities must live on one (supersystem) grid");
    for (uint32_t j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return c->fail(XCGPU_ERR_INVALID, "nadd_all: one plan per subsystem");
  }
  cudaSetDevice(c->device);
  const bool gga = xc::is_gga(func), mixed = precision == XCGPU_PREC_MIXED;
  const long n = A->grid->n;
  for (uint32_t i = 0; i < n_sub; ++i) XC_TRY(ensure_work(plans[i], nspin, gga, mixed));
  std::vector<const double*> Pd(n_sub);
  std::vector<double*> Vd(n_sub);
  for (uint32_t i = 0; i < n_sub; ++i) {
    xcgpu_plan* q = plans[i];
    const size_t cnt = (size_t)nspin * q->basis->nbf * q->basis->nbf;
    if (mem == XCGPU_MEM_HOST) {
      XC_TRY(upload(c, q->w_P, P[i], cnt));
      XC_TRY(q->w_V.alloc(c, cnt * sizeof(double)));
      Pd[i] = q->w_P.as<double>();
      Vd[i] = q->w_V.as<double>();
    } else {
      Pd[i] = P[i];
      Vd[i] = V[i];
    }
    XC_TRY(q->n_dfdrho.alloc(c, (size_t)nspin * n * sizeof(double)));
    if (gga) XC_TRY(q->n_dfdgrad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
  }
  int* counter = nullptr;
  XC_TRY(c->aux(&counter));
  int* err = counter + 2;
  XC_TRY(c->cuda(cudaMemsetAsync(counter, 0, 4 * sizeof(int), c->stream), "memset aux"));
  // 1. all subsystem densities (one batched launch in mixed precision)
  std::vector<MixedWork> work;
  for (uint32_t i = 0; i < n_sub; ++i) {
    xcgpu_plan* q = plans[i];
    double* grad = gga ? q->w_grad.as<double>() : nullptr;
    if (mixed) {
      XC_TRY(mixed_split(c, Pd[i], nspin, q->basis->nbf, q->w_psplit.as<float>()));
      work.push_back(MixedWork{&q->basis->dev, &q->dev, nspin, q->w_psplit.as<float>(), q->w_rho.as<double>(), grad,
                               q->n_dfdrho.as<double>(), gga ? q->n_dfdgrad.as<double>() : nullptr,
                               q->w_skip.as<unsigned char>(), Vd[i]});
    } else {
      XC_TRY(stage_density(q, nspin, Pd[i], q->w_rho.as<double>(), grad));
    }
  }
  if (mixed) XC_TRY(mixed_density_batch(c, work, counter, err));
  // 2. supersystem density in the first plan's buffers
  XC_TRY(A->n_rho.alloc(c, (size_t)nspin * n * sizeof(double)));
  XC_TRY(A->n_epuv.alloc(c, (size_t)n * sizeof(double)));
  if (gga) XC_TRY(A->n_grad.alloc(c, (size_t)nspin * 3 * n * sizeof(double)));
  XC_TRY(A->n_partials.alloc(c, 2 * ((n + 127) / 128) * sizeof(double) + 16));
  XC_TRY(A->n_fskip.alloc(c, (size_t)(n + kSkipBlock - 1) / kSkipBlock + 1));
  XC_TRY(A->n_sums.alloc(c, 2 * (n_sub + 1) * sizeof(double)));
  XC_TRY(c->cuda(cudaMemcpyAsync(A->n_rho.p, A->w_rho.p, (size_t)nspin * n * sizeof(double), cudaMemcpyDeviceToDevice,
                                 c->stream), "supersystem density"));
  if (gga)
    XC_TRY(c->cuda(cudaMemcpyAsync(A->n_grad.p, A->w_grad.p, (size_t)nspin * 3 * n * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream), "supersystem gradient"));
  for (uint32_t i = 1; i < n_sub; ++i) {
    XC_TRY(launch_axpy(c, (long)nspin * n, plans[i]->w_rho.as<double>(), A->n_rho.as<double>()));
    if (gga) XC_TRY(launch_axpy(c, (long)nspin * 3 * n, plans[i]->w_grad.as<double>(), A->n_grad.as<double>()));
  }
  // 3. functionals: the supersystem's into the first plan's difference buffers (it is
  //    subtracted last), each subsystem's into its own work buffers
  double* sums = A->n_sums.as<double>();
  auto functional = [&](const double* rho, const double* grad, double* epuv, double* dfdrho, double* dfdgrad,
                        double* partials, unsigned char* fskip, double* out) -> xcgpu_status {
    int nparts = 0;
    xcgpu_status st = launch_functional(c, func, nspin, n, kSkipBlock, rho, gga ? grad : nullptr, epuv, dfdrho,
                                        gga ? dfdgrad : nullptr, A->dev.w, partials, &nparts, fskip);
    if (st) return st;
    if (nparts) return launch_sum_partials(c, partials, nparts, 2, out);
    return c->cuda(cudaMemsetAsync(out, 0, 2 * sizeof(double), c->stream), "memset sums");
  };
  XC_TRY(functional(A->n_rho.as<double>(), A->n_grad.as<double>(), A->n_epuv.as<double>(), A->n_dfdrho.as<double>(),
                    A->n_dfdgrad.as<double>(), A->n_partials.as<double>(), A->n_fskip.as<unsigned char>(), sums));
  for (uint32_t i = 0; i < n_sub; ++i) {
    xcgpu_plan* q = plans[i];
    XC_TRY(functional(q->w_rho.as<double>(), q->w_grad.as<double>(), q->w_epuv.as<double>(), q->w_dfdrho.as<double>(),
                      q->w_dfdgrad.as<double>(), q->w_partials.as<double>(), q->w_fskip.as<unsigned char>(),
                      sums + 2 * (i + 1)));
  }
  // 4. per subsystem: dF[rho_tot] - dF[rho_i] (the first plan's buffers hold dF[rho_tot])
  for (uint32_t k = 0; k < n_sub; ++k) {
    const uint32_t i = (k + 1) % n_sub;  // the first subsystem last
    xcgpu_plan* q = plans[i];
    if (i != 0) {
      XC_TRY(c->cuda(cudaMemcpyAsync(q->n_dfdrho.p, A->n_dfdrho.p, (size_t)nspin * n * sizeof(double),
                                     cudaMemcpyDeviceToDevice, c->stream), "copy potential"));
      if (gga)
        XC_TRY(c->cuda(cudaMemcpyAsync(q->n_dfdgrad.p, A->n_dfdgrad.p, (size_t)nspin * 3 * n * sizeof(double),
                                       cudaMemcpyDeviceToDevice, c->stream), "copy potential gradient"));
    }
    XC_TRY(launch_scale_add(c, (long)nspin * n, -1.0, q->w_dfdrho.as<double>(), q->n_dfdrho.as<double>()));
    if (gga)
      XC_TRY(launch_scale_add(c, (long)nspin * 3 * n, -1.0, q->w_dfdgrad.as<double>(), q->n_dfdgrad.as<double>()));
  }
  // 5. every subsystem's adder (one batched launch in mixed precision)
  for (uint32_t i = 0; i < n_sub; ++i) {
    xcgpu_plan* q = plans[i];
    const int nbf = q->basis->nbf;
    const double* gv = gga ? q->n_dfdgrad.as<double>() : nullptr;
    XC_TRY(c->cuda(cudaMemsetAsync(Vd[i], 0, (size_t)nspin * nbf * nbf * sizeof(double), c->stream), "memset V"));
    if (mixed)
      XC_TRY(launch_block_skip_flags(c, q->dev, nspin, q->n_dfdrho.as<double>(), gv, thr,
                                     q->w_skip.as<unsigned char>()));
    else
      XC_TRY(stage_adder(q, nspin, q->n_dfdrho.as<double>(), gv, thr, Vd[i]));
  }
  if (mixed) XC_TRY(mixed_adder_batch(c, work, counter + 1, err));
  std::vector<double> hs(2 * (n_sub + 1));
  int herr = 0;
  XC_TRY(c->cuda(cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                 "sums"));
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  if (mem == XCGPU_MEM_HOST)
    for (uint32_t i = 0; i < n_sub; ++i) {
      const int nbf = plans[i]->basis->nbf;
      XC_TRY(c->cuda(cudaMemcpyAsync(V[i], Vd[i], (size_t)nspin * nbf * nbf * sizeof(double), cudaMemcpyDeviceToHost,
                                     c->stream), "V"));
    }
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "nadd_all"));
  if (herr) return device_error(c, herr, "nadd_all");
  if (E_nadd) {
    double e = hs[0];  // E_xc[rho_tot] - sum_i E_xc[rho_i]
    for (uint32_t i = 0; i < n_sub; ++i) e -= hs[2 * (i + 1)];
    *E_nadd = e;
  }
  return XCGPU_OK;
}

xcgpu_status xcgpu_check_async(xcgpu_ctx* c) {
  if (!c) return XCGPU_ERR_INVALID;
  int herr = 0;
  int* aux = nullptr;
  XC_TRY(c->aux(&aux));
  XC_TRY(c->cuda(cudaMemcpyAsync(&herr, aux + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error word"));
  XC_TRY(c->cuda(cudaStreamSynchronize(c->stream), "check_async"));
  if (herr) return device_error(c, herr, "check_async");
  return XCGPU_OK;
}

xcgpu_status xcgpu_graph_begin(xcgpu_ctx* c) {
  if (!c) return XCGPU_ERR_INVALID;
  if (c->stream == nullptr) return c->fail(XCGPU_ERR_INVALID, "graph capture needs a non-default stream");
  return c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
}

xcgpu_status xcgpu_graph_end(xcgpu_ctx* c, void** graph_exec) {
  if (!c || !graph_exec) return XCGPU_ERR_INVALID;
  cudaGraph_t g = nullptr;
  XC_TRY(c->cuda(cudaStreamEndCapture(c->stream, &g), "end capture"));
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  XC_TRY(c->cuda(e, "graph instantiate"));
  *graph_exec = ge;
  return XCGPU_OK;
}

xcgpu_status xcgpu_graph_launch(xcgpu_ctx* c, void* graph_exec) {
  if (!c || !graph_exec) return XCGPU_ERR_INVALID;
  return c->cuda(cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph_exec), c->stream), "graph launch");
}

void xcgpu_graph_destroy(void* graph_exec) {
  if (graph_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph_exec));
}

}  // extern "C"
