// C ABI entry points of the Wigner-transport library (see include/wigner_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kline.cuh"
#include "problem.h"

namespace {

thread_local std::string g_err;

int fail(wg::Problem* P, int code, const std::string& msg) {
  if (P) P->err = msg;
  g_err = msg;
  return code;
}

#define API_CK(P, expr)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(P, WG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #expr); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count, double& bytes) {
  bytes += (double)sizeof(T) * (double)count;
  return cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
}

void free_all(wg::Problem& P) {
  for (wg::ArnoldiGraphs& G : P.graphs) {
    for (cudaGraphExec_t x : G.exec)
      if (x) cudaGraphExecDestroy(x);
    G.exec.clear();
  }
  wg::prof_release(P);
  wg::mixed_free(P);
  for (cudaEvent_t& e : P.ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  wg::gummel_free(P);
  void* ptrs[] = {P.phi, P.kvec, P.xi_edge, P.kap, P.betai, P.pre_dinv, P.pre_h, P.kmap_a, P.kmap_s, P.cosm, P.pinv, P.pp, P.flr, P.fxi, P.qd, P.beta, P.xq, P.pot_x,
                  P.pot_v, P.vslope, P.m_nodes, P.rhs, P.tr_b, P.x, P.w, P.z, P.r, P.V, P.xh, P.yh, P.H, P.cs, P.sn, P.g, P.hcol,
                  P.ycoef, P.partial, P.nrm_partial, P.nrm, P.nrm_keep, P.inv64, P.target, P.active, P.reorth, P.res_mask, P.res_digits, P.md_count, P.gs_count, P.kused, P.any_active};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (P.stream) cudaStreamDestroy(P.stream);
  P.stream = nullptr;
}

// Small dense inverse (row-major) for the k-line factors.
bool inv_small(const double* A, double* out, int n) {
  double a[wg::kMaxLocal * wg::kMaxLocal];
  std::memcpy(a, A, sizeof(double) * n * n);
  for (int i = 0; i < n * n; ++i) out[i] = 0;
  for (int i = 0; i < n; ++i) out[i * n + i] = 1;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (a[piv * n + c] == 0.0) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[piv * n + k]);
        std::swap(out[c * n + k], out[piv * n + k]);
      }
    const double d = a[c * n + c];
    for (int k = 0; k < n; ++k) { a[c * n + k] /= d; out[c * n + k] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r * n + c];
      for (int k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; out[r * n + k] -= f * out[c * n + k]; }
    }
  }
  return true;
}

}  // namespace

namespace wg {

double estimate_bytes(const Shape& s, int batch, int restart, int restart_inner, int precision, bool fp64_tc,
                      bool basis16) {
  const int nK = s.nK;
  const double N = (double)s.n_el * nK * s.nk, BN = N * batch, ncols = (double)batch * s.n_el * nK;
  const double nx = (double)s.n_el * (nK - 1) + 1;
  double est = 16.0 * BN * (5 + restart + 1) + 16.0 * 2 * s.nxi * ncols +
               8.0 * batch * s.n_el * nK * nK * (s.nxi + 1) + 16.0 * s.nxi * s.nk;
  est += 8.0 * batch * (nx * (8 + 2 * kMaxLocal) + 3.0 * s.n_el * nK + 12);   // Gummel state
  if (precision == WG_PREC_MIXED) est += mixed_bytes(s, batch, restart_inner, basis16);
  if (precision == WG_PREC_MIXED || fp64_tc)   // digit slices of the FP64 emulation
    est += 2.0 * 8 * ncols * 2 * std::max(s.nk, s.nxi) + 2.0 * 2 * 8 * 4.0 * s.nxi * s.nk;
  return est;
}

// k-line factors of the flux part of A + sigma I, per problem b and wave number k:
// D_b(k) = (k K1 + |k| K2 + (sigma / qd_b) I)^-1 and h = D_b(k) * upwind coupling column
// (the line operator of get_LineTransversePreconditioner_full2D.m:174-197 in 1D; the
// kernels multiply by 1 / qd_b).  With sigma = 0 and k = 0 (odd Nk) the flux vanishes
// and the shift 0.003 max|k| |K| of get_LineTransversePreconditioner_full2D.m:50-71
// keeps the factor regular.
int set_kline_factors(Problem& P) {
  const Shape& s = P.s;
  const int nK = s.nK, B = P.batch;
  const size_t per_d = (size_t)s.nk * nK * nK, per_h = (size_t)s.nk * nK;
  std::vector<double> dinv(per_d * B), hv(per_h * B);
  double kmax = 0;
  for (double kk : s.k) kmax = std::max(kmax, std::fabs(kk));
  for (int b = 0; b < B; ++b) {
    double rel = 0;
    if (P.shift != 0) {
      if (!P.hp[b].ready || !(P.hp[b].qd > 0)) {
        P.err = "shifted k-line factors need wg_set_potential for problem " + std::to_string(b);
        return WG_ERR_ARG;
      }
      rel = P.shift / P.hp[b].qd;
    } else if (b > 0) {
      std::copy(dinv.begin(), dinv.begin() + per_d, dinv.begin() + per_d * b);
      std::copy(hv.begin(), hv.begin() + per_h, hv.begin() + per_h * b);
      continue;
    }
    for (int j = 0; j < s.nk; ++j) {
      const double k = s.k[j], ak = std::fabs(k);
      double D[kMaxLocal * kMaxLocal], Di[kMaxLocal * kMaxLocal], g[kMaxLocal];
      for (int i = 0; i < nK * nK; ++i) D[i] = k * s.K1[i] + ak * s.K2[i];
      for (int i = 0; i < nK; ++i) D[i * nK + i] += rel;
      bool ok = (k != 0.0 || rel != 0.0) && inv_small(D, Di, nK);
      if (!ok) {
        if (rel != 0.0) {
          P.err = "singular shifted k-line block";
          return WG_ERR_NUMERIC;
        }
        for (int i = 0; i < nK * nK; ++i) Di[i] = 0;
        double nrm = 0;
        for (int i = 0; i < nK * nK; ++i) nrm = std::max(nrm, std::fabs(s.K1[i]) + std::fabs(s.K2[i]));
        const double sigma = 0.003 * kmax * std::max(nrm, 1e-300);
        for (int i = 0; i < nK; ++i) Di[i * nK + i] = 1.0 / sigma;
      }
      for (int a = 0; a < nK; ++a)
        g[a] = k > 0 ? (k + ak) * s.K3[a * nK + nK - 1] : (k < 0 ? (k - ak) * s.K5[a * nK + 0] : 0.0);
      for (int a = 0; a < nK; ++a) {
        double acc = 0;
        for (int c = 0; c < nK; ++c) acc += Di[a * nK + c] * g[c];
        hv[per_h * b + (size_t)j * nK + a] = acc;
      }
      for (int i = 0; i < nK * nK; ++i) dinv[per_d * b + (size_t)j * nK * nK + i] = Di[i];
    }
  }
  cudaError_t e = cudaMemcpyAsync(P.pre_dinv, dinv.data(), sizeof(double) * dinv.size(), cudaMemcpyHostToDevice,
                                  P.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P.pre_h, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice, P.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);   // host vectors go out of scope
  if (e != cudaSuccess) {
    P.err = std::string("k-line factors: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  return WG_OK;
}

}  // namespace wg

extern "C" {

const char* wg_global_error(void) { return g_err.c_str(); }

const char* wg_last_error(const wg_problem* h) { return h ? h->P.err.c_str() : g_err.c_str(); }

int wg_problem_create(const wg_params* prm, int batch, wg_problem** out) {
  if (!prm || !out || batch < 1) return fail(nullptr, WG_ERR_ARG, "wg_problem_create: null argument or batch < 1");
  *out = nullptr;
  wg_problem* h = new (std::nothrow) wg_problem();
  if (!h) return fail(nullptr, WG_ERR_OOM, "host allocation failed");
  wg::Problem& P = h->P;
  std::string e = wg::build_shape_cached(P.s, prm->n_el, prm->n_local, prm->nk, prm->n_xi, prm->l_xi, prm->m_diff, prm->mpc);
  if (!e.empty()) {
    delete h;
    return fail(nullptr, WG_ERR_ARG, "wg_problem_create: " + e);
  }
  if (prm->precision != WG_PREC_FP64 && prm->precision != WG_PREC_MIXED) {
    delete h;
    return fail(nullptr, WG_ERR_ARG, "wg_problem_create: unknown precision");
  }
  P.batch = batch;
  P.precision = prm->precision;
  P.restart = prm->restart > 0 ? prm->restart : 50;
  P.restart_inner = prm->inner_restart > 0 ? prm->inner_restart : 40;
  P.restart_max = std::max(P.restart, P.restart_inner);
  P.inner_tol = prm->inner_tol > 0 ? prm->inner_tol : 1e-3;
  if (prm->reorth != 0) P.reorth_eta = prm->reorth;
  P.inner_reorth_eta = prm->inner_reorth != 0 ? prm->inner_reorth : -1.0;
  if (P.restart_max > 256) {
    delete h;
    return fail(nullptr, WG_ERR_ARG, "wg_problem_create: restart lengths must be <= 256");
  }
  if (P.precision == WG_PREC_MIXED) {
    const std::string me = wg::mixed_check_shape(P.s);
    if (!me.empty()) {
      delete h;
      return fail(nullptr, WG_ERR_ARG, "wg_problem_create: " + me);
    }
  }
  P.mem_budget = prm->mem_budget_bytes;
  const wg::Shape& s = P.s;
  const int nK = s.nK;
  P.N = (long long)s.n_el * nK * s.nk;
  P.ncols = (long long)batch * s.n_el * nK;
  P.nx = s.n_el * (nK - 1) + 1;
  P.nchunk = (int)std::max<long long>(1, (P.N + 2047) / 2048);
  P.nblk = (int)std::max<long long>(1, (P.N + 255) / 256);
  const long long BN = P.N * batch;
  const int mp1 = P.restart + 1;
  const int pst = P.restart_max + 1;
  // memory estimate before allocating (GmresMemoryLimit analogue)
  P.fp64_tc = prm->fp64_tc != 0 && P.precision == WG_PREC_FP64;
  P.inner_basis16 = prm->inner_basis_fp32 == 0;
  const double est = wg::estimate_bytes(s, batch, P.restart, P.restart_inner, P.precision, P.fp64_tc,
                                        P.inner_basis16);
  if (P.mem_budget > 0 && est > P.mem_budget) {
    delete h;
    return fail(nullptr, WG_ERR_OOM,
                "wg_problem_create: estimated device memory " + std::to_string(est / 1073741824.0) +
                    " GiB exceeds the admission budget");
  }
  P.fb.nK = nK;
  for (int i = 0; i < nK * nK; ++i) {
    P.fb.K1[i] = s.K1[i];
    P.fb.K2[i] = s.K2[i];
    P.fb.K3[i] = s.K3[i];
    P.fb.K5[i] = s.K5[i];
    P.fb.invM[i] = s.invM[i];
  }
  wg::finish_flux_blocks(P.fb);
  double bytes = 0;
  cudaError_t ce = cudaSuccess;
  auto A = [&](cudaError_t r) {
    if (ce == cudaSuccess) ce = r;
  };
  A(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
  A(dalloc(&P.phi, (size_t)s.nxi * s.nk, bytes));
  A(dalloc(&P.kvec, s.nk, bytes));
  A(dalloc(&P.xi_edge, s.nxi + 1, bytes));
  A(dalloc(&P.kap, (size_t)nK * nK * wg::kNqx, bytes));
  A(dalloc(&P.betai, (size_t)nK * nK * (s.nxi + 1), bytes));
  A(dalloc(&P.pre_dinv, (size_t)batch * s.nk * nK * nK, bytes));
  A(dalloc(&P.pre_h, (size_t)batch * s.nk * nK, bytes));
  {
    // chunk maps for any chunk length the autotuner may pick (at most kMaxChunks chunks)
    P.kline_L = wg::kline::chunk_len(s.n_el);
    const size_t nmap = (size_t)batch * std::max(wg::kline::chunk_count(s.n_el), wg::kline::kMaxChunks) * s.nk;
    double* a = nullptr;
    double2* m = nullptr;
    A(dalloc(&a, nmap, bytes));
    A(dalloc(&m, nmap, bytes));
    P.kmap_a = a;
    P.kmap_s = m;
  }
  A(dalloc(&P.cosm, (size_t)s.nxi * s.nk, bytes));
  A(dalloc(&P.pinv, (size_t)s.nk * s.nxi, bytes));
  A(dalloc(&P.pp, (size_t)batch * wg::kPP, bytes));
  A(dalloc(&P.flr, (size_t)batch * 2 * s.nk, bytes));
  A(dalloc(&P.fxi, (size_t)batch * 2 * s.nxi, bytes));
  A(dalloc(&P.qd, batch, bytes));
  A(dalloc(&P.beta, (size_t)batch * s.n_el * nK * nK * (s.nxi + 1), bytes));
  A(dalloc(&P.xq, (size_t)batch * s.n_el * wg::kNqx, bytes));
  A(dalloc(&P.pot_x, (size_t)batch * P.nx, bytes));
  A(dalloc(&P.pot_v, (size_t)batch * P.nx, bytes));
  A(dalloc(&P.vslope, (size_t)batch * P.nx, bytes));
  A(dalloc(&P.m_nodes, (size_t)batch * s.n_el * nK, bytes));
  A(dalloc(&P.rhs, BN, bytes));
  A(dalloc(&P.x, BN, bytes));
  A(dalloc(&P.w, BN, bytes));
  A(dalloc(&P.z, BN, bytes));
  A(dalloc(&P.r, BN, bytes));
  A(dalloc(&P.V, (size_t)BN * mp1, bytes));
  A(dalloc(&P.xh, (size_t)s.nxi * P.ncols, bytes));
  A(dalloc(&P.yh, (size_t)s.nxi * P.ncols, bytes));
  A(dalloc(&P.H, (size_t)batch * pst * P.restart_max, bytes));
  A(dalloc(&P.cs, (size_t)batch * P.restart_max, bytes));
  A(dalloc(&P.sn, (size_t)batch * P.restart_max, bytes));
  A(dalloc(&P.g, (size_t)batch * pst, bytes));
  A(dalloc(&P.hcol, (size_t)batch * pst, bytes));
  A(dalloc(&P.ycoef, (size_t)batch * P.restart_max, bytes));
  A(dalloc(&P.partial, (size_t)batch * pst * P.nchunk, bytes));
  A(dalloc(&P.nrm_partial, (size_t)batch * std::max(P.nchunk, P.nblk), bytes));
  A(dalloc(&P.nrm, batch, bytes));
  A(dalloc(&P.nrm_keep, batch, bytes));
  A(dalloc(&P.inv64, batch, bytes));
  A(dalloc(&P.target, batch, bytes));
  A(dalloc(&P.active, batch, bytes));
  A(dalloc(&P.reorth, batch, bytes));
  A(dalloc(&P.res_mask, batch, bytes));
  A(dalloc(&P.res_digits, batch, bytes));
  A(dalloc(&P.md_count, batch, bytes));
  A(dalloc(&P.gs_count, batch, bytes));
  A(dalloc(&P.kused, batch, bytes));
  A(dalloc(&P.any_active, 1, bytes));
  P.device_bytes = bytes;
  if (ce != cudaSuccess) {
    std::string msg = std::string("wg_problem_create: device allocation failed: ") + cudaGetErrorString(ce);
    free_all(P);
    delete h;
    cudaGetLastError();
    return fail(nullptr, ce == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA, msg);
  }
  // constant data
  std::vector<double2> phi((size_t)s.nxi * s.nk);
  for (size_t i = 0; i < phi.size(); ++i) phi[i] = make_double2(s.phi[i].real(), s.phi[i].imag());
  std::vector<double> betai((size_t)nK * nK * (s.nxi + 1));
  for (int ac = 0; ac < nK * nK; ++ac)
    for (int i = 0; i <= s.nxi; ++i)
      betai[(size_t)ac * (s.nxi + 1) + i] = -(s.delta_xi / 4 * s.mpc) * s.kap_sum[ac] * s.cap[i];
  API_CK(&P, cudaMemcpyAsync(P.phi, phi.data(), sizeof(double2) * phi.size(), cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.kvec, s.k.data(), sizeof(double) * s.nk, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.xi_edge, s.xi_edge.data(), sizeof(double) * (s.nxi + 1), cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.kap, s.kap.data(), sizeof(double) * s.kap.size(), cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.betai, betai.data(), sizeof(double) * betai.size(), cudaMemcpyHostToDevice, P.stream));
  {
    const int rc = wg::set_kline_factors(P);
    if (rc) return fail(&P, rc, P.err);
  }
  API_CK(&P, cudaMemcpyAsync(P.cosm, s.cosm.data(), sizeof(double) * s.cosm.size(), cudaMemcpyHostToDevice, P.stream));
  {
    std::vector<double2> pinv(s.pinv.size());
    for (size_t i = 0; i < pinv.size(); ++i) pinv[i] = make_double2(s.pinv[i].real(), s.pinv[i].imag());
    API_CK(&P, cudaMemcpyAsync(P.pinv, pinv.data(), sizeof(double2) * pinv.size(), cudaMemcpyHostToDevice, P.stream));
    API_CK(&P, cudaStreamSynchronize(P.stream));
  }
  API_CK(&P, cudaMemsetAsync(P.rhs, 0, sizeof(double2) * BN, P.stream));
  API_CK(&P, cudaMemsetAsync(P.x, 0, sizeof(double2) * BN, P.stream));
  API_CK(&P, cudaMemsetAsync(P.beta, 0, sizeof(double) * batch * s.n_el * nK * nK * (s.nxi + 1), P.stream));
  // a problem never given data is a zero operator with a zero rhs: it is converged and inert
  API_CK(&P, cudaMemsetAsync(P.qd, 0, sizeof(double) * batch, P.stream));
  API_CK(&P, cudaMemsetAsync(P.md_count, 0, sizeof(int) * batch, P.stream));
  API_CK(&P, cudaMemsetAsync(P.nrm, 0, sizeof(double) * batch, P.stream));   // residuals kept by masked problems
  API_CK(&P, cudaMemsetAsync(P.gs_count, 0, sizeof(int) * batch, P.stream));
  API_CK(&P, cudaMemsetAsync(P.pp, 0, sizeof(double) * batch * wg::kPP, P.stream));
  API_CK(&P, cudaMemsetAsync(P.flr, 0, sizeof(double) * batch * 2 * s.nk, P.stream));
  API_CK(&P, cudaMemsetAsync(P.pot_v, 0, sizeof(double) * batch * P.nx, P.stream));
  API_CK(&P, cudaMemsetAsync(P.pot_x, 0, sizeof(double) * batch * P.nx, P.stream));
  API_CK(&P, cudaMemsetAsync(P.m_nodes, 0, sizeof(double) * batch * s.n_el * nK, P.stream));
  API_CK(&P, cudaMemsetAsync(P.xq, 0, sizeof(double) * batch * s.n_el * wg::kNqx, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  if (P.precision == WG_PREC_MIXED || P.fp64_tc) {
    const int mr = P.precision == WG_PREC_MIXED ? wg::mixed_alloc(P) : wg::ozaki_alloc(P);
    if (mr != WG_OK) {
      std::string msg = "wg_problem_create: " + P.err;
      free_all(P);
      delete h;
      return fail(nullptr, mr, msg);
    }
  }
  P.hp.resize(batch);
  P.h_nrm.resize(batch);
  P.h_active.resize(batch);
  P.h_kused.resize(batch);
  *out = h;
  return WG_OK;
}

int wg_problem_bytes(const wg_params* prm, int batch, double* bytes) {
  if (!prm || !bytes || batch < 1) return fail(nullptr, WG_ERR_ARG, "wg_problem_bytes: null argument or batch < 1");
  wg::Shape s;
  const std::string e =
      wg::build_shape_light(s, prm->n_el, prm->n_local, prm->nk, prm->n_xi, prm->l_xi, prm->m_diff, prm->mpc);
  if (!e.empty()) return fail(nullptr, WG_ERR_ARG, "wg_problem_bytes: " + e);
  const int restart = prm->restart > 0 ? prm->restart : 50, inner = prm->inner_restart > 0 ? prm->inner_restart : 40;
  *bytes = wg::estimate_bytes(s, batch, restart, inner, prm->precision, prm->fp64_tc != 0,
                              prm->inner_basis_fp32 == 0);
  return WG_OK;
}

int wg_problem_destroy(wg_problem* h) {
  if (!h) return WG_OK;
  if (h->P.stream) cudaStreamSynchronize(h->P.stream);
  free_all(h->P);
  delete h;
  return WG_OK;
}

int wg_problem_sizes(const wg_problem* h, long long* n_per_problem, int* batch, double* device_bytes) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  if (n_per_problem) *n_per_problem = h->P.N;
  if (batch) *batch = h->P.batch;
  if (device_bytes) *device_bytes = h->P.device_bytes;
  return WG_OK;
}

int wg_runtime_stats_get(const wg_problem* h, wg_runtime_stats* out) {
  if (!h || !out) return fail(h ? const_cast<wg::Problem*>(&h->P) : nullptr, WG_ERR_ARG, "wg_runtime_stats_get: null argument");
  const wg::Problem& P = h->P;
  wg_runtime_stats r{};
  for (const wg::ArnoldiGraphs& G : P.graphs) {
    r.graph_replays += G.replays;
    for (cudaGraphExec_t x : G.exec) r.graphs_captured += x ? 1 : 0;
    r.graphs_disabled |= G.disabled ? 1 : 0;
  }
  r.tuned = P.tuned ? 1 : 0;
  r.kline_chunk = P.kline_L;
  r.stencil_cells = P.st_cells;
  *out = r;
  return WG_OK;
}

int wg_set_launch_shapes(wg_problem* h, int kline_chunk, int stencil_cells) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (kline_chunk < 0 || kline_chunk > P.s.n_el ||
      (kline_chunk > 0 && wg::kline::chunk_count_for(P.s.n_el, kline_chunk) > wg::kline::kMaxChunks))
    return fail(&P, WG_ERR_ARG, "wg_set_launch_shapes: kline_chunk must give 1 .. 64 chunks of at most n_el elements");
  if (stencil_cells != 0 && stencil_cells != 2 && stencil_cells != 4)
    return fail(&P, WG_ERR_ARG, "wg_set_launch_shapes: stencil_cells must be 2 or 4");
  if (kline_chunk) P.kline_L = kline_chunk;
  if (stencil_cells) P.st_cells = stencil_cells;
  P.tuned = true;
  return WG_OK;
}

int wg_set_potential(wg_problem* h, int b, const wg_device* dev, const double* esub_ev, double ef_l, double ef_r) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_set_potential: batch index out of range");
  if (!dev || !esub_ev || !dev->x_nm || !dev->m_kg) return fail(&P, WG_ERR_ARG, "wg_set_potential: null argument");
  if (dev->nx != P.nx)
    return fail(&P, WG_ERR_ARG, "wg_set_potential: nx must equal n_el*(n_local-1)+1 = " + std::to_string(P.nx));
  const wg::Shape& s = P.s;
  const int nK = s.nK, nx = dev->nx;
  for (int i = 0; i < nx; ++i) {
    if (!std::isfinite(esub_ev[i]) || !std::isfinite(dev->x_nm[i]) || !std::isfinite(dev->m_kg[i]))
      return fail(&P, WG_ERR_ARG, "wg_set_potential: non-finite potential, grid or mass");
    if (i > 0 && !(dev->x_nm[i] > dev->x_nm[i - 1]))
      return fail(&P, WG_ERR_ARG, "wg_set_potential: x_nm must be strictly increasing");
  }
  if (dev->x_nm[0] != 0.0) return fail(&P, WG_ERR_ARG, "wg_set_potential: x_nm[0] must be 0");
  if (!std::isfinite(ef_l) || !std::isfinite(ef_r)) return fail(&P, WG_ERR_ARG, "wg_set_potential: non-finite Fermi level");
  wg::HostProblem& hp = P.hp[b];
  hp.l_chi = dev->x_nm[nx - 1] * 1e-9;
  const double detJ = hp.l_chi / s.n_el / 2;
  hp.qd = s.q_diff / detJ * s.mpc;
  hp.ef_l = ef_l;
  hp.ef_r = ef_r;
  {
    double vmax = esub_ev[0];
    for (int i = 1; i < nx; ++i) vmax = std::max(vmax, esub_ev[i]);
    if (!(vmax + 0.3 > 0)) return fail(&P, WG_ERR_ARG, "wg_set_potential: max(Esub)+0.3 must be positive (kz range of verteilung.m:140)");
    if (!(dev->me_z > 0) || !(dev->temp > 0) || !(dev->m_kg[0] > 0) || !(dev->m_kg[nx - 1] > 0))
      return fail(&P, WG_ERR_ARG, "wg_set_potential: masses and Temp must be positive");
  }
  hp.m_nodes.resize((size_t)s.n_el * nK);
  for (int el = 0; el < s.n_el; ++el)
    for (int a = 0; a < nK; ++a) hp.m_nodes[(size_t)el * nK + a] = dev->m_kg[el * (nK - 1) + a];
  std::vector<double> xq, xg(nx);
  wg::quad_points(s, hp.l_chi, xq);
  for (int i = 0; i < nx; ++i) xg[i] = dev->x_nm[i] * 1e-9;
  double pp[wg::kPP] = {};
  pp[wg::PP_LX] = hp.l_chi;
  pp[wg::PP_QD] = hp.qd;
  pp[wg::PP_M0] = dev->m_kg[0];
  pp[wg::PP_M1] = dev->m_kg[nx - 1];
  pp[wg::PP_MEZ] = dev->me_z;
  pp[wg::PP_TEMP] = dev->temp;
  pp[wg::PP_EFL] = ef_l;
  pp[wg::PP_EFR] = ef_r;
  API_CK(&P, cudaMemcpyAsync(P.pp + (long long)b * wg::kPP, pp, sizeof(pp), cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.xq + (long long)b * s.n_el * wg::kNqx, xq.data(), sizeof(double) * xq.size(),
                             cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.pot_x + (long long)b * nx, xg.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.pot_v + (long long)b * nx, esub_ev, sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.m_nodes + (long long)b * s.n_el * nK, hp.m_nodes.data(), sizeof(double) * hp.m_nodes.size(),
                             cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaMemcpyAsync(P.qd + b, &hp.qd, sizeof(double), cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, wg::launch_potential_update(P, b, b + 1));
  // host vectors above go out of scope: wait for the copies
  API_CK(&P, cudaStreamSynchronize(P.stream));
  hp.ready = true;
  return WG_OK;
}

int wg_solve(wg_problem* h, const wg_solve_opts* opts, const double* rho0, wg_solve_info* info) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (!info) return fail(&P, WG_ERR_ARG, "wg_solve: info must hold batch entries");
  for (int b = 0; b < P.batch; ++b)
    if (!P.hp[b].ready) return fail(&P, WG_ERR_ARG, "wg_solve: wg_set_potential not called for problem " + std::to_string(b));
  wg_solve_opts o{};
  if (opts) o = *opts;
  if (o.tol < 0 || !std::isfinite(o.tol)) return fail(&P, WG_ERR_ARG, "wg_solve: tol must be >= 0 and finite");
  bool warm = false;
  if (rho0) {
    const long long n = P.N * P.batch;
    for (long long i = 0; i < 2 * n; ++i)
      if (!std::isfinite(rho0[i])) return fail(&P, WG_ERR_ARG, "wg_solve: rho0 must contain only finite values");
    API_CK(&P, cudaMemcpyAsync(P.x, rho0, sizeof(double2) * n, cudaMemcpyHostToDevice, P.stream));
    warm = true;
  } else if (o.use_rho0) {
    warm = true;
  }
  std::memset(info, 0, sizeof(wg_solve_info) * P.batch);
  int rc = wg::solve_dispatch(P, o, warm, info);
  if (rc == WG_ERR_CUDA || rc == WG_ERR_NUMERIC) fail(&P, rc, P.err);
  return rc;
}

int wg_get_rho(wg_problem* h, int b, double* rho) {
  if (!h || !rho) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_get_rho: null argument");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_get_rho: batch index out of range");
  API_CK(&P, cudaMemcpyAsync(rho, P.x + (long long)b * P.N, sizeof(double2) * P.N, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_set_rho(wg_problem* h, int b, const double* rho) {
  if (!h || !rho) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_set_rho: null argument");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_set_rho: batch index out of range");
  API_CK(&P, cudaMemcpyAsync(P.x + (long long)b * P.N, rho, sizeof(double2) * P.N, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_set_rhs(wg_problem* h, int b, const double* rhs) {
  if (!h || !rhs) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_set_rhs: null argument");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_set_rhs: batch index out of range");
  API_CK(&P, cudaMemcpyAsync(P.rhs + (long long)b * P.N, rhs, sizeof(double2) * P.N, cudaMemcpyHostToDevice,
                             P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_get_observables(wg_problem* h, int b, double* n_dg, double* j) {
  if (!h || !n_dg || !j) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_get_observables: null argument");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_get_observables: batch index out of range");
  const int ncol = P.s.n_el * P.s.nK;
  // two small outputs: reuse the norm-partial scratch when it is large enough, else the xh buffer
  double* dn = reinterpret_cast<double*>(P.xh);
  API_CK(&P, wg::launch_observables(P, b, dn, dn + ncol));
  API_CK(&P, cudaMemcpyAsync(n_dg, dn, sizeof(double) * ncol, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaMemcpyAsync(j, dn + ncol, sizeof(double) * ncol, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_get_rho_xi(wg_problem* h, int b, double* rho_u) {
  if (!h || !rho_u) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_get_rho_xi: null argument");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_get_rho_xi: batch index out of range");
  const long long n = (long long)P.s.n_el * P.s.nK * P.s.nxi;
  API_CK(&P, wg::launch_rho_xi(P, b, P.yh));
  API_CK(&P, cudaMemcpyAsync(rho_u, P.yh, sizeof(double2) * n, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_apply(wg_problem* h, const double* x, double* y) {
  if (!h || !x || !y) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_apply: null argument");
  wg::Problem& P = h->P;
  const long long n = P.N * P.batch;
  API_CK(&P, cudaMemcpyAsync(P.z, x, sizeof(double2) * n, cudaMemcpyHostToDevice, P.stream));
  if (P.precision == WG_PREC_MIXED) API_CK(&P, wg::launch_apply_f64_tc(P, P.z, P.w));
  else API_CK(&P, wg::launch_apply(P, P.z, P.w));
  API_CK(&P, cudaMemcpyAsync(y, P.w, sizeof(double2) * n, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  if (P.mx.err) {
    int herr = 0;
    API_CK(&P, cudaMemcpy(&herr, P.mx.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail(&P, WG_ERR_TIMEOUT, "wg_apply: tensor-core GEMM barrier wait timed out");
  }
  return WG_OK;
}

int wg_apply_lowprec(wg_problem* h, const double* x, double* y) {
  if (!h || !x || !y) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_apply_lowprec: null argument");
  wg::Problem& P = h->P;
  if (P.precision != WG_PREC_MIXED) return fail(&P, WG_ERR_ARG, "wg_apply_lowprec: handle is not mixed precision");
  const long long n = P.N * P.batch;
  API_CK(&P, cudaMemcpyAsync(P.z, x, sizeof(double2) * n, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, wg::apply_mixed_f64(P, P.z, P.w));
  API_CK(&P, cudaMemcpyAsync(y, P.w, sizeof(double2) * n, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  int herr = 0;
  API_CK(&P, cudaMemcpy(&herr, P.mx.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return fail(&P, WG_ERR_TIMEOUT, "wg_apply_lowprec: tensor-core GEMM barrier wait timed out");
  return WG_OK;
}

int wg_precondition(wg_problem* h, const double* r, double* z) {
  if (!h || !r || !z) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_precondition: null argument");
  wg::Problem& P = h->P;
  const long long n = P.N * P.batch;
  API_CK(&P, cudaMemcpyAsync(P.r, r, sizeof(double2) * n, cudaMemcpyHostToDevice, P.stream));
  API_CK(&P, wg::launch_precondition(P, P.r, P.N, P.z));
  API_CK(&P, cudaMemcpyAsync(z, P.z, sizeof(double2) * n, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int wg_gummel_set(wg_problem* h, int b, const wg_device* dev, const wg_rtd_1d* rtd) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_gummel_set: batch index out of range");
  if (!dev || !rtd || !dev->x_nm || !rtd->vc_ev || !rtd->nd_m3 || !rtd->eps_r || !rtd->phi0)
    return fail(&P, WG_ERR_ARG, "wg_gummel_set: null argument");
  if (dev->nx != P.nx) return fail(&P, WG_ERR_ARG, "wg_gummel_set: nx must equal n_el*(n_local-1)+1");
  if (!std::isfinite(rtd->bias) || !std::isfinite(rtd->ef_offset))
    return fail(&P, WG_ERR_ARG, "wg_gummel_set: non-finite bias or Fermi offset");
  // transport data for the initial potential V = Vc - phi0, E_F from the contact band edges
  std::vector<double> v(P.nx);
  for (int i = 0; i < P.nx; ++i) v[i] = rtd->vc_ev[i] - rtd->phi0[i];
  const double efl = rtd->vc_ev[0] + rtd->ef_offset;
  const double efr = rtd->vc_ev[P.nx - 1] + rtd->ef_offset - rtd->bias;
  int rc = wg_set_potential(h, b, dev, v.data(), efl, efr);
  if (rc) return rc;
  rc = wg::gummel_set(P, b, *dev, *rtd);
  if (rc) return fail(&P, rc, P.err);
  return WG_OK;
}

int wg_gummel_run(wg_problem* h, const wg_gummel_opts* opts, wg_gummel_info* info) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (!info) return fail(&P, WG_ERR_ARG, "wg_gummel_run: info must hold batch entries");
  wg_gummel_opts o{};
  if (opts) o = *opts;
  if (o.mixing < 0 || o.mixing > 1) return fail(&P, WG_ERR_ARG, "wg_gummel_run: mixing must be in (0, 1]");
  const int rc = wg::gummel_run(P, o, info);
  if (rc != WG_OK && rc != WG_NOT_CONVERGED) return fail(&P, rc, P.err);
  return rc;
}

int wg_transient_set_bias(wg_problem* h, int b, double bias) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_transient_set_bias: batch index out of range");
  if (!std::isfinite(bias)) return fail(&P, WG_ERR_ARG, "wg_transient_set_bias: non-finite bias");
  const int rc = wg::transient_set_bias(P, b, bias);
  if (rc) return fail(&P, rc, P.err);
  return WG_OK;
}

int wg_transient_run(wg_problem* h, const wg_transient_opts* opts, double* n_hist, double* j_hist,
                     wg_transient_info* info) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (!opts || !info) return fail(&P, WG_ERR_ARG, "wg_transient_run: opts and info (batch entries) are required");
  const int rc = wg::transient_run(P, *opts, n_hist, j_hist, info);
  if (rc != WG_OK && rc != WG_NOT_CONVERGED) return fail(&P, rc, P.err);
  return rc;
}

int wg_gummel_get(wg_problem* h, int b, double* phi, double* n_dg, double* j) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  if (b < 0 || b >= P.batch) return fail(&P, WG_ERR_ARG, "wg_gummel_get: batch index out of range");
  const int rc = wg::gummel_get(P, b, phi, n_dg, j);
  if (rc) return fail(&P, rc, P.err);
  return WG_OK;
}

int wg_apply_noalloc(const wg_operator_view* op, const double* x, double* y, void* stream) {
  if (!op) return fail(nullptr, WG_ERR_ARG, "wg_apply_noalloc: null operator view");
  std::string err;
  const int rc = wg::apply_noalloc(*op, x, y, stream, err);
  if (rc) return fail(nullptr, rc, err);
  return WG_OK;
}

int wg_debug_gemm_bf16(const float* A, const float* B, float* C, int M, int N, int K) {
  if (!A || !B || !C) return fail(nullptr, WG_ERR_ARG, "wg_debug_gemm_bf16: null argument");
  std::string err;
  const int rc = wg::debug_gemm_bf16(A, B, C, M, N, K, err);
  if (rc) return fail(nullptr, rc, "wg_debug_gemm_bf16: " + err);
  return WG_OK;
}

int wg_debug_wait_timeout(long long spin_limit) {
  if (spin_limit < 1 || spin_limit > (1ll << 24))
    return fail(nullptr, WG_ERR_ARG, "wg_debug_wait_timeout: spin_limit must be in 1 .. 2^24");
  std::string err;
  const int rc = wg::debug_wait_timeout(spin_limit, err);
  if (rc) return fail(nullptr, rc, "wg_debug_wait_timeout: " + err);
  return WG_OK;
}

int wg_debug_gemm_f64_tc(const double* A, const double* B, double* C, int M, int N, int K) {
  if (!A || !B || !C) return fail(nullptr, WG_ERR_ARG, "wg_debug_gemm_f64_tc: null argument");
  std::string err;
  const int rc = wg::debug_gemm_f64_tc(A, B, C, M, N, K, err);
  if (rc) return fail(nullptr, rc, "wg_debug_gemm_f64_tc: " + err);
  return WG_OK;
}

int wg_debug_gemm_f64_tc_digits(const double* A, const double* B, double* C, int M, int N, int K, int nd) {
  if (!A || !B || !C || nd < 1 || nd > 8) return fail(nullptr, WG_ERR_ARG, "wg_debug_gemm_f64_tc_digits: null argument or nd outside 1 .. 8");
  std::string err;
  const int rc = wg::debug_gemm_f64_tc(A, B, C, M, N, K, err, nd);
  if (rc) return fail(nullptr, rc, "wg_debug_gemm_f64_tc_digits: " + err);
  return WG_OK;
}

int wg_apply_repeat(wg_problem* h, int which, int n, double* ms) {
  if (!h || !ms || n < 1 || which < 0 || which > 2) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_apply_repeat: bad argument");
  wg::Problem& P = h->P;
  if (which > 0 && P.precision != WG_PREC_MIXED)
    return fail(&P, WG_ERR_ARG, "wg_apply_repeat: the low-precision and tensor-core FP64 operators need a mixed handle");
  cudaEvent_t a = nullptr, b = nullptr;
  API_CK(&P, cudaEventCreate(&a));
  API_CK(&P, cudaEventCreate(&b));
  cudaError_t e = cudaSuccess;
  if (which == 1) {
    e = wg::apply_mixed_repeat(P, P.x, 1);   // conversion and first touch, untimed
    if (e == cudaSuccess) e = cudaEventRecord(a, P.stream);
    if (e == cudaSuccess) e = wg::apply_mixed_repeat(P, P.x, n);
  } else {
    e = which == 2 ? wg::launch_apply_f64_tc(P, P.x, P.w) : wg::launch_apply(P, P.x, P.w);
    if (e == cudaSuccess) e = cudaEventRecord(a, P.stream);
    for (int i = 0; i < n && e == cudaSuccess; ++i)
      e = which == 2 ? wg::launch_apply_f64_tc(P, P.x, P.w) : wg::launch_apply(P, P.x, P.w);
  }
  if (e == cudaSuccess) e = cudaEventRecord(b, P.stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  API_CK(&P, e);
  *ms = t / n;
  return WG_OK;
}

int wg_event_record(wg_problem* h, int slot) {
  if (!h || slot < 0 || slot >= 16) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_event_record: bad slot");
  wg::Problem& P = h->P;
  if (!P.ev[slot]) API_CK(&P, cudaEventCreate(&P.ev[slot]));
  API_CK(&P, cudaEventRecord(P.ev[slot], P.stream));
  return WG_OK;
}

int wg_event_wait(wg_problem* waiter, wg_problem* signaler, int slot) {
  if (!waiter || !signaler || slot < 0 || slot >= 16 || !signaler->P.ev[slot])
    return fail(waiter ? &waiter->P : nullptr, WG_ERR_ARG, "wg_event_wait: null handle or unrecorded slot");
  API_CK(&waiter->P, cudaStreamWaitEvent(waiter->P.stream, signaler->P.ev[slot], 0));
  return WG_OK;
}

int wg_event_elapsed(wg_problem* h, int a, int b, double* ms) {
  if (!h || !ms || a < 0 || b < 0 || a >= 16 || b >= 16 || !h->P.ev[a] || !h->P.ev[b])
    return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_event_elapsed: unrecorded slot");
  wg::Problem& P = h->P;
  API_CK(&P, cudaEventSynchronize(P.ev[b]));
  float f = 0;
  API_CK(&P, cudaEventElapsedTime(&f, P.ev[a], P.ev[b]));
  *ms = f;
  return WG_OK;
}

int wg_profile_enable(wg_problem* h, int on) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  h->P.prof.on = on != 0;
  return WG_OK;
}

int wg_profile_read(wg_problem* h, double* ms, long long* timed, long long* launches, double* bytes, double* flops,
                    int reset) {
  if (!h) return fail(nullptr, WG_ERR_ARG, "null handle");
  wg::Problem& P = h->P;
  API_CK(&P, wg::prof_collect(P));
  for (int i = 0; i < wg::PROF_N; ++i) {
    if (ms) ms[i] = P.prof.ms[i];
    if (timed) timed[i] = P.prof.timed[i];
    if (launches) launches[i] = P.prof.launches[i];
    if (bytes) bytes[i] = P.prof.bytes[i];
    if (flops) flops[i] = P.prof.flops[i];
  }
  if (reset)
    for (int i = 0; i < wg::PROF_N; ++i) {
      P.prof.ms[i] = 0;
      P.prof.timed[i] = 0;
      P.prof.launches[i] = 0;
      P.prof.bytes[i] = 0;
      P.prof.flops[i] = 0;
    }
  return WG_OK;
}

int wg_get_rhs(wg_problem* h, double* rhs) {
  if (!h || !rhs) return fail(h ? &h->P : nullptr, WG_ERR_ARG, "wg_get_rhs: null argument");
  wg::Problem& P = h->P;
  API_CK(&P, cudaMemcpyAsync(rhs, P.rhs, sizeof(double2) * P.N * P.batch, cudaMemcpyDeviceToHost, P.stream));
  API_CK(&P, cudaStreamSynchronize(P.stream));
  return WG_OK;
}

}  // extern "C"
