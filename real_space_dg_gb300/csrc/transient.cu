// Transient self-consistent solve of the 1D RTD on the device (sm_103a).
//
// DG_code/solve_transport_DG_2D_transient_SC_new.m:124-212 for every problem of
// a Gummel handle, from its resident state:
//   d rho / dt = s_r rhs - s_A A rho          (A scaled by 2e-10 at :148)
//   before step t, if (t-1) % E == 0 or t < F: operator and inflow rebuilt from
//                                              the potential (:131-149)
//   step: RK4 (:153-158) or Crank-Nicolson, one shifted GMRES solve
//   after step t: n, j at the DG nodes (:161-185); if t % E == 0 or t < F the
//                 linear Poisson problem for that density (:204-211 with
//                 solve_Poisson2D_transient.m)
// Crank-Nicolson divided by dt s_A / 2 reads
//   (A + sigma I) rho' = (sigma I - A) rho + (2 s_r / s_A) rhs,  sigma = 2 / (dt s_A),
// which keeps the operator kernels (the flux kernel adds sigma x) and the k-line
// preconditioner (factors of the shifted flux blocks).  Every step's GMRES starts
// from the previous state.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "problem.h"

namespace wg {

namespace {

__global__ void cn_rhs_kernel(const double2* __restrict__ rhs, const double2* __restrict__ w,
                              double2* __restrict__ b, double g, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double2 r = rhs[t], v = w[t];
  b[t] = make_double2(g * r.x - v.x, g * r.y - v.y);
}

// One RK4 stage with k = s_r rhs - s_A w (w = A u):
//   mode 0: acc = k,       u = x + cu k
//   mode 1: acc += 2 k,    u = x + cu k
//   mode 2: x += dt/6 (acc + k)
__global__ void rk4_stage_kernel(const double2* __restrict__ rhs, const double2* __restrict__ w,
                                 double2* __restrict__ x, double2* __restrict__ u, double2* __restrict__ acc,
                                 double sr, double sa, double cu, double dt6, int mode, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double2 r = rhs[t], v = w[t];
  const double2 k = make_double2(sr * r.x - sa * v.x, sr * r.y - sa * v.y);
  const double2 xv = x[t];
  if (mode == 2) {
    const double2 a = acc[t];
    x[t] = make_double2(xv.x + dt6 * (a.x + k.x), xv.y + dt6 * (a.y + k.y));
    return;
  }
  if (mode == 0) {
    acc[t] = k;
  } else {
    const double2 a = acc[t];
    acc[t] = make_double2(a.x + 2.0 * k.x, a.y + 2.0 * k.y);
  }
  u[t] = make_double2(xv.x + cu * k.x, xv.y + cu * k.y);
}

unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

#define TK(expr)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (expr);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      P.err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #expr;          \
      return WG_ERR_CUDA;                                                             \
    }                                                                                 \
  } while (0)

int transient_set_bias(Problem& P, int b, double bias) {
  if (!P.gd.phi || !P.gh[b].ready) {
    P.err = "wg_transient_set_bias: wg_gummel_set was not called for problem " + std::to_string(b);
    return WG_ERR_ARG;
  }
  GummelHost& gh = P.gh[b];
  HostProblem& hp = P.hp[b];
  // E_F,R = Vc(end) + offset - bias (solve2D_rtd_self_consistent.m:110-116)
  hp.ef_r += gh.bias - bias;
  gh.bias = bias;
  gh.step_pending = true;
  TK(cudaMemcpyAsync(P.gd.bias + b, &gh.bias, sizeof(double), cudaMemcpyHostToDevice, P.stream));
  TK(cudaMemcpyAsync(P.pp + (long long)b * kPP + PP_EFR, &hp.ef_r, sizeof(double), cudaMemcpyHostToDevice,
                     P.stream));
  TK(cudaStreamSynchronize(P.stream));
  return WG_OK;
}

namespace {

// Restores the stationary operator (no shift, unshifted k-line factors) on every exit.
struct ShiftGuard {
  Problem& P;
  bool shifted = false;
  ~ShiftGuard() {
    if (!shifted) return;
    P.shift = 0;
    std::string keep = P.err;
    set_kline_factors(P);
    P.err = keep;
  }
};

cudaError_t apply_f64(Problem& P, const double2* x, double2* y) {
  return P.precision == WG_PREC_MIXED ? launch_apply_f64_tc(P, x, y) : launch_apply(P, x, y);
}

}  // namespace

int transient_run(Problem& P, const wg_transient_opts& o, double* n_hist, double* j_hist, wg_transient_info* info) {
  const int B = P.batch, ncol = P.s.n_el * P.s.nK;
  if (!P.gd.phi) {
    P.err = "wg_transient_run: wg_gummel_set was not called";
    return WG_ERR_ARG;
  }
  for (int b = 0; b < B; ++b)
    if (!P.gh[b].ready || !P.hp[b].ready) {
      P.err = "wg_transient_run: problem " + std::to_string(b) + " lacks wg_gummel_set";
      return WG_ERR_ARG;
    }
  if (!(o.dt > 0) || !std::isfinite(o.dt) || o.nsteps < 0 || (o.method != WG_TRANSIENT_CN && o.method != WG_TRANSIENT_RK4) ||
      o.scale_a < 0 || o.scale_rhs < 0 || o.tol < 0 || o.record_every < 0) {
    P.err = "wg_transient_run: need dt > 0, nsteps >= 0, a known method and non-negative scales, tol, record_every";
    return WG_ERR_ARG;
  }
  const double sa = o.scale_a > 0 ? o.scale_a : 2e-10;
  const double sr = o.scale_rhs > 0 ? o.scale_rhs : sa;
  const int E = o.refresh_every == 0 ? 20 : o.refresh_every;   // < 0: never
  const int F = o.refresh_first == 0 ? 50 : std::max(0, o.refresh_first);
  const bool cn = o.method == WG_TRANSIENT_CN;
  const long long tot = P.N * B;
  const int rec = o.record_every;
  const int nrec = rec > 0 ? o.nsteps / rec : 0;
  GummelDev& G = P.gd;
  for (int b = 0; b < B; ++b) std::memset(&info[b], 0, sizeof(wg_transient_info));
  const auto t0 = std::chrono::steady_clock::now();

  // device history [nrec][2][B][ncol]
  double* hist = nullptr;
  struct Free {
    double*& p;
    ~Free() {
      if (p) cudaFree(p);
    }
  } free_hist{hist};
  if (nrec > 0 && (n_hist || j_hist)) TK(cudaMalloc(&hist, sizeof(double) * 2 * (size_t)nrec * B * ncol));
  if (cn && !P.tr_b) {
    TK(cudaMalloc(&P.tr_b, sizeof(double2) * tot));
    P.device_bytes += 16.0 * tot;
  }

  std::vector<int> ones(B, 1), pend(B, 0);
  bool any_pending = false;
  for (int b = 0; b < B; ++b) {
    pend[b] = P.gh[b].step_pending ? 1 : 0;
    any_pending |= pend[b] != 0;
  }
  // a bias step: potential for the current density with the new contact value
  if (any_pending) {
    TK(cudaMemcpyAsync(G.active, pend.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
    TK(cudaMemcpyAsync(G.mix, pend.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
    TK(gummel_observables(P));
    TK(gummel_poisson(P, G.active, true));
    TK(gummel_mix(P, G.mix, 1.0));
    for (int b = 0; b < B; ++b)
      if (pend[b]) {
        ++info[b].poisson_solves;
        P.gh[b].step_pending = false;
      }
  }
  TK(cudaMemcpyAsync(G.active, ones.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
  TK(cudaMemcpyAsync(G.mix, ones.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));

  ShiftGuard guard{P};
  const double sigma = 2.0 / (o.dt * sa);
  if (cn) {
    guard.shifted = true;
    P.shift = sigma;
    const int rc = set_kline_factors(P);
    if (rc) return rc;
  }
  wg_solve_opts so{};
  so.tol = o.tol > 0 ? o.tol : 1e-10;
  so.maxit = o.maxit > 0 ? o.maxit : 20;
  so.use_rho0 = 1;
  std::vector<wg_solve_info> sinfo(B);
  int irec = 0;
  for (int t = 1; t <= o.nsteps; ++t) {
    if (t == 1 || (E > 0 && ((t - 1) % E == 0 || t < F))) {
      TK(gummel_potential(P, G.active));
      // the update rebuilds the operator and the inflow; a fixed right-hand side is kept in r
      // (free between steps) and put back
      if (o.fixed_rhs) TK(cudaMemcpyAsync(P.r, P.rhs, sizeof(double2) * tot, cudaMemcpyDeviceToDevice, P.stream));
      TK(launch_potential_update(P, 0, B));
      if (o.fixed_rhs) TK(cudaMemcpyAsync(P.rhs, P.r, sizeof(double2) * tot, cudaMemcpyDeviceToDevice, P.stream));
      for (int b = 0; b < B; ++b) ++info[b].refreshes;
    }
    if (cn) {
      // b = (2 s_r / s_A) rhs - (A - sigma I) rho^n
      P.shift = -sigma;
      TK(apply_f64(P, P.x, P.w));
      P.prof.launches[PROF_OTHER] += 1;
      cn_rhs_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.rhs, P.w, P.tr_b, 2.0 * sr / sa, tot);
      TK(cudaGetLastError());
      P.shift = sigma;
      std::swap(P.rhs, P.tr_b);
      const int rc = solve_dispatch(P, so, /*warm=*/true, sinfo.data());
      std::swap(P.rhs, P.tr_b);
      if (rc != WG_OK && rc != WG_NOT_CONVERGED) return rc;
      for (int b = 0; b < B; ++b) {
        info[b].gmres_iterations += sinfo[b].iterations;
        const double rr = sinfo[b].relres;
        info[b].max_relres = std::isfinite(rr) ? std::max(info[b].max_relres, rr) : INFINITY;
        if (sinfo[b].flag != 0 || !std::isfinite(rr)) info[b].status = 1;
      }
    } else {
      const double cu[3] = {o.dt / 2, o.dt / 2, o.dt};
      for (int st = 0; st < 4; ++st) {
        TK(apply_f64(P, st == 0 ? P.x : P.z, P.w));
        P.prof.launches[PROF_OTHER] += 1;
        rk4_stage_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.rhs, P.w, P.x, P.z, P.r, sr, sa,
                                                                st < 3 ? cu[st] : 0.0, o.dt / 6,
                                                                st == 0 ? 0 : (st == 3 ? 2 : 1), tot);
        TK(cudaGetLastError());
      }
    }
    TK(gummel_observables(P));
    if (hist && t % rec == 0 && irec < nrec) {
      const size_t slab = (size_t)B * ncol;
      TK(cudaMemcpyAsync(hist + (size_t)irec * 2 * slab, G.ndg, sizeof(double) * slab, cudaMemcpyDeviceToDevice,
                         P.stream));
      TK(cudaMemcpyAsync(hist + ((size_t)irec * 2 + 1) * slab, G.jdg, sizeof(double) * slab,
                         cudaMemcpyDeviceToDevice, P.stream));
      ++irec;
    }
    if (E > 0 && (t % E == 0 || t < F)) {
      TK(gummel_poisson(P, G.active, true));
      TK(gummel_mix(P, G.mix, 1.0));
      for (int b = 0; b < B; ++b) ++info[b].poisson_solves;
    }
    for (int b = 0; b < B; ++b) info[b].steps = t;
  }
  TK(cudaStreamSynchronize(P.stream));
  if (hist) {
    const size_t slab = (size_t)B * ncol;
    std::vector<double> h((size_t)irec * 2 * slab);
    TK(cudaMemcpy(h.data(), hist, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
    for (int r = 0; r < irec; ++r) {
      if (n_hist) std::memcpy(n_hist + r * slab, &h[(size_t)r * 2 * slab], sizeof(double) * slab);
      if (j_hist) std::memcpy(j_hist + r * slab, &h[((size_t)r * 2 + 1) * slab], sizeof(double) * slab);
    }
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int b = 0; b < B; ++b) info[b].seconds = secs;
  if (cn) {
    guard.shifted = false;
    P.shift = 0;
    const int rc = set_kline_factors(P);
    if (rc) return rc;
  }
  for (int b = 0; b < B; ++b)
    if (info[b].status != 0) return WG_NOT_CONVERGED;
  return WG_OK;
}

}  // namespace wg
