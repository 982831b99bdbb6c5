// Gummel self-consistency loop of the 1D RTD on the device (sm_103a).
//
// Restates, for Ny = 1 and Dirichlet contacts, the fixed point of
// RTD/solve2D_rtd_self_consistent.m:88-205 with the built-in Poisson step:
//   - project the DG nodal density onto the Poisson control volumes, exact
//     elementwise integrals of the DG polynomial (RTD/project_DG_density_RTD.m:16-31)
//   - one approximate-Newton Poisson update: F = A phi - q (n - N_D),
//     J = A_ff - diag(q^2 n / (kB T)), delta = -J^-1 F (RTD/solve_Poisson2D_rtd.m:113-165)
//     with A the harmonic-mean div(eps grad) stencil (RTD/eval_Poisson2D_rtd.m:108-200)
//   - convergence on the unmixed potential defect, the density change and the
//     Poisson residual; mixing phi <- phi + alpha (phi* - phi) otherwise
//     (solve2D_rtd_self_consistent.m:145-187)
// Every problem of the batch runs its own loop; a converged problem freezes and
// costs nothing in the later transport solves (its GMRES starts converged).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "problem.h"

namespace wg {

namespace {

constexpr double kQP = 1.602176634e-19;   // solve_Poisson2D_rtd.m:79
constexpr double kKBP = 1.380649e-23;     // solve_Poisson2D_rtd.m:80
constexpr double kEps0 = 8.8541878128e-12;  // eval_Poisson2D_rtd.m:28
constexpr int kPcrMax = 2048;                // Poisson unknowns per problem (block of 256 threads)

__device__ double bmax(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = -INFINITY;
  for (int i = 0; i < nw; ++i) r = fmax(r, sh[i]);
  return r;  // every thread
}

__device__ double bsum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  for (int i = 0; i < nw; ++i) r += sh[i];
  return r;
}

// V = Vc - phi on the material grid (electron energy, eV).
__global__ void potential_from_phi_kernel(const double* __restrict__ vc, const double* __restrict__ phi,
                                          double* __restrict__ pot_v, const int* __restrict__ active, int nx) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx || !active[b]) return;
  pot_v[(long long)b * nx + i] = vc[(long long)b * nx + i] - phi[(long long)b * nx + i];
}

// n and j at the DG nodes of every problem (solve_transport_DG_2D.m:147-156),
// n scaled by |Vsub|^2 / dy.  One warp per (node, problem).
__global__ void observables_batched_kernel(const double2* __restrict__ x, const double2* __restrict__ phi,
                                           const double* __restrict__ m_nodes, const double* __restrict__ scale,
                                           double* __restrict__ n_out, double* __restrict__ j_out, int nk, int nxi,
                                           int ncol, long long N, double delta_xi, double pref) {
  const int b = blockIdx.y;
  const int col = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (col >= ncol) return;
  const bool odd = nxi & 1;
  const int c1 = odd ? (nxi - 1) / 2 - 1 : nxi / 2 - 1;
  const int c2 = odd ? (nxi - 1) / 2 + 1 : nxi / 2;
  const int cm = (nxi - 1) / 2;
  double u1r = 0, u1i = 0, u2r = 0, u2i = 0, umr = 0;
  const double2* rx = x + (long long)b * N + (long long)col * nk;
  for (int j = lane; j < nk; j += 32) {
    const double2 r = rx[j];
    const double2 p1 = phi[(long long)c1 * nk + j], p2 = phi[(long long)c2 * nk + j];
    u1r += p1.x * r.x - p1.y * r.y;
    u1i += p1.x * r.y + p1.y * r.x;
    u2r += p2.x * r.x - p2.y * r.y;
    u2i += p2.x * r.y + p2.y * r.x;
    if (odd) {
      const double2 pm = phi[(long long)cm * nk + j];
      umr += pm.x * r.x - pm.y * r.y;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    u1r += __shfl_xor_sync(0xffffffffu, u1r, o);
    u1i += __shfl_xor_sync(0xffffffffu, u1i, o);
    u2r += __shfl_xor_sync(0xffffffffu, u2r, o);
    u2i += __shfl_xor_sync(0xffffffffu, u2i, o);
    umr += __shfl_xor_sync(0xffffffffu, umr, o);
  }
  if (lane == 0) {
    const double m = m_nodes[(long long)b * ncol + col];
    const double pm = m > 0 ? pref / m : 0.0;   // a problem without data stays zero
    double n, jj;
    if (odd) {
      n = umr;
      jj = pm * (u2i - u1i) / 2 / delta_xi;
    } else {
      n = (u1r + u2r) / 2;
      jj = pm * (u2i - u1i) / delta_xi;
    }
    n_out[(long long)b * ncol + col] = n * scale[b];
    j_out[(long long)b * ncol + col] = jj;
  }
}

// One approximate-Newton Poisson step per problem (block per problem).
// diag[b][0..7] = {defect, density change, relres before, linear relres, max|delta|, finite, -, -}
// newton = 1: approximate-Newton step of the Gummel loop; newton = 0: the linear
// Poisson problem A v = q (n - N_D) of the transient (solve_Poisson2D_transient.m),
// solved exactly by the same step with J = A.
__global__ void __launch_bounds__(256) poisson_kernel(const GummelDev G, const int* __restrict__ active, int nx,
                                                      int ncol, int nK, double temp_default, double newton) {
  const int b = blockIdx.x;
  if (!active[b]) return;
  const long long ox = (long long)b * nx;
  const double* phi = G.phi + ox;
  const double* nd = G.nd + ox;
  const double* lo = G.tri + 3 * ox;
  const double* di = lo + nx;
  const double* up = di + nx;
  double* ncv = G.ncv + ox;
  double* cand = G.cand + ox;
  double* wd = G.work + 2 * ox + nx;   // right-hand side -F, then the Newton step
  const double* ndg = G.ndg + (long long)b * ncol;
  const double bias = G.bias[b];
  const double temp = G.temp[b] > 0 ? G.temp[b] : temp_default;
  // 1. control-volume density
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    double acc = 0;
    for (int t = 0; t < 2; ++t) {
      const int e = G.proje[(ox + i) * 2 + t];
      if (e < 0) continue;
      const double* c = G.projc + ((ox + i) * 2 + t) * kMaxLocal;
      for (int a = 0; a < nK; ++a) acc += c[a] * ndg[e * nK + a];
    }
    ncv[i] = acc;
  }
  __syncthreads();
  // 2. residual F = A v - q (n - N_D) on the free nodes, v = phi with Dirichlet values
  double mqn = 0, mqd = 0, mav = 0, mf = 0;
  for (int i = 1 + threadIdx.x; i < nx - 1; i += blockDim.x) {
    const double vm = (i - 1 == 0) ? 0.0 : phi[i - 1];
    const double vp = (i + 1 == nx - 1) ? bias : phi[i + 1];
    const double av = lo[i] * vm + di[i] * phi[i] + up[i] * vp;
    const double f = av - kQP * (ncv[i] - nd[i]);
    wd[i] = -f;
    mqn = fmax(mqn, fabs(kQP * ncv[i]));
    mqd = fmax(mqd, fabs(kQP * nd[i]));
    mav = fmax(mav, fabs(av));
    mf = fmax(mf, fabs(f));
  }
  mqn = bmax(mqn);
  mqd = bmax(mqd);
  mav = bmax(mav);
  mf = bmax(mf);
  const double scale = fmax(fmax(mqn, mqd), fmax(mav, kQP));
  __syncthreads();
  // 3. J delta = -F over the free nodes 1..nx-2 by parallel cyclic reduction in shared
  //    memory (kPcrMax unknowns at most; J is diagonally dominant, so PCR is stable)
  {
    // a, b, c, d and 1/b: 5 x n.  Each row's owner keeps the reciprocal of its diagonal, so a
    // reduction step divides once per row instead of once per (row, neighbour) pair (FP64
    // divisions on one SM are this kernel's cost)
    extern __shared__ double pcr[];
    const int n = nx - 2;
    double* pa = pcr;
    double* pb = pa + n;
    double* pc = pb + n;
    double* pd = pc + n;
    double* pi = pd + n;
    const double g = newton * kQP * kQP / (kKBP * temp);
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      const int i = q + 1;
      pa[q] = q > 0 ? lo[i] : 0.0;
      pb[q] = di[i] - g * ncv[i];
      pi[q] = 1.0 / pb[q];
      pc[q] = q < n - 1 ? up[i] : 0.0;
      pd[q] = wd[i];
    }
    __syncthreads();
    constexpr int R = kPcrMax / 256;
    for (int st = 1; st < n; st <<= 1) {
      double na[R], nb[R], nc[R], nd2[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int q = threadIdx.x + r * 256;
        if (q >= n) continue;
        double a = pa[q], bb = pb[q], c = pc[q], d = pd[q];
        double an = 0.0, cn = 0.0;
        if (q - st >= 0) {
          const double k1 = a * pi[q - st];
          an = -pa[q - st] * k1;
          bb -= pc[q - st] * k1;
          d -= pd[q - st] * k1;
        }
        if (q + st < n) {
          const double k2 = c * pi[q + st];
          cn = -pc[q + st] * k2;
          bb -= pa[q + st] * k2;
          d -= pd[q + st] * k2;
        }
        na[r] = an;
        nb[r] = bb;
        nc[r] = cn;
        nd2[r] = d;
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int q = threadIdx.x + r * 256;
        if (q >= n) continue;
        pa[q] = na[r];
        pb[q] = nb[r];
        pi[q] = 1.0 / nb[r];
        pc[q] = nc[r];
        pd[q] = nd2[r];
      }
      __syncthreads();
    }
    for (int q = threadIdx.x; q < n; q += blockDim.x) wd[q + 1] = pd[q] / pb[q];
  }
  __syncthreads();
  // 4. candidate, defect, linear residual |J delta + F|
  double mdef = 0, mlin = 0, mstep = 0, fin = 1;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    double c;
    if (i == 0) c = 0.0;
    else if (i == nx - 1) c = bias;
    else {
      c = phi[i] + wd[i];
      const double dm = (i > 1) ? wd[i - 1] : 0.0, dp = (i < nx - 2) ? wd[i + 1] : 0.0;
      const double g = newton * kQP * kQP / (kKBP * temp);
      const double jd = lo[i] * dm + (di[i] - g * ncv[i]) * wd[i] + up[i] * dp;
      const double vm = (i - 1 == 0) ? 0.0 : phi[i - 1];
      const double vp = (i + 1 == nx - 1) ? bias : phi[i + 1];
      const double f = lo[i] * vm + di[i] * phi[i] + up[i] * vp - kQP * (ncv[i] - nd[i]);
      mlin = fmax(mlin, fabs(jd + f));
      mstep = fmax(mstep, fabs(wd[i]));
    }
    cand[i] = c;
    mdef = fmax(mdef, fabs(c - phi[i]));
    if (!isfinite(c)) fin = 0;
  }
  mdef = bmax(mdef);
  mlin = bmax(mlin);
  mstep = bmax(mstep);
  fin = -bmax(-fin);
  // 5. density change of the DG nodal density
  double s2 = 0, n2 = 0, p2 = 0;
  const double* np = G.nprev + (long long)b * ncol;
  for (int i = threadIdx.x; i < ncol; i += blockDim.x) {
    const double d = ndg[i] - np[i];
    s2 += d * d;
    n2 += ndg[i] * ndg[i];
    p2 += np[i] * np[i];
  }
  s2 = bsum(s2);
  n2 = bsum(n2);
  p2 = bsum(p2);
  if (threadIdx.x == 0) {
    double* d = G.diag + (long long)b * 8;
    d[0] = mdef;
    d[1] = sqrt(s2) / fmax(fmax(sqrt(n2), sqrt(p2)), 2.2250738585072014e-308);
    d[2] = mf / scale;
    d[3] = mlin / fmax(mf, kQP);
    d[4] = mstep;
    d[5] = fin;
  }
}

// mix[b] == 1: phi <- phi + alpha (cand - phi) and nprev <- n;  mix[b] == 2: nprev <- n only.
__global__ void mix_kernel(const GummelDev G, const int* __restrict__ mix, double alpha, int nx, int ncol) {
  const int b = blockIdx.y;
  if (!mix[b]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nx && mix[b] == 1) {
    const long long o = (long long)b * nx + i;
    G.phi[o] = G.phi[o] + alpha * (G.cand[o] - G.phi[o]);
  }
  if (i < ncol) G.nprev[(long long)b * ncol + i] = G.ndg[(long long)b * ncol + i];
}

// Lagrange basis l_a(r) on the Gauss-Lobatto nodes.
double lagrange(const std::vector<double>& r, int a, double x) {
  double v = 1;
  for (size_t k = 0; k < r.size(); ++k)
    if ((int)k != a) v *= (x - r[k]) / (r[a] - r[k]);
  return v;
}

}  // namespace

cudaError_t gummel_observables(Problem& P) {
  const int ncol = P.s.n_el * P.s.nK;
  const double pref = kQ * (kHV / 2 / M_PI);
  P.prof.launches[PROF_OTHER] += 1;
  observables_batched_kernel<<<dim3((ncol * 32 + 255) / 256, P.batch), 256, 0, P.stream>>>(
      P.x, P.phi, P.m_nodes, P.gd.scale, P.gd.ndg, P.gd.jdg, P.s.nk, P.s.nxi, ncol, P.N, P.s.delta_xi, pref);
  return cudaGetLastError();
}

cudaError_t gummel_poisson(Problem& P, const int* active_dev, bool linear) {
  static const cudaError_t attr = cudaFuncSetAttribute(poisson_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)(5 * sizeof(double) * kPcrMax));
  if (attr != cudaSuccess) return attr;
  P.prof.launches[PROF_OTHER] += 1;
  const size_t smem = 5 * sizeof(double) * (size_t)std::max(1, P.nx - 2);
  poisson_kernel<<<P.batch, 256, smem, P.stream>>>(P.gd, active_dev, P.nx, P.s.n_el * P.s.nK, P.s.nK, 300.0,
                                                   linear ? 0.0 : 1.0);
  return cudaGetLastError();
}

cudaError_t gummel_potential(Problem& P, const int* active_dev) {
  P.prof.launches[PROF_OTHER] += 1;
  potential_from_phi_kernel<<<dim3((P.nx + 255) / 256, P.batch), 256, 0, P.stream>>>(P.gd.vc, P.gd.phi, P.pot_v,
                                                                                     active_dev, P.nx);
  return cudaGetLastError();
}

cudaError_t gummel_mix(Problem& P, const int* mix_dev, double alpha) {
  const int nx = P.nx, ncol = P.s.n_el * P.s.nK;
  P.prof.launches[PROF_OTHER] += 1;
  mix_kernel<<<dim3((std::max(nx, ncol) + 255) / 256, P.batch), 256, 0, P.stream>>>(P.gd, mix_dev, alpha, nx, ncol);
  return cudaGetLastError();
}

int gummel_alloc(Problem& P) {
  if (P.gd.phi) return WG_OK;
  const int B = P.batch, nx = P.nx, ncol = P.s.n_el * P.s.nK;
  GummelDev& G = P.gd;
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(cudaMalloc(&G.vc, sizeof(double) * B * nx));
  A(cudaMalloc(&G.nd, sizeof(double) * B * nx));
  A(cudaMalloc(&G.phi, sizeof(double) * B * nx));
  A(cudaMalloc(&G.phi0, sizeof(double) * B * nx));
  A(cudaMalloc(&G.cand, sizeof(double) * B * nx));
  A(cudaMalloc(&G.ncv, sizeof(double) * B * nx));
  A(cudaMalloc(&G.tri, sizeof(double) * B * 3 * nx));
  A(cudaMalloc(&G.work, sizeof(double) * B * 2 * nx));
  A(cudaMalloc(&G.projc, sizeof(double) * B * nx * 2 * kMaxLocal));
  A(cudaMalloc(&G.proje, sizeof(int) * B * nx * 2));
  A(cudaMalloc(&G.ndg, sizeof(double) * B * ncol));
  A(cudaMalloc(&G.jdg, sizeof(double) * B * ncol));
  A(cudaMalloc(&G.nprev, sizeof(double) * B * ncol));
  A(cudaMalloc(&G.diag, sizeof(double) * B * 8));
  A(cudaMalloc(&G.bias, sizeof(double) * B));
  A(cudaMalloc(&G.temp, sizeof(double) * B));
  A(cudaMalloc(&G.scale, sizeof(double) * B));
  A(cudaMalloc(&G.active, sizeof(int) * B));
  A(cudaMalloc(&G.mix, sizeof(int) * B));
  if (e != cudaSuccess) {
    P.err = std::string("gummel allocation failed: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  cudaMemsetAsync(G.nprev, 0, sizeof(double) * B * ncol, P.stream);
  P.device_bytes += 8.0 * B * (nx * (8 + 2 * kMaxLocal) + 3 * ncol + 12) + 4.0 * B * nx * 2;
  P.gh.assign(B, GummelHost{});
  return WG_OK;
}

void gummel_free(Problem& P) {
  GummelDev& G = P.gd;
  void* ptrs[] = {G.vc, G.nd, G.phi, G.phi0, G.cand, G.ncv, G.tri, G.work, G.projc, G.proje, G.ndg, G.jdg, G.nprev,
                  G.diag, G.bias, G.temp, G.scale, G.active, G.mix};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  G = GummelDev{};
}

#define GK(expr)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (expr);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      P.err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #expr;          \
      return WG_ERR_CUDA;                                                             \
    }                                                                                 \
  } while (0)

int gummel_set(Problem& P, int b, const wg_device& dev, const wg_rtd_1d& rtd) {
  int rc = gummel_alloc(P);
  if (rc) return rc;
  const int nx = P.nx, nK = P.s.nK, n_el = P.s.n_el;
  if (nx - 2 > kPcrMax || nx < 3) {
    P.err = "wg_gummel_set: the Poisson grid needs 3 to " + std::to_string(kPcrMax + 2) + " nodes";
    return WG_ERR_ARG;
  }
  const double* x = dev.x_nm;
  const double dx = x[1] - x[0];
  for (int i = 1; i < nx; ++i)
    if (std::fabs((x[i] - x[i - 1]) - dx) > 1e-10 * dx) {
      P.err = "wg_gummel_set: the Poisson grid must be uniform (eval_Poisson2D_rtd.m checkUniformGrid)";
      return WG_ERR_ARG;
    }
  for (int i = 0; i < nx; ++i)
    if (!std::isfinite(rtd.vc_ev[i]) || !std::isfinite(rtd.nd_m3[i]) || !(rtd.eps_r[i] > 0) ||
        !std::isfinite(rtd.phi0[i]) || rtd.nd_m3[i] < 0) {
      P.err = "wg_gummel_set: Vc, N_D, eps_r and phi0 must be finite (eps_r > 0, N_D >= 0)";
      return WG_ERR_ARG;
    }
  if (!(rtd.dy_nm > 0)) {
    P.err = "wg_gummel_set: dy_nm must be positive";
    return WG_ERR_ARG;
  }
  // Poisson stencil (eval_Poisson2D_rtd.m:114-197), Dirichlet rows at both contacts
  std::vector<double> tri(3 * nx, 0.0);
  const double cx = kEps0 * 1e18 / (dx * dx);
  for (int i = 1; i < nx - 1; ++i) {
    const double e0 = rtd.eps_r[i];
    const double cm = cx * (2 * e0 * rtd.eps_r[i - 1] / (e0 + rtd.eps_r[i - 1]));
    const double cp = cx * (2 * e0 * rtd.eps_r[i + 1] / (e0 + rtd.eps_r[i + 1]));
    tri[i] = cm;
    tri[nx + i] = -(cm + cp);
    tri[2 * nx + i] = cp;
  }
  // projection DG -> dual control volumes (project_DG_density_RTD.m:32-61)
  std::vector<double> projc((size_t)nx * 2 * kMaxLocal, 0.0);
  std::vector<int> proje((size_t)nx * 2, -1);
  const double gq_x[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)};
  const double gq_w[3] = {5.0 / 9, 8.0 / 9, 5.0 / 9};
  for (int i = 0; i < nx; ++i) {
    const double a = i == 0 ? x[0] : 0.5 * (x[i - 1] + x[i]);
    const double bnd = i == nx - 1 ? x[nx - 1] : 0.5 * (x[i] + x[i + 1]);
    const double width = bnd - a;
    int slot = 0;
    for (int e = 0; e < n_el && slot < 2; ++e) {
      const double left = x[e * (nK - 1)], right = x[(e + 1) * (nK - 1)];
      const double lo_ = std::max(a, left), hi_ = std::min(bnd, right);
      if (!(hi_ > lo_)) continue;
      const double jac = (right - left) / 2;
      proje[(size_t)i * 2 + slot] = e;
      for (int q = 0; q < 3; ++q) {
        const double xs = (lo_ + hi_) / 2 + (hi_ - lo_) / 2 * gq_x[q];
        const double r = (xs - (left + right) / 2) / jac;
        for (int aa = 0; aa < nK; ++aa)
          projc[((size_t)i * 2 + slot) * kMaxLocal + aa] += (hi_ - lo_) / 2 * gq_w[q] * lagrange(P.s.r, aa, r) / width;
      }
      ++slot;
    }
  }
  GummelHost& gh = P.gh[b];
  gh.ready = true;
  gh.bias = rtd.bias;
  const long long ox = (long long)b * nx;
  GummelDev& G = P.gd;
  const double scale = 1.0 / (rtd.dy_nm * 1e-9);
  GK(cudaMemcpyAsync(G.vc + ox, rtd.vc_ev, sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.nd + ox, rtd.nd_m3, sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.phi + ox, rtd.phi0, sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.phi0 + ox, rtd.phi0, sizeof(double) * nx, cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.tri + 3 * ox, tri.data(), sizeof(double) * 3 * nx, cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.projc + ox * 2 * kMaxLocal, projc.data(), sizeof(double) * projc.size(), cudaMemcpyHostToDevice,
                     P.stream));
  GK(cudaMemcpyAsync(G.proje + ox * 2, proje.data(), sizeof(int) * proje.size(), cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.bias + b, &rtd.bias, sizeof(double), cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.temp + b, &dev.temp, sizeof(double), cudaMemcpyHostToDevice, P.stream));
  GK(cudaMemcpyAsync(G.scale + b, &scale, sizeof(double), cudaMemcpyHostToDevice, P.stream));
  GK(cudaStreamSynchronize(P.stream));
  return WG_OK;
}

namespace {

struct LoopOpts {
  int maxit;
  double alpha, tol_v, tol_n, tol_p, tol, cap;
  int transport_maxit;
  bool inexact;
  int defer;   // iterations a loosely converged problem may wait for the batched final re-solve (0: none)
};

LoopOpts loop_opts(const wg_gummel_opts& o) {
  LoopOpts L;
  L.maxit = o.max_iterations > 0 ? o.max_iterations : 100;
  L.alpha = o.mixing > 0 ? o.mixing : 0.1;
  L.tol_v = o.potential_tol > 0 ? o.potential_tol : 5e-4;
  L.tol_n = o.density_tol > 0 ? o.density_tol : 5e-4;
  L.tol_p = o.poisson_residual_tol > 0 ? o.poisson_residual_tol : 8e-2;
  L.tol = o.transport_tol > 0 ? o.transport_tol : 1e-8;
  L.transport_maxit = o.transport_maxit > 0 ? o.transport_maxit : 50;
  // Inexact Gummel (opt-in): transport tolerance tied to the potential defect,
  // tol_b = clamp(factor * defect_b, final tol, cap); convergence is accepted only
  // after a transport solve at the final tolerance with the same potential.
  L.inexact = o.inexact_factor > 0;
  L.cap = o.inexact_cap > 0 ? o.inexact_cap : 1e-4;
  L.defer = !L.inexact || o.defer_final < 0 ? 0 : (o.defer_final > 0 ? o.defer_final : 64);
  return L;
}

double clock_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int gummel_start(Problem& P, int b, const wg_gummel_opts& o, bool warm, bool from_phi0) {
  if (!P.gd.phi || !P.gh[b].ready || !P.hp[b].ready) {
    P.err = "Gummel start: problem " + std::to_string(b) + " lacks wg_set_potential/wg_gummel_set";
    return WG_ERR_ARG;
  }
  const int nx = P.nx, ncol = P.s.n_el * P.s.nK;
  const LoopOpts L = loop_opts(o);
  GummelHost& gh = P.gh[b];
  gh.running = 1;
  gh.waiting = -1;
  gh.it = 0;
  gh.tol = L.inexact ? std::max(L.cap, L.tol) : L.tol;
  gh.t0 = clock_s();
  std::memset(&gh.info, 0, sizeof(wg_gummel_info));
  gh.info.status = WG_GUMMEL_ITERATION_LIMIT;
  gh.info.density_change = INFINITY;
  GummelDev& G = P.gd;
  GK(cudaMemsetAsync(G.nprev + (long long)b * ncol, 0, sizeof(double) * ncol, P.stream));
  if (from_phi0)
    GK(cudaMemcpyAsync(G.phi + (long long)b * nx, G.phi0 + (long long)b * nx, sizeof(double) * nx,
                       cudaMemcpyDeviceToDevice, P.stream));
  if (!warm) GK(cudaMemsetAsync(P.x + (long long)b * P.N, 0, sizeof(double2) * P.N, P.stream));
  return WG_OK;
}

int gummel_iterate(Problem& P, const wg_gummel_opts& o, int* still_running) {
  const int B = P.batch;
  const LoopOpts L = loop_opts(o);
  GummelDev& G = P.gd;
  std::vector<int> active(B, 0), mix(B, 0);
  int n_run = 0, n_loose = 0;
  for (int b = 0; b < B; ++b) n_loose += P.gh[b].running && P.gh[b].waiting < 0;
  for (int b = 0; b < B; ++b) {
    GummelHost& gh = P.gh[b];
    // a problem waiting for its final re-solve runs once no other is in its loose phase or its
    // wait is over; until then it is frozen (its iterates do not depend on when they run)
    if (gh.running && gh.waiting >= 0 && (n_loose == 0 || gh.waiting >= L.defer)) gh.waiting = -1;
    active[b] = gh.running && gh.waiting < 0;
    n_run += gh.running;
  }
  *still_running = n_run;
  if (!n_run) return WG_OK;
  for (int b = 0; b < B; ++b)
    if (P.gh[b].running && P.gh[b].waiting >= 0) ++P.gh[b].waiting;
  std::vector<double> diag(8 * B);
  std::vector<wg_solve_info> sinfo(B);
  struct TolGuard {
    Problem& P;
    ~TolGuard() { P.tol_pp.clear(); }
  } guard{P};
  GK(cudaMemcpyAsync(G.active, active.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
  GK(gummel_potential(P, G.active));
  GK(launch_potential_update(P, 0, B, G.active));
  // problems outside their loop keep their state: an unreachable target freezes them
  P.tol_pp.assign(B, 1e300);
  for (int b = 0; b < B; ++b)
    if (active[b]) P.tol_pp[b] = P.gh[b].tol;
  wg_solve_opts so{};
  so.tol = L.tol;
  so.maxit = L.transport_maxit;
  int rc = solve_dispatch(P, so, /*warm=*/true, sinfo.data());
  if (rc != WG_OK && rc != WG_NOT_CONVERGED) return rc;
  GK(gummel_observables(P));
  GK(gummel_poisson(P, G.active, false));
  GK(cudaMemcpyAsync(diag.data(), G.diag, sizeof(double) * 8 * B, cudaMemcpyDeviceToHost, P.stream));
  GK(cudaStreamSynchronize(P.stream));
  const double tnow = clock_s();
  for (int b = 0; b < B; ++b) {
    if (!active[b]) continue;
    GummelHost& gh = P.gh[b];
    wg_gummel_info& in = gh.info;
    const int it = ++gh.it;
    in.iterations = it;
    in.seconds = tnow - gh.t0;
    in.gmres_iterations += sinfo[b].iterations;
    in.transport_relres = sinfo[b].relres;
    gh.running = 0;
    if (sinfo[b].flag != 0 || !std::isfinite(sinfo[b].relres)) {
      in.status = WG_GUMMEL_TRANSPORT_FAILED;
      continue;
    }
    const double* d = &diag[8 * b];
    in.potential_defect = d[0];
    in.density_change = it == 1 ? INFINITY : d[1];
    in.poisson_relres = d[2];
    if (d[5] == 0 || !(d[3] < 1e-8)) {
      in.status = WG_GUMMEL_POISSON_FAILED;
      continue;
    }
    const bool conv = in.potential_defect <= L.tol_v && in.density_change <= L.tol_n && in.poisson_relres <= L.tol_p;
    if (conv && gh.tol <= L.tol) {
      in.status = WG_GUMMEL_CONVERGED;
      continue;
    }
    if (it >= L.maxit) continue;  // never hand back a potential newer than the transport state
    gh.running = 1;
    if (conv) {
      // converged on a loose transport solve: re-solve at the final tolerance, same potential
      // (batched with the other problems' final solves when waiting is allowed)
      gh.tol = L.tol;
      mix[b] = 2;
      if (L.defer > 0) gh.waiting = 0;
      continue;
    }
    if (L.inexact) gh.tol = std::min(L.cap, std::max(L.tol, o.inexact_factor * in.potential_defect));
    mix[b] = 1;
  }
  GK(cudaMemcpyAsync(G.mix, mix.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
  GK(gummel_mix(P, G.mix, L.alpha));
  GK(cudaStreamSynchronize(P.stream));   // mix[] is a host vector
  n_run = 0;
  for (int b = 0; b < B; ++b) n_run += P.gh[b].running;
  *still_running = n_run;
  return WG_OK;
}

int gummel_run(Problem& P, const wg_gummel_opts& o, wg_gummel_info* info) {
  const int B = P.batch;
  if (!P.gd.phi) {
    P.err = "wg_gummel_run: wg_gummel_set was not called";
    return WG_ERR_ARG;
  }
  for (int b = 0; b < B; ++b)
    if (!P.gh[b].ready || !P.hp[b].ready) {
      P.err = "wg_gummel_run: problem " + std::to_string(b) + " lacks wg_set_potential/wg_gummel_set";
      return WG_ERR_ARG;
    }
  for (int b = 0; b < B; ++b) {
    const int rc = gummel_start(P, b, o, o.warm_start != 0, o.restart_from_phi0 != 0);
    if (rc) return rc;
  }
  int running = B;
  while (running > 0) {
    const int rc = gummel_iterate(P, o, &running);
    if (rc) return rc;
  }
  int status = WG_OK;
  for (int b = 0; b < B; ++b) {
    info[b] = P.gh[b].info;
    if (info[b].status != WG_GUMMEL_CONVERGED) status = WG_NOT_CONVERGED;
  }
  return status;
}

int gummel_get(Problem& P, int b, double* phi, double* n_dg, double* j) {
  if (!P.gd.phi) {
    P.err = "wg_gummel_get: wg_gummel_set was not called";
    return WG_ERR_ARG;
  }
  const int nx = P.nx, ncol = P.s.n_el * P.s.nK;
  if (phi) GK(cudaMemcpyAsync(phi, P.gd.phi + (long long)b * nx, sizeof(double) * nx, cudaMemcpyDeviceToHost, P.stream));
  if (n_dg) GK(cudaMemcpyAsync(n_dg, P.gd.ndg + (long long)b * ncol, sizeof(double) * ncol, cudaMemcpyDeviceToHost, P.stream));
  if (j) GK(cudaMemcpyAsync(j, P.gd.jdg + (long long)b * ncol, sizeof(double) * ncol, cudaMemcpyDeviceToHost, P.stream));
  GK(cudaStreamSynchronize(P.stream));
  return WG_OK;
}

}  // namespace wg
