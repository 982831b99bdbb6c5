// Device-side rebuild of everything that depends on the potential (sm_103a).
//
// For problems [b0, b1) of a handle, from the potential V(x) on the material grid:
//   minmax_kernel   min V (V(x >= Lx) of V_transient.m:6) and max V (kz range of
//                   verteilung.m:140)
//   fermi_kernel    f_L(k), f_R(k): Fermi-Dirac occupation integrated over 1001 kz
//                   (verteilung.m:139-152), one block per (k, problem)
//   inflow_kernel   cosine transform to the xi cells, least-squares projection on
//                   Phi (pseudo-inverse, verteilung.m:158-168) and the contact
//                   inflow blocks of the rhs (get_Diff.m:77-83)
//   vw_kernel       Wigner-potential weights beta[e][ab][s] (the Vw(x,k) rebuild of
//                   get_Drift_accel_trial_permutedShell.m:64-147, contracted with the
//                   element quadrature)
#include <cuda_runtime.h>

#include "problem.h"

namespace wg {

namespace {

constexpr double kPi = 3.141592653589793;

__device__ double block_reduce(double v, bool is_max) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, t) : (v + t);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < nw ? sh[threadIdx.x] : (is_max ? -INFINITY : 0.0);
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(0xffffffffu, v, o);
      v = is_max ? fmax(v, t) : (v + t);
    }
  return v;  // valid in warp 0
}

__global__ void minmax_kernel(const double* __restrict__ pot_v, double* __restrict__ pp, int nx, int b0,
                              const int* __restrict__ mask) {
  const int b = b0 + blockIdx.x;
  if (mask && !mask[b]) return;
  const double* v = pot_v + (long long)b * nx;
  double mx = -INFINITY, mn = INFINITY;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    mx = fmax(mx, v[i]);
    mn = fmin(mn, v[i]);
  }
  mx = block_reduce(mx, true);
  const double mneg = block_reduce(-mn, true);
  if (threadIdx.x == 0) {
    pp[b * kPP + PP_VMAX] = mx;
    pp[b * kPP + PP_VMIN] = -mneg;
  }
}

// f_{L,R}(k_j) = 2/pi dkz sum_z 1/(1 + exp(q (E_{L,R}(k) + E_kz - E_F) / (kB T)))
__global__ void fermi_kernel(const double* __restrict__ pot_v, const double* __restrict__ pp,
                             const double* __restrict__ kvec, double* __restrict__ flr, int nx, int nk, int b0,
                             const int* __restrict__ mask) {
  const int j = blockIdx.x, b = b0 + blockIdx.y;
  if (mask && !mask[b]) return;
  const double* P = pp + b * kPP;
  const double hb = kHV / 2 / kPi;
  const double k = kvec[j];
  const double v0 = pot_v[(long long)b * nx], v1 = pot_v[(long long)b * nx + nx - 1];
  const double EL = v0 + hb * hb * k * k / 2 / P[PP_M0] / kQV;
  const double ER = v1 + hb * hb * k * k / 2 / P[PP_M1] / kQV;
  const double me_z = P[PP_MEZ], temp = P[PP_TEMP];
  const double kz_max = sqrt(2 * 2 * kM0V * me_z * kQV * (P[PP_VMAX] + 0.3)) / hb;
  const double dkz = kz_max / (kNkz - 1);
  double sl = 0, sr = 0;
  for (int z = threadIdx.x; z < kNkz; z += blockDim.x) {
    const double kz = (z == kNkz - 1) ? kz_max : z * dkz;
    const double ekz = hb * hb * kz * kz / 2 / kM0V / me_z / kQV;
    sl += 1.0 / (1.0 + exp(kQV * (EL + ekz - P[PP_EFL]) / (kKBV * temp)));
    sr += 1.0 / (1.0 + exp(kQV * (ER + ekz - P[PP_EFR]) / (kKBV * temp)));
  }
  sl = block_reduce(sl, false);
  sr = block_reduce(sr, false);
  if (threadIdx.x == 0) {
    flr[((long long)b * 2 + 0) * nk + j] = 2 / kPi * dkz * sl;
    flr[((long long)b * 2 + 1) * nk + j] = 2 / kPi * dkz * sr;
  }
}

// fLn(s) = sum_j cos(xi_s k_j) f(k_j) dk/(2 pi); fnl = Phi^+ fLn; rhs blocks.
__global__ void inflow_kernel(const double* __restrict__ flr, const double* __restrict__ cosm,
                              const double2* __restrict__ pinv, const double* __restrict__ kvec,
                              const double* __restrict__ pp, double2* __restrict__ rhs, FluxBlocks fb, int nk,
                              int nxi, int n_el, long long N, double q_diff, double mpc, int b0,
                              const int* __restrict__ mask) {
  extern __shared__ double sm[];  // [2][nxi]
  const int b = b0 + blockIdx.x;
  if (mask && !mask[b]) return;
  const double* fL = flr + (long long)b * 2 * nk;
  const double* fR = fL + nk;
  const double dk = fabs(kvec[1] - kvec[0]);
  for (int s = threadIdx.x; s < nxi; s += blockDim.x) {
    double al = 0, ar = 0;
    const double* c = cosm + (long long)s * nk;
    for (int j = 0; j < nk; ++j) {
      al += c[j] * fL[j];
      ar += c[j] * fR[j];
    }
    sm[s] = al * dk / 2 / kPi;
    sm[nxi + s] = ar * dk / 2 / kPi;
  }
  __syncthreads();
  const int nK = fb.nK;
  const double detJ = pp[b * kPP + PP_LX] / n_el / 2;
  double2* rfirst = rhs + (long long)b * N;
  double2* rlast = rfirst + (long long)(n_el - 1) * nK * nk;
  for (int j = threadIdx.x; j < nk; j += blockDim.x) {
    double2 zl = make_double2(0, 0), zr = make_double2(0, 0);
    const double2* pr = pinv + (long long)j * nxi;
    for (int s = 0; s < nxi; ++s) {
      const double2 w = pr[s];
      zl.x += w.x * sm[s];
      zl.y += w.y * sm[s];
      zr.x += w.x * sm[nxi + s];
      zr.y += w.y * sm[nxi + s];
    }
    const double k = kvec[j], ak = fabs(k);
    const double fl = k > 0 ? 1.0 : 0.0, fr = k < 0 ? 1.0 : 0.0;
    for (int a = 0; a < nK; ++a) {
      const double q1 = fb.invM[a * nK + 0] / detJ, q2 = fb.invM[a * nK + nK - 1] / detJ;
      rfirst[(long long)a * nk + j] =
          make_double2(mpc * (q_diff * (q1 * (fl * (ak * zl.x)))), mpc * (q_diff * (q1 * (fl * (ak * zl.y)))));
      rlast[(long long)a * nk + j] =
          make_double2(mpc * (q_diff * (q2 * (fr * (ak * zr.x)))), mpc * (q_diff * (q2 * (fr * (ak * zr.y)))));
    }
  }
}

__device__ double v_lookup(double x, const double* __restrict__ xg, const double* __restrict__ vg, int nx, double lx,
                           double vmin) {
  if (x < 0) return vg[0];
  if (x >= lx) return vmin;
  int lo = 0, hi = nx - 1;
  if (x >= xg[hi]) return vg[hi];
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xg[mid] <= x) lo = mid; else hi = mid;
  }
  const double slope = (vg[lo + 1] - vg[lo]) / (xg[lo + 1] - xg[lo]);
  return slope * (x - xg[lo]) + vg[lo];
}

// beta[b][e][ac][s] = (dxi/4) mpc sum_q kap[ac][q] (V(x_q + xi_s/2) - V(x_q - xi_s/2))
template <int NK>
__global__ void vw_kernel(double* __restrict__ beta, const double* __restrict__ xq, const double* __restrict__ xi_edge,
                          const double* __restrict__ kap, const double* __restrict__ pot_x,
                          const double* __restrict__ pot_v, const double* __restrict__ pp, int nx, int n_el, int nxi,
                          double scale, int b0, const int* __restrict__ mask) {
  if (mask && !mask[b0 + blockIdx.y]) return;
  const int ne = nxi + 1;
  const int b = b0 + blockIdx.y;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_el * ne) return;
  const int s = (int)(t % ne);
  const int e = (int)(t / ne);
  const double xi = xi_edge[s];
  const double* xg = pot_x + (long long)b * nx;
  const double* vg = pot_v + (long long)b * nx;
  const double lx = pp[b * kPP + PP_LX], vmin = pp[b * kPP + PP_VMIN];
  const double* xqb = xq + (long long)b * n_el * kNqx + e * kNqx;
  double dv[kNqx];
#pragma unroll
  for (int q = 0; q < kNqx; ++q) {
    const double x = xqb[q];
    dv[q] = v_lookup(x + 0.5 * xi, xg, vg, nx, lx, vmin) - v_lookup(x - 0.5 * xi, xg, vg, nx, lx, vmin);
  }
  double* be = beta + ((long long)b * n_el + e) * NK * NK * ne;
#pragma unroll
  for (int ac = 0; ac < NK * NK; ++ac) {
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < kNqx; ++q) acc += kap[ac * kNqx + q] * dv[q];
    be[(long long)ac * ne + s] = acc * scale;
  }
}

}  // namespace

cudaError_t launch_potential_update(Problem& P, int b0, int b1, const int* mask) {
  const int nb = b1 - b0;
  if (nb <= 0) return cudaSuccess;
  const Shape& s = P.s;
  cudaEvent_t ev = prof_begin(P, PROF_OTHER, 4);
  minmax_kernel<<<nb, 256, 0, P.stream>>>(P.pot_v, P.pp, P.nx, b0, mask);
  fermi_kernel<<<dim3(s.nk, nb), 128, 0, P.stream>>>(P.pot_v, P.pp, P.kvec, P.flr, P.nx, s.nk, b0, mask);
  inflow_kernel<<<nb, 256, sizeof(double) * 2 * s.nxi, P.stream>>>(P.flr, P.cosm, P.pinv, P.kvec, P.pp, P.rhs, P.fb,
                                                                   s.nk, s.nxi, s.n_el, P.N, s.q_diff, s.mpc, b0,
                                                                   mask);
  const int ne = s.nxi + 1;
  dim3 g((unsigned)(((long long)s.n_el * ne + 127) / 128), nb);
  const double scale = s.delta_xi / 4 * s.mpc;
  switch (s.nK) {
    case 2: vw_kernel<2><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.pp, P.nx,
                                                  s.n_el, s.nxi, scale, b0, mask); break;
    case 3: vw_kernel<3><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.pp, P.nx,
                                                  s.n_el, s.nxi, scale, b0, mask); break;
    default: vw_kernel<4><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.pp, P.nx,
                                                   s.n_el, s.nxi, scale, b0, mask); break;
  }
  prof_end(P, PROF_OTHER, ev);
  return cudaGetLastError();
}

}  // namespace wg
