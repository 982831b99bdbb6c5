// Device-side rebuild of everything that depends on the potential (sm_103a).
//
// For problems [b0, b1) of a handle, from the potential V(x) on the material grid:
//   minmax_kernel   min V (V(x >= Lx) of V_transient.m:6) and max V (kz range of
//                   verteilung.m:140)
//   fermi_kernel    f_L(k), f_R(k): Fermi-Dirac occupation integrated over 1001 kz
//                   (verteilung.m:139-152), 16 k per block, kz factors shared
//   inflow_xi_kernel cosine transform to the xi cells (verteilung.m:158-161)
//   inflow_kernel   least-squares projection on Phi (pseudo-inverse,
//                   verteilung.m:167-168) and the contact inflow blocks of the rhs
//                   (get_Diff.m:77-83)
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

// min V, max V and the slopes (V[i+1] - V[i]) / (x[i+1] - x[i]) of the linear interpolation.
__global__ void minmax_kernel(const double* __restrict__ pot_v, const double* __restrict__ pot_x,
                              double* __restrict__ vslope, double* __restrict__ pp, int nx, int b0,
                              const int* __restrict__ mask) {
  const int b = b0 + blockIdx.x;
  if (mask && !mask[b]) return;
  const double* v = pot_v + (long long)b * nx;
  const double* x = pot_x + (long long)b * nx;
  double mx = -INFINITY, mn = INFINITY;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    mx = fmax(mx, v[i]);
    mn = fmin(mn, v[i]);
    if (i < nx - 1) vslope[(long long)b * nx + i] = (v[i + 1] - v[i]) / (x[i + 1] - x[i]);
  }
  mx = block_reduce(mx, true);
  const double mneg = block_reduce(-mn, true);
  if (threadIdx.x == 0) {
    pp[b * kPP + PP_VMAX] = mx;
    pp[b * kPP + PP_VMIN] = -mneg;
  }
}

// f_{L,R}(k_j) = 2/pi dkz sum_z 1/(1 + exp(q (E_{L,R}(k) + E_kz - E_F) / (kB T)))
// 1 / d for d >= 1 by Newton-Raphson from the FP32 reciprocal: two steps take the
// ~23 correct bits to full double precision (within an ulp or two) without the
// FP64 divide sequence.
__device__ __forceinline__ double recip_ge1(double d) {
  if (!(d < 1e30)) return isinf(d) ? 0.0 : 1.0 / d;   // outside FP32 range (rare): plain division
  double r = (double)__frcp_rn((float)d);
  r = r * fma(-d, r, 2.0);
  r = r * fma(-d, r, 2.0);
  return r;
}

// f_L(k_j), f_R(k_j) for kFermiJ consecutive j of problem b.  The Fermi factor of
// (j, kz) is 1 / (1 + a_j g(kz)) with a_j = exp((E_j - E_F) / kT) and
// g(kz) = exp(hbar^2 kz^2 / (2 m_z kT)): the kz factors are computed once per block
// in shared memory, the j factors once per j, instead of one exponential per (j, kz).
// Four j per block, one warp each: a small batch still spreads over the SMs (16 j per block left
// 32 blocks for a 2-problem handle at Nk = 256).
constexpr int kFermiJ = 4;
__global__ void __launch_bounds__(32 * kFermiJ) fermi_kernel(const double* __restrict__ pot_v, const double* __restrict__ pp,
                                                    const double* __restrict__ kvec, double* __restrict__ flr,
                                                    int nx, int nk, int b0, const int* __restrict__ mask) {
  __shared__ double g[kNkz];
  const int b = b0 + blockIdx.y;
  if (mask && !mask[b]) return;
  const double* P = pp + b * kPP;
  const double hb = kHV / 2 / kPi;
  const double me_z = P[PP_MEZ], temp = P[PP_TEMP];
  const double kz_max = sqrt(2 * 2 * kM0V * me_z * kQV * (P[PP_VMAX] + 0.3)) / hb;
  const double dkz = kz_max / (kNkz - 1);
  const double inv_kt = kQV / (kKBV * temp);
  const double cz = hb * hb / 2 / kM0V / me_z / kQV;
  for (int z = threadIdx.x; z < kNkz; z += blockDim.x) {
    const double kz = (z == kNkz - 1) ? kz_max : z * dkz;
    g[z] = exp(cz * kz * kz * inv_kt);
  }
  __syncthreads();
  const double v0 = pot_v[(long long)b * nx], v1 = pot_v[(long long)b * nx + nx - 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int jj = warp; jj < kFermiJ; jj += nw) {
    const int j = blockIdx.x * kFermiJ + jj;
    if (j >= nk) break;
    const double k = kvec[j];
    const double EL = v0 + hb * hb * k * k / 2 / P[PP_M0] / kQV;
    const double ER = v1 + hb * hb * k * k / 2 / P[PP_M1] / kQV;
    const double aL = exp((EL - P[PP_EFL]) * inv_kt), aR = exp((ER - P[PP_EFR]) * inv_kt);
    double sl = 0, sr = 0;
    for (int z = lane; z < kNkz; z += 32) {
      sl += recip_ge1(1.0 + aL * g[z]);
      sr += recip_ge1(1.0 + aR * g[z]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sl += __shfl_xor_sync(0xffffffffu, sl, o);
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
    }
    if (lane == 0) {
      flr[((long long)b * 2 + 0) * nk + j] = 2 / kPi * dkz * sl;
      flr[((long long)b * 2 + 1) * nk + j] = 2 / kPi * dkz * sr;
    }
  }
}

// fLn(s) = sum_j cos(xi_s k_j) f(k_j) dk/(2 pi); fnl = Phi^+ fLn; rhs blocks.
// Cosine transform of f_L, f_R to the xi cells (verteilung.m:158-161): one warp per
// (xi cell, problem), lanes over k.  fxi[b][2][nxi].
__global__ void __launch_bounds__(256) inflow_xi_kernel(const double* __restrict__ flr, const double* __restrict__ cosm,
                                                        const double* __restrict__ kvec, double* __restrict__ fxi,
                                                        int nk, int nxi, int b0, const int* __restrict__ mask) {
  const int b = b0 + blockIdx.y;
  if (mask && !mask[b]) return;
  const int s = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (s >= nxi) return;
  const double* fL = flr + (long long)b * 2 * nk;
  const double* fR = fL + nk;
  const double* c = cosm + (long long)s * nk;
  double al = 0, ar = 0;
  for (int j = lane; j < nk; j += 32) {
    al += c[j] * fL[j];
    ar += c[j] * fR[j];
  }
  for (int o = 16; o > 0; o >>= 1) {
    al += __shfl_xor_sync(0xffffffffu, al, o);
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
  }
  if (lane == 0) {
    const double dk = fabs(kvec[1] - kvec[0]);
    fxi[((long long)b * 2 + 0) * nxi + s] = al * dk / 2 / kPi;
    fxi[((long long)b * 2 + 1) * nxi + s] = ar * dk / 2 / kPi;
  }
}

// Least-squares projection on Phi (pseudo-inverse, verteilung.m:167-168) and the contact
// inflow blocks of the rhs (get_Diff.m:77-83): one warp per (k, problem), lanes over xi.
__global__ void __launch_bounds__(256) inflow_kernel(const double* __restrict__ fxi, const double2* __restrict__ pinv,
                                                     const double* __restrict__ kvec, const double* __restrict__ pp,
                                                     double2* __restrict__ rhs, FluxBlocks fb, int nk, int nxi,
                                                     int n_el, long long N, double q_diff, double mpc, int b0,
                                                     const int* __restrict__ mask) {
  const int b = b0 + blockIdx.y;
  if (mask && !mask[b]) return;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= nk) return;
  const double* sL = fxi + (long long)b * 2 * nxi;
  const double* sR = sL + nxi;
  const double2* pr = pinv + (long long)j * nxi;
  double2 zl = make_double2(0, 0), zr = make_double2(0, 0);
  for (int s = lane; s < nxi; s += 32) {
    const double2 w = pr[s];
    zl.x += w.x * sL[s];
    zl.y += w.y * sL[s];
    zr.x += w.x * sR[s];
    zr.y += w.y * sR[s];
  }
  for (int o = 16; o > 0; o >>= 1) {
    zl.x += __shfl_xor_sync(0xffffffffu, zl.x, o);
    zl.y += __shfl_xor_sync(0xffffffffu, zl.y, o);
    zr.x += __shfl_xor_sync(0xffffffffu, zr.x, o);
    zr.y += __shfl_xor_sync(0xffffffffu, zr.y, o);
  }
  const int nK = fb.nK;
  if (lane < nK) {
    const int a = lane;
    const double detJ = pp[b * kPP + PP_LX] / n_el / 2;
    double2* rfirst = rhs + (long long)b * N;
    double2* rlast = rfirst + (long long)(n_el - 1) * nK * nk;
    const double k = kvec[j], ak = fabs(k);
    const double fl = k > 0 ? 1.0 : 0.0, fr = k < 0 ? 1.0 : 0.0;
    const double q1 = fb.invM[a * nK + 0] / detJ, q2 = fb.invM[a * nK + nK - 1] / detJ;
    rfirst[(long long)a * nk + j] =
        make_double2(mpc * (q_diff * (q1 * (fl * (ak * zl.x)))), mpc * (q_diff * (q1 * (fl * (ak * zl.y)))));
    rlast[(long long)a * nk + j] =
        make_double2(mpc * (q_diff * (q2 * (fr * (ak * zr.x)))), mpc * (q_diff * (q2 * (fr * (ak * zr.y)))));
  }
}

// V(x) by linear interpolation on the material grid, V(x < 0) = V(0), V(x >= Lx) = min V
// (V_transient.m:1-8).  The interval is guessed from a uniform grid (inv_span =
// (nx-1) / (x[nx-1] - x[0])) and corrected by comparisons; slopes are precomputed.
__device__ double v_lookup(double x, const double* __restrict__ xg, const double* __restrict__ vg,
                           const double* __restrict__ slope, int nx, double lx, double vmin, double inv_span) {
  if (x < 0) return vg[0];
  if (x >= lx) return vmin;
  int hi = nx - 1;
  if (x >= xg[hi]) return vg[hi];
  int lo = (int)((x - xg[0]) * inv_span);
  lo = max(0, min(nx - 2, lo));
  int steps = 0;
  while (steps < 4 && lo > 0 && xg[lo] > x) { --lo; ++steps; }
  while (steps < 4 && lo < nx - 2 && xg[lo + 1] <= x) { ++lo; ++steps; }
  if (xg[lo] > x || xg[lo + 1] <= x) {
    lo = 0;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (xg[mid] <= x) lo = mid; else hi = mid;
    }
  }
  return slope[lo] * (x - xg[lo]) + vg[lo];
}

// beta[b][e][ac][s] = (dxi/4) mpc sum_q kap[ac][q] (V(x_q + xi_s/2) - V(x_q - xi_s/2)).
// The xi edges are symmetric about 0 (xi_{ne-1-s} = -xi_s up to the rounding of their grid), so
// the difference is odd in xi: one thread computes the edges s and ne-1-s (FP64-bound kernel).
template <int NK>
__global__ void vw_kernel(double* __restrict__ beta, const double* __restrict__ xq, const double* __restrict__ xi_edge,
                          const double* __restrict__ kap, const double* __restrict__ pot_x,
                          const double* __restrict__ pot_v, const double* __restrict__ vslope,
                          const double* __restrict__ pp, int nx, int n_el, int nxi, double scale, int b0,
                          const int* __restrict__ mask) {
  if (mask && !mask[b0 + blockIdx.y]) return;
  const int ne = nxi + 1, nh = (ne + 1) / 2;
  const int b = b0 + blockIdx.y;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_el * nh) return;
  const int s = (int)(t % nh);
  const int e = (int)(t / nh);
  const int sm = ne - 1 - s;   // the mirrored edge (== s at the centre of an odd edge count)
  const double xi = xi_edge[s];
  const double* xg = pot_x + (long long)b * nx;
  const double* vg = pot_v + (long long)b * nx;
  const double lx = pp[b * kPP + PP_LX], vmin = pp[b * kPP + PP_VMIN];
  const double* sl = vslope + (long long)b * nx;
  const double inv_span = (nx - 1) / (xg[nx - 1] - xg[0]);
  const double* xqb = xq + (long long)b * n_el * kNqx + e * kNqx;
  double dv[kNqx];
#pragma unroll
  for (int q = 0; q < kNqx; ++q) {
    const double x = xqb[q];
    dv[q] = v_lookup(x + 0.5 * xi, xg, vg, sl, nx, lx, vmin, inv_span) -
            v_lookup(x - 0.5 * xi, xg, vg, sl, nx, lx, vmin, inv_span);
  }
  double* be = beta + ((long long)b * n_el + e) * NK * NK * ne;
  // the weights are symmetric in (a, c) (symmetric inverse mass, products W(q,a) W(q,c)):
  // one contraction per unordered pair
#pragma unroll
  for (int a = 0; a < NK; ++a)
#pragma unroll
    for (int c = a; c < NK; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < kNqx; ++q) acc += kap[(a * NK + c) * kNqx + q] * dv[q];
      acc *= scale;
      be[(long long)(a * NK + c) * ne + s] = acc;
      if (c != a) be[(long long)(c * NK + a) * ne + s] = acc;
      if (sm != s) {
        be[(long long)(a * NK + c) * ne + sm] = -acc;
        if (c != a) be[(long long)(c * NK + a) * ne + sm] = -acc;
      }
    }
}

}  // namespace

cudaError_t launch_potential_update(Problem& P, int b0, int b1, const int* mask) {
  const int nb = b1 - b0;
  if (nb <= 0) return cudaSuccess;
  const Shape& s = P.s;
  cudaEvent_t ev = prof_begin(P, PROF_OTHER, 5);
  minmax_kernel<<<nb, 256, 0, P.stream>>>(P.pot_v, P.pot_x, P.vslope, P.pp, P.nx, b0, mask);
  fermi_kernel<<<dim3((s.nk + kFermiJ - 1) / kFermiJ, nb), 32 * kFermiJ, 0, P.stream>>>(P.pot_v, P.pp, P.kvec, P.flr,
                                                                                       P.nx, s.nk, b0, mask);
  inflow_xi_kernel<<<dim3((s.nxi + 7) / 8, nb), 256, 0, P.stream>>>(P.flr, P.cosm, P.kvec, P.fxi, s.nk, s.nxi, b0,
                                                                     mask);
  inflow_kernel<<<dim3((s.nk + 7) / 8, nb), 256, 0, P.stream>>>(P.fxi, P.pinv, P.kvec, P.pp, P.rhs, P.fb, s.nk,
                                                                  s.nxi, s.n_el, P.N, s.q_diff, s.mpc, b0, mask);
  const int ne = s.nxi + 1;
  dim3 g((unsigned)(((long long)s.n_el * ((ne + 1) / 2) + 127) / 128), nb);
  const double scale = s.delta_xi / 4 * s.mpc;
  switch (s.nK) {
    case 2: vw_kernel<2><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.vslope, P.pp,
                                                  P.nx, s.n_el, s.nxi, scale, b0, mask); break;
    case 3: vw_kernel<3><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.vslope, P.pp,
                                                  P.nx, s.n_el, s.nxi, scale, b0, mask); break;
    default: vw_kernel<4><<<g, 128, 0, P.stream>>>(P.beta, P.xq, P.xi_edge, P.kap, P.pot_x, P.pot_v, P.vslope, P.pp,
                                                   P.nx, s.n_el, s.nxi, scale, b0, mask); break;
  }
  prof_end(P, PROF_OTHER, ev);
  return cudaGetLastError();
}

}  // namespace wg
