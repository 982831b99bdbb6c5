// FP64 operator kernels of the 1D Wigner transport solve (sm_103a).
//
// y = A x is applied matrix-free in three parts (the factorised form of
// get_SysM.m:1-16 = get_Diff.m:66-84 + get_Drift_accel_trial_permutedShell.m:64-333):
//   1. flux_kernel       upwind x-flux times diag(k): per k a block-bidiagonal
//                        stencil over elements (HBM-bound streaming kernel)
//   2. zgemm_kernel      X^ = Phi X over every DG node of the batch (one GEMM),
//      stencil_kernel    Y^_{e,a} = sum_b T(beta_{e,ab}) X^_{e,b} (xi-tridiagonal),
//      zgemm_kernel      y += i Phi^H Y^ (second GEMM, accumulating epilogue)
// plus the k-line preconditioner, the Vw(x,k) rebuild and the observables.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "kline.cuh"
#include "problem.h"

namespace wg {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// ---------------------------------------------------------------------------
// 1. Upwind flux: y_{e,.,j} = qd_b [ (k K1 + |k| K2) x_e + (k+|k|) K3 x_{e-1}
//                                   + (k-|k|) K5 x_{e+1} ]_j  + shift x_{e,.,j}
// Grid (batch * n_el, ceil(nk / 128)): one block row per element, one thread per
// k, k fastest so every load/store is coalesced; no integer division per thread.
// shift = 0 for the stationary operator, sigma for the shifted (Crank-Nicolson) one.
// ---------------------------------------------------------------------------
constexpr int kFluxThreads = 128;

template <int NK>
__global__ void __launch_bounds__(kFluxThreads) flux_kernel(const double2* __restrict__ x, double2* __restrict__ y,
                                                            const double* __restrict__ kvec,
                                                            const double* __restrict__ qd, FluxBlocks fb, int n_el,
                                                            int nk, double shift, const int* __restrict__ mask) {
  const int be = blockIdx.x;                  // b * n_el + e
  const int j = blockIdx.y * kFluxThreads + threadIdx.x;
  if (j >= nk) return;
  const int b = be / n_el;
  if (mask && !mask[b]) return;
  const int e = be - b * n_el;
  const double k = kvec[j];
  const double ak = fabs(k);
  const double s = qd[b];
  const double2* xe = x + (long long)be * NK * nk + j;
  double2 xv[NK];
#pragma unroll
  for (int c = 0; c < NK; ++c) xv[c] = xe[(long long)c * nk];
  double2 acc[NK];
  if (fb.single) {
    // k K1 + |k| K2 = k (K1 +- K2); the upwind neighbour enters through one node:
    // y = qd k [ Kpm x_e + K3c x_{e-1}[nK-1]  (k > 0)  or  K5c x_{e+1}[0]  (k < 0) ] + shift x
    const bool pos = k > 0;
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      double2 v = make_double2(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < NK; ++c) {
        const double m = pos ? fb.Kp[a * NK + c] : fb.Km[a * NK + c];
        v.x += m * xv[c].x;
        v.y += m * xv[c].y;
      }
      acc[a] = v;
    }
    if (k > 0 && e > 0) {
      const double2 xn = xe[-(long long)NK * nk + (long long)(NK - 1) * nk];
#pragma unroll
      for (int a = 0; a < NK; ++a) {
        acc[a].x += fb.K3c[a] * xn.x;
        acc[a].y += fb.K3c[a] * xn.y;
      }
    } else if (k < 0 && e < n_el - 1) {
      const double2 xn = xe[(long long)NK * nk];
#pragma unroll
      for (int a = 0; a < NK; ++a) {
        acc[a].x += fb.K5c[a] * xn.x;
        acc[a].y += fb.K5c[a] * xn.y;
      }
    }
    const double sk = s * k;
    double2* ye = y + (long long)be * NK * nk + j;
#pragma unroll
    for (int a = 0; a < NK; ++a)
      ye[(long long)a * nk] = make_double2(sk * acc[a].x + shift * xv[a].x, sk * acc[a].y + shift * xv[a].y);
    return;
  }
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    double2 v = make_double2(0.0, 0.0);
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      const double m = k * fb.K1[a * NK + c] + ak * fb.K2[a * NK + c];
      v.x += m * xv[c].x;
      v.y += m * xv[c].y;
    }
    acc[a] = v;
  }
  if (k > 0 && e > 0) {
    const double2* xl = xe - (long long)NK * nk;
    double2 xp[NK];
#pragma unroll
    for (int c = 0; c < NK; ++c) xp[c] = xl[(long long)c * nk];
#pragma unroll
    for (int a = 0; a < NK; ++a)
#pragma unroll
      for (int c = 0; c < NK; ++c) {
        const double m = (k + ak) * fb.K3[a * NK + c];
        acc[a].x += m * xp[c].x;
        acc[a].y += m * xp[c].y;
      }
  } else if (k < 0 && e < n_el - 1) {
    const double2* xr = xe + (long long)NK * nk;
    double2 xp[NK];
#pragma unroll
    for (int c = 0; c < NK; ++c) xp[c] = xr[(long long)c * nk];
#pragma unroll
    for (int a = 0; a < NK; ++a)
#pragma unroll
      for (int c = 0; c < NK; ++c) {
        const double m = (k - ak) * fb.K5[a * NK + c];
        acc[a].x += m * xp[c].x;
        acc[a].y += m * xp[c].y;
      }
  }
  double2* ye = y + (long long)be * NK * nk + j;
#pragma unroll
  for (int a = 0; a < NK; ++a)
    ye[(long long)a * nk] = make_double2(s * acc[a].x + shift * xv[a].x, s * acc[a].y + shift * xv[a].y);
}

// ---------------------------------------------------------------------------
// 2a. Complex FP64 GEMM  C(M x Ncol) = op(A)(M x K) * B(K x Ncol), column-major
// B and C with leading dimensions ldb = K, ldc = M.
//   MODE 0: A(m,k) = phi[m*lda + k]        C  = acc        (X^ = Phi X)
//   MODE 1: A(m,k) = conj(phi[k*lda + m])  C += i * acc    (y += i Phi^H Y^)
// 64x64 output tile, 256 threads, 4x4 complex outputs per thread, BK = 8.
// ---------------------------------------------------------------------------
constexpr int GBM = 64, GBN = 64, GBK = 8;

template <int MODE>
__global__ void __launch_bounds__(256) zgemm_kernel(const double2* __restrict__ A, int lda,
                                                   const double2* __restrict__ Bm, double2* __restrict__ C, int M,
                                                   int K, long long Ncol) {
  __shared__ double2 As[2][GBK][GBM];
  __shared__ double2 Bs[2][GBK][GBN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * GBM;
  const long long n0 = (long long)blockIdx.x * GBN;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) acc[i][jj] = make_double2(0.0, 0.0);

  auto load = [&](int buf, int k0) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (MODE == 0) { mm = idx >> 3; kk = idx & 7; } else { kk = idx >> 6; mm = idx & 63; }
      const int gm = m0 + mm, gk = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (gm < M && gk < K) {
        if (MODE == 0) {
          v = A[(long long)gm * lda + gk];
        } else {
          v = A[(long long)gk * lda + gm];
          v.y = -v.y;
        }
      }
      As[buf][kk][mm] = v;
      const int nn = idx >> 3, kb = idx & 7;
      const long long gn = n0 + nn;
      double2 bv = make_double2(0.0, 0.0);
      if (gn < Ncol && k0 + kb < K) bv = Bm[gn * K + k0 + kb];
      Bs[buf][kb][nn] = bv;
    }
  };

  const int nkt = (K + GBK - 1) / GBK;
  load(0, 0);
  __syncthreads();
  for (int kt = 0; kt < nkt; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < nkt) load(cur ^ 1, (kt + 1) * GBK);
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[cur][kk][tx + 16 * i];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) b[jj] = Bs[cur][kk][ty + 16 * jj];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          acc[i][jj].x = fma(a[i].x, b[jj].x, fma(-a[i].y, b[jj].y, acc[i][jj].x));
          acc[i][jj].y = fma(a[i].x, b[jj].y, fma(a[i].y, b[jj].x, acc[i][jj].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tx + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const long long gn = n0 + ty + 16 * jj;
      if (gn >= Ncol) continue;
      double2* c = C + gn * M + gm;
      if (MODE == 0) {
        *c = acc[i][jj];
      } else {
        double2 o = *c;
        o.x -= acc[i][jj].y;
        o.y += acc[i][jj].x;
        *c = o;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 2b. xi stencil: Y^_{e,a}(s) = sum_c beta_{ac}(s) (X^_c(s) + X^_c(s-1))
//                               + beta_{ac}(s+1) (X^_c(s) + X^_c(s+1))
// beta = betar[b][e][ac][s] + i * betai[ac][s] (potential + CAP parts).
// One thread per (element of the batch, s); s fastest.
// ---------------------------------------------------------------------------
template <int NK>
__global__ void __launch_bounds__(kFluxThreads) stencil_kernel(const double2* __restrict__ xh,
                                                               double2* __restrict__ yh,
                                                               const double* __restrict__ betar,
                                                               const double* __restrict__ betai, int nxi,
                                                               int n_el, const int* __restrict__ mask) {
  // grid (batch * n_el, ceil(nxi / 128)): one block row per element, one thread per xi cell
  const int be = blockIdx.x;
  const int s = blockIdx.y * kFluxThreads + threadIdx.x;
  if (s >= nxi || (mask && !mask[be / n_el])) return;
  const int ne = nxi + 1;
  const double2* X = xh + (long long)be * NK * nxi;
  double2 sm[NK], sp[NK];
#pragma unroll
  for (int c = 0; c < NK; ++c) {
    const double2 x0 = X[c * nxi + s];
    const double2 xm = s > 0 ? X[c * nxi + s - 1] : make_double2(0.0, 0.0);
    const double2 xp = s < nxi - 1 ? X[c * nxi + s + 1] : make_double2(0.0, 0.0);
    sm[c] = cadd(x0, xm);
    sp[c] = cadd(x0, xp);
  }
  const double* br = betar + (long long)be * NK * NK * ne;
  double2* Y = yh + (long long)be * NK * nxi;
  // beta = betar + i betai with both parts real: Y = R + i I, R = sum betar (.), I = sum betai (.),
  // 8 FP64 FMAs per (a, c) instead of two complex products; the CAP part betai vanishes outside
  // the absorbing layers of the xi interval, where its FMAs are skipped (FP64-bound kernel)
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    double2 vr = make_double2(0.0, 0.0), vi = make_double2(0.0, 0.0);
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      const int ac = a * NK + c;
      const double r0 = br[ac * ne + s], r1 = br[ac * ne + s + 1];
      vr.x = fma(r0, sm[c].x, fma(r1, sp[c].x, vr.x));
      vr.y = fma(r0, sm[c].y, fma(r1, sp[c].y, vr.y));
      const double i0 = betai[ac * ne + s], i1 = betai[ac * ne + s + 1];
      // i0 != 0 || i1 != 0 tested on the bit patterns: an FP64 compare would take the FP64 pipe
      if ((((unsigned long long)__double_as_longlong(i0) | (unsigned long long)__double_as_longlong(i1)) << 1) != 0) {
        vi.x = fma(i0, sm[c].x, fma(i1, sp[c].x, vi.x));
        vi.y = fma(i0, sm[c].y, fma(i1, sp[c].y, vi.y));
      }
    }
    Y[a * nxi + s] = make_double2(vr.x - vi.y, vr.y + vi.x);
  }
}

// ---------------------------------------------------------------------------
// Observables: rho_u(s) = sum_j Phi(s,j) rho_{x,j} at the centre xi rows,
// n = Re rho_u(centre), j = q hbar / m Im d rho_u / d xi
// (solve_transport_DG_2D.m:114-156).  One warp per DG node.
// ---------------------------------------------------------------------------
__global__ void observables_kernel(const double2* __restrict__ rho, const double2* __restrict__ phi,
                                   const double* __restrict__ m_nodes, double* __restrict__ n_out,
                                   double* __restrict__ j_out, int nk, int nxi, int ncol, double delta_xi,
                                   double pref) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncol) return;
  const bool odd = nxi & 1;
  const int c1 = odd ? (nxi - 1) / 2 - 1 : nxi / 2 - 1;
  const int c2 = odd ? (nxi - 1) / 2 + 1 : nxi / 2;
  const int cm = (nxi - 1) / 2;
  double2 u1 = make_double2(0, 0), u2 = make_double2(0, 0), um = make_double2(0, 0);
  const double2* rx = rho + (long long)warp * nk;
  for (int j = lane; j < nk; j += 32) {
    const double2 rv = rx[j];
    u1 = cadd(u1, cmul(phi[(long long)c1 * nk + j], rv));
    u2 = cadd(u2, cmul(phi[(long long)c2 * nk + j], rv));
    if (odd) um = cadd(um, cmul(phi[(long long)cm * nk + j], rv));
  }
  for (int o = 16; o > 0; o >>= 1) {
    u1.x += __shfl_xor_sync(0xffffffffu, u1.x, o);
    u1.y += __shfl_xor_sync(0xffffffffu, u1.y, o);
    u2.x += __shfl_xor_sync(0xffffffffu, u2.x, o);
    u2.y += __shfl_xor_sync(0xffffffffu, u2.y, o);
    um.x += __shfl_xor_sync(0xffffffffu, um.x, o);
    um.y += __shfl_xor_sync(0xffffffffu, um.y, o);
  }
  if (lane == 0) {
    const double m = m_nodes[warp];
    if (odd) {
      n_out[warp] = um.x;
      j_out[warp] = pref / m * (u2.y - u1.y) / 2 / delta_xi;
    } else {
      n_out[warp] = (u1.x + u2.x) / 2;
      j_out[warp] = pref / m * (u2.y - u1.y) / delta_xi;
    }
  }
}

template <int NK>
void flux_launch(const double2* x, double2* y, const double* kvec, const double* qd, const FluxBlocks& fb, int batch,
                 int n_el, int nk, double shift, cudaStream_t st, const int* mask = nullptr) {
  const dim3 grid((unsigned)(batch * n_el), (unsigned)((nk + kFluxThreads - 1) / kFluxThreads));
  flux_kernel<NK><<<grid, kFluxThreads, 0, st>>>(x, y, kvec, qd, fb, n_el, nk, shift, mask);
}

template <int NK>
void stencil_launch(const double2* xh, double2* yh, const double* beta, const double* betai, int batch, int n_el,
                    int nxi, cudaStream_t st, const int* mask = nullptr) {
  const dim3 grid((unsigned)(batch * n_el), (unsigned)((nxi + kFluxThreads - 1) / kFluxThreads));
  stencil_kernel<NK><<<grid, kFluxThreads, 0, st>>>(xh, yh, beta, betai, nxi, n_el, mask);
}

template <int NK>
cudaError_t apply_nk(Problem& P, const double2* x, double2* y) {
  const double BN = (double)P.N * P.batch, ncols = (double)P.ncols, nxi = P.s.nxi, nk = P.s.nk;
  const double gemm_flops = 8.0 * nxi * nk * ncols;
  cudaEvent_t ev = prof_begin(P, PROF_FLUX64, 1, 32.0 * BN, 8.0 * NK * BN);
  flux_launch<NK>(x, y, P.kvec, P.qd, P.fb, P.batch, P.s.n_el, P.s.nk, P.shift, P.stream);
  prof_end(P, PROF_FLUX64, ev);
  dim3 g1((unsigned)((P.ncols + GBN - 1) / GBN), (P.s.nxi + GBM - 1) / GBM);
  ev = prof_begin(P, PROF_GEMM_F64, 1, 16.0 * (BN + nxi * ncols), gemm_flops);
  zgemm_kernel<0><<<g1, 256, 0, P.stream>>>(P.phi, P.s.nk, x, P.xh, P.s.nxi, P.s.nk, P.ncols);
  prof_end(P, PROF_GEMM_F64, ev);
  ev = prof_begin(P, PROF_STENCIL64, 1, 32.0 * nxi * ncols + 8.0 * P.batch * P.s.n_el * NK * NK * (nxi + 1),
                  16.0 * NK * nxi * ncols);
  stencil_launch<NK>(P.xh, P.yh, P.beta, P.betai, P.batch, P.s.n_el, P.s.nxi, P.stream);
  prof_end(P, PROF_STENCIL64, ev);
  dim3 g2((unsigned)((P.ncols + GBN - 1) / GBN), (P.s.nk + GBM - 1) / GBM);
  ev = prof_begin(P, PROF_GEMM_F64, 1, 16.0 * (2 * BN + nxi * ncols), gemm_flops);
  zgemm_kernel<1><<<g2, 256, 0, P.stream>>>(P.phi, P.s.nk, P.yh, y, P.s.nk, P.s.nxi, P.ncols);
  prof_end(P, PROF_GEMM_F64, ev);
  return cudaGetLastError();
}

template <int NK>
cudaError_t precond_nk(Problem& P, const double2* r, long long r_stride, double2* z, const double* rscale,
                       double2* rout, long long rout_stride) {
  const int L = P.kline_L, nc = kline::chunk_count_for(P.s.n_el, L);
  const dim3 grid((P.s.nk + 31) / 32, (nc + kline::kChunksPerBlock - 1) / kline::kChunksPerBlock, P.batch);
  const dim3 block(32, kline::kChunksPerBlock);
  double* ma = static_cast<double*>(P.kmap_a);
  double2* ms = static_cast<double2*>(P.kmap_s);
  cudaEvent_t ev = prof_begin(P, PROF_PRECOND, 2, (48.0 + (rout ? 16.0 : 0.0)) * P.N * P.batch);
  kline::kline_maps_kernel<NK, double><<<grid, block, 0, P.stream>>>(r, P.kvec, P.pre_dinv, P.pre_h, P.qd, ma, ms,
                                                                     P.s.n_el, P.s.nk, P.N, r_stride, L, nc,
                                                                     nullptr, rscale);
  kline::kline_apply_kernel<NK, double><<<grid, block, 0, P.stream>>>(r, z, nullptr, P.kvec, P.pre_dinv, P.pre_h,
                                                                      P.qd, ma, ms, P.s.n_el, P.s.nk, P.N,
                                                                      r_stride, L, nc, nullptr, rscale, rout,
                                                                      rout_stride);
  prof_end(P, PROF_PRECOND, ev);
  return cudaGetLastError();
}

}  // namespace

// Fraction of the batch a masked launch processes (out[0]) and, for an emulated FP64
// GEMM with nd > 0 digits (per problem nd_pp[b] when given), its digit-slice products
// per problem relative to one product (out[1]); out[1] = out[0] without digits.
__global__ void prof_count_kernel(const int* __restrict__ mask, const int* __restrict__ nd_pp, int nd, int batch,
                                  double* __restrict__ out) {
  double act = 0, wt = 0;
  for (int b = threadIdx.x; b < batch; b += 32) {
    if (mask && !mask[b]) continue;
    act += 1.0;
    const int d = nd_pp ? nd_pp[b] : nd;
    wt += d > 0 ? 0.5 * d * (d + 1) : 1.0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    act += __shfl_xor_sync(0xffffffffu, act, o);
    wt += __shfl_xor_sync(0xffffffffu, wt, o);
  }
  if (threadIdx.x == 0) {
    out[0] = act / batch;
    out[1] = wt / batch;
  }
}

cudaEvent_t prof_begin(Problem& P, int cls, int n, double bytes, double flops, const int* mask, int nd,
                       const int* nd_pp) {
  P.prof.launches[cls] += n;
  if (!P.prof.on) return nullptr;
  int slot = -1;
  if (mask || nd > 0 || nd_pp) {
    if (!P.prof.d_frac && cudaMalloc(&P.prof.d_frac, sizeof(double) * 2 * Profiler::kProfSlots) != cudaSuccess)
      P.prof.d_frac = nullptr;
    if (P.prof.d_frac && (int)P.prof.pending.size() < Profiler::kProfSlots) {
      slot = (int)P.prof.pending.size();
      prof_count_kernel<<<1, 32, 0, P.stream>>>(mask, nd_pp, nd, P.batch, P.prof.d_frac + 2 * slot);
    }
  }
  P.prof.pend_bytes.push_back(bytes);
  P.prof.pend_flops.push_back(flops);
  P.prof.pend_slot.push_back(slot);
  cudaEvent_t a;
  if (P.prof.pool.empty()) {
    if (cudaEventCreate(&a) != cudaSuccess) {
      P.prof.pend_bytes.pop_back();
      P.prof.pend_flops.pop_back();
      P.prof.pend_slot.pop_back();
      return nullptr;
    }
  } else {
    a = P.prof.pool.back();
    P.prof.pool.pop_back();
  }
  cudaEventRecord(a, P.stream);
  return a;
}

void prof_end(Problem& P, int cls, cudaEvent_t a) {
  if (!a) return;
  cudaEvent_t b;
  if (P.prof.pool.empty()) {
    if (cudaEventCreate(&b) != cudaSuccess) {
      P.prof.pool.push_back(a);
      P.prof.pend_bytes.pop_back();
      P.prof.pend_flops.pop_back();
      P.prof.pend_slot.pop_back();
      return;
    }
  } else {
    b = P.prof.pool.back();
    P.prof.pool.pop_back();
  }
  cudaEventRecord(b, P.stream);
  P.prof.pending.push_back({cls, a, b});
  if (P.prof.pending.size() >= 8192) prof_collect(P);
}

cudaError_t prof_collect(Problem& P) {
  if (P.prof.pending.empty()) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(P.stream);
  std::vector<double> frac;
  bool any = false;
  for (int s : P.prof.pend_slot) any = any || s >= 0;
  if (any && e == cudaSuccess) {
    frac.resize(2 * P.prof.pending.size());
    e = cudaMemcpy(frac.data(), P.prof.d_frac, sizeof(double) * frac.size(), cudaMemcpyDeviceToHost);
  }
  for (size_t i = 0; i < P.prof.pending.size(); ++i) {
    const auto& r = P.prof.pending[i];
    float ms = 0;
    if (e == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      const int slot = P.prof.pend_slot[i];
      const double fb = slot >= 0 ? frac[2 * slot] : 1.0, ff = slot >= 0 ? frac[2 * slot + 1] : 1.0;
      P.prof.ms[r.cls] += ms;
      P.prof.timed[r.cls] += 1;
      P.prof.bytes[r.cls] += fb * P.prof.pend_bytes[i];
      P.prof.flops[r.cls] += ff * P.prof.pend_flops[i];
    }
    P.prof.pool.push_back(r.a);
    P.prof.pool.push_back(r.b);
  }
  P.prof.pending.clear();
  P.prof.pend_bytes.clear();
  P.prof.pend_flops.clear();
  P.prof.pend_slot.clear();
  return e;
}

void prof_release(Problem& P) {
  prof_collect(P);
  for (cudaEvent_t e : P.prof.pool) cudaEventDestroy(e);
  P.prof.pool.clear();
  if (P.prof.d_frac) cudaFree(P.prof.d_frac);
  P.prof.d_frac = nullptr;
}

cudaError_t launch_apply(Problem& P, const double2* x, double2* y) {
  if (P.fp64_tc && P.mx.ozaki) return launch_apply_f64_tc(P, x, y);
  switch (P.s.nK) {
    case 2: return apply_nk<2>(P, x, y);
    case 3: return apply_nk<3>(P, x, y);
    default: return apply_nk<4>(P, x, y);
  }
}

cudaError_t launch_flux_f64(Problem& P, const double2* x, double2* y, const int* mask) {
  cudaEvent_t ev = prof_begin(P, PROF_FLUX64, 1, 32.0 * P.N * P.batch, 8.0 * P.s.nK * P.N * P.batch, mask);
  switch (P.s.nK) {
    case 2: flux_launch<2>(x, y, P.kvec, P.qd, P.fb, P.batch, P.s.n_el, P.s.nk, P.shift, P.stream, mask); break;
    case 3: flux_launch<3>(x, y, P.kvec, P.qd, P.fb, P.batch, P.s.n_el, P.s.nk, P.shift, P.stream, mask); break;
    default: flux_launch<4>(x, y, P.kvec, P.qd, P.fb, P.batch, P.s.n_el, P.s.nk, P.shift, P.stream, mask); break;
  }
  prof_end(P, PROF_FLUX64, ev);
  return cudaGetLastError();
}

cudaError_t launch_stencil_f64(Problem& P, const double2* xh, double2* yh, const int* mask) {
  const int nK = P.s.nK;
  cudaEvent_t ev = prof_begin(P, PROF_STENCIL64, 1,
                              32.0 * P.s.nxi * P.ncols + 8.0 * P.batch * P.s.n_el * nK * nK * (P.s.nxi + 1),
                              16.0 * nK * P.s.nxi * P.ncols, mask);
  switch (nK) {
    case 2: stencil_launch<2>(xh, yh, P.beta, P.betai, P.batch, P.s.n_el, P.s.nxi, P.stream, mask); break;
    case 3: stencil_launch<3>(xh, yh, P.beta, P.betai, P.batch, P.s.n_el, P.s.nxi, P.stream, mask); break;
    default: stencil_launch<4>(xh, yh, P.beta, P.betai, P.batch, P.s.n_el, P.s.nxi, P.stream, mask); break;
  }
  prof_end(P, PROF_STENCIL64, ev);
  return cudaGetLastError();
}

cudaError_t launch_precondition(Problem& P, const double2* r, long long r_stride, double2* z, const double* rscale,
                                double2* rout, long long rout_stride) {
  switch (P.s.nK) {
    case 2: return precond_nk<2>(P, r, r_stride, z, rscale, rout, rout_stride);
    case 3: return precond_nk<3>(P, r, r_stride, z, rscale, rout, rout_stride);
    default: return precond_nk<4>(P, r, r_stride, z, rscale, rout, rout_stride);
  }
}

cudaError_t launch_rho_xi(Problem& P, int b, double2* out) {
  const long long ncol = (long long)P.s.n_el * P.s.nK;
  dim3 g1((unsigned)((ncol + GBN - 1) / GBN), (P.s.nxi + GBM - 1) / GBM);
  zgemm_kernel<0><<<g1, 256, 0, P.stream>>>(P.phi, P.s.nk, P.x + (long long)b * P.N, out, P.s.nxi, P.s.nk, ncol);
  return cudaGetLastError();
}

cudaError_t launch_observables(Problem& P, int b, double* n_dg, double* j) {
  const int ncol = P.s.n_el * P.s.nK;
  const double pref = kQ * (kHV / 2 / M_PI);
  const double2* rho = P.x + (long long)b * P.N;
  const unsigned grid = (unsigned)((ncol * 32 + 255) / 256);
  observables_kernel<<<grid, 256, 0, P.stream>>>(rho, P.phi, P.m_nodes + (long long)b * ncol, n_dg, j, P.s.nk,
                                                 P.s.nxi, ncol, P.s.delta_xi, pref);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free operator apply.
//
// For callers that must not allocate device memory while they call in: a host
// application that owns every device allocation through its own pool (a MATLAB
// MEX gateway working on gpuArray storage, a framework's caching allocator with
// a hard budget, an embedding that has reserved the whole device up front).
// The caller passes its own device buffers for the operator data, x and y; the
// only scratch, the transformed state X^ and the stencil output Y^, lives in the
// file-scope array below.  Its size is fixed (kNoAllocScratch complex doubles,
// 16 MiB) and every GPU that loads the library keeps it until the process exits.
// All calls share it: two calls whose kernels overlap on the GPU (different
// streams, or devices shared by threads without ordering) race on it and must be
// serialised by the caller.  Both halves are fully written before they are read
// in every call, so nothing is cleared.
// ---------------------------------------------------------------------------
constexpr long long kNoAllocScratch = 1ll << 20;      // complex doubles: two halves for X^ and Y^
static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocScratch];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double2* g_noalloc_ptr[kMaxDevices] = {};
unsigned long long g_noalloc_ctx[kMaxDevices] = {};   // context the cached address belongs to

// Identifier of the current CUDA context (driver entry points loaded once; 0 when
// no context is current or the driver does not offer them).  A device reset
// (cudaDeviceReset, MATLAB's reset(gpuDevice)) destroys the primary context, and
// the context made afterwards has a new identifier.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(p);
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  return get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of the scratch array for the current device.  The first call on
// a device (and the first after a device reset replaced its context) looks it up
// with cudaGetSymbolAddress, which does not allocate; make that first call before
// any stream capture.
cudaError_t noalloc_scratch(double2** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<double2*>(p);
    g_noalloc_ctx[dev] = current_context_id();   // the lookup made the primary context current
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

template <int NK>
cudaError_t apply_noalloc_nk(const wg_operator_view& v, const FluxBlocks& fb, const double2* x, double2* y,
                             double2* xh, double2* yh, cudaStream_t st) {
  const long long ncols = (long long)v.batch * v.n_el * NK;
  flux_launch<NK>(x, y, v.kvec, v.qd, fb, v.batch, v.n_el, v.nk, 0.0, st);
  const double2* phi = reinterpret_cast<const double2*>(v.phi);
  dim3 g1((unsigned)((ncols + GBN - 1) / GBN), (v.n_xi + GBM - 1) / GBM);
  zgemm_kernel<0><<<g1, 256, 0, st>>>(phi, v.nk, x, xh, v.n_xi, v.nk, ncols);
  stencil_launch<NK>(xh, yh, v.beta, v.betai, v.batch, v.n_el, v.n_xi, st);
  dim3 g2((unsigned)((ncols + GBN - 1) / GBN), (v.nk + GBM - 1) / GBM);
  zgemm_kernel<1><<<g2, 256, 0, st>>>(phi, v.nk, yh, y, v.nk, v.n_xi, ncols);
  return cudaGetLastError();
}

}  // namespace

int apply_noalloc(const wg_operator_view& v, const double* x, double* y, void* stream, std::string& err) {
  if (v.n_local < 2 || v.n_local > kMaxLocal || v.n_el < 1 || v.nk < 1 || v.n_xi < 1 || v.batch < 1) {
    err = "wg_apply_noalloc: sizes must be positive and n_local in 2..4";
    return WG_ERR_ARG;
  }
  if (!v.phi || !v.kvec || !v.qd || !v.beta || !v.betai || !x || !y) {
    err = "wg_apply_noalloc: null device pointer";
    return WG_ERR_ARG;
  }
  const long long need = (long long)v.n_xi * v.batch * v.n_el * v.n_local;
  if (need > kNoAllocScratch / 2) {
    err = "wg_apply_noalloc: n_xi*batch*n_el*n_local = " + std::to_string(need) + " exceeds the fixed scratch of " +
          std::to_string(kNoAllocScratch / 2) + " complex values per transform (use wg_apply on a handle)";
    return WG_ERR_ARG;
  }
  double2* scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) {
    err = std::string("wg_apply_noalloc: scratch address: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  FluxBlocks fb{};
  fb.nK = v.n_local;
  for (int i = 0; i < v.n_local * v.n_local; ++i) {
    fb.K1[i] = v.K1[i];
    fb.K2[i] = v.K2[i];
    fb.K3[i] = v.K3[i];
    fb.K5[i] = v.K5[i];
  }
  finish_flux_blocks(fb);
  const double2* xx = reinterpret_cast<const double2*>(x);
  double2* yy = reinterpret_cast<double2*>(y);
  double2* xh = scratch;
  double2* yh = scratch + kNoAllocScratch / 2;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (v.n_local) {
    case 2: e = apply_noalloc_nk<2>(v, fb, xx, yy, xh, yh, st); break;
    case 3: e = apply_noalloc_nk<3>(v, fb, xx, yy, xh, yh, st); break;
    default: e = apply_noalloc_nk<4>(v, fb, xx, yy, xh, yh, st); break;
  }
  if (e != cudaSuccess) {
    err = std::string("wg_apply_noalloc: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  return WG_OK;
}

}  // namespace wg
