// Batched restarted GMRES(m) with right preconditioning, FP64 (sm_103a).
//
// Semantics of the reference's Krylov wrapper (DG_code/solve_transport_DG_full2D.m):
//  - right preconditioning: Krylov space of A M^-1, x = x0 + M^-1 V y (:462-484)
//  - warm start as a correction about rho0 with the absolute target tol*|b| (:474)
//  - an independent true-residual check that downgrades a converged flag (:314-320)
// Arnoldi uses classical Gram-Schmidt applied twice (CGS2), block reductions
// with warp shuffles; the Givens rotations and the Hessenberg back substitution
// run on the device, one thread per problem.  Every problem of the batch has
// its own basis, Hessenberg matrix and convergence state; a problem that meets
// its target freezes while the others continue.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "problem.h"

namespace wg {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of a double2 (blockDim.x == 256).
__device__ double2 block_sum2(double2 v) {
  __shared__ double sx[8], sy[8];
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sx[w] = v.x; sy[w] = v.y; }
  __syncthreads();
  double2 r = make_double2(0, 0);
  if (threadIdx.x < 32) {
    r.x = lane < 8 ? sx[lane] : 0.0;
    r.y = lane < 8 ? sy[lane] : 0.0;
    r.x = warp_sum(r.x);
    r.y = warp_sum(r.y);
  }
  __syncthreads();
  return r;
}

__device__ double block_sum1(double v) {
  __shared__ double s[8];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) s[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = lane < 8 ? s[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// partial[b][i][c] = sum over chunk c of conj(V_i) . w       grid (nchunk, nv, B)
__global__ void __launch_bounds__(256) dot_partial_kernel(const double2* __restrict__ V, const double2* __restrict__ w,
                                                          double2* __restrict__ partial, const int* __restrict__ active,
                                                          long long N, int mp1, int nchunk) {
  const int b = blockIdx.z, i = blockIdx.y, c = blockIdx.x;
  if (!active[b]) return;
  const double2* v = V + ((long long)b * mp1 + i) * N;
  const double2* ww = w + (long long)b * N;
  double2 acc = make_double2(0, 0);
  for (long long n = (long long)c * 256 + threadIdx.x; n < N; n += (long long)nchunk * 256) {
    const double2 t = cmulc(v[n], ww[n]);
    acc.x += t.x;
    acc.y += t.y;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) partial[((long long)b * mp1 + i) * nchunk + c] = acc;
}

// hcol[b][i] = sum_c partial; H[b][k][i] (+)= hcol           grid (B), block 32*8
__global__ void dot_reduce_kernel(const double2* __restrict__ partial, double2* __restrict__ hcol,
                                  double2* __restrict__ H, const int* __restrict__ active, int nv, int k, int mp1,
                                  int m, int nchunk, int first) {
  const int b = blockIdx.x;
  if (!active[b]) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = w; i < nv; i += nw) {
    double2 acc = make_double2(0, 0);
    for (int c = lane; c < nchunk; c += 32) {
      const double2 t = partial[((long long)b * mp1 + i) * nchunk + c];
      acc.x += t.x;
      acc.y += t.y;
    }
    acc.x = warp_sum(acc.x);
    acc.y = warp_sum(acc.y);
    if (lane == 0) {
      hcol[b * mp1 + i] = acc;
      double2* h = H + (long long)b * mp1 * m + (long long)k * mp1 + i;
      if (first) *h = acc;
      else { h->x += acc.x; h->y += acc.y; }
    }
  }
}

// w -= sum_i V_i hcol_i                                       grid over B*N
__global__ void __launch_bounds__(256) gs_update_kernel(const double2* __restrict__ V, double2* __restrict__ w,
                                                        const double2* __restrict__ hcol, const int* __restrict__ active,
                                                        long long N, int nv, int mp1, int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  if (!active[b]) return;
  const long long n = t - (long long)b * N;
  double2 acc = w[t];
  const double2* v = V + (long long)b * mp1 * N + n;
  for (int i = 0; i < nv; ++i) {
    const double2 h = hcol[b * mp1 + i];
    const double2 vi = v[(long long)i * N];
    acc.x -= vi.x * h.x - vi.y * h.y;
    acc.y -= vi.x * h.y + vi.y * h.x;
  }
  w[t] = acc;
}

// nrm_partial[b][c] = sum |v|^2 over chunk c                  grid (nchunk, B)
__global__ void __launch_bounds__(256) norm_partial_kernel(const double2* __restrict__ v, double* __restrict__ out,
                                                           long long N, int nchunk) {
  const int b = blockIdx.y, c = blockIdx.x;
  const double2* vv = v + (long long)b * N;
  double acc = 0;
  for (long long n = (long long)c * 256 + threadIdx.x; n < N; n += (long long)nchunk * 256) {
    const double2 t = vv[n];
    acc += t.x * t.x + t.y * t.y;
  }
  acc = block_sum1(acc);
  if (threadIdx.x == 0) out[b * nchunk + c] = acc;
}

// out[b] = sqrt(sum_c partial); optionally H[b][k][k+1] = out[b]   grid (B), block 32
__global__ void norm_reduce_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                   double2* __restrict__ H, const int* __restrict__ active, int nchunk, int k,
                                   int mp1, int m) {
  const int b = blockIdx.x;
  double acc = 0;
  for (int c = threadIdx.x; c < nchunk; c += 32) acc += partial[b * nchunk + c];
  acc = warp_sum(acc);
  if (threadIdx.x == 0) {
    const double v = sqrt(acc);
    out[b] = v;
    if (H && active[b]) H[(long long)b * mp1 * m + (long long)k * mp1 + k + 1] = make_double2(v, 0.0);
  }
}

// dst = src / s[b]  (s from a norm array or from H[b][k][k+1])
__global__ void __launch_bounds__(256) scale_kernel(const double2* __restrict__ src, double2* __restrict__ dst,
                                                    const double* __restrict__ nrm, const int* __restrict__ active,
                                                    long long N, long long dst_stride, int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  if (!active[b]) return;
  const long long n = t - (long long)b * N;
  const double s = nrm[b];
  const double inv = s > 0 ? 1.0 / s : 0.0;
  const double2 v = src[t];
  dst[(long long)b * dst_stride + n] = make_double2(v.x * inv, v.y * inv);
}

__global__ void __launch_bounds__(256) scale_h_kernel(const double2* __restrict__ src, double2* __restrict__ dst,
                                                      const double2* __restrict__ H, const int* __restrict__ active,
                                                      long long N, long long dst_stride, int k, int mp1, int m,
                                                      int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  if (!active[b]) return;
  const long long n = t - (long long)b * N;
  const double s = H[(long long)b * mp1 * m + (long long)k * mp1 + k + 1].x;
  const double inv = s > 0 ? 1.0 / s : 0.0;
  const double2 v = src[t];
  dst[(long long)b * dst_stride + n] = make_double2(v.x * inv, v.y * inv);
}

// r = rhs - Ax
__global__ void __launch_bounds__(256) residual_kernel(const double2* __restrict__ rhs, const double2* __restrict__ ax,
                                                       double2* __restrict__ r, long long total) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const double2 a = rhs[t], b = ax[t];
  r[t] = make_double2(a.x - b.x, a.y - b.y);
}

__global__ void __launch_bounds__(256) axpy_kernel(double2* __restrict__ x, const double2* __restrict__ z,
                                                   long long total) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const double2 a = x[t], b = z[t];
  x[t] = make_double2(a.x + b.x, a.y + b.y);
}

// Cycle start: g = [beta, 0, ...], kused = 0, active from the residual norm.
__global__ void cycle_init_kernel(const double* __restrict__ nrm, const double* __restrict__ target,
                                  double2* __restrict__ g, int* __restrict__ active, int* __restrict__ kused, int mp1,
                                  int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const double beta = nrm[b];
  const int act = (beta > target[b]) && isfinite(beta);
  active[b] = act;
  kused[b] = 0;
  for (int i = 0; i < mp1; ++i) g[b * mp1 + i] = make_double2(i == 0 ? beta : 0.0, 0.0);
}

// Givens rotations of column k, residual estimate, convergence test.  One thread per problem.
__global__ void givens_kernel(double2* __restrict__ H, double2* __restrict__ cs, double2* __restrict__ sn,
                              double2* __restrict__ g, int* __restrict__ active, int* __restrict__ kused,
                              const double* __restrict__ target, int k, int mp1, int m, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch || !active[b]) return;
  double2* col = H + (long long)b * mp1 * m + (long long)k * mp1;
  double2* c = cs + b * m;
  double2* s = sn + b * m;
  double2* gg = g + b * mp1;
  for (int i = 0; i < k; ++i) {
    const double2 hi = col[i], hj = col[i + 1];
    const double2 t = make_double2(c[i].x * hi.x - c[i].y * hi.y + s[i].x * hj.x - s[i].y * hj.y,
                                   c[i].x * hi.y + c[i].y * hi.x + s[i].x * hj.y + s[i].y * hj.x);
    // -conj(s) hi + conj(c) hj
    const double2 u = make_double2(-(s[i].x * hi.x + s[i].y * hi.y) + (c[i].x * hj.x + c[i].y * hj.y),
                                   -(s[i].x * hi.y - s[i].y * hi.x) + (c[i].x * hj.y - c[i].y * hj.x));
    col[i] = t;
    col[i + 1] = u;
  }
  const double2 a = col[k], bb = col[k + 1];
  const double den = sqrt(a.x * a.x + a.y * a.y + bb.x * bb.x + bb.y * bb.y);
  double2 cc, ss;
  if (den == 0.0) {
    cc = make_double2(1.0, 0.0);
    ss = make_double2(0.0, 0.0);
  } else {
    cc = make_double2(a.x / den, -a.y / den);    // conj(a/den)
    ss = make_double2(bb.x / den, -bb.y / den);  // conj(b/den)
  }
  c[k] = cc;
  s[k] = ss;
  col[k] = make_double2(den, 0.0);
  col[k + 1] = make_double2(0.0, 0.0);
  const double2 gk = gg[k];
  gg[k + 1] = make_double2(-(ss.x * gk.x + ss.y * gk.y), -(ss.x * gk.y - ss.y * gk.x));  // -conj(s) g_k
  gg[k] = make_double2(cc.x * gk.x - cc.y * gk.y, cc.x * gk.y + cc.y * gk.x);
  kused[b] = k + 1;
  const double res = sqrt(gg[k + 1].x * gg[k + 1].x + gg[k + 1].y * gg[k + 1].y);
  if (!(res > target[b]) || bb.x == 0.0 || !isfinite(res)) active[b] = 0;
}

// y = R^-1 g for the leading kused x kused triangle.  One thread per problem.
__global__ void backsolve_kernel(const double2* __restrict__ H, const double2* __restrict__ g,
                                 double2* __restrict__ y, const int* __restrict__ kused, int mp1, int m, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const int kk = kused[b];
  const double2* Hb = H + (long long)b * mp1 * m;
  double2* yb = y + b * m;
  for (int i = m - 1; i >= kk; --i) yb[i] = make_double2(0, 0);
  for (int i = kk - 1; i >= 0; --i) {
    double2 acc = g[b * mp1 + i];
    for (int c = i + 1; c < kk; ++c) {
      const double2 t = cmul(Hb[(long long)c * mp1 + i], yb[c]);
      acc.x -= t.x;
      acc.y -= t.y;
    }
    const double2 d = Hb[(long long)i * mp1 + i];
    const double dd = d.x * d.x + d.y * d.y;
    yb[i] = dd > 0 ? make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd)
                   : make_double2(0, 0);
  }
}

// u = sum_{i < kused} V_i y_i
__global__ void __launch_bounds__(256) combine_kernel(const double2* __restrict__ V, const double2* __restrict__ y,
                                                      const int* __restrict__ kused, double2* __restrict__ u,
                                                      long long N, int mp1, int m, int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  const long long n = t - (long long)b * N;
  const int kk = kused[b];
  double2 acc = make_double2(0, 0);
  const double2* v = V + (long long)b * mp1 * N + n;
  for (int i = 0; i < kk; ++i) {
    const double2 t2 = cmul(v[(long long)i * N], y[b * m + i]);
    acc.x += t2.x;
    acc.y += t2.y;
  }
  u[t] = acc;
}

inline unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

#define WG_CK(expr)                                                        \
  do {                                                                     \
    cudaError_t e_ = (expr);                                               \
    if (e_ != cudaSuccess) {                                               \
      P.err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #expr; \
      return WG_ERR_CUDA;                                                  \
    }                                                                      \
  } while (0)

// r = rhs - A x ; nrm[b] = |r_b|
int true_residual(Problem& P) {
  const long long tot = P.N * P.batch;
  P.prof.launches[PROF_OTHER] += 3;
  WG_CK(launch_apply(P, P.x, P.w));
  residual_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.rhs, P.w, P.r, tot);
  norm_partial_kernel<<<dim3(P.nchunk, P.batch), 256, 0, P.stream>>>(P.r, P.nrm_partial, P.N, P.nchunk);
  norm_reduce_kernel<<<P.batch, 32, 0, P.stream>>>(P.nrm_partial, P.nrm, nullptr, P.active, P.nchunk, 0, 0, 0);
  WG_CK(cudaGetLastError());
  return WG_OK;
}

}  // namespace

int gmres_solve_fp64(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info) {
  const int B = P.batch, m = P.restart, mp1 = m + 1;
  const long long N = P.N, tot = N * B;
  const double tol = o.tol > 0 ? o.tol : 1e-10;
  const int maxit = o.maxit > 0 ? o.maxit : 50;
  if (!warm) WG_CK(cudaMemsetAsync(P.x, 0, sizeof(double2) * tot, P.stream));
  // |b|
  P.prof.launches[PROF_OTHER] += 2;
  norm_partial_kernel<<<dim3(P.nchunk, B), 256, 0, P.stream>>>(P.rhs, P.nrm_partial, N, P.nchunk);
  norm_reduce_kernel<<<B, 32, 0, P.stream>>>(P.nrm_partial, P.nrm, nullptr, P.active, P.nchunk, 0, 0, 0);
  std::vector<double> bnorm(B), initial(B);
  WG_CK(cudaMemcpyAsync(bnorm.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
  WG_CK(cudaStreamSynchronize(P.stream));
  std::vector<double> tgt(B);
  for (int b = 0; b < B; ++b) tgt[b] = tol * bnorm[b];
  WG_CK(cudaMemcpyAsync(P.target, tgt.data(), sizeof(double) * B, cudaMemcpyHostToDevice, P.stream));
  int rc = true_residual(P);
  if (rc) return rc;
  WG_CK(cudaMemcpyAsync(initial.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
  WG_CK(cudaStreamSynchronize(P.stream));
  std::vector<int> iters(B, 0), cycles(B, 0);
  std::vector<double> res(B);
  for (int b = 0; b < B; ++b) res[b] = initial[b];
  for (int cyc = 0; cyc < maxit; ++cyc) {
    bool any = false;
    for (int b = 0; b < B; ++b) any |= (res[b] > tgt[b]) && std::isfinite(res[b]);
    if (!any) break;
    P.prof.launches[PROF_OTHER] += 2;
    cycle_init_kernel<<<(B + 127) / 128, 128, 0, P.stream>>>(P.nrm, P.target, P.g, P.active, P.kused, mp1, B);
    // V_0 = r / |r|
    scale_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.r, P.V, P.nrm, P.active, N, (long long)mp1 * N, B);
    for (int k = 0; k < m; ++k) {
      // z = M^-1 V_k  (problem b's k-th basis vector sits at stride (m+1) N)
      WG_CK(launch_precondition(P, P.V + (long long)k * N, (long long)mp1 * N, P.z));
      WG_CK(launch_apply(P, P.z, P.w));
      const int nv = k + 1;
      cudaEvent_t ev = prof_begin(P, PROF_KRYLOV, 10);
      for (int pass = 0; pass < 2; ++pass) {
        dot_partial_kernel<<<dim3(P.nchunk, nv, B), 256, 0, P.stream>>>(P.V, P.w, P.partial, P.active, N, mp1,
                                                                       P.nchunk);
        dot_reduce_kernel<<<B, 256, 0, P.stream>>>(P.partial, P.hcol, P.H, P.active, nv, k, mp1, m, P.nchunk,
                                                   pass == 0);
        gs_update_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.V, P.w, P.hcol, P.active, N, nv, mp1, B);
      }
      norm_partial_kernel<<<dim3(P.nchunk, B), 256, 0, P.stream>>>(P.w, P.nrm_partial, N, P.nchunk);
      norm_reduce_kernel<<<B, 32, 0, P.stream>>>(P.nrm_partial, P.nrm, P.H, P.active, P.nchunk, k, mp1, m);
      scale_h_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.w, P.V + (long long)(k + 1) * N, P.H, P.active, N,
                                                            (long long)mp1 * N, k, mp1, m, B);
      givens_kernel<<<(B + 127) / 128, 128, 0, P.stream>>>(P.H, P.cs, P.sn, P.g, P.active, P.kused, P.target, k, mp1,
                                                          m, B);
      prof_end(P, PROF_KRYLOV, ev);
      WG_CK(cudaGetLastError());
      // early exit of the cycle once every problem has met its target
      if ((k & 3) == 3 || k == m - 1) {
        WG_CK(cudaMemcpyAsync(P.h_active.data(), P.active, sizeof(int) * B, cudaMemcpyDeviceToHost, P.stream));
        WG_CK(cudaStreamSynchronize(P.stream));
        bool still = false;
        for (int b = 0; b < B; ++b) still |= P.h_active[b] != 0;
        if (!still) break;
      }
    }
    P.prof.launches[PROF_OTHER] += 4;
    backsolve_kernel<<<(B + 127) / 128, 128, 0, P.stream>>>(P.H, P.g, P.ycoef, P.kused, mp1, m, B);
    combine_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.V, P.ycoef, P.kused, P.w, N, mp1, m, B);
    WG_CK(launch_precondition(P, P.w, N, P.z));
    axpy_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.x, P.z, tot);
    WG_CK(cudaGetLastError());
    rc = true_residual(P);
    if (rc) return rc;
    WG_CK(cudaMemcpyAsync(P.h_kused.data(), P.kused, sizeof(int) * B, cudaMemcpyDeviceToHost, P.stream));
    WG_CK(cudaMemcpyAsync(res.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
    WG_CK(cudaStreamSynchronize(P.stream));
    for (int b = 0; b < B; ++b) {
      iters[b] += P.h_kused[b];
      if (P.h_kused[b] > 0) cycles[b] += 1;
    }
  }
  int status = WG_OK;
  for (int b = 0; b < B; ++b) {
    wg_solve_info& in = info[b];
    const double bn = bnorm[b] > 0 ? bnorm[b] : 1.0;
    in.rhs_norm = bnorm[b];
    in.relres = res[b] / bn;
    in.initial_relres = initial[b] / bn;
    in.iterations = iters[b];
    in.cycles = cycles[b];
    in.refinements = 0;
    in.flag = (std::isfinite(res[b]) && res[b] <= tgt[b]) ? 0 : 1;
    if (bnorm[b] == 0) in.flag = 0;
    if (!std::isfinite(res[b])) {
      P.err = "non-finite residual (NaN/Inf in operator data or rhs)";
      status = WG_ERR_NUMERIC;
    }
    if (in.flag && status == WG_OK) status = WG_NOT_CONVERGED;
  }
  return status;
}

int solve_dispatch(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info) {
  return gmres_solve_fp64(P, o, warm, info);
}

}  // namespace wg
