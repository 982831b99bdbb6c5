// Batched restarted GMRES(m) with right preconditioning (sm_103a).
//
// Semantics of the reference's Krylov wrapper (DG_code/solve_transport_DG_full2D.m):
//  - right preconditioning: Krylov space of A M^-1, x = x0 + M^-1 V y (:462-484)
//  - warm start as a correction about rho0 with the absolute target tol*|b| (:474)
//  - an independent true-residual check that downgrades a converged flag (:314-320)
// Arnoldi uses classical Gram-Schmidt applied twice (CGS2) with block reductions
// and warp shuffles; Givens rotations and the Hessenberg back substitution run on
// the device, one thread per problem.  Every problem of a batch has its own basis,
// Hessenberg matrix and convergence state; a converged problem freezes.
//
// Two drivers share the Arnoldi step, templated on the basis vector type:
//  - gmres_solve_fp64:  FP64 basis and operator (the drop-in plain form);
//  - gmres_solve_mixed: FP64 iterative refinement.  The outer residual
//    r = b - A x is FP64; each correction solves A d = r/|r| with one GMRES cycle
//    whose basis is stored in FP16 (FP32 with inner_basis_fp32), with FP32
//    arithmetic, and whose operator runs the BF16 tensor-core transforms and the
//    FP32 flux / preconditioner.  Inner products and norms are combined in FP64
//    (see AccF32), Givens rotations and the Hessenberg solve are FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <type_traits>

#include "problem.h"

namespace wg {

namespace {

constexpr int kMaxRestart = 256;   // Krylov length bound of the device Givens / staging buffers

__device__ __forceinline__ double2 ld2(const double2& v) { return v; }
__device__ __forceinline__ double2 ld2(const float2& v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ void st2(double2& d, double2 v) { d = v; }
__device__ __forceinline__ void st2(float2& d, double2 v) { d = make_float2((float)v.x, (float)v.y); }

// Basis loads of the FP32 inner solve: two consecutive complex values (16 bytes of an FP32
// basis, 8 bytes of an FP16 one) as one float4; one complex value as float2.
__device__ __forceinline__ float4 ld_pair(const float2* v, long long n4) {
  return reinterpret_cast<const float4*>(v)[n4];
}
__device__ __forceinline__ float4 ld_pair(const __half2* v, long long n4) {
  const uint2 u = reinterpret_cast<const uint2*>(v)[n4];
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float2 ld_one(const float2& v) { return v; }
__device__ __forceinline__ double2 ld_one(const double2& v) { return v; }
__device__ __forceinline__ float2 ld_one(const __half2& v) { return __half22float2(v); }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Inner-product accumulators.  FP64 vectors accumulate in FP64.  FP32 basis
// vectors (mixed form) multiply and add in FP32 within a thread (at most 8
// complex terms) and across the warp (a 5-level tree), then in FP64 across warps,
// blocks and chunks.  The error, a few 1e-7 of sum |a_i b_i|, matches the rounding
// of the FP32 basis itself; the inner GMRES it serves targets 1e-3.  (Error-free
// FP32 transformations per element measured at a third of the HBM rate, and
// double-float merges per warp level made the kernels issue-bound.)
struct Acc64 {
  double2 v = make_double2(0.0, 0.0);
  __device__ __forceinline__ void add_cdot(const double2& a, const double2& x) {  // += conj(a) x
    v.x += a.x * x.x + a.y * x.y;
    v.y += a.x * x.y - a.y * x.x;
  }
  __device__ __forceinline__ void add_norm(const double2& a) { v.x += a.x * a.x + a.y * a.y; }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
  }
  __device__ __forceinline__ double2 get() const { return v; }
  // block-level staging: one slot of 4 doubles per warp
  __device__ __forceinline__ void stage(double* slot) const { slot[0] = v.x; slot[1] = v.y; }
  __device__ __forceinline__ static double2 combine(const double* slots, int n) {
    double2 r = make_double2(0, 0);
    for (int q = 0; q < n; ++q) { r.x += slots[4 * q]; r.y += slots[4 * q + 1]; }
    return r;
  }
};

struct AccF32 {
  float re = 0.f, im = 0.f;
  // two consecutive complex values per float4
  __device__ __forceinline__ void add_cdot4(const float4& a, const float4& x) {
    re = fmaf(a.x, x.x, fmaf(a.y, x.y, fmaf(a.z, x.z, fmaf(a.w, x.w, re))));
    im = fmaf(a.x, x.y, fmaf(-a.y, x.x, fmaf(a.z, x.w, fmaf(-a.w, x.z, im))));
  }
  __device__ __forceinline__ void add_norm(const float2& a) { re = fmaf(a.x, a.x, fmaf(a.y, a.y, re)); }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
  }
  __device__ __forceinline__ void stage(double* slot) const {
    float* f = reinterpret_cast<float*>(slot);
    f[0] = re;
    f[1] = im;
  }
  __device__ __forceinline__ static double2 combine(const double* slots, int n) {
    double2 r = make_double2(0, 0);
    for (int q = 0; q < n; ++q) {
      const float* f = reinterpret_cast<const float*>(slots + 4 * q);
      r.x += (double)f[0];
      r.y += (double)f[1];
    }
    return r;
  }
};

template <typename T> struct AccFor;
template <> struct AccFor<double2> { using type = Acc64; };
template <> struct AccFor<float2> { using type = AccF32; };

// Complex multiply-subtract in the vector's own precision: w -= v h.
__device__ __forceinline__ void cms(double2& w, const double2& v, const double2& h) {
  w.x -= v.x * h.x - v.y * h.y;
  w.y -= v.x * h.y + v.y * h.x;
}
__device__ __forceinline__ void cms(float2& w, const float2& v, const float2& h) {
  w.x = fmaf(-v.x, h.x, fmaf(v.y, h.y, w.x));
  w.y = fmaf(-v.x, h.y, fmaf(-v.y, h.x, w.y));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over a block of up to 256 threads; the result is valid in warp 0.
__device__ double block_sum1(double v) {
  __shared__ double s[8];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  if (lane == 0) s[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = lane < nw ? s[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// The last block of a problem to finish a grid-wide pass (per-problem ticket
// counter; the threadFenceReduction pattern: every block fences its partial
// results, takes a ticket, and the block holding the last ticket reduces them and
// resets the counter for the next launch on the stream).  No block waits.
__device__ __forceinline__ bool last_block_of_problem(int* __restrict__ count, int b) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&count[b], 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// hcol[b][i] = sum_c partial[b][i][c] (FP64); H[b][k][i] = (first) or += hcol.  One block.
__device__ void dot_reduce_block(const double2* __restrict__ partial, double2* __restrict__ hcol,
                                 float2* __restrict__ hcol32, double2* __restrict__ H, int b, int nv, int k,
                                 int pstride, int m, int nchunk, int first) {
  // warp w takes the coefficients w, w + nw, w + 2 nw, w + 3 nw together, so that the loads
  // of four partial rows are in flight at once (this tail runs after the grid's last block)
  constexpr int U = 4;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i0 = w; i0 < nv; i0 += U * nw) {
    double2 acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = make_double2(0, 0);
#pragma unroll 2
    for (int c = lane; c < nchunk; c += 32) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * nw;
        if (i < nv) {
          const double2 t = __ldcg(&partial[((long long)b * pstride + i) * nchunk + c]);
          acc[u].x += t.x;
          acc[u].y += t.y;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * nw;
      if (i >= nv) continue;   // warp-uniform
      acc[u].x = warp_sum(acc[u].x);
      acc[u].y = warp_sum(acc[u].y);
      if (lane == 0) {
        hcol[b * pstride + i] = acc[u];
        if (hcol32) hcol32[b * pstride + i] = make_float2((float)acc[u].x, (float)acc[u].y);
        double2* h = H + (long long)b * pstride * m + (long long)k * pstride + i;
        if (first) *h = acc[u];
        else { h->x += acc[u].x; h->y += acc[u].y; }
      }
    }
  }
}

// Givens step k of problem b (one warp): rotate the new Hessenberg column by the
// previous rotations, make the next rotation, update g and deactivate the problem
// once the residual estimate |g[k+1]| reaches its target.  H is column-major per
// problem (H[b][col*(m+1)+row]), cs/sn/g per problem; staging in shared memory.
__device__ void givens_warp(double2* __restrict__ H, double2* __restrict__ cs, double2* __restrict__ sn,
                            double2* __restrict__ g, int* __restrict__ active, int* __restrict__ kused,
                            const double* __restrict__ target, int b, int k, int pstride, int m, double2* col_s,
                            double2* c_s, double2* s_s) {
  const int lane = threadIdx.x & 31;
  double2* col = H + (long long)b * pstride * m + (long long)k * pstride;
  double2* c = cs + b * m;
  double2* s = sn + b * m;
  for (int i = lane; i <= k + 1; i += 32) col_s[i] = col[i];
  for (int i = lane; i < k; i += 32) {
    c_s[i] = c[i];
    s_s[i] = s[i];
  }
  __syncwarp();
  if (lane == 0) {
    double2* gg = g + b * pstride;
    double2 hi = col_s[0];
    for (int i = 0; i < k; ++i) {
      const double2 hj = col_s[i + 1];
      const double2 ci = c_s[i], si = s_s[i];
      col_s[i] = make_double2(ci.x * hi.x - ci.y * hi.y + si.x * hj.x - si.y * hj.y,
                              ci.x * hi.y + ci.y * hi.x + si.x * hj.y + si.y * hj.x);
      hi = make_double2(-(si.x * hi.x + si.y * hi.y) + (ci.x * hj.x + ci.y * hj.y),
                        -(si.x * hi.y - si.y * hi.x) + (ci.x * hj.y - ci.y * hj.x));
    }
    const double2 a = hi, bb = col_s[k + 1];
    const double den = sqrt(a.x * a.x + a.y * a.y + bb.x * bb.x + bb.y * bb.y);
    double2 cc, ss;
    if (den == 0.0) {
      cc = make_double2(1.0, 0.0);
      ss = make_double2(0.0, 0.0);
    } else {
      const double inv = 1.0 / den;
      cc = make_double2(a.x * inv, -a.y * inv);
      ss = make_double2(bb.x * inv, -bb.y * inv);
    }
    c[k] = cc;
    s[k] = ss;
    col_s[k] = make_double2(den, 0.0);
    col_s[k + 1] = make_double2(0.0, 0.0);
    const double2 gk = gg[k];
    gg[k + 1] = make_double2(-(ss.x * gk.x + ss.y * gk.y), -(ss.x * gk.y - ss.y * gk.x));
    gg[k] = make_double2(cc.x * gk.x - cc.y * gk.y, cc.x * gk.y + cc.y * gk.x);
    kused[b] = k + 1;
    const double res = sqrt(gg[k + 1].x * gg[k + 1].x + gg[k + 1].y * gg[k + 1].y);
    if (!(res > target[b]) || bb.x == 0.0 || !isfinite(res)) active[b] = 0;
  }
  __syncwarp();
  for (int i = lane; i <= k + 1; i += 32) col[i] = col_s[i];
}

// Arguments of the per-problem tail work done by the last block of a launch.
struct KrylovTail {
  int* md_count;       // [B] tickets of the multi-dot
  int* gs_count;       // [B] tickets of the update
  double2* partial;    // multi-dot partials
  double2* hcol;       // FP64 coefficients
  float2* hcol32;      // FP32 copy (mixed form) or null
  double2* H;
  double2 *cs, *sn, *g;
  int* active;
  int* kused;
  int* reorth;
  const double* target;
  double* nrm;
  double* inv64;
  float* inv32;
  double eta2;         // DGKS threshold squared
  int k, pstride, m, first;
};

// Multi-dot: partial[b][i][c] = sum over chunk c of conj(V_i) . w for every i < nv.
// One block per (chunk of 256*E elements, problem): w stays in registers, each V_i
// chunk is read once, warps drop their partial sums in shared memory and the
// block adds them at the end (no block barrier per coefficient).
constexpr int kMdE = 8;
template <typename T, typename VB = T>
__global__ void __launch_bounds__(256) multidot_kernel(const VB* __restrict__ V, const T* __restrict__ w,
                                                       double2* __restrict__ partial, const int* __restrict__ active,
                                                       long long N, int nv, int mp1, int pstride, int nchunk,
                                                       KrylovTail tl) {
  extern __shared__ double red[];  // [nv][8 warps][4 doubles]
  const int b = blockIdx.y, c = blockIdx.x;
  if (!active[b]) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (std::is_same<T, float2>::value) {
    // two complex values per 16-byte load (N is even for the mixed form)
    constexpr int E4 = kMdE / 2;
    const long long base4 = (long long)c * 256 * E4 + threadIdx.x, N4 = N / 2;
    const float4* wb = reinterpret_cast<const float4*>(w + (long long)b * N);
    float4 wv[E4];
#pragma unroll
    for (int j = 0; j < E4; ++j) {
      const long long n = base4 + (long long)j * 256;
      wv[j] = n < N4 ? wb[n] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    int i = 0;
    // four basis vectors per pass: 16 loads in flight per thread between two reductions
    for (; i + 3 < nv; i += 4) {
      const VB* v0 = V + ((long long)b * mp1 + i) * N;
      float4 a[4][E4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < E4; ++j) {
          const long long n = base4 + (long long)j * 256;
          a[u][j] = n < N4 ? ld_pair(v0 + (long long)u * N, n) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      AccF32 s4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int j = 0; j < E4; ++j) s4[u].add_cdot4(a[u][j], wv[j]);
        s4[u].warp_reduce();
      }
      if (lane == 0)
#pragma unroll
        for (int u = 0; u < 4; ++u) s4[u].stage(red + ((i + u) * 8 + warp) * 4);
    }
    for (; i + 1 < nv; i += 2) {
      const VB* v0 = V + ((long long)b * mp1 + i) * N;
      const VB* v1 = v0 + N;
      float4 a0[E4], a1[E4];
#pragma unroll
      for (int j = 0; j < E4; ++j) {
        const long long n = base4 + (long long)j * 256;
        a0[j] = n < N4 ? ld_pair(v0, n) : make_float4(0.f, 0.f, 0.f, 0.f);
        a1[j] = n < N4 ? ld_pair(v1, n) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      AccF32 s0, s1;
#pragma unroll
      for (int j = 0; j < E4; ++j) {
        s0.add_cdot4(a0[j], wv[j]);
        s1.add_cdot4(a1[j], wv[j]);
      }
      s0.warp_reduce();
      s1.warp_reduce();
      if (lane == 0) {
        s0.stage(red + (i * 8 + warp) * 4);
        s1.stage(red + ((i + 1) * 8 + warp) * 4);
      }
    }
    if (i < nv) {
      const VB* v0 = V + ((long long)b * mp1 + i) * N;
      AccF32 s0;
#pragma unroll
      for (int j = 0; j < E4; ++j) {
        const long long n = base4 + (long long)j * 256;
        if (n < N4) s0.add_cdot4(ld_pair(v0, n), wv[j]);
      }
      s0.warp_reduce();
      if (lane == 0) s0.stage(red + (i * 8 + warp) * 4);
    }
  } else {
    const long long base = (long long)c * 256 * kMdE + threadIdx.x;
    const T* wb = w + (long long)b * N;
    T wv[kMdE];
#pragma unroll
    for (int j = 0; j < kMdE; ++j) {
      const long long n = base + (long long)j * 256;
      if (n < N) wv[j] = wb[n];
      else { wv[j].x = 0; wv[j].y = 0; }
    }
    for (int i = 0; i < nv; ++i) {
      const VB* v = V + ((long long)b * mp1 + i) * N;
      typename AccFor<T>::type a;
#pragma unroll
      for (int j = 0; j < kMdE; ++j) {
        const long long n = base + (long long)j * 256;
        if (n < N) a.add_cdot(v[n], wv[j]);
      }
      a.warp_reduce();
      if (lane == 0) a.stage(red + (i * 8 + warp) * 4);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nv; i += blockDim.x)
    partial[((long long)b * pstride + i) * nchunk + c] = AccFor<T>::type::combine(red + i * 8 * 4, 8);
  // the last chunk of problem b reduces the partials into the Hessenberg column
  if (!last_block_of_problem(tl.md_count, b)) return;
  dot_reduce_block(partial, tl.hcol, tl.hcol32, tl.H, b, nv, tl.k, pstride, tl.m, nchunk, tl.first);
  if (threadIdx.x == 0) tl.md_count[b] = 0;
}



// w -= sum_i V_i hcol_i.  FP64 vectors: grid (ceil(N/256), B), one complex value per
// thread; FP32 vectors: grid (ceil(N/(256 kGsPairs)), B), 128 threads of kGsPairs 16-byte
// accesses (two complex values each); the coefficients are staged in shared memory.
// MODE 0: update only.  MODE >= 1: also nrm_partial[b][block] = sum |w|^2, and the last
// block of problem b finishes the step: MODE 1 runs the DGKS test (reorth[b]) and, when
// no second pass is needed, MODE 2's work: |w|, H[k+1][k], inverse norm, Givens step.
constexpr int kGsPairs = 2;
template <typename T, int MODE, typename VB = T>
__global__ void __launch_bounds__(256) gs_update_kernel(const VB* __restrict__ V, T* __restrict__ w,
                                                        const T* __restrict__ hcol, const int* __restrict__ mask,
                                                        double* __restrict__ nrm_partial, long long N, int nv, int mp1,
                                                        int pstride, int nblk, KrylovTail tl) {
  const int b = blockIdx.y;
  if (!mask[b]) return;
  __shared__ T hs[kMaxRestart + 1];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = hcol[b * pstride + i];
  __syncthreads();
  typename AccFor<T>::type a;
  if constexpr (std::is_same<T, float2>::value) {
    // kGsPairs float4 (two complex values each) per thread, 128 apart: the grid of a handle
    // fits one wave of resident blocks and every basis pass has kGsPairs loads per thread
    const long long N4 = N / 2;
    const long long n40 = (long long)blockIdx.x * (128 * kGsPairs) + threadIdx.x;
    float4* wp = reinterpret_cast<float4*>(w + (long long)b * N);
    float4 acc[kGsPairs];
#pragma unroll
    for (int g = 0; g < kGsPairs; ++g) {
      const long long n4 = n40 + 128 * g;
      acc[g] = n4 < N4 ? wp[n4] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const VB* v = V + (long long)b * mp1 * N;
    // the loads of four basis vectors are issued before their updates are applied
    constexpr int U = 4;
    for (int i0 = 0; i0 < nv; i0 += U) {
      float4 x[U][kGsPairs];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int g = 0; g < kGsPairs; ++g) {
          const long long n4 = n40 + 128 * g;
          x[u][g] = (i0 + u < nv && n4 < N4) ? ld_pair(v, (long long)(i0 + u) * N4 + n4)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        // past nv the coefficient is zero and the (zero) loads change nothing
        const float2 h = i0 + u < nv ? hs[i0 + u] : make_float2(0.f, 0.f);
#pragma unroll
        for (int g = 0; g < kGsPairs; ++g) {
          acc[g].x = fmaf(-x[u][g].x, h.x, fmaf(x[u][g].y, h.y, acc[g].x));
          acc[g].y = fmaf(-x[u][g].x, h.y, fmaf(-x[u][g].y, h.x, acc[g].y));
          acc[g].z = fmaf(-x[u][g].z, h.x, fmaf(x[u][g].w, h.y, acc[g].z));
          acc[g].w = fmaf(-x[u][g].z, h.y, fmaf(-x[u][g].w, h.x, acc[g].w));
        }
      }
    }
#pragma unroll
    for (int g = 0; g < kGsPairs; ++g) {
      const long long n4 = n40 + 128 * g;
      if (n4 < N4) {
        wp[n4] = acc[g];
        if (MODE) {
          a.add_norm(make_float2(acc[g].x, acc[g].y));
          a.add_norm(make_float2(acc[g].z, acc[g].w));
        }
      }
    }
  } else {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n < N) {
      const long long t = (long long)b * N + n;
      T acc = w[t];
      const VB* v = V + (long long)b * mp1 * N + n;
#pragma unroll 4
      for (int i = 0; i < nv; ++i) cms(acc, v[(long long)i * N], hs[i]);
      w[t] = acc;
      if (MODE) a.add_norm(acc);
    }
  }
  if constexpr (MODE >= 1) {
    __shared__ double wsum[8 * 4];
    a.warp_reduce();
    if ((threadIdx.x & 31) == 0) a.stage(wsum + (threadIdx.x >> 5) * 4);
    __syncthreads();
    if (threadIdx.x == 0)
      nrm_partial[(long long)b * nblk + blockIdx.x] = AccFor<T>::type::combine(wsum, blockDim.x >> 5).x;
    if (!last_block_of_problem(tl.gs_count, b)) return;
    // the whole last block adds the partial norms (independent loads), warp 0 finishes the step
    double w2p = 0;
#pragma unroll 8
    for (int c = threadIdx.x; c < nblk; c += blockDim.x) w2p += __ldcg(&nrm_partial[(long long)b * nblk + c]);
    const double w2b = block_sum1(w2p);
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      const double w2 = w2b;
      bool finish = true;
      if (MODE == 1) {
        double h2 = 0;
        for (int i = lane; i < nv; i += 32) {
          const double2 h = tl.hcol[(long long)b * pstride + i];
          h2 += h.x * h.x + h.y * h.y;
        }
        h2 = warp_sum(h2);
        const int re = w2 < tl.eta2 * (w2 + h2) ? 1 : 0;
        if (lane == 0) tl.reorth[b] = re;
        finish = !re;
      }
      if (finish) {
        __shared__ double2 col_s[kMaxRestart + 1], c_s[kMaxRestart], s_s[kMaxRestart];
        if (lane == 0) {
          const double v = sqrt(w2);
          tl.nrm[b] = v;
          if (tl.inv64) tl.inv64[b] = v > 0 ? 1.0 / v : 0.0;
          if (tl.inv32) tl.inv32[b] = v > 0 ? (float)(1.0 / v) : 0.f;
          tl.H[(long long)b * pstride * tl.m + (long long)tl.k * pstride + tl.k + 1] = make_double2(v, 0.0);
        }
        __syncwarp();
        givens_warp(tl.H, tl.cs, tl.sn, tl.g, tl.active, tl.kused, tl.target, b, tl.k, pstride, tl.m, col_s, c_s,
                    s_s);
      }
    }
    if (threadIdx.x == 0) tl.gs_count[b] = 0;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) norm_partial_kernel(const T* __restrict__ v, double* __restrict__ out,
                                                           long long N, int nchunk,
                                                           const int* __restrict__ mask = nullptr) {
  const int b = blockIdx.y, c = blockIdx.x;
  if (mask && !mask[b]) return;
  const T* vv = v + (long long)b * N;
  typename AccFor<T>::type a;
  for (long long n = (long long)c * 256 + threadIdx.x; n < N; n += (long long)nchunk * 256) a.add_norm(vv[n]);
  const double acc = block_sum1(a.get().x);
  if (threadIdx.x == 0) out[b * nchunk + c] = acc;
}

// out[b] = sqrt(sum_c partial); optionally H[b][k][k+1] = out[b]
__global__ void norm_reduce_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                   double2* __restrict__ H, const int* __restrict__ active, int nchunk, int k,
                                   int pstride, int m, double* __restrict__ inv64 = nullptr,
                                   float* __restrict__ inv32 = nullptr, const int* __restrict__ mask = nullptr) {
  const int b = blockIdx.x;
  if (mask && !mask[b]) return;   // problems outside the mask keep their norm
  double acc = 0;
  for (int c = threadIdx.x; c < nchunk; c += 32) acc += partial[b * nchunk + c];
  acc = warp_sum(acc);
  if (threadIdx.x == 0) {
    const double v = sqrt(acc);
    out[b] = v;
    if (inv64) inv64[b] = v > 0 ? 1.0 / v : 0.0;
    if (inv32) inv32[b] = v > 0 ? (float)(1.0 / v) : 0.f;
    if (H && active[b]) H[(long long)b * pstride * m + (long long)k * pstride + k + 1] = make_double2(v, 0.0);
  }
}

// dst = src * inv[b]  (inverse norms precomputed per problem)
template <typename S, typename D>
__global__ void __launch_bounds__(256) scale_kernel(const S* __restrict__ src, D* __restrict__ dst,
                                                    const double* __restrict__ nrm, const int* __restrict__ active,
                                                    long long N, long long dst_stride, int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  if (!active[b]) return;
  const long long n = t - (long long)b * N;
  const double inv = nrm[b];   // inverse norm
  const double2 v = ld2(src[t]);
  st2(dst[(long long)b * dst_stride + n], make_double2(v.x * inv, v.y * inv));
}

__global__ void __launch_bounds__(256) residual_kernel(const double2* __restrict__ rhs, const double2* __restrict__ ax,
                                                       double2* __restrict__ r, long long total, long long N,
                                                       const int* __restrict__ mask) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total || (mask && !mask[t / N])) return;
  const double2 a = rhs[t], b = ax[t];
  r[t] = make_double2(a.x - b.x, a.y - b.y);
}

// x += s[b] * z  (s = nullptr: s = 1; problems with mask[b] == 0 are left as they are)
template <typename T>
__global__ void __launch_bounds__(256) axpy_kernel(double2* __restrict__ x, const T* __restrict__ z,
                                                   const double* __restrict__ s, long long N, int batch,
                                                   const int* __restrict__ mask = nullptr) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  if (mask && !mask[b]) return;
  const double f = s ? s[b] : 1.0;
  const double2 a = x[t], v = ld2(z[t]);
  x[t] = make_double2(a.x + f * v.x, a.y + f * v.y);
}

__global__ void cycle_init_kernel(const double* __restrict__ nrm, const double* __restrict__ target,
                                  double2* __restrict__ g, int* __restrict__ active, int* __restrict__ kused,
                                  int pstride, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const double beta = nrm[b];
  const int act = (beta > target[b]) && isfinite(beta);
  active[b] = act;
  kused[b] = 0;
  for (int i = 0; i < pstride; ++i) g[b * pstride + i] = make_double2(i == 0 ? beta : 0.0, 0.0);
}


// y = R^-1 g for the rotated Hessenberg matrix R (upper triangular, column-major per
// problem), one warp per problem: column-oriented back substitution, the lanes update
// the remaining right-hand side with column i of R.  The inverse diagonal is formed for
// all rows at once first, and column i - 1 is loaded into registers while column i is
// applied, so the serial sweep waits on neither a division nor a load per row.
__global__ void backsolve_kernel(const double2* __restrict__ H, const double2* __restrict__ g,
                                 double2* __restrict__ y, float2* __restrict__ y32, const int* __restrict__ kused,
                                 int pstride, int m, int batch) {
  constexpr int JT = kMaxRestart / 32;   // column entries per lane
  __shared__ double2 acc[kMaxRestart + 1];
  __shared__ double2 dinv[kMaxRestart];
  const int b = blockIdx.x;
  const int lane = threadIdx.x;
  if (b >= batch) return;
  const int kk = kused[b];
  const double2* Hb = H + (long long)b * pstride * m;
  double2* yb = y + b * m;
  for (int i = lane; i < m; i += 32) {
    acc[i] = i < kk ? g[b * pstride + i] : make_double2(0, 0);
    if (i >= kk) yb[i] = make_double2(0, 0);
  }
  for (int i = lane; i < kk; i += 32) {
    const double2 d = Hb[(long long)i * pstride + i];
    const double dd = d.x * d.x + d.y * d.y;
    dinv[i] = dd > 0 ? make_double2(d.x / dd, -d.y / dd) : make_double2(0, 0);
  }
  double2 cur[JT], nxt[JT];
#pragma unroll
  for (int t = 0; t < JT; ++t) {
    const int j = lane + 32 * t;
    cur[t] = (kk > 0 && j < kk - 1) ? Hb[(long long)(kk - 1) * pstride + j] : make_double2(0, 0);
  }
  __syncwarp();
  for (int i = kk - 1; i >= 0; --i) {
#pragma unroll
    for (int t = 0; t < JT; ++t) {
      const int j = lane + 32 * t;
      nxt[t] = (i > 0 && j < i - 1) ? Hb[(long long)(i - 1) * pstride + j] : make_double2(0, 0);
    }
    const double2 yi = cmul(acc[i], dinv[i]);
    if (lane == 0) yb[i] = yi;
#pragma unroll
    for (int t = 0; t < JT; ++t) {
      const int j = lane + 32 * t;
      if (j < i) {
        const double2 u = cmul(cur[t], yi);
        acc[j].x -= u.x;
        acc[j].y -= u.y;
      }
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < JT; ++t) cur[t] = nxt[t];
  }
  __syncwarp();
  if (y32)
    for (int i = lane; i < m; i += 32) {
      const double2 v = i < kk ? yb[i] : make_double2(0, 0);
      y32[b * m + i] = make_float2((float)v.x, (float)v.y);
    }
}

template <typename T, typename VB = T>
__global__ void __launch_bounds__(256) combine_kernel(const VB* __restrict__ V, const T* __restrict__ y,
                                                      const int* __restrict__ kused, T* __restrict__ u, long long N,
                                                      int mp1, int m, int batch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * batch) return;
  const int b = (int)(t / N);
  const long long n = t - (long long)b * N;
  const int kk = kused[b];
  T acc;
  acc.x = 0;
  acc.y = 0;
  const VB* v = V + (long long)b * mp1 * N + n;
  for (int i = 0; i < kk; ++i) {
    T h = y[b * m + i];
    h.x = -h.x;
    h.y = -h.y;
    cms(acc, ld_one(v[(long long)i * N]), h);   // acc += v y
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

// One Arnoldi step k on basis V (stride (m+1) N per problem): z = M^-1 V_k,
// w = A z, CGS2 against V_0..V_k, V_{k+1} = w / |w|, Givens.  `prec` and `apply`
// are the operator pair of the basis precision.
template <typename T> T* coef_col(Problem& P);
template <> double2* coef_col<double2>(Problem& P) { return P.hcol; }
template <> float2* coef_col<float2>(Problem& P) { return P.mx.hcol; }
template <typename T> float2* coef_col32(Problem& P);
template <> float2* coef_col32<double2>(Problem&) { return nullptr; }
template <> float2* coef_col32<float2>(Problem& P) { return P.mx.hcol; }

template <typename T, typename VB = T, typename Prec, typename Apply>
int arnoldi_step(Problem& P, VB* V, T* w, int k, int m, Prec prec, Apply apply) {
  const int B = P.batch, mp1 = m + 1, ps = P.restart_max + 1, mm = P.restart_max;
  const long long N = P.N;
  // V_k: step 0 reads the basis vector the cycle start wrote; later steps take the previous
  // step's w and its inverse norm, and the preconditioner writes V_k = w / |w| as it reads it
  // (no separate scaling pass per step).  An FP16 basis: the cycle start leaves V_0 in FP32
  // in w, and the preconditioner stores its FP16 rounding as V_0.
  if (k == 0) {
    if constexpr (std::is_same<VB, T>::value) WG_CK(prec(V, (long long)mp1 * N, nullptr, nullptr));
    else WG_CK(prec(w, N, nullptr, V));
  } else {
    const T* wprev = w;
    if constexpr (std::is_same<T, float2>::value)
      WG_CK(prec(wprev, N, P.mx.inv, V + (long long)k * N));
    else
      WG_CK(prec(wprev, N, P.inv64, V + (long long)k * N));
  }
  WG_CK(apply());
  const int nv = k + 1;
  const double vec = (double)N * B * sizeof(T), vecb = (double)N * B * sizeof(VB);
  // the FP32 update covers 256 kGsPairs complex values per block of 128 threads
  const long long per_blk = sizeof(T) == sizeof(float2) ? 256LL * kGsPairs : 256LL;
  const dim3 gu((unsigned)((N + per_blk - 1) / per_blk), B);
  const int nblk = (int)gu.x;
  // classical Gram-Schmidt; the second pass runs for the problems that fail the DGKS
  // test (its kernels see P.reorth as their activity mask), for all with eta >= 1,
  // for none with eta < 0.  The reductions, the norm and the Givens step run in the
  // last block of each problem's multi-dot / update launch (KrylovTail).
  const double eta = sizeof(T) == sizeof(float2) ? P.inner_reorth_eta : P.reorth_eta;
  const int passes = eta < 0 ? 1 : 2;
  KrylovTail tl{P.md_count, P.gs_count, P.partial, P.hcol, coef_col32<T>(P), P.H, P.cs, P.sn, P.g, P.active,
                P.kused, P.reorth, P.target, P.nrm, sizeof(T) == sizeof(float2) ? nullptr : P.inv64,
                sizeof(T) == sizeof(float2) ? P.mx.inv : nullptr, eta * eta, k, ps, mm, 1};
  const unsigned gthreads = sizeof(T) == sizeof(float2) ? 128 : 256;
  // the DGKS flags are written only for problems that take part in the first pass
  if (passes == 2 && eta < 1) WG_CK(cudaMemsetAsync(P.reorth, 0, sizeof(int) * B, P.stream));
  for (int pass = 0; pass < passes; ++pass) {
    const int* mask = (pass == 0 || eta >= 1) ? P.active : P.reorth;
    tl.first = pass == 0;
    cudaEvent_t ev = prof_begin(P, PROF_MULTIDOT, 1, nv * vecb + vec, 8.0 * nv * N * B, mask);
    multidot_kernel<T, VB><<<dim3(P.nchunk, B), 256, sizeof(double) * 32 * nv, P.stream>>>(V, w, P.partial, mask,
                                                                                          N, nv, mp1, ps, P.nchunk,
                                                                                          tl);
    prof_end(P, PROF_MULTIDOT, ev);
    ev = prof_begin(P, PROF_GSUPDATE, 1, nv * vecb + 2 * vec, 8.0 * nv * N * B, mask);
    if (pass == passes - 1)
      gs_update_kernel<T, 2, VB><<<gu, gthreads, 0, P.stream>>>(V, w, coef_col<T>(P), mask, P.nrm_partial, N, nv,
                                                                 mp1, ps, nblk, tl);
    else if (eta < 1)
      gs_update_kernel<T, 1, VB><<<gu, gthreads, 0, P.stream>>>(V, w, coef_col<T>(P), mask, P.nrm_partial, N, nv,
                                                                 mp1, ps, nblk, tl);
    else
      gs_update_kernel<T, 0, VB><<<gu, gthreads, 0, P.stream>>>(V, w, coef_col<T>(P), mask, P.nrm_partial, N, nv,
                                                                 mp1, ps, nblk, tl);
    prof_end(P, PROF_GSUPDATE, ev);
  }
  // V_{k+1} = w / |w| is written by the next step's preconditioner
  WG_CK(cudaGetLastError());
  return WG_OK;
}

// r = rhs - A x ; nrm[b] = |r_b|  (FP64)
// r = b - A x and |r| (FP64; the mixed form's transforms on the tensor cores).  mask
// (device, optional): only problems with mask[b] != 0 are evaluated, the others keep
// their previous r and |r| (their x has not changed since).
int true_residual(Problem& P, const int* mask = nullptr, int nd = 8, const int* nd_pp = nullptr) {
  const long long tot = P.N * P.batch;
  P.prof.launches[PROF_OTHER] += 3;
  if (P.precision == WG_PREC_MIXED) WG_CK(launch_apply_f64_tc(P, P.x, P.w, mask, nd, nd_pp));
  else WG_CK(launch_apply(P, P.x, P.w));
  residual_kernel<<<blocks_for(tot), 256, 0, P.stream>>>(P.rhs, P.w, P.r, tot, P.N, mask);
  norm_partial_kernel<double2><<<dim3(P.nchunk, P.batch), 256, 0, P.stream>>>(P.r, P.nrm_partial, P.N, P.nchunk,
                                                                             mask);
  norm_reduce_kernel<<<P.batch, 32, 0, P.stream>>>(P.nrm_partial, P.nrm, nullptr, P.active, P.nchunk, 0, 0, 0,
                                                   P.inv64, nullptr, mask);
  WG_CK(cudaGetLastError());
  return WG_OK;
}

// Leading digits of the emulated FP64 transforms for the mixed form's true residual: enough
// that the residual's error (~2^(-6 nd) |A||x|, with a margin of 2^21 for |A||x| / |b|) stays
// below the loosest target among the problems it is evaluated for; 8 (the full split) for
// tolerances of 1e-7 and below.  WG_RESIDUAL_DIGITS (1 .. 8) fixes it.
int digits_for(double t) {
  if (!(t > 0) || !(t < 1e299)) return 8;
  const int d = (int)std::ceil((std::log2(1.0 / t) + 21.0) / 6.0);
  return std::max(4, std::min(8, d));
}

int residual_digits(const Problem& P, double tol, const std::vector<int>* hmask) {
  static const int forced = [] {
    const char* v = std::getenv("WG_RESIDUAL_DIGITS");
    const int d = v ? std::atoi(v) : 0;
    return (d >= 1 && d <= 8) ? d : 0;
  }();
  if (forced) return forced;
  double tmin = INFINITY;
  for (int b = 0; b < P.batch; ++b) {
    if (hmask && (int)hmask->size() == P.batch && !(*hmask)[b]) continue;
    tmin = std::min(tmin, P.tol_pp.empty() ? tol : P.tol_pp[b]);
  }
  return digits_for(tmin);
}

// Digits per problem (the emulated GEMM's column tiles take the largest of their problems);
// uploads them and returns the device array, or nullptr when one count serves all.
const int* residual_digits_pp(Problem& P, double tol) {
  if (P.tol_pp.empty() || std::getenv("WG_RESIDUAL_DIGITS")) return nullptr;
  P.h_res_digits.assign(P.batch, 8);
  for (int b = 0; b < P.batch; ++b) P.h_res_digits[b] = digits_for(P.tol_pp[b]);
  if (cudaMemcpyAsync(P.res_digits, P.h_res_digits.data(), sizeof(int) * P.batch, cudaMemcpyHostToDevice,
                      P.stream) != cudaSuccess)
    return nullptr;
  return P.res_digits;
}

// Shared set-up: |b| per problem, targets, initial true residual.
int solve_begin(Problem& P, double tol, bool warm, std::vector<double>& bnorm, std::vector<double>& tgt,
                std::vector<double>& res) {
  const int B = P.batch;
  if (!warm) WG_CK(cudaMemsetAsync(P.x, 0, sizeof(double2) * P.N * B, P.stream));
  P.prof.launches[PROF_OTHER] += 2;
  norm_partial_kernel<double2><<<dim3(P.nchunk, B), 256, 0, P.stream>>>(P.rhs, P.nrm_partial, P.N, P.nchunk);
  norm_reduce_kernel<<<B, 32, 0, P.stream>>>(P.nrm_partial, P.nrm, nullptr, P.active, P.nchunk, 0, 0, 0);
  bnorm.resize(B);
  WG_CK(cudaMemcpyAsync(bnorm.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
  WG_CK(cudaStreamSynchronize(P.stream));
  tgt.resize(B);
  for (int b = 0; b < B; ++b) tgt[b] = (P.tol_pp.empty() ? tol : P.tol_pp[b]) * bnorm[b];
  // problems frozen by an unreachable tolerance keep their residual
  const int* mask = nullptr;
  int nd = 8;
  if (P.precision == WG_PREC_MIXED) {
    if (!P.tol_pp.empty()) {
      P.h_res_mask.assign(B, 1);
      for (int b = 0; b < B; ++b) P.h_res_mask[b] = P.tol_pp[b] < 1e299 ? 1 : 0;
      WG_CK(cudaMemcpyAsync(P.res_mask, P.h_res_mask.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
      mask = P.res_mask;
      nd = residual_digits(P, tol, &P.h_res_mask);
    } else {
      nd = residual_digits(P, tol, nullptr);
    }
  }
  int rc = true_residual(P, mask, nd, P.precision == WG_PREC_MIXED ? residual_digits_pp(P, tol) : nullptr);
  if (rc) return rc;
  res.resize(B);
  WG_CK(cudaMemcpyAsync(res.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
  WG_CK(cudaStreamSynchronize(P.stream));
  return WG_OK;
}

int solve_end(Problem& P, const std::vector<double>& bnorm, const std::vector<double>& tgt,
              const std::vector<double>& initial, const std::vector<double>& res, const std::vector<int>& iters,
              const std::vector<int>& cycles, const std::vector<int>& refinements, wg_solve_info* info) {
  int status = WG_OK;
  for (int b = 0; b < P.batch; ++b) {
    wg_solve_info& in = info[b];
    const double bn = bnorm[b] > 0 ? bnorm[b] : 1.0;
    in.rhs_norm = bnorm[b];
    in.relres = res[b] / bn;
    in.initial_relres = initial[b] / bn;
    in.iterations = iters[b];
    in.cycles = cycles[b];
    in.refinements = refinements[b];
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

bool all_done(const std::vector<int>& act) {
  for (int a : act)
    if (a) return false;
  return true;
}

bool graphs_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("WG_CUDA_GRAPHS");
    return !(v && v[0] == '0');
  }();
  return on;
}

void reset_graphs(ArnoldiGraphs& G) {
  for (cudaGraphExec_t x : G.exec)
    if (x) cudaGraphExecDestroy(x);
  G.exec.clear();
  G.launches.clear();
  G.eager.clear();
}

// Arnoldi steps k0 .. k0+3 (fewer at the end of the cycle) of a cycle of length m, run
// eagerly (`run`) or replayed from the chunk's CUDA graph.  A chunk is captured on its
// second use, so the launch helpers' one-time set-up has run outside the capture; any
// failure to capture or instantiate falls back to eager launches for the handle.
// Chunks of a cycle: steps [0,1), [1,2), [2,4), then 4 at a time.  The host checks the
// problems' convergence after every chunk; the short first chunks keep a cycle that
// converges in one or two steps (loose transport tolerances) from running masked steps.
int chunk_end(int k0, int m) { return std::min(m, k0 < 2 ? k0 + 1 : (k0 < 4 ? 4 : k0 + 4)); }
int chunk_index(int k0) { return k0 < 2 ? k0 : (k0 < 4 ? 2 : 2 + k0 / 4); }
int chunk_count(int m) { return m <= 2 ? m : (m <= 4 ? 3 : 2 + (m + 3) / 4); }

template <typename Run>
int run_arnoldi_chunk(Problem& P, ArnoldiGraphs& G, int m, int k0, Run run) {
  if (G.disabled || P.prof.on || !graphs_enabled()) return run();
  const int nchunk = chunk_count(m), c = chunk_index(k0);
  if (G.m != m || G.shift != P.shift || G.kline_L != P.kline_L || G.st_cells != P.st_cells ||
      (int)G.exec.size() != nchunk) {
    reset_graphs(G);
    G.m = m;
    G.shift = P.shift;
    G.kline_L = P.kline_L;
    G.st_cells = P.st_cells;
    G.exec.assign(nchunk, nullptr);
    G.launches.assign(nchunk, {});
    G.eager.assign(nchunk, 0);
  }
  if (G.exec[c]) {
    const cudaError_t e = cudaGraphLaunch(G.exec[c], P.stream);
    if (e != cudaSuccess) {
      P.err = std::string("CUDA graph launch: ") + cudaGetErrorString(e);
      return WG_ERR_CUDA;
    }
    for (int i = 0; i < PROF_N; ++i) P.prof.launches[i] += G.launches[c][i];
    ++G.replays;
    return WG_OK;
  }
  if (G.eager[c]++ == 0) return run();
  std::array<long long, PROF_N> before;
  for (int i = 0; i < PROF_N; ++i) before[i] = P.prof.launches[i];
  auto fall_back = [&]() {
    cudaGetLastError();
    G.disabled = true;
    reset_graphs(G);
    for (int i = 0; i < PROF_N; ++i) P.prof.launches[i] = before[i];
    return run();
  };
  if (cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fall_back();
  const int rc = run();
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(P.stream, &g);
  if (rc != WG_OK || ec != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    return fall_back();
  }
  cudaGraphExec_t x = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess || !x) return fall_back();
  G.exec[c] = x;
  for (int i = 0; i < PROF_N; ++i) G.launches[c][i] = P.prof.launches[i] - before[i];
  const cudaError_t e = cudaGraphLaunch(x, P.stream);
  if (e != cudaSuccess) {
    P.err = std::string("CUDA graph launch: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  return WG_OK;
}

}  // namespace

int gmres_solve_fp64(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info) {
  const int B = P.batch, m = P.restart, mp1 = m + 1, ps = P.restart_max + 1, mm = P.restart_max;
  const long long N = P.N, tot = N * B;
  const double tol = o.tol > 0 ? o.tol : 1e-10;
  const int maxit = o.maxit > 0 ? o.maxit : 50;
  std::vector<double> bnorm, tgt, initial;
  int rc = solve_begin(P, tol, warm, bnorm, tgt, initial);
  if (rc) return rc;
  WG_CK(cudaMemcpyAsync(P.target, tgt.data(), sizeof(double) * B, cudaMemcpyHostToDevice, P.stream));
  std::vector<int> iters(B, 0), cycles(B, 0), refs(B, 0);
  std::vector<double> res = initial;
  auto prec = [&](const double2* r, long long stride, const double* rscale, double2* rout) {
    return launch_precondition(P, r, stride, P.z, rscale, rout, (long long)mp1 * N);
  };
  auto apply = [&]() { return launch_apply(P, P.z, P.w); };
  for (int cyc = 0; cyc < maxit; ++cyc) {
    bool any = false;
    for (int b = 0; b < B; ++b) any |= (res[b] > tgt[b]) && std::isfinite(res[b]);
    if (!any) break;
    P.prof.launches[PROF_OTHER] += 2;
    cycle_init_kernel<<<(B + 127) / 128, 128, 0, P.stream>>>(P.nrm, P.target, P.g, P.active, P.kused, ps, B);
    scale_kernel<double2, double2><<<blocks_for(tot), 256, 0, P.stream>>>(P.r, P.V, P.inv64, P.active, N,
                                                                         (long long)mp1 * N, B);
    for (int k0 = 0; k0 < m; k0 = chunk_end(k0, m)) {
      const int k1 = chunk_end(k0, m);
      rc = run_arnoldi_chunk(P, P.graphs[0], m, k0, [&]() {
        for (int k = k0; k < k1; ++k) {
          const int r = arnoldi_step<double2>(P, P.V, P.w, k, m, prec, apply);
          if (r) return r;
        }
        return (int)WG_OK;
      });
      if (rc) return rc;
      WG_CK(cudaMemcpyAsync(P.h_active.data(), P.active, sizeof(int) * B, cudaMemcpyDeviceToHost, P.stream));
      WG_CK(cudaStreamSynchronize(P.stream));
      if (all_done(P.h_active)) break;
    }
    P.prof.launches[PROF_OTHER] += 3;
    backsolve_kernel<<<B, 32, 0, P.stream>>>(P.H, P.g, P.ycoef, nullptr, P.kused, ps, mm, B);
    combine_kernel<double2><<<blocks_for(tot), 256, 0, P.stream>>>(P.V, P.ycoef, P.kused, P.w, N, mp1, mm, B);
    WG_CK(launch_precondition(P, P.w, N, P.z));
    axpy_kernel<double2><<<blocks_for(tot), 256, 0, P.stream>>>(P.x, P.z, nullptr, N, B);
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
  if (P.fp64_tc && P.mx.err) {
    int herr = 0;
    WG_CK(cudaMemcpy(&herr, P.mx.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      P.err = "FP64 tensor-core GEMM: bounded barrier wait timed out";
      return WG_ERR_TIMEOUT;
    }
  }
  return solve_end(P, bnorm, tgt, initial, res, iters, cycles, refs, info);
}

// FP64 iterative refinement around one FP32/BF16 GMRES cycle per correction.
int gmres_solve_mixed(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info) {
  const int B = P.batch, m = P.restart_inner, mp1 = m + 1, ps = P.restart_max + 1, mm = P.restart_max;
  const long long N = P.N, tot = N * B;
  const double tol = o.tol > 0 ? o.tol : 1e-10;
  const int max_ref = o.maxit > 0 ? o.maxit : 50;
  MixedBuffers& M = P.mx;
  WG_CK(mixed_sync_weights(P));
  std::vector<double> bnorm, tgt, initial;
  int rc = solve_begin(P, tol, warm, bnorm, tgt, initial);
  if (rc) return rc;
  std::vector<int> iters(B, 0), cycles(B, 0), refs(B, 0);
  std::vector<double> res = initial, itgt(B), ones(B, 1.0);
  // the inner Arnoldi steps skip problems that have converged in this cycle (P.active)
  auto prec = [&](const float2* r, long long stride, const float* rscale, float2* rout) {
    return launch_precondition_mixed(P, r, stride, M.z, M.zb16, P.active, rscale, rout, (long long)mp1 * N);
  };
  auto prec_h = [&](const float2* r, long long stride, const float* rscale, __half2* rout) {
    return launch_precondition_mixed_h(P, r, stride, M.z, M.zb16, P.active, rscale, rout, (long long)mp1 * N);
  };
  auto apply = [&]() { return launch_apply_mixed(P, M.z, M.zb16, M.w, P.active); };
  for (int ref = 0; ref < max_ref; ++ref) {
    bool any = false;
    for (int b = 0; b < B; ++b) any |= (res[b] > tgt[b]) && std::isfinite(res[b]);
    if (!any) break;
    // inner target on the normalised residual: reach the outer target, never below inner_tol
    P.h_res_mask.assign(B, 0);
    for (int b = 0; b < B; ++b) {
      const bool act = (res[b] > tgt[b]) && std::isfinite(res[b]);
      itgt[b] = act ? std::max(P.inner_tol, 0.5 * tgt[b] / res[b]) : INFINITY;
      P.h_res_mask[b] = act ? 1 : 0;
    }
    WG_CK(cudaMemcpyAsync(P.target, itgt.data(), sizeof(double) * B, cudaMemcpyHostToDevice, P.stream));
    WG_CK(cudaMemcpyAsync(P.res_mask, P.h_res_mask.data(), sizeof(int) * B, cudaMemcpyHostToDevice, P.stream));
    // keep |r| for the update, start the inner cycle from the unit-norm residual
    WG_CK(cudaMemcpyAsync(P.nrm_keep, P.nrm, sizeof(double) * B, cudaMemcpyDeviceToDevice, P.stream));
    WG_CK(cudaMemcpyAsync(P.nrm, ones.data(), sizeof(double) * B, cudaMemcpyHostToDevice, P.stream));
    P.prof.launches[PROF_OTHER] += 2;
    cycle_init_kernel<<<(B + 127) / 128, 128, 0, P.stream>>>(P.nrm, P.target, P.g, P.active, P.kused, ps, B);
    // V_0 = r / |r| (an FP16 basis: in FP32 in w, stored by the first step's preconditioner)
    if (M.basis16)
      scale_kernel<double2, float2><<<blocks_for(tot), 256, 0, P.stream>>>(P.r, M.w, P.inv64, P.active, N, N, B);
    else
      scale_kernel<double2, float2><<<blocks_for(tot), 256, 0, P.stream>>>(P.r, M.V, P.inv64, P.active, N,
                                                                          (long long)mp1 * N, B);
    for (int k0 = 0; k0 < m; k0 = chunk_end(k0, m)) {
      const int k1 = chunk_end(k0, m);
      rc = run_arnoldi_chunk(P, P.graphs[1], m, k0, [&]() {
        for (int k = k0; k < k1; ++k) {
          const int r = M.basis16 ? arnoldi_step<float2, __half2>(P, M.Vh, M.w, k, m, prec_h, apply)
                                  : arnoldi_step<float2>(P, M.V, M.w, k, m, prec, apply);
          if (r) return r;
        }
        return (int)WG_OK;
      });
      if (rc) return rc;
      WG_CK(cudaMemcpyAsync(P.h_active.data(), P.active, sizeof(int) * B, cudaMemcpyDeviceToHost, P.stream));
      WG_CK(cudaStreamSynchronize(P.stream));
      if (all_done(P.h_active)) break;
    }
    // d = M^-1 (V y) in FP32, x += |r| d in FP64
    P.prof.launches[PROF_OTHER] += 3;
    backsolve_kernel<<<B, 32, 0, P.stream>>>(P.H, P.g, P.ycoef, M.y, P.kused, ps, mm, B);
    if (M.basis16)
      combine_kernel<float2, __half2><<<blocks_for(tot), 256, 0, P.stream>>>(M.Vh, M.y, P.kused, M.w, N, mp1, mm, B);
    else
      combine_kernel<float2><<<blocks_for(tot), 256, 0, P.stream>>>(M.V, M.y, P.kused, M.w, N, mp1, mm, B);
    WG_CK(launch_precondition_mixed(P, M.w, N, M.d, nullptr, P.res_mask));
    axpy_kernel<float2><<<blocks_for(tot), 256, 0, P.stream>>>(P.x, M.d, P.nrm_keep, N, B, P.res_mask);
    WG_CK(cudaGetLastError());
    // problems that did not move this refinement keep r and |r|; the others are re-evaluated
    WG_CK(cudaMemcpyAsync(P.nrm, P.nrm_keep, sizeof(double) * B, cudaMemcpyDeviceToDevice, P.stream));
    rc = true_residual(P, P.res_mask, residual_digits(P, tol, &P.h_res_mask), residual_digits_pp(P, tol));
    if (rc) return rc;
    int herr = 0;
    WG_CK(cudaMemcpyAsync(&herr, M.err, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
    WG_CK(cudaMemcpyAsync(P.h_kused.data(), P.kused, sizeof(int) * B, cudaMemcpyDeviceToHost, P.stream));
    WG_CK(cudaMemcpyAsync(res.data(), P.nrm, sizeof(double) * B, cudaMemcpyDeviceToHost, P.stream));
    WG_CK(cudaStreamSynchronize(P.stream));
    if (herr) {
      P.err = "tensor-core GEMM: bounded barrier wait timed out";
      return WG_ERR_TIMEOUT;
    }
    for (int b = 0; b < B; ++b) {
      iters[b] += P.h_kused[b];
      if (P.h_kused[b] > 0) {
        cycles[b] += 1;
        refs[b] += 1;
      }
    }
  }
  WG_CK(cudaMemcpyAsync(P.target, tgt.data(), sizeof(double) * B, cudaMemcpyHostToDevice, P.stream));
  WG_CK(cudaStreamSynchronize(P.stream));
  return solve_end(P, bnorm, tgt, initial, res, iters, cycles, refs, info);
}

int solve_dispatch(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info) {
  if (!P.tuned) {
    const int rt = autotune(P);
    if (rt) return rt;
  }
  if (P.precision == WG_PREC_MIXED) return gmres_solve_mixed(P, o, warm, info);
  return gmres_solve_fp64(P, o, warm, info);
}

}  // namespace wg
