// k-line preconditioner sweep, two kernels over (k line, element chunk, problem).
//
// In 1D the flux operator of wave number k is block-bidiagonal over the elements
// with an upwind coupling that touches one node of the neighbour element
// (get_LineTransversePreconditioner_full2D.m:174-239 reduced to one line per k):
//   z_e = D_b(k) r_e / qd_b - h_b(k) s_{e-1},   s_e = z_e[st]
// (st = the last local node for k > 0, sweeping e upwards; the first for k < 0,
// sweeping downwards).  The scalar recurrence s_e = a s_{e-1} + c_e is affine, so
// the elements are cut into chunks of L:
//   kline_maps_kernel   each (k, chunk) composes its chunk's map s -> A s + S from a
//                       zero start (one pass over the chunk's r);
//   kline_apply_kernel  each (k, chunk) folds the maps of the chunks upwind of it
//                       into its incoming s, then sweeps its chunk writing z.
// Threads: x = 32 consecutive k (coalesced rows), y = 4 chunks; grid
// (ceil(nk/32), ceil(n_chunks/4), batch) covers every SM even for one problem.
// Optional: r enters scaled by rscale[b] (the Arnoldi step's w / |w|), and the apply kernel
// writes the scaled r to rout (the next basis vector), which replaces a separate scaling pass.
// With an FP16 basis (rout of type __half2) both kernels round the scaled r to FP16 before
// they use it, so z is the preconditioned image of exactly the stored basis vector.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include <vector>

namespace wg {
namespace kline {

constexpr int kChunksPerBlock = 4;

template <typename R> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }

// r value as the basis stores it: unchanged, or rounded to FP16 (RH)
template <bool RH, typename T>
__device__ __forceinline__ T basis_round(T v) {
  if constexpr (RH) {
    const float2 f = __half22float2(__floats2half2_rn((float)v.x, (float)v.y));
    v.x = f.x;
    v.y = f.y;
  }
  return v;
}
__device__ __forceinline__ void basis_store(float2& d, float2 v) { d = v; }
__device__ __forceinline__ void basis_store(double2& d, double2 v) { d = v; }
__device__ __forceinline__ void basis_store(__half2& d, float2 v) { d = __floats2half2_rn(v.x, v.y); }

template <int NK, typename R, bool RH = false>
__global__ void __launch_bounds__(32 * kChunksPerBlock) kline_maps_kernel(
    const typename Cplx<R>::type* __restrict__ r, const R* __restrict__ kvec, const R* __restrict__ dinv,
    const R* __restrict__ hvec, const R* __restrict__ qd, R* __restrict__ mapA, typename Cplx<R>::type* __restrict__ mapS,
    int n_el, int nk, long long N, long long r_stride, int L, int nchunk, const int* __restrict__ mask,
    const R* __restrict__ rscale = nullptr) {
  using T = typename Cplx<R>::type;
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int c = blockIdx.y * kChunksPerBlock + threadIdx.y;
  const int b = blockIdx.z;
  if (j >= nk || c >= nchunk || (mask && !mask[b])) return;
  const long long bj = (long long)b * nk + j;
  const bool fwd = kvec[j] > R(0);
  const int st = fwd ? NK - 1 : 0;
  const R sc = rscale ? rscale[b] : R(1);   // r enters scaled (the basis vector w / |w|)
  R Dst[NK];
#pragma unroll
  for (int q = 0; q < NK; ++q) Dst[q] = dinv[bj * NK * NK + st * NK + q];
  const R alpha = -hvec[bj * NK + st];
  const R inv_qd = qd[b] > R(0) ? rcp(qd[b]) : R(0);   // a problem without data stays zero
  const int e_lo = c * L, e_hi = min(n_el, e_lo + L);
  const T* rb = r + (long long)b * r_stride + j;
  R A = R(1);
  T s;
  s.x = R(0);
  s.y = R(0);
  for (int i = 0; i < e_hi - e_lo; ++i) {
    const int e = fwd ? e_lo + i : e_hi - 1 - i;
    const T* re = rb + (long long)e * NK * nk;
    R ux = R(0), uy = R(0);
#pragma unroll
    for (int q = 0; q < NK; ++q) {
      T rv = re[(long long)q * nk];
      if constexpr (RH) {
        rv.x *= sc;
        rv.y *= sc;
        rv = basis_round<RH>(rv);
      }
      ux += Dst[q] * rv.x;
      uy += Dst[q] * rv.y;
    }
    const R scm = RH ? R(1) : sc;   // RH: the scale is already in rv
    s.x = ux * scm * inv_qd + alpha * s.x;
    s.y = uy * scm * inv_qd + alpha * s.y;
    A *= alpha;
  }
  const long long m = ((long long)b * nchunk + c) * nk + j;
  mapA[m] = A;
  mapS[m] = s;
}

template <int NK, typename R, typename O = typename Cplx<R>::type>
__global__ void __launch_bounds__(32 * kChunksPerBlock) kline_apply_kernel(
    const typename Cplx<R>::type* __restrict__ r, typename Cplx<R>::type* __restrict__ z,
    __nv_bfloat162* __restrict__ zb, const R* __restrict__ kvec, const R* __restrict__ dinv,
    const R* __restrict__ hvec, const R* __restrict__ qd, const R* __restrict__ mapA,
    const typename Cplx<R>::type* __restrict__ mapS, int n_el, int nk, long long N, long long r_stride, int L,
    int nchunk, const int* __restrict__ mask, const R* __restrict__ rscale = nullptr,
    O* __restrict__ rout = nullptr, long long rout_stride = 0) {
  using T = typename Cplx<R>::type;
  constexpr bool RH = std::is_same<O, __half2>::value;
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int c = blockIdx.y * kChunksPerBlock + threadIdx.y;
  const int b = blockIdx.z;
  if (j >= nk || c >= nchunk || (mask && !mask[b])) return;
  const long long bj = (long long)b * nk + j;
  const bool fwd = kvec[j] > R(0);
  const int st = fwd ? NK - 1 : 0;
  // incoming state: the maps of the chunks upwind of c, in sweep order
  T s;
  s.x = R(0);
  s.y = R(0);
  const long long mb = (long long)b * nchunk * nk + j;
  if (fwd) {
#pragma unroll 4
    for (int cc = 0; cc < c; ++cc) {
      const R a = mapA[mb + (long long)cc * nk];
      const T v = mapS[mb + (long long)cc * nk];
      s.x = a * s.x + v.x;
      s.y = a * s.y + v.y;
    }
  } else {
#pragma unroll 4
    for (int cc = nchunk - 1; cc > c; --cc) {
      const R a = mapA[mb + (long long)cc * nk];
      const T v = mapS[mb + (long long)cc * nk];
      s.x = a * s.x + v.x;
      s.y = a * s.y + v.y;
    }
  }
  R D[NK * NK], h[NK];
#pragma unroll
  for (int q = 0; q < NK * NK; ++q) D[q] = dinv[bj * NK * NK + q];
#pragma unroll
  for (int q = 0; q < NK; ++q) h[q] = hvec[bj * NK + q];
  const R inv_qd = qd[b] > R(0) ? rcp(qd[b]) : R(0);
  const R sc = rscale ? rscale[b] : R(1);
  const int e_lo = c * L, e_hi = min(n_el, e_lo + L);
  const T* rb = r + (long long)b * r_stride + j;
  T* zbase = z + (long long)b * N + j;
  O* obase = rout ? rout + (long long)b * rout_stride + j : nullptr;
  for (int i = 0; i < e_hi - e_lo; ++i) {
    const int e = fwd ? e_lo + i : e_hi - 1 - i;
    const T* re = rb + (long long)e * NK * nk;
    T rv[NK];
#pragma unroll
    for (int q = 0; q < NK; ++q) {
      rv[q] = re[(long long)q * nk];
      if (rscale) {
        rv[q].x *= sc;
        rv[q].y *= sc;
      }
      rv[q] = basis_round<RH>(rv[q]);
      // the scaled input is the next Krylov basis vector: written here, so no separate pass
      if (obase) basis_store(obase[(long long)e * NK * nk + (long long)q * nk], rv[q]);
    }
    T snew = s;
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      R ux = R(0), uy = R(0);
#pragma unroll
      for (int q = 0; q < NK; ++q) {
        ux += D[a * NK + q] * rv[q].x;
        uy += D[a * NK + q] * rv[q].y;
      }
      T zv;
      zv.x = ux * inv_qd - h[a] * s.x;
      zv.y = uy * inv_qd - h[a] * s.y;
      const long long o = (long long)e * NK * nk + (long long)a * nk;
      zbase[o] = zv;
      if (zb) zb[(long long)b * N + j + o] = __floats2bfloat162_rn((float)zv.x, (float)zv.y);
      if (a == st) snew = zv;
    }
    s = snew;
  }
}

// Elements per chunk L.  The default: about 32 chunks per line (the incoming-state fold
// costs one map read per upwind chunk), at least 4 elements each; the autotuner times
// the candidates below and keeps the fastest per shape.  At most kMaxChunks chunks (the
// map buffers are sized for that).
constexpr int kMaxChunks = 64;
inline int chunk_len(int n_el) { return n_el / 32 > 4 ? (n_el + 31) / 32 : 4; }
inline int chunk_count_for(int n_el, int L) { return (n_el + L - 1) / L; }
inline int chunk_count(int n_el) { return chunk_count_for(n_el, chunk_len(n_el)); }
inline std::vector<int> chunk_len_candidates(int n_el) {
  std::vector<int> out;
  int last = -1;
  for (int L : {2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128}) {
    if (L > n_el && !out.empty()) break;
    const int nc = chunk_count_for(n_el, L);
    if (nc > kMaxChunks || nc == last) continue;
    out.push_back(L);
    last = nc;
  }
  if (out.empty()) out.push_back(chunk_len(n_el));
  return out;
}

}  // namespace kline
}  // namespace wg
