// Mixed-precision operator of the 1D Wigner solve (sm_103a).
//
// The complex plane-wave transforms become real BF16 GEMMs on the tensor cores:
// with real and imaginary parts interleaved along K and M, a complex coefficient
// c = a + ib acts as the 2x2 block [[a, -b], [b, a]], so the interleaved complex
// state (column-major, Nk complex per DG node) IS the K-major B operand and the
// FP32 accumulator, stored column-major, IS the interleaved complex result.
//   GEMM 1: X^ (2 N_xi x ncols) = Phi'      (2 N_xi x 2 Nk) * x (2 Nk x ncols)
//   GEMM 2: y  (2 Nk x ncols)  += (i Phi^H)' (2 Nk x 2 N_xi) * Y^ (2 N_xi x ncols)
// The flux, the xi stencil and the k-line preconditioner run in FP32; the stencil
// and the preconditioner write the BF16 GEMM operands directly.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "kline.cuh"
#include "ozaki.cuh"
#include "problem.h"
#include "ozaki_api.h"
#include "tc_gemm.cuh"

namespace wg {

namespace {

using bf16 = __nv_bfloat16;
using bf162 = __nv_bfloat162;

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  // initialised once, thread-safe (handles may be created from several host threads)
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeTiledFn>(p);
    return nullptr;
  }();
  return fn;
}

// K-major bf16 operand of `rows` rows and K columns, 64 x box_rows boxes, 128-byte swizzle.
bool make_map(CUtensorMap* m, const void* base, long long rows, int K, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// bf16 digit stack [S][rows][K] (K-major), BK x box_rows x 1 boxes (64-byte rows), 64-byte swizzle.
bool make_map3(CUtensorMap* m, const void* base, long long rows, int K, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)oz::S};
  cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * (cuuint64_t)rows};
  cuuint32_t box[3] = {(cuuint32_t)oz::BK, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Digits of the rows of a row-major M x K FP64 matrix (host), the split of
// slice_columns_kernel: row r with max|a| < 2^m has F = round(a 2^(6S-1-m)) written
// in balanced base-64 digits, a = 2^e[r] sum_p t_p 2^(-6(p+1)), e[r] = m + 1.
void slice_rows_host(const std::vector<double>& A, int M, int K, std::vector<bf16>& dig, std::vector<int>& e) {
  dig.assign((size_t)oz::S * M * K, __float2bfloat16(0.f));
  e.assign(M, 0);
  for (int r = 0; r < M; ++r) {
    double mx = 0;
    for (int k = 0; k < K; ++k) mx = std::max(mx, std::fabs(A[(size_t)r * K + k]));
    if (mx == 0) continue;
    int m;
    std::frexp(mx, &m);   // mx = f 2^m, 0.5 <= f < 1
    e[r] = m + 1;
    for (int k = 0; k < K; ++k) {
      const double a = A[(size_t)r * K + k];
      // |a| 2^(6S-1-m) < 2^47: adding one half is exact
      long long F = (long long)std::floor(std::ldexp(std::fabs(a), oz::BETA * oz::S - 1 - m) + 0.5);
      if (a < 0) F = -F;
      for (int p = oz::S - 1; p > 0; --p) {
        const long long d = ((F + 32) & 63) - 32;
        dig[((size_t)p * M + r) * K + k] = __float2bfloat16((float)d);
        F = (F - d) >> oz::BETA;
      }
      dig[(size_t)r * K + k] = __float2bfloat16((float)F);
    }
  }
}

unsigned slice_blocks(long long ncol) {
  return (unsigned)((ncol + oz::kSliceColsPerBlock - 1) / oz::kSliceColsPerBlock);
}

template <int EPI>
cudaError_t launch_ozaki(const CUtensorMap& a, const CUtensorMap& b, const int* ea, const int* eb, double* C, int M,
                         long long Ncol, int K, int* err, cudaStream_t st, const int* mask = nullptr,
                         int cols_per_problem = 1, int nd = oz::S, const int* nd_pp = nullptr) {
  static const cudaError_t attr = cudaFuncSetAttribute(oz::gemm_ozaki_kernel<EPI>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, oz::SMEM_BYTES);
  if (attr != cudaSuccess) return attr;
  if (nd < 1 || nd > oz::S) return cudaErrorInvalidValue;
  dim3 grid((M + oz::BM - 1) / oz::BM, (unsigned)((Ncol + oz::BN - 1) / oz::BN));
  oz::gemm_ozaki_kernel<EPI><<<grid, oz::THREADS, oz::SMEM_BYTES, st>>>(a, b, ea, eb, C, M, Ncol, K, err, mask,
                                                                 cols_per_problem, nd, nd_pp);
  return cudaGetLastError();
}

// GEMM 1 with the xi stencil in its epilogue (tc::gemm_stencil_kernel): yh16 from x (BF16 via tmB).
template <int NK>
cudaError_t launch_gemm_stencil(Problem& P, const CUtensorMap& tmB, const int* mask) {
  MixedBuffers& M = P.mx;
  const Shape& s = P.s;
  static const cudaError_t attr = cudaFuncSetAttribute(tc::gemm_stencil_kernel<NK>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       tc::ST_SMEM_BYTES);
  if (attr != cudaSuccess) return attr;
  constexpr int EPT = tc::BN2 / NK;
  const long long nel = (long long)P.batch * s.n_el;
  const unsigned grid = (unsigned)((nel + EPT - 1) / EPT);
  tc::gemm_stencil_kernel<NK><<<grid, tc::ST_THREADS, tc::ST_SMEM_BYTES, P.stream>>>(
      M.tmA1, tmB, M.yh16, M.beta, M.betai, s.nxi, M.ne4, nel, s.n_el, 2 * s.nk, M.err, mask);
  return cudaGetLastError();
}

// GEMM 2 with the FP32 flux in its epilogue: y = i Phi^H Y^ + flux(x).
template <int NK>
cudaError_t launch_gemm_flux(Problem& P, const float2* x, float2* y, const int* mask) {
  MixedBuffers& M = P.mx;
  const Shape& s = P.s;
  static const cudaError_t attr = cudaFuncSetAttribute(tc::gemm_bf16_kernel<2, NK, 256>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
  if (attr != cudaSuccess) return attr;
  tc::FluxEpi ep{};
  ep.x = reinterpret_cast<const float*>(x);
  ep.kvec = M.kvec;
  ep.qd = M.qd;
  for (int i = 0; i < NK * NK; ++i) {
    ep.kp[i] = M.fb.Kp[i];
    ep.km[i] = M.fb.Km[i];
  }
  for (int a = 0; a < NK; ++a) {
    ep.k3c[a] = M.fb.K3c[a];
    ep.k5c[a] = M.fb.K5c[a];
  }
  ep.n_el = s.n_el;
  ep.shift = (float)P.shift;
  const int Mr = 2 * s.nk;
  dim3 grid((Mr + tc::BM - 1) / tc::BM, (unsigned)((P.ncols + tc::BN - 1) / tc::BN));
  tc::gemm_bf16_kernel<2, NK, 256><<<grid, 256, tc::SMEM_BYTES, P.stream>>>(
      M.tmA2, M.tmB2, reinterpret_cast<float*>(y), Mr, P.ncols, 2 * s.nxi, M.err, mask, s.n_el * NK, ep);
  return cudaGetLastError();
}

template <int EPI>
cudaError_t launch_gemm(const CUtensorMap& a, const CUtensorMap& b, float* D, int M, long long Ncol, int K, int* err,
                        cudaStream_t st, const int* mask = nullptr, int cols_per_problem = 1) {
  static const cudaError_t attr = cudaFuncSetAttribute(tc::gemm_bf16_kernel<EPI>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
  if (attr != cudaSuccess) return attr;
  dim3 grid((M + tc::BM - 1) / tc::BM, (unsigned)((Ncol + tc::BN - 1) / tc::BN));
  tc::gemm_bf16_kernel<EPI><<<grid, 128, tc::SMEM_BYTES, st>>>(a, b, D, M, Ncol, K, err, mask, cols_per_problem);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP32 upwind flux (the FP64 flux_kernel in single precision), two k per thread
// with 16-byte loads and stores.  Grid (batch * n_el, ceil(nk / 256)).  k changes
// sign only between j = nk/2 - 1 and nk/2, so for nk % 4 == 0 (required by the
// mixed form) both k of a pair share the upwind side.  xb (optional) receives x in
// BF16, the B operand of the following GEMM, so no separate conversion pass is needed.
// ---------------------------------------------------------------------------
constexpr int kFlux32Threads = 128;

template <int NK>
__global__ void __launch_bounds__(kFlux32Threads) flux32_kernel(const float2* __restrict__ x, float2* __restrict__ y,
                                                                bf162* __restrict__ xb,
                                                                const float* __restrict__ kvec,
                                                                const float* __restrict__ qd, FluxBlocks32 fb,
                                                                int n_el, int nk, float shift,
                                                                const int* __restrict__ mask) {
  const int be = blockIdx.x;
  const int j = 2 * (blockIdx.y * kFlux32Threads + threadIdx.x);
  if (j >= nk) return;
  const int b = be / n_el;
  if (mask && !mask[b]) return;
  const int e = be - b * n_el;
  const float k0 = kvec[j], k1 = kvec[j + 1];
  const float s = qd[b];
  const long long base = (long long)be * NK * nk + j;
  float4 xv[NK];
#pragma unroll
  for (int c = 0; c < NK; ++c) xv[c] = *reinterpret_cast<const float4*>(x + base + (long long)c * nk);
  if (xb) {
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      bf162 lo = __floats2bfloat162_rn(xv[c].x, xv[c].y), hi = __floats2bfloat162_rn(xv[c].z, xv[c].w);
      uint2 pk;
      pk.x = *reinterpret_cast<uint32_t*>(&lo);
      pk.y = *reinterpret_cast<uint32_t*>(&hi);
      *reinterpret_cast<uint2*>(xb + base + (long long)c * nk) = pk;
    }
  }
  // k K1 + |k| K2 = k (K1 +- K2); the upwind neighbour enters through one node
  const bool pos = k0 > 0;
  float4 acc[NK];
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      const float m = pos ? fb.Kp[a * NK + c] : fb.Km[a * NK + c];
      v.x = fmaf(m, xv[c].x, v.x);
      v.y = fmaf(m, xv[c].y, v.y);
      v.z = fmaf(m, xv[c].z, v.z);
      v.w = fmaf(m, xv[c].w, v.w);
    }
    acc[a] = v;
  }
  const bool left = pos && e > 0, right = k0 < 0 && e < n_el - 1;
  if (left || right) {
    const float4 xp = *reinterpret_cast<const float4*>(
        x + base + (left ? -(long long)NK * nk + (long long)(NK - 1) * nk : (long long)NK * nk));
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      const float m = left ? fb.K3c[a] : fb.K5c[a];
      acc[a].x = fmaf(m, xp.x, acc[a].x);
      acc[a].y = fmaf(m, xp.y, acc[a].y);
      acc[a].z = fmaf(m, xp.z, acc[a].z);
      acc[a].w = fmaf(m, xp.w, acc[a].w);
    }
  }
  const float s0 = s * k0, s1 = s * k1;
#pragma unroll
  for (int a = 0; a < NK; ++a)
    *reinterpret_cast<float4*>(y + base + (long long)a * nk) =
        make_float4(fmaf(s0, acc[a].x, shift * xv[a].x), fmaf(s0, acc[a].y, shift * xv[a].y),
                    fmaf(s1, acc[a].z, shift * xv[a].z), fmaf(s1, acc[a].w, shift * xv[a].w));
}

// ---------------------------------------------------------------------------
// FP32 xi stencil, output as the BF16 B operand of GEMM 2:
//   y_a(s) = sum_c beta_ac(s) (x_c(s) + x_c(s-1)) + beta_ac(s+1) (x_c(s) + x_c(s+1)),
// beta = betar (symmetric in a, c: pairs a <= c stored) + i betai.  Each thread owns
// CELLS (2 or 4, picked per shape by the autotuner) consecutive xi cells: vector loads
// of x (16 bytes per two cells), of the weights (4 bytes per cell) and vector stores of
// the BF16 output; the cells s0-1 and s0+CELLS come from the neighbouring lanes.  Grid
// (batch * n_el, ceil(nxi / (64 CELLS))) of 64 threads; nxi % 4 == 0 (mixed form).
// ---------------------------------------------------------------------------
constexpr int kSt4Threads = 64;

__host__ __device__ constexpr int pair_count(int nk) { return nk * (nk + 1) / 2; }
// index of the pair (a, c), a <= c, in the order (0,0) (0,1) .. (0,nK-1) (1,1) ..
__host__ __device__ constexpr int pair_index(int nk, int a, int c) { return a * nk - a * (a - 1) / 2 + (c - a); }

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }

// CELLS consecutive floats (CELLS * 4 bytes aligned) into v[0..CELLS)
template <int CELLS>
__device__ __forceinline__ void ld_cells(const float* p, float* v) {
  if constexpr (CELLS == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x; v[1] = t.y;
  }
}

template <int NK, int CELLS>
__global__ void __launch_bounds__(kSt4Threads) stencil32_kernel(const float2* __restrict__ xh,
                                                                bf162* __restrict__ yh,
                                                                const float* __restrict__ betar,
                                                                const float* __restrict__ betai, int nxi, int ne4,
                                                                int n_el, const int* __restrict__ mask) {
  static_assert(CELLS == 2 || CELLS == 4, "two or four cells per thread");
  const int be = blockIdx.x;
  if (mask && !mask[be / n_el]) return;
  const int lane = threadIdx.x & 31;
  const int s0 = (blockIdx.y * kSt4Threads + threadIdx.x) * CELLS;
  const bool valid = s0 < nxi;                       // nxi % 4 == 0: then all CELLS cells are
  const bool edge = lane == 31 || s0 + CELLS >= nxi;  // s0 + CELLS not held by the next lane
  const float2* X = xh + (long long)be * NK * nxi;
  const float2 z2 = make_float2(0.f, 0.f);
  float2 sm[NK][CELLS], sp[NK][CELLS];
#pragma unroll
  for (int c = 0; c < NK; ++c) {
    float2 x[CELLS];
#pragma unroll
    for (int h = 0; h < CELLS / 2; ++h) {
      float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
      if (valid) t = *reinterpret_cast<const float4*>(X + c * nxi + s0 + 2 * h);
      x[2 * h] = make_float2(t.x, t.y);
      x[2 * h + 1] = make_float2(t.z, t.w);
    }
    float2 xm, xp;
    xm.x = __shfl_up_sync(0xffffffffu, x[CELLS - 1].x, 1);
    xm.y = __shfl_up_sync(0xffffffffu, x[CELLS - 1].y, 1);
    xp.x = __shfl_down_sync(0xffffffffu, x[0].x, 1);
    xp.y = __shfl_down_sync(0xffffffffu, x[0].y, 1);
    if (lane == 0) xm = (valid && s0 > 0) ? X[c * nxi + s0 - 1] : z2;
    if (edge) xp = (valid && s0 + CELLS < nxi) ? X[c * nxi + s0 + CELLS] : z2;
    if (s0 == 0) xm = z2;
#pragma unroll
    for (int j = 0; j < CELLS; ++j) {
      sm[c][j] = f2add(x[j], j == 0 ? xm : x[j - 1]);
      sp[c][j] = f2add(x[j], j == CELLS - 1 ? xp : x[j + 1]);
    }
  }
  const float* br = betar + (long long)be * pair_count(NK) * ne4;
  bf162* Y = yh + (long long)be * NK * nxi;
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    float vx[CELLS], vy[CELLS];
#pragma unroll
    for (int j = 0; j < CELLS; ++j) vx[j] = vy[j] = 0.f;
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      const float* rr = br + pair_index(NK, a < c ? a : c, a < c ? c : a) * ne4;
      const float* ri = betai + (a * NK + c) * ne4;
      float r0[CELLS], i0[CELLS];
#pragma unroll
      for (int j = 0; j < CELLS; ++j) r0[j] = i0[j] = 0.f;
      if (valid) {
        ld_cells<CELLS>(rr + s0, r0);
        ld_cells<CELLS>(ri + s0, i0);
      }
      // the weight of edge s0 + CELLS: the next lane's first, loaded at the warp's edge
      float rn = __shfl_down_sync(0xffffffffu, r0[0], 1), in = __shfl_down_sync(0xffffffffu, i0[0], 1);
      if (edge) {
        rn = valid ? rr[s0 + CELLS] : 0.f;
        in = valid ? ri[s0 + CELLS] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < CELLS; ++j) {
        const float b1r = j == CELLS - 1 ? rn : r0[j + 1], b1i = j == CELLS - 1 ? in : i0[j + 1];
        vx[j] += r0[j] * sm[c][j].x - i0[j] * sm[c][j].y + b1r * sp[c][j].x - b1i * sp[c][j].y;
        vy[j] += r0[j] * sm[c][j].y + i0[j] * sm[c][j].x + b1r * sp[c][j].y + b1i * sp[c][j].x;
      }
    }
    if (valid) {
      uint32_t o[CELLS];
#pragma unroll
      for (int j = 0; j < CELLS; ++j) {
        bf162 t = __floats2bfloat162_rn(vx[j], vy[j]);
        o[j] = *reinterpret_cast<uint32_t*>(&t);
      }
      if constexpr (CELLS == 4)
        *reinterpret_cast<uint4*>(Y + a * nxi + s0) = make_uint4(o[0], o[1], o[2], o[3]);
      else
        *reinterpret_cast<uint2*>(Y + a * nxi + s0) = make_uint2(o[0], o[1]);
    }
  }
}

template <int NK>
void launch_stencil32(Problem& P, const int* mask) {
  const Shape& s = P.s;
  MixedBuffers& M = P.mx;
  const int cells = P.st_cells == 2 ? 2 : 4;
  const dim3 grid((unsigned)(P.batch * s.n_el), (unsigned)((s.nxi + cells * kSt4Threads - 1) / (cells * kSt4Threads)));
  if (cells == 2)
    stencil32_kernel<NK, 2><<<grid, kSt4Threads, 0, P.stream>>>(reinterpret_cast<const float2*>(M.xh), M.yh16,
                                                                M.beta, M.betai, s.nxi, M.ne4, s.n_el, mask);
  else
    stencil32_kernel<NK, 4><<<grid, kSt4Threads, 0, P.stream>>>(reinterpret_cast<const float2*>(M.xh), M.yh16,
                                                                M.beta, M.betai, s.nxi, M.ne4, s.n_el, mask);
}

// FP32 packed copies of the potential weights: out[r][p][s] = beta[r][a*nK+c][s] for the
// pairs p = (a <= c) (npair = nK(nK+1)/2; npair = nK*nK with all = true copies every
// (a, c)), rows padded from ne to ne4 with zeros.
__global__ void pack_weights_kernel(const double* __restrict__ beta, float* __restrict__ out, long long nrows,
                                    int nk, int npair, bool all, int ne, int ne4) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows * npair * ne4) return;
  const int s = (int)(t % ne4);
  const long long rp = t / ne4;
  const int p = (int)(rp % npair);
  const long long r = rp / npair;
  int a = 0, c = p;
  if (all) {
    a = p / nk;
    c = p % nk;
  } else {
    int rem = p;
    while (rem >= nk - a) {
      rem -= nk - a;
      ++a;
    }
    c = a + rem;
  }
  out[t] = s < ne ? (float)beta[(r * nk * nk + a * nk + c) * ne + s] : 0.f;
}

__global__ void c2f_kernel(const double2* __restrict__ x, float2* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = make_float2((float)x[t].x, (float)x[t].y);
}

__global__ void f2c_kernel(const float2* __restrict__ x, double2* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = make_double2(x[t].x, x[t].y);
}

__global__ void d2f_kernel(const double* __restrict__ x, float* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = (float)x[t];
}

__global__ void to_bf16_kernel(const float4* __restrict__ x, uint2* __restrict__ xb, long long n2,
                               const int* __restrict__ mask, long long n2_per_problem) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n2 || (mask && !mask[t / n2_per_problem])) return;
  const float4 v = x[t];
  bf162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
  uint2 pk;
  pk.x = *reinterpret_cast<uint32_t*>(&lo);
  pk.y = *reinterpret_cast<uint32_t*>(&hi);
  xb[t] = pk;
}

template <int NK>
cudaError_t apply_mixed_nk(Problem& P, const float2* x, const bf162* xb, float2* y, const int* mask) {
  MixedBuffers& M = P.mx;
  if (xb && xb != M.xin16 && xb != M.zb16) return cudaErrorInvalidValue;
  const Shape& s = P.s;
  const long long BN = P.N * P.batch;
  if (M.fused) {
    // two launches: GEMM 1 + stencil (X^ stays in TMEM), GEMM 2 + flux (y written once)
    const double ncols = (double)P.ncols, nxi = s.nxi, nkd = s.nk;
    const double gemm_flops = 2.0 * (2 * nxi) * (2 * nkd) * ncols;
    if (!xb) {
      // the BF16 copy of x (the preconditioner writes it in the Arnoldi step)
      cudaEvent_t ev = prof_begin(P, PROF_FLUX, 1, 12.0 * BN, 0, mask);
      const long long n2 = BN / 2;
      to_bf16_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, P.stream>>>(
          reinterpret_cast<const float4*>(x), reinterpret_cast<uint2*>(M.xin16), n2, mask, P.N / 2);
      prof_end(P, PROF_FLUX, ev);
      xb = M.xin16;
    }
    cudaEvent_t ev = prof_begin(P, PROF_GEMM_STENCIL, 1,
                                4.0 * BN + 4.0 * nxi * ncols + 4.0 * P.batch * s.n_el * pair_count(NK) * M.ne4,
                                gemm_flops, mask);
    cudaError_t e = launch_gemm_stencil<NK>(P, xb == M.xin16 ? M.tmB1n : M.tmB1zn, mask);
    prof_end(P, PROF_GEMM_STENCIL, ev);
    if (e != cudaSuccess) return e;
    ev = prof_begin(P, PROF_GEMM_FLUX, 1, 4.0 * nxi * ncols + 16.0 * BN, gemm_flops, mask);
    e = launch_gemm_flux<NK>(P, x, y, mask);
    prof_end(P, PROF_GEMM_FLUX, ev);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  // without a BF16 copy of x the flux kernel writes one into xin16
  bf162* xb_out = xb ? nullptr : M.xin16;
  if (!xb) xb = M.xin16;
  const double ncols = (double)P.ncols, nxi = s.nxi, nkd = s.nk;
  const double gemm_flops = 2.0 * (2 * nxi) * (2 * nkd) * ncols;
  cudaEvent_t ev = prof_begin(P, PROF_FLUX, 1, (xb_out ? 20.0 : 16.0) * BN, 0, mask);
  const dim3 fgrid((unsigned)(P.batch * s.n_el), (unsigned)((s.nk / 2 + kFlux32Threads - 1) / kFlux32Threads));
  flux32_kernel<NK><<<fgrid, kFlux32Threads, 0, P.stream>>>(x, y, xb_out, M.kvec, M.qd, M.fb, s.n_el, s.nk,
                                                            (float)P.shift, mask);
  prof_end(P, PROF_FLUX, ev);
  ev = prof_begin(P, PROF_GEMM_BF16, 1, 4.0 * BN + 8.0 * nxi * ncols, gemm_flops, mask);
  // GEMM 1 reads its B operand through the tensor map of whichever bf16 buffer holds x
  const int cpp = s.n_el * s.nK;   // GEMM columns per problem
  cudaError_t e = launch_gemm<0>(M.tmA1, xb == M.xin16 ? M.tmB1 : M.tmB1z, reinterpret_cast<float*>(M.xh), 2 * s.nxi,
                                 P.ncols, 2 * s.nk, M.err, P.stream, mask, cpp);
  prof_end(P, PROF_GEMM_BF16, ev);
  if (e != cudaSuccess) return e;
  ev = prof_begin(P, PROF_STENCIL, 1, 12.0 * nxi * ncols + 4.0 * P.batch * s.n_el * pair_count(NK) * M.ne4, 0,
                  mask);
  launch_stencil32<NK>(P, mask);
  prof_end(P, PROF_STENCIL, ev);
  ev = prof_begin(P, PROF_GEMM_BF16, 1, 4.0 * nxi * ncols + 16.0 * BN, gemm_flops, mask);
  e = launch_gemm<1>(M.tmA2, M.tmB2, reinterpret_cast<float*>(y), 2 * s.nk, P.ncols, 2 * s.nxi, M.err, P.stream, mask,
                     cpp);
  prof_end(P, PROF_GEMM_BF16, ev);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <int NK, typename O>
cudaError_t precond_mixed_nk(Problem& P, const float2* r, long long r_stride, float2* z, bf162* zb, const int* mask,
                             const float* rscale, O* rout, long long rout_stride) {
  constexpr bool RH = std::is_same<O, __half2>::value;
  const int L = P.kline_L, nc = kline::chunk_count_for(P.s.n_el, L);
  const dim3 grid((P.s.nk + 31) / 32, (nc + kline::kChunksPerBlock - 1) / kline::kChunksPerBlock, P.batch);
  const dim3 block(32, kline::kChunksPerBlock);
  float* ma = static_cast<float*>(P.kmap_a);
  float2* ms = static_cast<float2*>(P.kmap_s);
  cudaEvent_t ev = prof_begin(P, PROF_PRECOND, 2,
                              ((zb ? 28.0 : 24.0) + (rout ? (double)sizeof(O) : 0.0)) * P.N * P.batch, 0, mask);
  kline::kline_maps_kernel<NK, float, RH><<<grid, block, 0, P.stream>>>(r, P.mx.kvec, P.mx.dinv, P.mx.h, P.mx.qd, ma,
                                                                        ms, P.s.n_el, P.s.nk, P.N, r_stride, L, nc,
                                                                        mask, rscale);
  kline::kline_apply_kernel<NK, float, O><<<grid, block, 0, P.stream>>>(r, z, zb, P.mx.kvec, P.mx.dinv, P.mx.h,
                                                                        P.mx.qd, ma, ms, P.s.n_el, P.s.nk, P.N,
                                                                        r_stride, L, nc, mask, rscale, rout,
                                                                        rout_stride);
  prof_end(P, PROF_PRECOND, ev);
  return cudaGetLastError();
}

}  // namespace

std::string mixed_check_shape(const Shape& s) {
  if (s.nk % 4 || s.nxi % 4) return "the mixed form needs Nk and N_xi divisible by 4 (16-byte TMA rows)";
  if (s.nk < 32 || s.nxi < 32) return "the mixed form needs Nk, N_xi >= 32 (one 64-wide BF16 K block)";
  return "";
}

double mixed_bytes(const Shape& s, int batch, int restart, bool basis16) {
  const double BN = (double)s.n_el * s.nK * s.nk * batch;
  const double ncols = (double)batch * s.n_el * s.nK;
  return 2.0 * 2 * (4.0 * s.nxi * s.nk) + 4.0 * BN + 8.0 * ncols * s.nxi + 4.0 * ncols * s.nxi +
         (basis16 ? 4.0 : 8.0) * BN * (restart + 1) + 8.0 * BN * 4 +
         4.0 * batch * s.n_el * pair_count(s.nK) * ((s.nxi + 4) & ~3);
}

int mixed_alloc(Problem& P) {
  MixedBuffers& M = P.mx;
  const Shape& s = P.s;
  const long long BN = P.N * P.batch;
  const int mp1 = P.restart_inner + 1;
  double bytes = 0;
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  auto alloc = [&](void** p, size_t n) { bytes += (double)n; A(cudaMalloc(p, n)); };
  alloc((void**)&M.phi1, sizeof(bf16) * 4 * (size_t)s.nxi * s.nk);
  alloc((void**)&M.phi2, sizeof(bf16) * 4 * (size_t)s.nxi * s.nk);
  alloc((void**)&M.xin16, sizeof(bf162) * BN);
  alloc((void**)&M.zb16, sizeof(bf162) * BN);
  alloc((void**)&M.yh16, sizeof(bf162) * (size_t)s.nxi * P.ncols);
  alloc((void**)&M.xh, sizeof(float2) * (size_t)s.nxi * P.ncols);
  M.basis16 = P.inner_basis16;
  if (M.basis16) alloc((void**)&M.Vh, sizeof(__half2) * BN * mp1);
  else alloc((void**)&M.V, sizeof(float2) * BN * mp1);
  alloc((void**)&M.w, sizeof(float2) * BN);
  alloc((void**)&M.z, sizeof(float2) * BN);
  alloc((void**)&M.r, sizeof(float2) * BN);
  alloc((void**)&M.d, sizeof(float2) * BN);
  M.ne4 = (s.nxi + 1 + 3) & ~3;
  alloc((void**)&M.beta, sizeof(float) * (size_t)P.batch * s.n_el * pair_count(s.nK) * M.ne4);
  alloc((void**)&M.betai, sizeof(float) * (size_t)s.nK * s.nK * M.ne4);
  alloc((void**)&M.err, sizeof(int));
  alloc((void**)&M.kvec, sizeof(float) * s.nk);
  alloc((void**)&M.qd, sizeof(float) * P.batch);
  alloc((void**)&M.dinv, sizeof(float) * (size_t)P.batch * s.nk * s.nK * s.nK);
  alloc((void**)&M.h, sizeof(float) * (size_t)P.batch * s.nk * s.nK);
  alloc((void**)&M.hcol, sizeof(float2) * (size_t)P.batch * (P.restart_max + 1));
  alloc((void**)&M.y, sizeof(float2) * (size_t)P.batch * P.restart_max);
  alloc((void**)&M.inv, sizeof(float) * P.batch);
  if (e != cudaSuccess) {
    P.err = std::string("mixed-precision buffers: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  if (!P.fb.single) {
    P.err = "the mixed form needs the single-node upwind coupling of the DG flux blocks";
    return WG_ERR_ARG;
  }
  M.fb.nK = s.nK;
  for (int i = 0; i < s.nK * s.nK; ++i) {
    M.fb.Kp[i] = (float)P.fb.Kp[i];
    M.fb.Km[i] = (float)P.fb.Km[i];
  }
  for (int a = 0; a < s.nK; ++a) {
    M.fb.K3c[a] = (float)P.fb.K3c[a];
    M.fb.K5c[a] = (float)P.fb.K5c[a];
  }
  P.device_bytes += bytes;
  cudaMemsetAsync(M.err, 0, sizeof(int), P.stream);
  // BF16 real embeddings of Phi (GEMM 1) and i Phi^H (GEMM 2), interleaved (re, im) along both axes
  const int nxi = s.nxi, nk = s.nk;
  std::vector<bf16> a1((size_t)4 * nxi * nk), a2((size_t)4 * nxi * nk);
  for (int si = 0; si < nxi; ++si)
    for (int j = 0; j < nk; ++j) {
      const double pr = s.phi[(size_t)si * nk + j].real(), pi = s.phi[(size_t)si * nk + j].imag();
      // GEMM 1 row 2s+o, column 2j+c: [[pr, -pi], [pi, pr]]
      const size_t K1 = 2 * (size_t)nk;
      a1[(2 * si + 0) * K1 + 2 * j + 0] = __float2bfloat16((float)pr);
      a1[(2 * si + 0) * K1 + 2 * j + 1] = __float2bfloat16((float)-pi);
      a1[(2 * si + 1) * K1 + 2 * j + 0] = __float2bfloat16((float)pi);
      a1[(2 * si + 1) * K1 + 2 * j + 1] = __float2bfloat16((float)pr);
      // GEMM 2: i conj(Phi(s,j)) = pi + i pr -> row 2j+o, column 2s+c: [[pi, -pr], [pr, pi]]
      const size_t K2 = 2 * (size_t)nxi;
      a2[(2 * j + 0) * K2 + 2 * si + 0] = __float2bfloat16((float)pi);
      a2[(2 * j + 0) * K2 + 2 * si + 1] = __float2bfloat16((float)-pr);
      a2[(2 * j + 1) * K2 + 2 * si + 0] = __float2bfloat16((float)pr);
      a2[(2 * j + 1) * K2 + 2 * si + 1] = __float2bfloat16((float)pi);
    }
  e = cudaMemcpyAsync(M.phi1, a1.data(), sizeof(bf16) * a1.size(), cudaMemcpyHostToDevice, P.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(M.phi2, a2.data(), sizeof(bf16) * a2.size(), cudaMemcpyHostToDevice, P.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);
  if (e != cudaSuccess) {
    P.err = std::string("mixed-precision set-up: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  bool ok = make_map(&M.tmA1, M.phi1, 2 * nxi, 2 * nk, tc::BM) && make_map(&M.tmB1, M.xin16, P.ncols, 2 * nk, tc::BN) &&
            make_map(&M.tmB1z, M.zb16, P.ncols, 2 * nk, tc::BN) && make_map(&M.tmA2, M.phi2, 2 * nk, 2 * nxi, tc::BM) &&
            make_map(&M.tmB2, M.yh16, P.ncols, 2 * nxi, tc::BN) &&
            make_map(&M.tmB1n, M.xin16, P.ncols, 2 * nk, tc::BN2) && make_map(&M.tmB1zn, M.zb16, P.ncols, 2 * nk, tc::BN2);
  // The two-launch fused apply (WG_FUSED_APPLY=1) keeps all 2 N_xi rows of a column tile in TMEM
  // (at most 8 accumulators) and reads whole 128-row tiles.  It is opt-in: on GB300 it measured
  // 130 us per C2 batch-16 apply against 90 us for the four-launch apply, whose stencil and flux
  // kernels hide their memory latency across thousands of resident warps while the fused
  // epilogues run after the tensor-core main loop with a few warps per SM.
  {
    const char* f = std::getenv("WG_FUSED_APPLY");
    M.fused = (f && f[0] == '1') && (2 * nxi) % tc::BM == 0 && 2 * nxi <= tc::BM * tc::ST_MAX_MT &&
              (2 * nk) % tc::BM == 0;
  }
  if (!ok) {
    P.err = "cuTensorMapEncodeTiled failed for the BF16 GEMM operands";
    return WG_ERR_CUDA;
  }
  // FP64 outer residual on the tensor cores when the grouped accumulation stays exact
  return ozaki_alloc(P);
}

int ozaki_alloc(Problem& P) {
  MixedBuffers& M = P.mx;
  const Shape& s = P.s;
  const int nk = s.nk, nxi = s.nxi;
  bool ok = true;
  if (!M.err) {
    if (cudaMalloc(&M.err, sizeof(int)) != cudaSuccess || cudaMemset(M.err, 0, sizeof(int)) != cudaSuccess) {
      P.err = "FP64 tensor-core buffers: error flag";
      return WG_ERR_CUDA;
    }
  }
  // exact grouped accumulation (K <= MAX_K) and 16-byte TMA rows of the digit slices
  M.ozaki = 2 * nk <= oz::MAX_K && 2 * nxi <= oz::MAX_K && nk % 4 == 0 && nxi % 4 == 0;
  if (M.ozaki) {
    const int kmax = 2 * std::max(nk, nxi);
    std::vector<double> A1((size_t)4 * nxi * nk), A2((size_t)4 * nxi * nk);
    for (int si = 0; si < nxi; ++si)
      for (int j = 0; j < nk; ++j) {
        const double pr = s.phi[(size_t)si * nk + j].real(), pi = s.phi[(size_t)si * nk + j].imag();
        const size_t K1 = 2 * (size_t)nk, K2 = 2 * (size_t)nxi;
        A1[(2 * si + 0) * K1 + 2 * j + 0] = pr;
        A1[(2 * si + 0) * K1 + 2 * j + 1] = -pi;
        A1[(2 * si + 1) * K1 + 2 * j + 0] = pi;
        A1[(2 * si + 1) * K1 + 2 * j + 1] = pr;
        A2[(2 * j + 0) * K2 + 2 * si + 0] = pi;
        A2[(2 * j + 0) * K2 + 2 * si + 1] = -pr;
        A2[(2 * j + 1) * K2 + 2 * si + 0] = pr;
        A2[(2 * j + 1) * K2 + 2 * si + 1] = pi;
      }
    std::vector<bf16> d1, d2;
    std::vector<int> e1, e2;
    slice_rows_host(A1, 2 * nxi, 2 * nk, d1, e1);
    slice_rows_host(A2, 2 * nk, 2 * nxi, d2, e2);
    cudaError_t ce = cudaSuccess;
    auto C2 = [&](cudaError_t r) { if (ce == cudaSuccess) ce = r; };
    C2(cudaMalloc(&M.oa1, sizeof(bf16) * d1.size()));
    C2(cudaMalloc(&M.oa2, sizeof(bf16) * d2.size()));
    C2(cudaMalloc(&M.ea1, sizeof(int) * e1.size()));
    C2(cudaMalloc(&M.ea2, sizeof(int) * e2.size()));
    C2(cudaMalloc(&M.ob, sizeof(bf16) * (size_t)oz::S * P.ncols * kmax));
    C2(cudaMalloc(&M.eb, sizeof(int) * (size_t)P.ncols));
    // columns of masked problems are not re-sliced: keep them finite from the start
    C2(cudaMemset(M.ob, 0, sizeof(bf16) * (size_t)oz::S * P.ncols * kmax));
    C2(cudaMemset(M.eb, 0, sizeof(int) * (size_t)P.ncols));
    C2(cudaMemcpy(M.oa1, d1.data(), sizeof(bf16) * d1.size(), cudaMemcpyHostToDevice));
    C2(cudaMemcpy(M.oa2, d2.data(), sizeof(bf16) * d2.size(), cudaMemcpyHostToDevice));
    C2(cudaMemcpy(M.ea1, e1.data(), sizeof(int) * e1.size(), cudaMemcpyHostToDevice));
    C2(cudaMemcpy(M.ea2, e2.data(), sizeof(int) * e2.size(), cudaMemcpyHostToDevice));
    if (ce != cudaSuccess) {
      P.err = std::string("FP64 tensor-core buffers: ") + cudaGetErrorString(ce);
      return ce == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
    }
    P.device_bytes += 2.0 * (d1.size() + d2.size()) + 4.0 * (e1.size() + e2.size()) +
                      2.0 * oz::S * P.ncols * kmax + 4.0 * P.ncols;
    ok = make_map3(&M.tmOA1, M.oa1, 2 * nxi, 2 * nk, oz::BM) && make_map3(&M.tmOA2, M.oa2, 2 * nk, 2 * nxi, oz::BM) &&
         make_map3(&M.tmOB1, M.ob, P.ncols, 2 * nk, oz::BN) && make_map3(&M.tmOB2, M.ob, P.ncols, 2 * nxi, oz::BN);
    if (!ok) {
      P.err = "cuTensorMapEncodeTiled failed for the FP64 tensor-core operands";
      return WG_ERR_CUDA;
    }
  }
  return WG_OK;
}

void mixed_free(Problem& P) {
  MixedBuffers& M = P.mx;
  void* ptrs[] = {M.phi1, M.phi2, M.xin16, M.zb16, M.yh16, M.xh, M.V, M.Vh, M.w, M.z, M.r, M.d, M.beta, M.betai,
                  M.err, M.kvec, M.qd, M.dinv, M.h, M.hcol, M.y, M.inv, M.oa1, M.oa2, M.ea1, M.ea2, M.ob, M.eb};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  M = MixedBuffers{};
}

// FP32 copies of the potential weights after every potential update.
cudaError_t mixed_sync_weights(Problem& P) {
  const Shape& s = P.s;
  const int ne = s.nxi + 1, ne4 = P.mx.ne4, np = pair_count(s.nK);
  const long long rows = (long long)P.batch * s.n_el;
  const long long nb = rows * np * ne4, ni = (long long)s.nK * s.nK * ne4;
  P.prof.launches[PROF_OTHER] += 6;
  pack_weights_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, P.stream>>>(P.beta, P.mx.beta, rows, s.nK, np, false,
                                                                          ne, ne4);
  pack_weights_kernel<<<(unsigned)((ni + 255) / 256), 256, 0, P.stream>>>(P.betai, P.mx.betai, 1, s.nK,
                                                                          s.nK * s.nK, true, ne, ne4);
  d2f_kernel<<<1, 256, 0, P.stream>>>(P.qd, P.mx.qd, P.batch);
  d2f_kernel<<<(unsigned)((s.nk + 255) / 256), 256, 0, P.stream>>>(P.kvec, P.mx.kvec, s.nk);
  const long long nd = (long long)P.batch * s.nk * s.nK * s.nK, nh = (long long)P.batch * s.nk * s.nK;
  d2f_kernel<<<(unsigned)((nd + 255) / 256), 256, 0, P.stream>>>(P.pre_dinv, P.mx.dinv, nd);
  d2f_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, P.stream>>>(P.pre_h, P.mx.h, nh);
  return cudaGetLastError();
}

cudaError_t launch_apply_mixed(Problem& P, const float2* x, const __nv_bfloat162* xb, float2* y, const int* mask) {
  switch (P.s.nK) {
    case 2: return apply_mixed_nk<2>(P, x, xb, y, mask);
    case 3: return apply_mixed_nk<3>(P, x, xb, y, mask);
    default: return apply_mixed_nk<4>(P, x, xb, y, mask);
  }
}

// y = A_lo x for FP64 device vectors (conversion, mixed apply, conversion back).
// n low-precision applies of the resident state (x in FP32 once, then M.z -> M.w repeatedly).
cudaError_t apply_mixed_repeat(Problem& P, const double2* x, int n_apply) {
  const long long n = P.N * P.batch;
  cudaError_t e = mixed_sync_weights(P);
  if (e != cudaSuccess) return e;
  c2f_kernel<<<(unsigned)((n + 255) / 256), 256, 0, P.stream>>>(x, P.mx.z, n);
  // the BF16 copy of the input once, as the preconditioner provides it in the Arnoldi step
  to_bf16_kernel<<<(unsigned)((n / 2 + 255) / 256), 256, 0, P.stream>>>(
      reinterpret_cast<const float4*>(P.mx.z), reinterpret_cast<uint2*>(P.mx.zb16), n / 2, nullptr, P.N / 2);
  for (int i = 0; i < n_apply && e == cudaSuccess; ++i) e = launch_apply_mixed(P, P.mx.z, P.mx.zb16, P.mx.w);
  return e;
}

cudaError_t apply_mixed_f64(Problem& P, const double2* x, double2* y) {
  const long long n = P.N * P.batch;
  cudaError_t e = mixed_sync_weights(P);
  if (e != cudaSuccess) return e;
  c2f_kernel<<<(unsigned)((n + 255) / 256), 256, 0, P.stream>>>(x, P.mx.z, n);
  e = launch_apply_mixed(P, P.mx.z, nullptr, P.mx.w);
  if (e != cudaSuccess) return e;
  f2c_kernel<<<(unsigned)((n + 255) / 256), 256, 0, P.stream>>>(P.mx.w, y, n);
  return cudaGetLastError();
}

cudaError_t launch_stencil_mixed(Problem& P) {
  switch (P.s.nK) {
    case 2: launch_stencil32<2>(P, nullptr); break;
    case 3: launch_stencil32<3>(P, nullptr); break;
    default: launch_stencil32<4>(P, nullptr); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_precondition_mixed(Problem& P, const float2* r, long long r_stride, float2* z,
                                      __nv_bfloat162* zb, const int* mask, const float* rscale, float2* rout,
                                      long long rout_stride) {
  switch (P.s.nK) {
    case 2: return precond_mixed_nk<2>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
    case 3: return precond_mixed_nk<3>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
    default: return precond_mixed_nk<4>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
  }
}

cudaError_t launch_precondition_mixed_h(Problem& P, const float2* r, long long r_stride, float2* z,
                                        __nv_bfloat162* zb, const int* mask, const float* rscale, __half2* rout,
                                        long long rout_stride) {
  switch (P.s.nK) {
    case 2: return precond_mixed_nk<2>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
    case 3: return precond_mixed_nk<3>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
    default: return precond_mixed_nk<4>(P, r, r_stride, z, zb, mask, rscale, rout, rout_stride);
  }
}

// One thread waits on an mbarrier that nothing arrives at: the bounded wait of the GEMM kernels
// must give up after `limit` polls, raise err and return.
__global__ void stuck_wait_kernel(int* err, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::mbar_wait_limit(&bar, 0, err, limit);
  }
}

int debug_wait_timeout(long long limit, std::string& err) {
  int* d = nullptr;
  int flag = 0;
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(int));
  if (e == cudaSuccess) {
    stuck_wait_kernel<<<1, 32>>>(d, limit);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&flag, d, sizeof(int), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    err = std::string("CUDA: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  if (flag) {
    err = "bounded barrier wait timed out";
    return WG_ERR_TIMEOUT;
  }
  return WG_OK;
}

// Stand-alone BF16 GEMM for diagnostics: C = bf16(A) bf16(B), A row-major M x K,
// B column-major K x N, C column-major M x N (fp32 host buffers).
int debug_gemm_bf16(const float* A, const float* B, float* C, int M, int N, int K, std::string& err) {
  if (M < 1 || N < 1 || K < 64 || K % 8) {
    err = "debug GEMM needs K >= 64 and K % 8 == 0";
    return WG_ERR_ARG;
  }
  std::vector<bf16> ha((size_t)M * K), hb((size_t)N * K);
  for (size_t i = 0; i < ha.size(); ++i) ha[i] = __float2bfloat16(A[i]);
  for (size_t i = 0; i < hb.size(); ++i) hb[i] = __float2bfloat16(B[i]);
  bf16 *da = nullptr, *db = nullptr;
  float* dc = nullptr;
  int* derr = nullptr;
  cudaError_t e = cudaMalloc(&da, ha.size() * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&db, hb.size() * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&dc, (size_t)M * N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(da, ha.data(), ha.size() * sizeof(bf16), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, hb.data(), hb.size() * sizeof(bf16), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dc, 0, (size_t)M * N * sizeof(float));
  CUtensorMap ma, mb;
  int rc = WG_OK;
  if (e == cudaSuccess) {
    if (!make_map(&ma, da, M, K, tc::BM) || !make_map(&mb, db, N, K, tc::BN)) {
      err = "cuTensorMapEncodeTiled failed";
      rc = WG_ERR_CUDA;
    } else {
      e = launch_gemm<0>(ma, mb, dc, M, N, K, derr, 0);
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      int herr = 0;
      if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(C, dc, (size_t)M * N * sizeof(float), cudaMemcpyDeviceToHost);
      if (herr) {
        err = "GEMM barrier wait timed out";
        rc = WG_ERR_TIMEOUT;
      }
    }
  }
  if (e != cudaSuccess) {
    err = std::string("CUDA: ") + cudaGetErrorString(e);
    rc = WG_ERR_CUDA;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dc);
  cudaFree(derr);
  return rc;
}

// FP64 operator apply of the mixed form's outer residual: flux and xi stencil in
// FP64, both transforms as digit-sliced FP64 GEMMs on the tensor cores.
cudaError_t launch_apply_f64_tc(Problem& P, const double2* x, double2* y, const int* mask, int nd,
                                const int* nd_pp) {
  MixedBuffers& M = P.mx;
  if (!M.ozaki) return launch_apply(P, x, y);
  const Shape& s = P.s;
  const int K1 = 2 * s.nk, K2 = 2 * s.nxi;
  const double ncols = (double)P.ncols;
  const int cpp = (int)(P.ncols / P.batch);   // columns (element, node) of one problem
  cudaError_t e = launch_flux_f64(P, x, y, mask);
  if (e != cudaSuccess) return e;
  // work of one GEMM: read the FP64 operand (slicing), write the FP64 result; flops of
  // ONE real-embedded BF16 digit-slice product, weighted by the products the digits need
  const double prod_flops = 2.0 * (2.0 * s.nxi) * (2.0 * s.nk) * ncols;
  cudaEvent_t ev = prof_begin(P, PROF_GEMM_F64TC, 2, 8.0 * P.N * P.batch + 16.0 * s.nxi * ncols, prod_flops, mask,
                              nd, nd_pp);
  oz::slice_columns_kernel<<<slice_blocks(P.ncols), 32 * oz::kSliceColsPerBlock, 0, P.stream>>>(
      reinterpret_cast<const double*>(x), K1, P.ncols, M.ob, M.eb, mask, cpp, 0, nd, nd_pp);
  e = launch_ozaki<0>(M.tmOA1, M.tmOB1, M.ea1, M.eb, reinterpret_cast<double*>(P.xh), K2, P.ncols, K1, M.err,
                      P.stream, mask, cpp, nd, nd_pp);
  prof_end(P, PROF_GEMM_F64TC, ev);
  if (e != cudaSuccess) return e;
  e = launch_stencil_f64(P, P.xh, P.yh, mask);
  if (e != cudaSuccess) return e;
  ev = prof_begin(P, PROF_GEMM_F64TC, 2, 16.0 * s.nxi * ncols + 16.0 * P.N * P.batch, prod_flops, mask, nd, nd_pp);
  oz::slice_columns_kernel<<<slice_blocks(P.ncols), 32 * oz::kSliceColsPerBlock, 0, P.stream>>>(
      reinterpret_cast<const double*>(P.yh), K2, P.ncols, M.ob, M.eb, mask, cpp, 0, nd, nd_pp);
  e = launch_ozaki<1>(M.tmOA2, M.tmOB2, M.ea2, M.eb, reinterpret_cast<double*>(y), K1, P.ncols, K2, M.err, P.stream,
                      mask, cpp, nd, nd_pp);
  prof_end(P, PROF_GEMM_F64TC, ev);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Stand-alone digit-sliced FP64 GEMM for diagnostics: C = A B with A row-major M x K,
// B column-major K x N, C column-major M x N (host FP64 buffers), K <= 1024, K % 8 == 0.
int debug_gemm_f64_tc(const double* A, const double* B, double* C, int M, int N, int K, std::string& err, int nd) {
  if (M < 1 || N < 1 || K < 64 || K % 8 || K > oz::MAX_K) {
    err = "debug FP64 GEMM needs 64 <= K <= 1024 and K % 8 == 0";
    return WG_ERR_ARG;
  }
  std::vector<double> a(A, A + (size_t)M * K);
  std::vector<bf16> da_h;
  std::vector<int> ea_h;
  slice_rows_host(a, M, K, da_h, ea_h);
  bf16 *da = nullptr, *db = nullptr;
  double *dB = nullptr, *dC = nullptr;
  int *dea = nullptr, *deb = nullptr, *derr = nullptr;
  cudaError_t e = cudaMalloc(&da, sizeof(bf16) * da_h.size());
  if (e == cudaSuccess) e = cudaMalloc(&db, sizeof(bf16) * (size_t)oz::S * N * K);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(double) * (size_t)N * K);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(double) * (size_t)M * N);
  if (e == cudaSuccess) e = cudaMalloc(&dea, sizeof(int) * M);
  if (e == cudaSuccess) e = cudaMalloc(&deb, sizeof(int) * N);
  if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(da, da_h.data(), sizeof(bf16) * da_h.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dea, ea_h.data(), sizeof(int) * M, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(double) * (size_t)N * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  int rc = WG_OK;
  if (e == cudaSuccess) {
    CUtensorMap ma, mb;
    if (!make_map3(&ma, da, M, K, oz::BM) || !make_map3(&mb, db, N, K, oz::BN)) {
      err = "cuTensorMapEncodeTiled failed";
      rc = WG_ERR_CUDA;
    } else {
      oz::slice_columns_kernel<<<slice_blocks(N), 32 * oz::kSliceColsPerBlock>>>(dB, K, N, db, deb);
      e = launch_ozaki<0>(ma, mb, dea, deb, dC, M, N, K, derr, 0, nullptr, 1, nd);
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      int herr = 0;
      if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(C, dC, sizeof(double) * (size_t)M * N, cudaMemcpyDeviceToHost);
      if (herr) {
        err = "FP64 tensor-core GEMM barrier wait timed out";
        rc = WG_ERR_TIMEOUT;
      }
    }
  }
  if (e != cudaSuccess) {
    err = std::string("CUDA: ") + cudaGetErrorString(e);
    rc = WG_ERR_CUDA;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dea);
  cudaFree(deb);
  cudaFree(derr);
  return rc;
}

// ---------------------------------------------------------------------------
// Emulated FP64 GEMM as a building block (ozaki_api.h).
// ---------------------------------------------------------------------------
int ozaki_rows_upload(const std::vector<double>& A, int M, int K, OzakiRowsDev& out, std::string& err) {
  if (M < 1 || K < 2 || K > oz::MAX_K || (int)A.size() != M * K) {
    err = "emulated GEMM: 1 <= M, 2 <= K <= 1024";
    return WG_ERR_ARG;
  }
  const int Kp = (K + 7) / 8 * 8;
  std::vector<double> Ap((size_t)M * Kp, 0.0);
  for (int r = 0; r < M; ++r)
    for (int k = 0; k < K; ++k) Ap[(size_t)r * Kp + k] = A[(size_t)r * K + k];
  std::vector<bf16> dig;
  std::vector<int> e;
  slice_rows_host(Ap, M, Kp, dig, e);
  cudaError_t ce = cudaMalloc(&out.dig, sizeof(bf16) * dig.size());
  if (ce == cudaSuccess) ce = cudaMalloc(&out.e, sizeof(int) * e.size());
  if (ce == cudaSuccess) ce = cudaMemcpy(out.dig, dig.data(), sizeof(bf16) * dig.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(out.e, e.data(), sizeof(int) * e.size(), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    err = std::string("emulated GEMM rows: ") + cudaGetErrorString(ce);
    ozaki_free(out);
    return ce == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  if (!make_map3(&out.map, out.dig, M, Kp, oz::BM)) {
    err = "emulated GEMM rows: tensor map";
    ozaki_free(out);
    return WG_ERR_CUDA;
  }
  out.M = M;
  out.K = K;
  out.Kp = Kp;
  return WG_OK;
}

int ozaki_cols_alloc(long long ncol, int K, OzakiColsDev& out, std::string& err) {
  const int Kp = (K + 7) / 8 * 8;
  cudaError_t ce = cudaMalloc(&out.dig, sizeof(bf16) * (size_t)oz::S * ncol * Kp);
  if (ce == cudaSuccess) ce = cudaMalloc(&out.e, sizeof(int) * (size_t)ncol);
  if (ce != cudaSuccess) {
    err = std::string("emulated GEMM columns: ") + cudaGetErrorString(ce);
    ozaki_free(out);
    return ce == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  if (!make_map3(&out.map, out.dig, ncol, Kp, oz::BN)) {
    err = "emulated GEMM columns: tensor map";
    ozaki_free(out);
    return WG_ERR_CUDA;
  }
  out.ncol = ncol;
  out.Kp = Kp;
  return WG_OK;
}

void ozaki_free(OzakiRowsDev& a) {
  cudaFree(a.dig);
  cudaFree(a.e);
  a = OzakiRowsDev{};
}

void ozaki_free(OzakiColsDev& b) {
  cudaFree(b.dig);
  cudaFree(b.e);
  b = OzakiColsDev{};
}

cudaError_t ozaki_accumulate(const OzakiRowsDev& A, OzakiColsDev& B, const double* X, double* C, int* err,
                             cudaStream_t st) {
  if (B.Kp != A.Kp) return cudaErrorInvalidValue;
  oz::slice_columns_kernel<<<slice_blocks(B.ncol), 32 * oz::kSliceColsPerBlock, 0, st>>>(X, A.K, B.ncol, B.dig, B.e,
                                                                                        nullptr, 1, B.Kp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_ozaki<1>(A.map, B.map, A.e, B.e, C, A.M, B.ncol, A.Kp, err, st);
}

cudaError_t ozaki_multiply(const OzakiRowsDev& A, OzakiColsDev& B, const double* X, double* C, int* err,
                           cudaStream_t st) {
  if (B.Kp != A.Kp) return cudaErrorInvalidValue;
  oz::slice_columns_kernel<<<slice_blocks(B.ncol), 32 * oz::kSliceColsPerBlock, 0, st>>>(X, A.K, B.ncol, B.dig, B.e,
                                                                                        nullptr, 1, B.Kp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_ozaki<0>(A.map, B.map, A.e, B.e, C, A.M, B.ncol, A.Kp, err, st);
}

}  // namespace wg
