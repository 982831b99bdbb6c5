// Full-2D (X, Y, rho_x, rho_y) matrix-free Wigner operator on the device (sm_103a).
//
// The device-resident apply of get_SysM_full2D.m:81,124-139 (sysInfo.makeGPUApply):
//   y = G_drift x + sum_parts c (R U) C^T
// with U the state reshaped [n_rel x n_center] (rho_x fastest, then rho_y, X, Y).
//
// Transport (get_Diff_full2D.m:618-639).  Every part of the reference's operator list
// acts on one centre axis and the matching relative axis only:
//   X parts: kron(I_Y, C_X) x kron(I_rho_y, R_x),   Y parts: kron(C_Y, I_X) x kron(R_y, I_rho_x),
// so an axis is a list of terms (c_t, C_t, R_t) with C_t block-tridiagonal over the DG
// elements (element blocks, wrapped on a periodic axis) and R_t a small CSR matrix on
// the FV cells (the central derivative, the dense characteristic |A|, ...).
//   f2d_center_kernel    G_t = F x_axis C_t for all terms (3 nk real MACs per entry);
//   f2d_relx_kernel      y += sum_t c_t R_t x_rho_x G_t: a column block of G_t staged in
//                        shared memory, each thread one rho_x row for 8 columns;
//   f2d_rely_kernel      the same along rho_y (rows of 12-40 cells: one thread per entry).
//
// Potential and CAP (applyFVConsistentDrift, get_Drift_full2D.m:331-364), per centre
// element e and quadrature point q:
//   f2d_interp_kernel    Uq[e][q][r] = sum_l W[q][l] U[r, id(e,l)]
//   f2d_vertex_kernel    Rq[e][q][cell] = sum over the cell's 4 vertices v of dV[e][q][v] x
//                        (sum of Uq over the <= 4 cells around v)   (P^T diag(dV) P)
//   f2d_project_kernel   y[r, id(e,l)] = pot/16 sum_q Cp[q][l] Rq[e][q][r] + capc cap[r] U[r, id(e,l)]
//   f2d_dv_kernel        dV from V on the material grid (bilinear, X clamped, Y clamped or wrapped).
// All arithmetic FP64 (the plain form).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "ozaki_api.h"
#include "wigner_gb300.h"

struct wg2d_problem {
  wg2d_shape s{};
  int nX = 0, nY = 0, nrx = 0, nry = 0, nrel = 0, ncen = 0, nel = 0, nloc = 0, nq = 0, nvert = 0;
  long long n = 0;
  cudaStream_t stream = nullptr;
  double2* x = nullptr;
  double2* y = nullptr;
  struct Axis {
    int T = 0;
    std::vector<double> coef;
    double* blocks = nullptr;   // [T][n_el][3][nk][nk]
    int* rp = nullptr;          // [T][n_rho + 1]
    int* col = nullptr;         // concatenated over the terms
    double2* val = nullptr;
    int* offs = nullptr;        // [T] start of term t in col / val
    double* dcoef = nullptr;    // [T]
    unsigned dense_mask = 0;    // terms applied by the emulated FP64 GEMM (rho_x axis)
    unsigned char* ymask = nullptr;   // rho_x axis: [T][nY] 1 where term t acts (closed X-face pieces); null: all
    std::vector<wg::OzakiRowsDev> dense;   // [T] digit slices of c_t R_t (real embedding) for those terms
  } ax[2];
  wg::OzakiColsDev cols;        // digit slices of the centre-applied state (rho_x columns)
  int* tc_err = nullptr;        // raised by a timed-out barrier wait of the emulated GEMM
  double2* G = nullptr;         // [Tmax][n] centre-applied state
  int g_terms = 0;
  // potential
  double *interp = nullptr, *proj = nullptr, *xq = nullptr, *yq = nullptr, *vx = nullptr, *vy = nullptr,
         *cap = nullptr, *dV = nullptr;
  double2 pot = {0, 0};
  double capc = 0;
  double2 *Uq = nullptr, *Rq = nullptr;
  bool drift_ready = false, potential_ready = false;
  cudaEvent_t ev[4] = {};
  // line-transverse preconditioner (modes of -i D_rho_x, X lines, dense transverse inverses)
  bool pre_ready = false;
  double sigma = 1.0;
  int nT = 0;
  wg::OzakiRowsDev UH, Us;        // real embeddings of U^H and U / sigma (tensor-core path)
  double2 *UHd = nullptr, *Usd = nullptr;   // the same as complex [nrx][nrx] row-major (FP64 path)
  double2 *xinv = nullptr, *xcpl = nullptr; // [nrx][n_el_x][nk][nk]
  double2* xmaps = nullptr;                  // chunk maps of the X-line sweep [chunk][nk*nk+nk][line]
  int x_chunk_len = 0, x_chunks = 1;
  int* fwd = nullptr;             // [nrx]
  double2* tinv = nullptr;        // [nrx][nT][nT]
  double2 *pa = nullptr, *pb = nullptr;     // [n] scratch of the preconditioner
  bool pre32 = false;             // the preconditioner in FP32 (its factors and scratch below)
  float2 *UH32 = nullptr, *Us32 = nullptr, *xinv32 = nullptr, *xcpl32 = nullptr, *tinv32 = nullptr;
  float2 *pa32 = nullptr, *pb32 = nullptr;
  // FP32 copies of the operator for the mixed solve's inner iterations
  bool d32_ready = false;
  float *blocks32[2] = {nullptr, nullptr}, *coef32[2] = {nullptr, nullptr};
  float2* val32[2] = {nullptr, nullptr};
  float *interp32 = nullptr, *proj32 = nullptr, *cap32 = nullptr, *dV32 = nullptr;
  float2 *Uq32 = nullptr, *Rq32 = nullptr, *G32 = nullptr;
  int vm32 = 0;
  float2 *V32 = nullptr, *Z32 = nullptr, *w32 = nullptr;
  __half2* Vh32 = nullptr;    // the inner basis stored in FP16 (V32 unused then)
  float2* vj32 = nullptr;     // FP32 copy of the current FP16 basis vector (the preconditioner's input)
  bool vbasis16 = false;      // the inner basis allocated in FP16
  // GMRES
  int vm = 0;                     // basis vectors allocated
  double2* Zb = nullptr;          // [m][n] preconditioned basis (flexible GMRES)
  double2 *V = nullptr, *r = nullptr, *w = nullptr, *z = nullptr, *b = nullptr, *xs = nullptr;
  double2 *H = nullptr, *g = nullptr, *sn = nullptr, *hc = nullptr, *hp = nullptr, *yc = nullptr;
  double *cs = nullptr, *partial = nullptr, *nrm = nullptr;
  double2 *bc_rt = nullptr, *bc_p = nullptr, *bc_ph = nullptr, *bc_sh = nullptr;   // BiCGSTAB vectors
  bool b_ready = false, xs_ready = false;   // resident right-hand side / solution of the last solve
  std::vector<double> resvec;               // residual norms of the last solve (initial, then per iteration)
  // observables at zero relative separation (get_Observables_full2D.m): the zero-cell weights and
  // derivative rows, the projection onto the material Y grid and the trapezoid weights over it
  wg2d_observables_desc obs{};
  bool obs_ready = false;
  double* obs_W = nullptr;    // [nty][nY]
  double* obs_wj = nullptr;   // [nty]
  double* obs_out = nullptr;  // nDG, jxDG, jyDG [nX][nY]; n, jx, jy [nX][nty]; j [nX]
  // hard-wall Y boundary (constrain_HardWall_full2D.m): active (rho_y cell, Y node) samples, the
  // exact-mass projection per (Y element, rho_y cell) and the weight of the constraint rows
  bool wall = false;
  double wall_scale = 0;
  unsigned char* wall_act = nullptr;   // [nY][nry]
  double* wall_T = nullptr;            // [n_el_y][nry][nk_y][nk_y] row-major
  float* wall_T32 = nullptr;
  double2* wall_u = nullptr;           // [n] masked input
  float2* wall_u32 = nullptr;
  std::string err;
};

namespace {

constexpr int kMaxNK = 4;
constexpr int kMaxTerms = 6;
constexpr int kRelxCols = 8;

__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {   // c + a b
  c.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
  c.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
  return c;
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  c.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x));
  c.y = fmaf(a.x, b.y, fmaf(a.y, b.x, c.y));
  return c;
}

template <typename T> __device__ __forceinline__ T czero();
template <> __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <> __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <typename T> __device__ __forceinline__ T cone();
template <> __device__ __forceinline__ double2 cone<double2>() { return make_double2(1.0, 0.0); }
template <> __device__ __forceinline__ float2 cone<float2>() { return make_float2(1.f, 0.f); }
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }

// G_t[r, X, Y] = sum_{e', b} C_t[e][dir][a][b] F[r, X'(e', b), Y] along X (axis 0) or Y (axis 1).
// grid (ceil(nrel/256), centre dofs of the other axis, n_el * nk of this axis).
template <int NK, typename T, typename R>
__global__ void __launch_bounds__(256) f2d_center_kernel(const T* __restrict__ F, T* __restrict__ G,
                                                         const R* __restrict__ blocks, int nterm, int axis,
                                                         int nrel, int nX, int nY, int n_el, int periodic,
                                                         long long n) {
  const int r = blockIdx.x * 256 + threadIdx.x;
  if (r >= nrel) return;
  const int other = blockIdx.y;        // Y dof (axis 0) or X dof (axis 1)
  const int d = blockIdx.z;            // dof along the axis = e * NK + a
  const int e = d / NK, a = d - e * NK;
  const int stride = axis == 0 ? nrel : nrel * nX;                     // between dofs of this axis
  const long long base = axis == 0 ? (long long)other * nX * nrel : (long long)other * nrel;
  T f[3][NK];
  bool has[3];
#pragma unroll
  for (int dir = 0; dir < 3; ++dir) {
    int en = e + dir - 1;
    has[dir] = true;
    if (en < 0 || en >= n_el) {
      if (periodic) en = (en + n_el) % n_el;
      else has[dir] = false;
    }
#pragma unroll
    for (int b = 0; b < NK; ++b)
      f[dir][b] = has[dir] ? F[base + (long long)(en * NK + b) * stride + r] : czero<T>();
  }
  const long long out = base + (long long)d * stride + r;
  for (int t = 0; t < nterm; ++t) {
    const R* B = blocks + ((long long)t * n_el + e) * 3 * NK * NK;
    T acc = czero<T>();
#pragma unroll
    for (int dir = 0; dir < 3; ++dir)
#pragma unroll
      for (int b = 0; b < NK; ++b) {
        const R c = B[(dir * NK + a) * NK + b];
        acc.x = fma(c, f[dir][b].x, acc.x);
        acc.y = fma(c, f[dir][b].y, acc.y);
      }
    G[(long long)t * n + out] = acc;
  }
}

// y[rx, col] += sum_t c_t sum_k val_t[k] G_t[col_t[k], col] for kRelxCols columns per block;
// the G_t columns are staged in shared memory, thread rx owns row rx (blockDim = nrx rounded
// up to a warp multiple, at most 512).
template <typename T, typename R>
__global__ void __launch_bounds__(512) f2d_relx_kernel(const T* __restrict__ G, T* __restrict__ y,
                                                       const int* __restrict__ rp, const int* __restrict__ col,
                                                       const T* __restrict__ val, const int* __restrict__ nnz_off,
                                                       const R* __restrict__ coef, int nterm, int nrx,
                                                       long long ncols, long long n, unsigned skip_mask,
                                                       const unsigned char* __restrict__ ymask = nullptr,
                                                       long long cols_per_y = 1, int nY = 1) {
  extern __shared__ __align__(16) unsigned char sgr_raw[];
  T* sg = reinterpret_cast<T*>(sgr_raw);   // [kRelxCols][nrx]
  const long long c0 = (long long)blockIdx.x * kRelxCols;
  const int nc = (int)min((long long)kRelxCols, ncols - c0);
  const int rx = threadIdx.x;
  T acc[kRelxCols];
#pragma unroll
  for (int j = 0; j < kRelxCols; ++j) acc[j] = czero<T>();
  for (int t = 0; t < nterm; ++t) {
    if ((skip_mask >> t) & 1u) continue;          // applied on the tensor cores
    __syncthreads();
    for (int i = threadIdx.x; i < kRelxCols * nrx; i += blockDim.x) {
      const int j = i / nrx, k = i - j * nrx;
      // a masked term (a closed X-face piece) acts only on its own Y dofs
      const bool on = j < nc && (!ymask || ymask[(long long)t * nY + (c0 + j) / cols_per_y]);
      sg[i] = on ? G[(long long)t * n + (c0 + j) * nrx + k] : czero<T>();
    }
    __syncthreads();
    if (rx < nrx) {
      const R ct = coef[t];
      const int* rpt = rp + t * (nrx + 1);
      const int off = nnz_off[t];
      for (int k = rpt[rx]; k < rpt[rx + 1]; ++k) {
        const int cidx = col[off + k];
        T v = val[off + k];
        v.x *= ct;
        v.y *= ct;
#pragma unroll
        for (int j = 0; j < kRelxCols; ++j) acc[j] = cfma(v, sg[j * nrx + cidx], acc[j]);
      }
    }
  }
  if (rx >= nrx) return;
#pragma unroll
  for (int j = 0; j < kRelxCols; ++j) {
    if (j < nc) {
      T* o = y + (c0 + j) * nrx + rx;
      o->x += acc[j].x;
      o->y += acc[j].y;
    }
  }
}

// y[rx, ry, c] += sum_t c_t sum_k val_t[k] G_t[rx, col_t[k], c]   (one thread per entry)
template <typename T, typename R>
__global__ void __launch_bounds__(256) f2d_rely_kernel(const T* __restrict__ G, T* __restrict__ y,
                                                       const int* __restrict__ rp, const int* __restrict__ col,
                                                       const T* __restrict__ val, const int* __restrict__ nnz_off,
                                                       const R* __restrict__ coef, int nterm, int nrx, int nry,
                                                       long long n) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const int rx = (int)(i % nrx);
  const long long q = i / nrx;
  const int ry = (int)(q % nry);
  const long long c = q / nry;
  const long long cbase = c * (long long)nrx * nry + rx;
  T acc = czero<T>();
  for (int t = 0; t < nterm; ++t) {
    const int* rpt = rp + t * (nry + 1);
    const int off = nnz_off[t];
    T s = czero<T>();
    for (int k = rpt[ry]; k < rpt[ry + 1]; ++k)
      s = cfma(val[off + k], G[(long long)t * n + cbase + (long long)col[off + k] * nrx], s);
    acc.x = fma(coef[t], s.x, acc.x);
    acc.y = fma(coef[t], s.y, acc.y);
  }
  y[i].x += acc.x;
  y[i].y += acc.y;
}

// centre dof of local node l of element e (local order X fastest, elements X fastest)
__device__ __forceinline__ long long center_id(int e, int l, int nex, int nkx, int nky, int nX) {
  const int ex = e % nex, ey = e / nex;
  const int lx = l % nkx, ly = l / nkx;
  return (long long)(ex * nkx + lx) + (long long)nX * (ey * nky + ly);
}

// Uq[e][q][r] = sum_l W[q][l] F[r, id(e, l)]; grid (ceil(nrel/128), n_el)
template <int NL, typename T, typename R>
__global__ void __launch_bounds__(128) f2d_interp_kernel(const T* __restrict__ F, T* __restrict__ Uq,
                                                         const R* __restrict__ W, int nq, int nrel, int nex,
                                                         int nkx, int nky, int nX) {
  const int r = blockIdx.x * 128 + threadIdx.x;
  const int e = blockIdx.y;
  if (r >= nrel) return;
  T u[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) u[l] = F[center_id(e, l, nex, nkx, nky, nX) * nrel + r];
  T* out = Uq + (long long)e * nq * nrel + r;
  for (int q = 0; q < nq; ++q) {
    T s = czero<T>();
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const R w = W[q * NL + l];
      s.x = fma(w, u[l].x, s.x);
      s.y = fma(w, u[l].y, s.y);
    }
    out[(long long)q * nrel] = s;
  }
}

// sum of Uq over the cells around relative vertex (vi, vj) (cells vi-1..vi, vj-1..vj)
template <typename T>
__device__ __forceinline__ T vertex_sum(const T* __restrict__ U, int vi, int vj, int nrx, int nry,
                                              bool periodic) {
  T s = czero<T>();
#pragma unroll
  for (int dj = -1; dj <= 0; ++dj) {
    int j = vj + dj;
    if (periodic) j = (j + nry) % nry;
    else if (j < 0 || j >= nry) continue;
#pragma unroll
    for (int di = -1; di <= 0; ++di) {
      const int i = vi + di;
      if (i < 0 || i >= nrx) continue;
      const T v = U[j * nrx + i];
      s.x += v.x;
      s.y += v.y;
    }
  }
  return s;
}

// Rq[e][q][cell] = sum_{vertices v of cell} dV[e][q][v] vertex_sum(v); grid (ceil(nrel/128), nq, n_el)
template <typename T, typename R>
__global__ void __launch_bounds__(128) f2d_vertex_kernel(const T* __restrict__ Uq, T* __restrict__ Rq,
                                                         const R* __restrict__ dV, int nrx, int nry, int nq,
                                                         int nvert, int periodic) {
  const int cell = blockIdx.x * 128 + threadIdx.x;
  const int nrel = nrx * nry;
  if (cell >= nrel) return;
  const int q = blockIdx.y, e = blockIdx.z;
  const long long slab = ((long long)e * nq + q);
  const T* U = Uq + slab * nrel;
  const R* D = dV + slab * nvert;
  const int i = cell % nrx, j = cell / nrx;
  const int nvx = nrx + 1;
  T acc = czero<T>();
#pragma unroll
  for (int b = 0; b <= 1; ++b) {
    int vj = j + b;
    if (periodic) vj %= nry;
#pragma unroll
    for (int a = 0; a <= 1; ++a) {
      const int vi = i + a;
      const R d = D[vj * nvx + vi];
      const T s = vertex_sum<T>(U, vi, vj, nrx, nry, periodic);
      acc.x = fma(d, s.x, acc.x);
      acc.y = fma(d, s.y, acc.y);
    }
  }
  Rq[slab * nrel + cell] = acc;
}

// y[r, id(e,l)] = pot/16 sum_q Cp[q][l] Rq[e][q][r] + capc cap[r] F[r, id(e,l)]; grid (ceil(nrel/128), n_el)
template <int NL, typename T, typename R>
__global__ void __launch_bounds__(128) f2d_project_kernel(const T* __restrict__ Rq, const T* __restrict__ F,
                                                          T* __restrict__ y, const R* __restrict__ Cp,
                                                          const R* __restrict__ cap, T pot16, R capc,
                                                          int nq, int nrel, int nex, int nkx, int nky, int nX) {
  const int r = blockIdx.x * 128 + threadIdx.x;
  const int e = blockIdx.y;
  if (r >= nrel) return;
  T s[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) s[l] = czero<T>();
  const T* Rr = Rq + (long long)e * nq * nrel + r;
  for (int q = 0; q < nq; ++q) {
    const T v = Rr[(long long)q * nrel];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const R c = Cp[q * NL + l];
      s[l].x = fma(c, v.x, s[l].x);
      s[l].y = fma(c, v.y, s[l].y);
    }
  }
  const R cr = capc * cap[r];
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    const long long idx = center_id(e, l, nex, nkx, nky, nX) * nrel + r;
    const T f = F[idx];
    T o;
    o.x = pot16.x * s[l].x - pot16.y * s[l].y + cr * f.x;
    o.y = pot16.x * s[l].y + pot16.y * s[l].x + cr * f.y;
    y[idx] = o;
  }
}

// interval i with g[i] <= v < g[i+1] on an ascending grid (v inside [g0, g_last])
__device__ __forceinline__ int grid_interval(const double* __restrict__ g, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (g[mid] <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ double v_bilinear(const double* __restrict__ gx, const double* __restrict__ gy,
                             const double* __restrict__ V, int nx, int ny, double qx, double qy, bool periodic) {
  qx = fmin(fmax(qx, gx[0]), gx[nx - 1]);
  if (periodic) {
    const double w = gy[ny - 1] - gy[0];
    qy = gy[0] + (qy - gy[0] - w * floor((qy - gy[0]) / w));
    if (qy > gy[ny - 1]) qy = gy[ny - 1];
  } else {
    qy = fmin(fmax(qy, gy[0]), gy[ny - 1]);
  }
  const int i = grid_interval(gx, nx, qx), j = grid_interval(gy, ny, qy);
  const double tx = (qx - gx[i]) / (gx[i + 1] - gx[i]);
  const double ty = (qy - gy[j]) / (gy[j + 1] - gy[j]);
  const double v00 = V[i + (long long)nx * j], v10 = V[i + 1 + (long long)nx * j];
  const double v01 = V[i + (long long)nx * (j + 1)], v11 = V[i + 1 + (long long)nx * (j + 1)];
  return (1 - tx) * (1 - ty) * v00 + tx * (1 - ty) * v10 + (1 - tx) * ty * v01 + tx * ty * v11;
}

// dV[e][q][v] = V(X_q + rho_v/2) - V(X_q - rho_v/2); grid (ceil(nvert/128), nq, n_el)
__global__ void __launch_bounds__(128) f2d_dv_kernel(double* __restrict__ dV, const double* __restrict__ xq,
                                                     const double* __restrict__ yq, const double* __restrict__ vx,
                                                     const double* __restrict__ vy, const double* __restrict__ gx,
                                                     const double* __restrict__ gy, const double* __restrict__ V,
                                                     int nx, int ny, int nq, int nvert, int periodic) {
  const int v = blockIdx.x * 128 + threadIdx.x;
  if (v >= nvert) return;
  const int q = blockIdx.y, e = blockIdx.z;
  const double X = xq[(long long)e * nq + q], Y = yq[(long long)e * nq + q];
  const double hx = 0.5 * vx[v], hy = 0.5 * vy[v];
  dV[((long long)e * nq + q) * nvert + v] = v_bilinear(gx, gy, V, nx, ny, X + hx, Y + hy, periodic) -
                                            v_bilinear(gx, gy, V, nx, ny, X - hx, Y - hy, periodic);
}

// out[rx, col] = scale sum_j A[rx][j] G[j, col]  (dense complex A [nrx][nrx] row-major; FP64 modal transforms)
template <typename T>
__global__ void __launch_bounds__(512) f2d_dense_rx_kernel(const T* __restrict__ A, const T* __restrict__ G,
                                                           T* __restrict__ out, int nrx, long long ncols) {
  extern __shared__ __align__(16) unsigned char sg_raw[];
  T* sg = reinterpret_cast<T*>(sg_raw);   // [kRelxCols][nrx]
  const long long c0 = (long long)blockIdx.x * kRelxCols;
  const int nc = (int)min((long long)kRelxCols, ncols - c0);
  for (int i = threadIdx.x; i < kRelxCols * nrx; i += blockDim.x) {
    const int j = i / nrx, k = i - j * nrx;
    sg[i] = j < nc ? G[(c0 + j) * nrx + k] : czero<T>();
  }
  __syncthreads();
  const int rx = threadIdx.x;
  if (rx >= nrx) return;
  T acc[kRelxCols];
#pragma unroll
  for (int j = 0; j < kRelxCols; ++j) acc[j] = czero<T>();
  const T* Ar = A + (long long)rx * nrx;
  for (int k = 0; k < nrx; ++k) {
    const T a = Ar[k];
#pragma unroll
    for (int j = 0; j < kRelxCols; ++j) acc[j] = cfma(a, sg[j * nrx + k], acc[j]);
  }
#pragma unroll
  for (int j = 0; j < kRelxCols; ++j)
    if (j < nc) out[(c0 + j) * nrx + rx] = acc[j];
}

// X lines per mode (xFactors / applyInverse of get_LineTransversePreconditioner_full2D.m:177-222):
// for mode k, transverse (ry, Y): sweep the X elements upwind (forward[k]: e = 0 .. ne-1), each
// element's nk values: prev = inv[k][e] (w_e - cpl[k][e] prev).  Thread per (k, ry, Y), k fastest.
template <int NK, typename T>
__global__ void __launch_bounds__(128) f2d_xline_kernel(const T* __restrict__ W, T* __restrict__ out,
                                                        const T* __restrict__ inv, const T* __restrict__ cpl,
                                                        const int* __restrict__ fwd, int nrx, int nry, int nX, int nY,
                                                        int ne) {
  const long long t = (long long)blockIdx.x * 128 + threadIdx.x;
  const long long lines = (long long)nrx * nry * nY;
  if (t >= lines) return;
  const int k = (int)(t % nrx);
  const long long q = t / nrx;
  const int ry = (int)(q % nry);
  const int Y = (int)(q / nry);
  const long long nrel = (long long)nrx * nry;
  const long long base = k + (long long)nrx * ry + nrel * (long long)nX * Y;
  const bool f = fwd[k] != 0;
  T prev[NK];
#pragma unroll
  for (int a = 0; a < NK; ++a) prev[a] = czero<T>();
  for (int i = 0; i < ne; ++i) {
    const int e = f ? i : ne - 1 - i;
    const T* Ci = cpl + ((long long)k * ne + e) * NK * NK;
    const T* Ii = inv + ((long long)k * ne + e) * NK * NK;
    T blk[NK];
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T v = W[base + nrel * (e * NK + a)];
#pragma unroll
      for (int b = 0; b < NK; ++b) {
        const T c = Ci[a * NK + b];
        v.x -= c.x * prev[b].x - c.y * prev[b].y;
        v.y -= c.x * prev[b].y + c.y * prev[b].x;
      }
      blk[a] = v;
    }
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T v = czero<T>();
#pragma unroll
      for (int b = 0; b < NK; ++b) v = cfma(Ii[a * NK + b], blk[b], v);
      prev[a] = v;
      out[base + nrel * (e * NK + a)] = v;
    }
  }
}

// The same sweep cut into chunks of L elements (sweep order).  The element recurrence is affine in
// the incoming state, prev_e = -Inv_e Cpl_e prev_{e-1} + Inv_e w_e, so a chunk composes to
// prev_out = M prev_in + b:
//   f2d_xline_maps_kernel   (line, chunk): M and b of the chunk from M = I, b = 0;
//   f2d_xline_apply_kernel  (line, chunk): the incoming state folded from the maps of the chunks
//                           upwind, then the chunk's elements swept as above, writing out.
// Threads (line, chunk) with the line fastest; maps stored [chunk][entry][line].
template <int NK, typename T>
__global__ void __launch_bounds__(128) f2d_xline_maps_kernel(const T* __restrict__ W, T* __restrict__ maps,
                                                             const T* __restrict__ inv, const T* __restrict__ cpl,
                                                             const int* __restrict__ fwd, int nrx, int nry, int nX,
                                                             int nY, int ne, int L, int nchunk) {
  const long long lines = (long long)nrx * nry * nY;
  const long long t = (long long)blockIdx.x * 128 + threadIdx.x;
  if (t >= lines * nchunk) return;
  const long long line = t % lines;
  const int c = (int)(t / lines);
  const int k = (int)(line % nrx);
  const long long q = line / nrx;
  const int ry = (int)(q % nry);
  const int Y = (int)(q / nry);
  const long long nrel = (long long)nrx * nry;
  const long long base = k + (long long)nrx * ry + nrel * (long long)nX * Y;
  const bool f = fwd[k] != 0;
  T M[NK][NK], b[NK];
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    b[a] = czero<T>();
#pragma unroll
    for (int j = 0; j < NK; ++j) M[a][j] = a == j ? cone<T>() : czero<T>();
  }
  const int i1 = min(ne, (c + 1) * L);
  for (int i = c * L; i < i1; ++i) {
    const int e = f ? i : ne - 1 - i;
    const T* Ci = cpl + ((long long)k * ne + e) * NK * NK;
    const T* Ii = inv + ((long long)k * ne + e) * NK * NK;
    T CM[NK][NK], r[NK];
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T v = W[base + nrel * (e * NK + a)];
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        T s = czero<T>();
#pragma unroll
        for (int m = 0; m < NK; ++m) s = cfma(Ci[a * NK + m], M[m][j], s);
        CM[a][j] = s;
      }
#pragma unroll
      for (int m = 0; m < NK; ++m) {
        const T cc = Ci[a * NK + m];
        v.x -= cc.x * b[m].x - cc.y * b[m].y;
        v.y -= cc.x * b[m].y + cc.y * b[m].x;
      }
      r[a] = v;
    }
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T bb = czero<T>();
#pragma unroll
      for (int m = 0; m < NK; ++m) bb = cfma(Ii[a * NK + m], r[m], bb);
      b[a] = bb;
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        T s = czero<T>();
#pragma unroll
        for (int m = 0; m < NK; ++m) s = cfma(Ii[a * NK + m], CM[m][j], s);
        M[a][j] = cneg(s);
      }
    }
  }
  T* o = maps + (long long)c * (NK * NK + NK) * lines + line;
#pragma unroll
  for (int a = 0; a < NK; ++a) {
#pragma unroll
    for (int j = 0; j < NK; ++j) o[(long long)(a * NK + j) * lines] = M[a][j];
    o[(long long)(NK * NK + a) * lines] = b[a];
  }
}

template <int NK, typename T>
__global__ void __launch_bounds__(128) f2d_xline_apply_kernel(const T* __restrict__ W, T* __restrict__ out,
                                                              const T* __restrict__ maps, const T* __restrict__ inv,
                                                              const T* __restrict__ cpl, const int* __restrict__ fwd,
                                                              int nrx, int nry, int nX, int nY, int ne, int L,
                                                              int nchunk) {
  const long long lines = (long long)nrx * nry * nY;
  const long long t = (long long)blockIdx.x * 128 + threadIdx.x;
  if (t >= lines * nchunk) return;
  const long long line = t % lines;
  const int c = (int)(t / lines);
  const int k = (int)(line % nrx);
  const long long q = line / nrx;
  const int ry = (int)(q % nry);
  const int Y = (int)(q / nry);
  const long long nrel = (long long)nrx * nry;
  const long long base = k + (long long)nrx * ry + nrel * (long long)nX * Y;
  const bool f = fwd[k] != 0;
  T prev[NK];
#pragma unroll
  for (int a = 0; a < NK; ++a) prev[a] = czero<T>();
  for (int cc = 0; cc < c; ++cc) {
    const T* o = maps + (long long)cc * (NK * NK + NK) * lines + line;
    T nxt[NK];
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T s = o[(long long)(NK * NK + a) * lines];
#pragma unroll
      for (int j = 0; j < NK; ++j) s = cfma(o[(long long)(a * NK + j) * lines], prev[j], s);
      nxt[a] = s;
    }
#pragma unroll
    for (int a = 0; a < NK; ++a) prev[a] = nxt[a];
  }
  const int i1 = min(ne, (c + 1) * L);
  for (int i = c * L; i < i1; ++i) {
    const int e = f ? i : ne - 1 - i;
    const T* Ci = cpl + ((long long)k * ne + e) * NK * NK;
    const T* Ii = inv + ((long long)k * ne + e) * NK * NK;
    T blk[NK];
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T v = W[base + nrel * (e * NK + a)];
#pragma unroll
      for (int m = 0; m < NK; ++m) {
        const T cc2 = Ci[a * NK + m];
        v.x -= cc2.x * prev[m].x - cc2.y * prev[m].y;
        v.y -= cc2.x * prev[m].y + cc2.y * prev[m].x;
      }
      blk[a] = v;
    }
#pragma unroll
    for (int a = 0; a < NK; ++a) {
      T v = czero<T>();
#pragma unroll
      for (int m = 0; m < NK; ++m) v = cfma(Ii[a * NK + m], blk[m], v);
      prev[a] = v;
      out[base + nrel * (e * NK + a)] = v;
    }
  }
}

constexpr int kTxTile = 32;
// transverse solve per mode k and X dof: v[k, t, X] <- Binv[k] v[k, :, X] over t = ry + nry Y.
// Block (k, tile of kTxTile X dofs); Binv[k] and the tile staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) f2d_transverse_kernel(const T* __restrict__ Vin, T* __restrict__ Vout,
                                                             const T* __restrict__ Binv, int nrx, int nry,
                                                             int nX, int nY, int nT) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* Bs = reinterpret_cast<T*>(sm_raw);   // [nT][nT] then [nT][kTxTile]
  T* Ts = Bs + (long long)nT * nT;
  const int k = blockIdx.y;
  const int X0 = blockIdx.x * kTxTile;
  const int nx = min(kTxTile, nX - X0);
  const long long nrel = (long long)nrx * nry;
  const T* Bk = Binv + (long long)k * nT * nT;
  for (int i = threadIdx.x; i < nT * nT; i += blockDim.x) Bs[i] = Bk[i];
  for (int i = threadIdx.x; i < nT * kTxTile; i += blockDim.x) {
    const int s = i / kTxTile, xx = i - s * kTxTile;
    const int ry = s % nry, Y = s / nry;
    Ts[i] = xx < nx ? Vin[k + (long long)nrx * ry + nrel * ((long long)(X0 + xx) + (long long)nX * Y)]
                    : czero<T>();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nT * kTxTile; i += blockDim.x) {
    const int tt = i / kTxTile, xx = i - tt * kTxTile;
    if (xx >= nx) continue;
    T acc = czero<T>();
    const T* Br = Bs + (long long)tt * nT;
    for (int s2 = 0; s2 < nT; ++s2) acc = cfma(Br[s2], Ts[s2 * kTxTile + xx], acc);
    const int ry = tt % nry, Y = tt / nry;
    Vout[k + (long long)nrx * ry + nrel * ((long long)(X0 + xx) + (long long)nX * Y)] = acc;
  }
}

__global__ void __launch_bounds__(256) f2d_to32(const double2* __restrict__ x, float2* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t < n) y[t] = make_float2((float)x[t].x, (float)x[t].y);
}

__global__ void __launch_bounds__(256) f2d_to64(const float2* __restrict__ x, double2* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t < n) y[t] = make_double2(x[t].x, x[t].y);
}

// Hard-wall Y boundary (constrain_HardWall_full2D.m:40-50): um = u on the active samples, 0 on the
// others.  Index g = rho_x + nrx (rho_y + nry (X + nX Y)); the flag is act[Y * nry + rho_y].
template <typename T>
__global__ void __launch_bounds__(256) f2d_wall_mask_kernel(const T* __restrict__ u, T* __restrict__ um,
                                                            const unsigned char* __restrict__ act, int nrx, int nry,
                                                            int nX, long long n) {
  const long long g = (long long)blockIdx.x * 256 + threadIdx.x;
  if (g >= n) return;
  const long long t = g / nrx;
  const int ry = (int)(t % nry);
  const long long Y = t / ((long long)nry * nX);
  T v = u[g];
  if (!act[Y * nry + ry]) v = czero<T>();
  um[g] = v;
}

// y <- T y on the Y nodes of each (rho_x, rho_y, X, Y element) group, and scale * u on the
// inactive samples (applyTransverse + the constraint rows of constrainedApply, :40-57).  One thread
// per group, rho_x fastest (coalesced); the group's NK nodes are NK Y dofs apart.
template <typename T, typename R, int NK>
__global__ void __launch_bounds__(256) f2d_wall_project_kernel(T* __restrict__ y, const T* __restrict__ u,
                                                               const unsigned char* __restrict__ act,
                                                               const R* __restrict__ Tb, R scale, int nrx, int nry,
                                                               int nX, int ney) {
  const long long q = (long long)blockIdx.x * 256 + threadIdx.x;
  const long long ngroups = (long long)nrx * nry * nX * ney;
  if (q >= ngroups) return;
  const int rx = (int)(q % nrx);
  long long t = q / nrx;
  const int ry = (int)(t % nry);
  t /= nry;
  const int X = (int)(t % nX);
  const int e = (int)(t / nX);
  const long long nrel = (long long)nrx * nry, ystride = nrel * nX;
  const long long base = rx + (long long)nrx * ry + nrel * X + ystride * ((long long)e * NK);
  T v[NK];
#pragma unroll
  for (int j = 0; j < NK; ++j) v[j] = y[base + ystride * j];
  const R* Te = Tb + ((long long)e * nry + ry) * NK * NK;
#pragma unroll
  for (int a = 0; a < NK; ++a) {
    const long long g = base + ystride * a;
    T o;
    if (act[(long long)(e * NK + a) * nry + ry]) {
      o = czero<T>();
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        o.x += Te[a * NK + j] * v[j].x;
        o.y += Te[a * NK + j] * v[j].y;
      }
    } else {
      const T uu = u[g];
      o.x = scale * uu.x;
      o.y = scale * uu.y;
    }
    y[g] = o;
  }
}

__global__ void __launch_bounds__(256) f2d_to32_scaled(const double2* __restrict__ x, float2* __restrict__ y,
                                                       const double* __restrict__ nrm, long long n) {
  __shared__ double sa;   // the reciprocal once per block
  if (threadIdx.x == 0) sa = nrm[0] > 0 ? 1.0 / nrm[0] : 0.0;
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  const double a = sa;
  if (t < n) y[t] = make_float2((float)(a * x[t].x), (float)(a * x[t].y));
}

// FP16 basis: the scaled vector rounded to FP16 is the basis vector; its FP32 value (exactly the
// stored one) also goes to `copy`, the preconditioner's input, so z = M^-1 v for the stored v.
__global__ void __launch_bounds__(256) f2d_to16_scaled(const double2* __restrict__ x, __half2* __restrict__ y,
                                                       float2* __restrict__ copy, const double* __restrict__ nrm,
                                                       long long n) {
  __shared__ double sa;
  if (threadIdx.x == 0) sa = nrm[0] > 0 ? 1.0 / nrm[0] : 0.0;
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const __half2 v = __floats2half2_rn((float)(sa * x[t].x), (float)(sa * x[t].y));
  y[t] = v;
  copy[t] = __half22float2(v);
}

__global__ void __launch_bounds__(256) f2d_scale16(const float2* __restrict__ x, __half2* __restrict__ out,
                                                   float2* __restrict__ copy, const double* __restrict__ nrm,
                                                   long long n) {
  __shared__ float sa;
  if (threadIdx.x == 0) sa = nrm[0] > 0 ? (float)(1.0 / nrm[0]) : 0.f;
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const __half2 v = __floats2half2_rn(sa * x[t].x, sa * x[t].y);
  out[t] = v;
  copy[t] = __half22float2(v);
}

__global__ void __launch_bounds__(256) f2d_d2f(const double* __restrict__ x, float* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t < n) y[t] = (float)x[t];
}

__device__ __forceinline__ float2 f2d_ld(const float2& v) { return v; }
__device__ __forceinline__ float2 f2d_ld(const __half2& v) { return __half22float2(v); }

// FP32 inner products, summed per thread in FP32 and across threads and blocks in FP64; the basis
// vectors V in FP32 or FP16 storage
template <typename VB>
__global__ void __launch_bounds__(256) f2d_dot_partial32(const VB* __restrict__ V, long long vstride,
                                                         const float2* __restrict__ w, double* __restrict__ partial,
                                                         long long n) {
  __shared__ double sre[256], sim[256];
  const int i = blockIdx.y;
  const VB* v = V + (long long)i * vstride;
  float re = 0.f, im = 0.f;
  for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n; t += (long long)gridDim.x * 256) {
    const float2 a = f2d_ld(v[t]), b = w[t];
    re = fmaf(a.x, b.x, fmaf(a.y, b.y, re));
    im = fmaf(a.x, b.y, fmaf(-a.y, b.x, im));
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sre[threadIdx.x] += sre[threadIdx.x + o];
      sim[threadIdx.x] += sim[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[((long long)i * gridDim.x + blockIdx.x) * 2] = sre[0];
    partial[((long long)i * gridDim.x + blockIdx.x) * 2 + 1] = sim[0];
  }
}

// w -= sum_i h_i V_i in FP32.  The coefficients are converted to FP32 once per block into shared memory:
// converting them per element put every element x vector through the FP64 pipe (98% busy, DRAM at 35%).
constexpr int kGsStage = 256;
template <typename VB>
__global__ void __launch_bounds__(256) f2d_gs_update32(const VB* __restrict__ V, long long vstride,
                                                       float2* __restrict__ w, const double2* __restrict__ h, int nv,
                                                       long long n) {
  __shared__ float2 hs[kGsStage];
  for (int i = threadIdx.x; i < min(nv, kGsStage); i += blockDim.x) hs[i] = make_float2((float)h[i].x, (float)h[i].y);
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  float2 acc = w[t];
  for (int i = 0; i < nv; ++i) {
    const float2 v = f2d_ld(V[(long long)i * vstride + t]);
    const float2 c = i < kGsStage ? hs[i] : make_float2((float)h[i].x, (float)h[i].y);
    acc.x -= c.x * v.x - c.y * v.y;
    acc.y -= c.x * v.y + c.y * v.x;
  }
  w[t] = acc;
}

__global__ void __launch_bounds__(256) f2d_scale32(const float2* __restrict__ x, float2* __restrict__ out,
                                                   const double* __restrict__ nrm, long long n) {
  // the reciprocal once per block (an FP64 division per element made this kernel FP64-bound)
  __shared__ float sa;
  if (threadIdx.x == 0) sa = nrm[0] > 0 ? (float)(1.0 / nrm[0]) : 0.f;
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const float a = sa;
  out[t] = make_float2(a * x[t].x, a * x[t].y);
}

// x += beta sum_i y_i Z_i (the FP32 correction of one refinement, added in FP64)
__global__ void __launch_bounds__(256) f2d_correct32(double2* __restrict__ x, const float2* __restrict__ Z,
                                                     long long zstride, const double2* __restrict__ y, int k,
                                                     const double* __restrict__ beta, long long n) {
  // The correction sum_i y_i Z_i of the FP32 inner solve is accumulated in FP32 (it is only FP32-
  // accurate; FP64 products here made the kernel FP64-pipe-bound), then added to the FP64 iterate.
  __shared__ float2 ys[64];
  for (int i = threadIdx.x; i < min(k, 64); i += blockDim.x) ys[i] = make_float2((float)y[i].x, (float)y[i].y);
  __syncthreads();
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  float2 acc = make_float2(0.f, 0.f);
  for (int i = 0; i < k; ++i) {
    const float2 z = Z[(long long)i * zstride + t];
    const float2 c = i < 64 ? ys[i] : make_float2((float)y[i].x, (float)y[i].y);
    acc.x = fmaf(c.x, z.x, fmaf(-c.y, z.y, acc.x));
    acc.y = fmaf(c.x, z.y, fmaf(c.y, z.x, acc.y));
  }
  x[t].x += beta[0] * (double)acc.x;
  x[t].y += beta[0] * (double)acc.y;
}

// ---------------- GMRES vector kernels (FP64, deterministic two-stage reductions)
constexpr int kDotBlocks = 1024;
// partial[(i * kDotBlocks + blk) * 2 + {0,1}] = sum over the block's chunk of conj(V_i) w
__global__ void __launch_bounds__(256) f2d_dot_partial(const double2* __restrict__ V, long long vstride,
                                                       const double2* __restrict__ w, double* __restrict__ partial,
                                                       long long n) {
  __shared__ double sre[256], sim[256];
  const int i = blockIdx.y;
  const double2* v = V + (long long)i * vstride;
  double re = 0.0, im = 0.0;
  for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n; t += (long long)gridDim.x * 256) {
    const double2 a = v[t], b = w[t];
    re = fma(a.x, b.x, fma(a.y, b.y, re));
    im = fma(a.x, b.y, fma(-a.y, b.x, im));
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sre[threadIdx.x] += sre[threadIdx.x + o];
      sim[threadIdx.x] += sim[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[((long long)i * gridDim.x + blockIdx.x) * 2] = sre[0];
    partial[((long long)i * gridDim.x + blockIdx.x) * 2 + 1] = sim[0];
  }
}

// out[i] = sum of the partials of vector i; one block per vector
__global__ void __launch_bounds__(256) f2d_dot_reduce(const double* __restrict__ partial, double2* __restrict__ out,
                                                      int nblk, int accumulate) {
  __shared__ double sre[256], sim[256];
  const int i = blockIdx.x;
  double re = 0.0, im = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 256) {
    re += partial[((long long)i * nblk + b) * 2];
    im += partial[((long long)i * nblk + b) * 2 + 1];
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sre[threadIdx.x] += sre[threadIdx.x + o];
      sim[threadIdx.x] += sim[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (accumulate) {
      out[i].x += sre[0];
      out[i].y += sim[0];
    } else {
      out[i] = make_double2(sre[0], sim[0]);
    }
  }
}

// w -= sum_i h[i] V_i
__global__ void __launch_bounds__(256) f2d_gs_update(const double2* __restrict__ V, long long vstride,
                                                     double2* __restrict__ w, const double2* __restrict__ h, int nv,
                                                     long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  double2 acc = w[t];
  for (int i = 0; i < nv; ++i) {
    const double2 v = V[(long long)i * vstride + t], c = h[i];
    acc.x -= c.x * v.x - c.y * v.y;
    acc.y -= c.x * v.y + c.y * v.x;
  }
  w[t] = acc;
}

// out = a * x (a = 1 / nrm[0] when inv, else a = nrm[0]); x may alias out
__global__ void __launch_bounds__(256) f2d_scale(const double2* __restrict__ x, double2* __restrict__ out,
                                                 const double* __restrict__ nrm, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const double a = nrm[0] > 0 ? 1.0 / nrm[0] : 0.0;
  out[t] = make_double2(a * x[t].x, a * x[t].y);
}

// y = x + a z (a complex on the host side as two doubles); r = b - y when residual
__global__ void __launch_bounds__(256) f2d_axpy(double2* __restrict__ x, const double2* __restrict__ z, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  x[t].x += z[t].x;
  x[t].y += z[t].y;
}

__global__ void __launch_bounds__(256) f2d_sub(const double2* __restrict__ b, double2* __restrict__ y, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  y[t] = make_double2(b[t].x - y[t].x, b[t].y - y[t].y);
}

// BiCGSTAB vector updates (complex scalars by value): p = r + beta (p - omega v); y += a x; y -= a x
__global__ void __launch_bounds__(256) f2d_bicg_p(double2* __restrict__ p, const double2* __restrict__ r,
                                                  const double2* __restrict__ v, double2 beta, double2 omega,
                                                  long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const double2 pv = p[t], vv = v[t], rv = r[t];
  const double2 d = make_double2(pv.x - (omega.x * vv.x - omega.y * vv.y), pv.y - (omega.x * vv.y + omega.y * vv.x));
  p[t] = make_double2(rv.x + beta.x * d.x - beta.y * d.y, rv.y + beta.x * d.y + beta.y * d.x);
}

__global__ void __launch_bounds__(256) f2d_caxpy(double2* __restrict__ y, const double2* __restrict__ x, double2 a,
                                                 long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  const double2 xv = x[t];
  y[t].x += a.x * xv.x - a.y * xv.y;
  y[t].y += a.x * xv.y + a.y * xv.x;
}

// |x|^2 of the dot result (real part) -> nrm[0] = sqrt
__global__ void f2d_sqrt_real(const double2* __restrict__ d, double* __restrict__ nrm) {
  nrm[0] = isnan(d[0].x) ? d[0].x : sqrt(fmax(d[0].x, 0.0));   // a NaN norm stays NaN (never "converged")
}

__global__ void __launch_bounds__(256) f2d_rscale(double2* __restrict__ v, double s, long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  v[t].x *= s;
  v[t].y *= s;
}

// Hessenberg column j (hc[0..j] from Gram-Schmidt, nrm[0] = |w|): previous Givens rotations, the
// new one, the rotated right-hand side; g[j+1] is the residual estimate.  One thread.
__global__ void f2d_givens(double2* __restrict__ H, const double2* __restrict__ hc, const double* __restrict__ nrm,
                           double* __restrict__ cs, double2* __restrict__ sn, double2* __restrict__ g, int j, int ldh) {
  double2* col = H + (long long)j * ldh;
  for (int i = 0; i <= j; ++i) col[i] = hc[i];
  col[j + 1] = make_double2(nrm[0], 0.0);
  for (int i = 0; i < j; ++i) {
    const double c = cs[i];
    const double2 s = sn[i], a = col[i], b = col[i + 1];
    // [c s; -conj(s) c] [a; b]
    col[i] = make_double2(c * a.x + s.x * b.x - s.y * b.y, c * a.y + s.x * b.y + s.y * b.x);
    col[i + 1] = make_double2(-(s.x * a.x + s.y * a.y) + c * b.x, -(s.x * a.y - s.y * a.x) + c * b.y);
  }
  const double2 a = col[j];
  const double bb = col[j + 1].x;
  const double aa = hypot(a.x, a.y);
  const double rho = hypot(aa, bb);
  double c;
  double2 s, top;
  if (rho == 0.0) {
    c = 1.0;
    s = make_double2(0.0, 0.0);
    top = a;
  } else if (aa == 0.0) {
    c = 0.0;
    s = make_double2(1.0, 0.0);
    top = make_double2(bb, 0.0);
  } else {
    c = aa / rho;
    const double2 ph = make_double2(a.x / aa, a.y / aa);
    s = make_double2(ph.x * bb / rho, ph.y * bb / rho);        // (a/|a|) conj(b) / rho, b real
    top = make_double2(ph.x * rho, ph.y * rho);
  }
  cs[j] = c;
  sn[j] = s;
  col[j] = top;
  col[j + 1] = make_double2(0.0, 0.0);
  const double2 gj = g[j];
  g[j] = make_double2(c * gj.x, c * gj.y);
  g[j + 1] = make_double2(-(s.x * gj.x + s.y * gj.y), -(s.x * gj.y - s.y * gj.x));
}

// y = R^-1 g for the leading k x k upper triangle of H; one thread
__global__ void f2d_backsolve(const double2* __restrict__ H, const double2* __restrict__ g, double2* __restrict__ y,
                              int k, int ldh) {
  for (int i = k - 1; i >= 0; --i) {
    double2 s = g[i];
    for (int j = i + 1; j < k; ++j) {
      const double2 h = H[(long long)j * ldh + i], v = y[j];
      s.x -= h.x * v.x - h.y * v.y;
      s.y -= h.x * v.y + h.y * v.x;
    }
    const double2 d = H[(long long)i * ldh + i];
    const double den = d.x * d.x + d.y * d.y;
    y[i] = den > 0 ? make_double2((s.x * d.x + s.y * d.y) / den, (s.y * d.x - s.x * d.y) / den)
                   : make_double2(0.0, 0.0);
  }
}

// u = sum_i y_i V_i
__global__ void __launch_bounds__(256) f2d_combine(const double2* __restrict__ V, long long vstride,
                                                   const double2* __restrict__ y, double2* __restrict__ u, int k,
                                                   long long n) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= n) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int i = 0; i < k; ++i) acc = cfma(y[i], V[(long long)i * vstride + t], acc);
  u[t] = acc;
}

int fail(wg2d_problem* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define F2_CK(expr)                                                         \
  do {                                                                      \
    cudaError_t e_ = (expr);                                                \
    if (e_ != cudaSuccess) return fail(h, WG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #expr); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1));
}

void free_axis(wg2d_problem::Axis& a) {
  for (wg::OzakiRowsDev& d : a.dense) wg::ozaki_free(d);
  cudaFree(a.blocks);
  cudaFree(a.rp);
  cudaFree(a.col);
  cudaFree(a.val);
  cudaFree(a.offs);
  cudaFree(a.dcoef);
  cudaFree(a.ymask);
  a = wg2d_problem::Axis{};
}

// Operator data of one precision: FP64 (the handle's own arrays) or the FP32 copies of the mixed solve.
template <typename T, typename R>
struct OpData {
  const R* blocks[2];
  const T* val[2];
  const R* coef[2];
  const R *interp, *proj, *cap, *dV;
  T *Uq, *Rq, *G;
  T pot16;
  R capc;
};

template <int NK, typename T, typename R>
void launch_center(wg2d_problem* h, int axis, const T* F, T* G, const R* blocks) {
  const int nk = axis == 0 ? h->s.nk_x : h->s.nk_y;
  const int n_el = axis == 0 ? h->s.n_el_x : h->s.n_el_y;
  const int other = axis == 0 ? h->nY : h->nX;
  const dim3 grid((unsigned)((h->nrel + 255) / 256), (unsigned)other, (unsigned)(n_el * nk));
  f2d_center_kernel<NK, T, R><<<grid, 256, 0, h->stream>>>(F, G, blocks, h->ax[axis].T, axis, h->nrel, h->nX, h->nY,
                                                           n_el, axis == 1 ? h->s.periodic_y : 0, h->n);
}

// y += transport terms of one axis; the terms in skip_mask are left to the caller
template <typename T, typename R>
void transport_terms(wg2d_problem* h, int axis, const OpData<T, R>& d, const T* F, T* y, unsigned skip_mask) {
  wg2d_problem::Axis& a = h->ax[axis];
  const int nk = axis == 0 ? h->s.nk_x : h->s.nk_y;
  switch (nk) {
    case 2: launch_center<2, T, R>(h, axis, F, d.G, d.blocks[axis]); break;
    case 3: launch_center<3, T, R>(h, axis, F, d.G, d.blocks[axis]); break;
    default: launch_center<4, T, R>(h, axis, F, d.G, d.blocks[axis]); break;
  }
  if (axis == 0) {
    const long long ncols = h->n / h->nrx;
    const size_t smem = sizeof(T) * kRelxCols * h->nrx;
    const int threads = (h->nrx + 31) / 32 * 32;
    if (skip_mask != (1u << a.T) - 1u)
      f2d_relx_kernel<T, R><<<(unsigned)((ncols + kRelxCols - 1) / kRelxCols), threads, smem, h->stream>>>(
          d.G, y, a.rp, a.col, d.val[0], a.offs, d.coef[0], a.T, h->nrx, ncols, h->n, skip_mask, a.ymask,
          (long long)h->nry * h->nX, h->nY);
  } else {
    f2d_rely_kernel<T, R><<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(d.G, y, a.rp, a.col, d.val[1], a.offs,
                                                                                d.coef[1], a.T, h->nrx, h->nry, h->n);
  }
}

OpData<double2, double> op64(wg2d_problem* h) {
  OpData<double2, double> d;
  for (int a = 0; a < 2; ++a) {
    d.blocks[a] = h->ax[a].blocks;
    d.val[a] = h->ax[a].val;
    d.coef[a] = h->ax[a].dcoef;
  }
  d.interp = h->interp;
  d.proj = h->proj;
  d.cap = h->cap;
  d.dV = h->dV;
  d.Uq = h->Uq;
  d.Rq = h->Rq;
  d.G = h->G;
  d.pot16 = make_double2(h->pot.x / 16.0, h->pot.y / 16.0);
  d.capc = h->capc;
  return d;
}

int apply_transport(wg2d_problem* h, int axis) {
  wg2d_problem::Axis& a = h->ax[axis];
  if (a.T == 0) return WG_OK;
  transport_terms<double2, double>(h, axis, op64(h), h->x, h->y, axis == 0 ? a.dense_mask : 0u);
  if (axis == 0)
    for (int t = 0; t < a.T; ++t)
      if ((a.dense_mask >> t) & 1u)
        F2_CK(wg::ozaki_accumulate(a.dense[t], h->cols, reinterpret_cast<const double*>(h->G + (long long)t * h->n),
                                   reinterpret_cast<double*>(h->y), h->tc_err, h->stream));
  F2_CK(cudaGetLastError());
  return WG_OK;
}

template <int NL, typename T, typename R>
void launch_drift(wg2d_problem* h, const OpData<T, R>& d, const T* F, T* y) {
  const wg2d_shape& s = h->s;
  const dim3 g1((unsigned)((h->nrel + 127) / 128), (unsigned)h->nel);
  f2d_interp_kernel<NL, T, R><<<g1, 128, 0, h->stream>>>(F, d.Uq, d.interp, h->nq, h->nrel, s.n_el_x, s.nk_x, s.nk_y,
                                                         h->nX);
  const dim3 g2((unsigned)((h->nrel + 127) / 128), (unsigned)h->nq, (unsigned)h->nel);
  f2d_vertex_kernel<T, R><<<g2, 128, 0, h->stream>>>(d.Uq, d.Rq, d.dV, h->nrx, h->nry, h->nq, h->nvert, s.periodic_y);
  f2d_project_kernel<NL, T, R><<<g1, 128, 0, h->stream>>>(d.Rq, F, y, d.proj, d.cap, d.pot16, d.capc, h->nq, h->nrel,
                                                          s.n_el_x, s.nk_x, s.nk_y, h->nX);
}

template <typename T, typename R>
void drift_terms(wg2d_problem* h, const OpData<T, R>& d, const T* F, T* y) {
  switch (h->nloc) {
    case 4: launch_drift<4, T, R>(h, d, F, y); break;
    case 6: launch_drift<6, T, R>(h, d, F, y); break;
    case 8: launch_drift<8, T, R>(h, d, F, y); break;
    case 9: launch_drift<9, T, R>(h, d, F, y); break;
    case 12: launch_drift<12, T, R>(h, d, F, y); break;
    default: launch_drift<16, T, R>(h, d, F, y); break;
  }
}

int apply_drift(wg2d_problem* h) {
  drift_terms<double2, double>(h, op64(h), h->x, h->y);
  F2_CK(cudaGetLastError());
  return WG_OK;
}

bool supported_nloc(int n) { return n == 4 || n == 6 || n == 8 || n == 9 || n == 12 || n == 16; }

}  // namespace

namespace {

// Observables at zero relative separation (get_Observables_full2D.m:19-79), one thread per DG X dof:
// the DG values over the Y dofs, then their projection onto the material Y points and the integral.
__global__ void __launch_bounds__(128) f2d_observables_kernel(const double2* __restrict__ F, wg2d_observables_desc d,
                                                              const double* __restrict__ W,
                                                              const double* __restrict__ wj, int nX, int nY, int nrx,
                                                              int nry, double* __restrict__ out) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= nX) return;
  const int nty = d.n_target_y;
  double* nDG = out;
  double* jxDG = out + (size_t)nX * nY;
  double* jyDG = out + (size_t)2 * nX * nY;
  double* n = out + (size_t)3 * nX * nY;
  double* jx = n + (size_t)nX * nty;
  double* jy = n + (size_t)2 * nX * nty;
  double* j = n + (size_t)3 * nX * nty;
  const long long nrel = (long long)nrx * nry;
  for (int yd = 0; yd < nY; ++yd) {
    const double2* c = F + ((long long)yd * nX + X) * nrel;
    double at0 = 0.0;
    double2 dx = make_double2(0.0, 0.0), dy = make_double2(0.0, 0.0);
    for (int a = 0; a < d.n_zero_y; ++a) {
      const double2* row = c + (long long)d.zero_y[a] * nrx;
      for (int b = 0; b < d.n_zero_x; ++b) at0 += d.w_zero_y[a] * d.w_zero_x[b] * row[d.zero_x[b]].x;
      for (int q = 0; q < d.n_dx; ++q) {
        const double w = d.w_zero_y[a] * d.dx_val[q];
        const double2 v = row[d.dx_idx[q]];
        dx.x += w * v.x;
        dx.y += w * v.y;
      }
    }
    for (int b = 0; b < d.n_zero_x; ++b)
      for (int q = 0; q < d.n_dy; ++q) {
        const double w = d.w_zero_x[b] * d.dy_val[q];
        const double2 v = c[(long long)d.dy_idx[q] * nrx + d.zero_x[b]];
        dy.x += w * v.x;
        dy.y += w * v.y;
      }
    nDG[(size_t)X * nY + yd] = at0;
    jxDG[(size_t)X * nY + yd] = d.scale_x * dx.y;
    jyDG[(size_t)X * nY + yd] = d.scale_y * dy.y;
  }
  double jsum = 0.0;
  for (int t = 0; t < nty; ++t) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int yd = 0; yd < nY; ++yd) {
      const double w = W[(size_t)t * nY + yd];
      s0 += w * nDG[(size_t)X * nY + yd];
      s1 += w * jxDG[(size_t)X * nY + yd];
      s2 += w * jyDG[(size_t)X * nY + yd];
    }
    n[(size_t)X * nty + t] = s0;
    jx[(size_t)X * nty + t] = s1;
    jy[(size_t)X * nty + t] = s2;
    jsum += wj[t] * s1;
  }
  j[X] = jsum;
}

}  // namespace

extern "C" {

static void free_solver(wg2d_problem* h);
static void free_preconditioner(wg2d_problem* h);
static void free32(wg2d_problem* h);

int wg2d_create(const wg2d_shape* s, wg2d_problem** out) {
  if (!s || !out) return WG_ERR_ARG;
  *out = nullptr;
  if (s->n_el_x < 1 || s->n_el_y < 1 || s->nk_x < 2 || s->nk_x > kMaxNK || s->nk_y < 2 || s->nk_y > kMaxNK ||
      s->n_rho_x < 2 || s->n_rho_x > 512 || s->n_rho_y < 2 || s->n_quad < 1 || !supported_nloc(s->nk_x * s->nk_y))
    return WG_ERR_ARG;
  if (s->periodic_y && (s->n_el_y < 2 || s->n_rho_y < 4)) return WG_ERR_ARG;
  wg2d_problem* h = new wg2d_problem;
  h->s = *s;
  h->nX = s->n_el_x * s->nk_x;
  h->nY = s->n_el_y * s->nk_y;
  h->nrx = s->n_rho_x;
  h->nry = s->n_rho_y;
  h->nrel = h->nrx * h->nry;
  h->ncen = h->nX * h->nY;
  h->nel = s->n_el_x * s->n_el_y;
  h->nloc = s->nk_x * s->nk_y;
  h->nq = s->n_quad;
  h->nvert = (h->nrx + 1) * (s->periodic_y ? h->nry : h->nry + 1);
  h->n = (long long)h->nrel * h->ncen;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  const size_t slab = (size_t)h->nel * h->nq;
  if (e == cudaSuccess) e = dalloc(&h->x, h->n);
  if (e == cudaSuccess) e = dalloc(&h->y, h->n);
  if (e == cudaSuccess) e = dalloc(&h->Uq, slab * h->nrel);
  if (e == cudaSuccess) e = dalloc(&h->Rq, slab * h->nrel);
  if (e == cudaSuccess) e = dalloc(&h->dV, slab * h->nvert);
  if (e == cudaSuccess) e = dalloc(&h->interp, (size_t)h->nq * h->nloc);
  if (e == cudaSuccess) e = dalloc(&h->proj, (size_t)h->nq * h->nloc);
  if (e == cudaSuccess) e = dalloc(&h->xq, slab);
  if (e == cudaSuccess) e = dalloc(&h->yq, slab);
  if (e == cudaSuccess) e = dalloc(&h->vx, h->nvert);
  if (e == cudaSuccess) e = dalloc(&h->vy, h->nvert);
  if (e == cudaSuccess) e = dalloc(&h->cap, h->nrel);
  if (e == cudaSuccess) e = dalloc(&h->tc_err, 1);
  if (e == cudaSuccess) e = cudaMemset(h->tc_err, 0, sizeof(int));
  for (cudaEvent_t& ev : h->ev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e == cudaSuccess && h->nrx * kRelxCols * sizeof(double2) > 48 * 1024)
    e = cudaFuncSetAttribute(f2d_relx_kernel<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(h->nrx * kRelxCols * sizeof(double2)));
  if (e != cudaSuccess) {
    wg2d_destroy(h);
    return e == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  *out = h;
  return WG_OK;
}

int wg2d_destroy(wg2d_problem* h) {
  if (!h) return WG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& a : h->ax) free_axis(a);
  free_solver(h);
  free_preconditioner(h);
  free32(h);
  wg::ozaki_free(h->cols);
  void* ptrs[] = {h->x, h->y, h->G, h->Uq, h->Rq, h->dV, h->interp, h->proj, h->xq, h->yq, h->vx, h->vy, h->cap,
                  h->tc_err, h->obs_W, h->obs_wj, h->obs_out, h->wall_act, h->wall_T, h->wall_T32, h->wall_u,
                  h->wall_u32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t ev : h->ev)
    if (ev) cudaEventDestroy(ev);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return WG_OK;
}

const char* wg2d_last_error(const wg2d_problem* h) { return h ? h->err.c_str() : "null handle"; }

int wg2d_set_transport(wg2d_problem* h, int axis, int n_terms, const double* coef, const double* center_blocks,
                       const int* row_ptr, const int* col, const double* val) {
  if (!h) return WG_ERR_ARG;
  if (axis < 0 || axis > 1 || n_terms < 0 || n_terms > kMaxTerms || (n_terms && (!coef || !center_blocks ||
                                                                                   !row_ptr || !col || !val)))
    return fail(h, WG_ERR_ARG, "wg2d_set_transport: axis 0/1, 0 .. 6 terms, non-null arrays");
  const int nk = axis == 0 ? h->s.nk_x : h->s.nk_y, n_el = axis == 0 ? h->s.n_el_x : h->s.n_el_y;
  const int nr = axis == 0 ? h->nrx : h->nry;
  std::vector<int> off(n_terms + 1, 0);
  for (int t = 0; t < n_terms; ++t) {
    const int* rp = row_ptr + t * (nr + 1);
    if (rp[0] != 0) return fail(h, WG_ERR_ARG, "wg2d_set_transport: row_ptr must start at 0");
    for (int i = 0; i < nr; ++i)
      if (rp[i + 1] < rp[i]) return fail(h, WG_ERR_ARG, "wg2d_set_transport: row_ptr must not decrease");
    off[t + 1] = off[t] + rp[nr];
  }
  for (int k = 0; k < off[n_terms]; ++k)
    if (col[k] < 0 || col[k] >= nr) return fail(h, WG_ERR_ARG, "wg2d_set_transport: column index out of range");
  cudaStreamSynchronize(h->stream);
  wg2d_problem::Axis& a = h->ax[axis];
  free_axis(a);
  h->d32_ready = false;
  a.T = n_terms;
  a.coef.assign(coef, coef + n_terms);
  if (n_terms == 0) return WG_OK;
  const int nrp = n_terms * (nr + 1);
  const size_t nb = (size_t)n_terms * n_el * 3 * nk * nk;
  F2_CK(dalloc(&a.blocks, nb));
  F2_CK(dalloc(&a.rp, nrp));
  F2_CK(dalloc(&a.col, off[n_terms]));
  F2_CK(dalloc(&a.val, off[n_terms]));
  F2_CK(dalloc(&a.offs, n_terms));
  F2_CK(dalloc(&a.dcoef, n_terms));
  F2_CK(cudaMemcpy(a.blocks, center_blocks, sizeof(double) * nb, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(a.rp, row_ptr, sizeof(int) * nrp, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(a.offs, off.data(), sizeof(int) * n_terms, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(a.dcoef, coef, sizeof(double) * n_terms, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(a.col, col, sizeof(int) * std::max(1, off[n_terms]), cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(a.val, val, sizeof(double2) * std::max(1, off[n_terms]), cudaMemcpyHostToDevice));
  // dense rho_x factors on the tensor cores: the real embedding of c_t R_t, digit-sliced once
  a.dense.assign(n_terms, wg::OzakiRowsDev{});
  a.dense_mask = 0;
  if (axis == 0 && h->s.tensor_cores) {
    for (int t = 0; t < n_terms; ++t) {
      const int nnz = off[t + 1] - off[t];
      if ((long long)nnz * 4 <= (long long)nr * nr) continue;
      std::vector<double> A((size_t)4 * nr * nr, 0.0);
      const int* rp = row_ptr + t * (nr + 1);
      for (int i = 0; i < nr; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
          const int j = col[off[t] + k];
          const double re = coef[t] * val[2 * (off[t] + k)], im = coef[t] * val[2 * (off[t] + k) + 1];
          A[(size_t)(2 * i) * 2 * nr + 2 * j] += re;
          A[(size_t)(2 * i) * 2 * nr + 2 * j + 1] += -im;
          A[(size_t)(2 * i + 1) * 2 * nr + 2 * j] += im;
          A[(size_t)(2 * i + 1) * 2 * nr + 2 * j + 1] += re;
        }
      const int rc = wg::ozaki_rows_upload(A, 2 * nr, 2 * nr, a.dense[t], h->err);
      if (rc) return rc;
      a.dense_mask |= 1u << t;
    }
    if (a.dense_mask && !h->cols.dig) {
      const int rc = wg::ozaki_cols_alloc(h->n / nr, 2 * nr, h->cols, h->err);
      if (rc) return rc;
    }
  }
  const int need = std::max(h->ax[0].T, h->ax[1].T);
  if (need > h->g_terms) {
    cudaFree(h->G);
    h->G = nullptr;
    h->g_terms = 0;
    F2_CK(dalloc(&h->G, (size_t)need * h->n));
    h->g_terms = need;
  }
  return WG_OK;
}

int wg2d_set_drift(wg2d_problem* h, const double* interp, const double* proj, const double* xq, const double* yq,
                   const double* vx, const double* vy, const double* pot, double cap_coef, const double* cap) {
  if (!h) return WG_ERR_ARG;
  if (!interp || !proj || !xq || !yq || !vx || !vy || !pot || !cap || !std::isfinite(cap_coef))
    return fail(h, WG_ERR_ARG, "wg2d_set_drift: null argument or non-finite coefficient");
  const size_t nql = (size_t)h->nq * h->nloc, slab = (size_t)h->nel * h->nq;
  F2_CK(cudaMemcpyAsync(h->interp, interp, sizeof(double) * nql, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->proj, proj, sizeof(double) * nql, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->xq, xq, sizeof(double) * slab, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->yq, yq, sizeof(double) * slab, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->vx, vx, sizeof(double) * h->nvert, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->vy, vy, sizeof(double) * h->nvert, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(h->cap, cap, sizeof(double) * h->nrel, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  h->pot = make_double2(pot[0], pot[1]);
  h->capc = cap_coef;
  h->drift_ready = true;
  h->d32_ready = false;
  return WG_OK;
}

int wg2d_set_potential(wg2d_problem* h, int nx, int ny, const double* gx, const double* gy, const double* V) {
  if (!h) return WG_ERR_ARG;
  if (!h->drift_ready) return fail(h, WG_ERR_ARG, "wg2d_set_potential: call wg2d_set_drift first");
  if (nx < 2 || ny < 2 || !gx || !gy || !V) return fail(h, WG_ERR_ARG, "wg2d_set_potential: need a 2 x 2 grid or larger");
  for (int i = 0; i + 1 < nx; ++i)
    if (!(gx[i + 1] > gx[i])) return fail(h, WG_ERR_ARG, "wg2d_set_potential: gx must increase");
  for (int j = 0; j + 1 < ny; ++j)
    if (!(gy[j + 1] > gy[j])) return fail(h, WG_ERR_ARG, "wg2d_set_potential: gy must increase");
  for (long long i = 0; i < (long long)nx * ny; ++i)
    if (!std::isfinite(V[i])) return fail(h, WG_ERR_ARG, "wg2d_set_potential: V must be finite");
  double *dgx = nullptr, *dgy = nullptr, *dV = nullptr;
  F2_CK(dalloc(&dgx, nx));
  F2_CK(dalloc(&dgy, ny));
  F2_CK(dalloc(&dV, (size_t)nx * ny));
  F2_CK(cudaMemcpyAsync(dgx, gx, sizeof(double) * nx, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(dgy, gy, sizeof(double) * ny, cudaMemcpyHostToDevice, h->stream));
  F2_CK(cudaMemcpyAsync(dV, V, sizeof(double) * nx * ny, cudaMemcpyHostToDevice, h->stream));
  const dim3 g((unsigned)((h->nvert + 127) / 128), (unsigned)h->nq, (unsigned)h->nel);
  f2d_dv_kernel<<<g, 128, 0, h->stream>>>(h->dV, h->xq, h->yq, h->vx, h->vy, dgx, dgy, dV, nx, ny, h->nq, h->nvert,
                                         h->s.periodic_y);
  const cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(h->stream);
  cudaFree(dgx);
  cudaFree(dgy);
  cudaFree(dV);
  if (e != cudaSuccess) return fail(h, WG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  h->potential_ready = true;
  h->d32_ready = false;
  return WG_OK;
}

}  // extern "C"

// The hard-wall constraint around an apply: mask the input before, project the output after.
template <typename T, typename R>
static int wall_project(wg2d_problem* h, T* y, const T* u, const R* Tb) {
  const long long groups = (long long)h->nrx * h->nry * h->nX * h->s.n_el_y;
  const unsigned nb = (unsigned)((groups + 255) / 256);
  const R sc = (R)h->wall_scale;
  switch (h->s.nk_y) {
    case 2: f2d_wall_project_kernel<T, R, 2><<<nb, 256, 0, h->stream>>>(y, u, h->wall_act, Tb, sc, h->nrx, h->nry,
                                                                         h->nX, h->s.n_el_y); break;
    case 3: f2d_wall_project_kernel<T, R, 3><<<nb, 256, 0, h->stream>>>(y, u, h->wall_act, Tb, sc, h->nrx, h->nry,
                                                                         h->nX, h->s.n_el_y); break;
    default: f2d_wall_project_kernel<T, R, 4><<<nb, 256, 0, h->stream>>>(y, u, h->wall_act, Tb, sc, h->nrx, h->nry,
                                                                          h->nX, h->s.n_el_y); break;
  }
  F2_CK(cudaGetLastError());
  return WG_OK;
}

extern "C" {

static int apply_device(wg2d_problem* h) {
  if (!h->potential_ready) return fail(h, WG_ERR_ARG, "wg2d_apply: set the drift data and the potential first");
  double2* u = h->x;
  if (h->wall) {
    f2d_wall_mask_kernel<double2><<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(u, h->wall_u, h->wall_act,
                                                                                     h->nrx, h->nry, h->nX, h->n);
    h->x = h->wall_u;
  }
  int rc = apply_drift(h);
  if (!rc) rc = apply_transport(h, 0);
  if (!rc) rc = apply_transport(h, 1);
  h->x = u;
  if (rc || !h->wall) return rc;
  return wall_project<double2, double>(h, h->y, u, h->wall_T);
}

// out = A in on device buffers (the kernels read h->x and write h->y at launch)
static int apply_op(wg2d_problem* h, double2* in, double2* out) {
  double2 *sx = h->x, *sy = h->y;
  h->x = in;
  h->y = out;
  const int rc = apply_device(h);
  h->x = sx;
  h->y = sy;
  return rc;
}

static unsigned blocks256(long long n) { return (unsigned)((n + 255) / 256); }

// z = M^-1 r (applyInverse of get_LineTransversePreconditioner_full2D.m:202-238): modes along rho_x,
// X lines per mode, transverse inverses per mode and X dof, back to rho_x.  FP32 (default for the
// solve: an approximate inverse; the flexible GMRES keeps the solve exact for what was applied) or
// FP64 with the mode transforms on the tensor cores.
}  // extern "C"

template <typename T>
static void precond_stages(wg2d_problem* h, const T* UH, const T* Us, const T* xinv, const T* xcpl, const T* tinv,
                           const T* r, T* pa, T* pb, T* z) {
  const long long ncols = h->n / h->nrx;
  const int threads = (h->nrx + 31) / 32 * 32;
  const size_t smem = sizeof(T) * kRelxCols * h->nrx;
  if (UH)
    f2d_dense_rx_kernel<T><<<(unsigned)((ncols + kRelxCols - 1) / kRelxCols), threads, smem, h->stream>>>(
        UH, r, pa, h->nrx, ncols);
  const long long lines = (long long)h->nrx * h->nry * h->nY;
  if (h->x_chunks > 1 && h->xmaps) {
    T* maps = reinterpret_cast<T*>(h->xmaps);
    const int L = h->x_chunk_len, C = h->x_chunks, ne = h->s.n_el_x;
    const unsigned cb = (unsigned)((lines * C + 127) / 128);
#define WG_XLINE_CHUNKED(NK_)                                                                                \
  f2d_xline_maps_kernel<NK_, T><<<cb, 128, 0, h->stream>>>(pa, maps, xinv, xcpl, h->fwd, h->nrx, h->nry, h->nX, \
                                                          h->nY, ne, L, C);                                   \
  f2d_xline_apply_kernel<NK_, T><<<cb, 128, 0, h->stream>>>(pa, pb, maps, xinv, xcpl, h->fwd, h->nrx, h->nry,  \
                                                           h->nX, h->nY, ne, L, C);
    switch (h->s.nk_x) {
      case 2: WG_XLINE_CHUNKED(2) break;
      case 3: WG_XLINE_CHUNKED(3) break;
      default: WG_XLINE_CHUNKED(4) break;
    }
#undef WG_XLINE_CHUNKED
  } else {
    const unsigned lb = (unsigned)((lines + 127) / 128);
    switch (h->s.nk_x) {
      case 2: f2d_xline_kernel<2, T><<<lb, 128, 0, h->stream>>>(pa, pb, xinv, xcpl, h->fwd, h->nrx, h->nry, h->nX,
                                                               h->nY, h->s.n_el_x); break;
      case 3: f2d_xline_kernel<3, T><<<lb, 128, 0, h->stream>>>(pa, pb, xinv, xcpl, h->fwd, h->nrx, h->nry, h->nX,
                                                               h->nY, h->s.n_el_x); break;
      default: f2d_xline_kernel<4, T><<<lb, 128, 0, h->stream>>>(pa, pb, xinv, xcpl, h->fwd, h->nrx, h->nry, h->nX,
                                                                h->nY, h->s.n_el_x); break;
    }
  }
  const size_t tsm = sizeof(T) * ((size_t)h->nT * h->nT + (size_t)h->nT * kTxTile);
  const dim3 tg((unsigned)((h->nX + kTxTile - 1) / kTxTile), (unsigned)h->nrx);
  f2d_transverse_kernel<T><<<tg, 256, tsm, h->stream>>>(pb, pa, tinv, h->nrx, h->nry, h->nX, h->nY, h->nT);
  if (Us)
    f2d_dense_rx_kernel<T><<<(unsigned)((ncols + kRelxCols - 1) / kRelxCols), threads, smem, h->stream>>>(
        Us, pa, z, h->nrx, ncols);
}

extern "C" {

static int precondition_device(wg2d_problem* h, const double2* r, double2* z) {
  if (!h->pre_ready) return fail(h, WG_ERR_ARG, "wg2d: set the preconditioner first");
  if (h->pre32) {
    f2d_to32<<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(r, h->pb32, h->n);
    precond_stages<float2>(h, h->UH32, h->Us32, h->xinv32, h->xcpl32, h->tinv32, h->pb32, h->pa32, h->pb32, h->pb32);
    f2d_to64<<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(h->pb32, z, h->n);
    F2_CK(cudaGetLastError());
    return WG_OK;
  }
  if (h->s.tensor_cores) {
    F2_CK(wg::ozaki_multiply(h->UH, h->cols, reinterpret_cast<const double*>(r), reinterpret_cast<double*>(h->pa),
                             h->tc_err, h->stream));
    precond_stages<double2>(h, nullptr, nullptr, h->xinv, h->xcpl, h->tinv, r, h->pa, h->pb, z);
    F2_CK(wg::ozaki_multiply(h->Us, h->cols, reinterpret_cast<const double*>(h->pa), reinterpret_cast<double*>(z),
                             h->tc_err, h->stream));
  } else {
    precond_stages<double2>(h, h->UHd, h->Usd, h->xinv, h->xcpl, h->tinv, r, h->pa, h->pb, z);
  }
  F2_CK(cudaGetLastError());
  return WG_OK;
}

// out[0..nv) = V_i^H w (accumulate: out += ...)
static void dots(wg2d_problem* h, const double2* V, int nv, const double2* w, double2* out, int accumulate) {
  f2d_dot_partial<<<dim3(kDotBlocks, nv), 256, 0, h->stream>>>(V, h->n, w, h->partial, h->n);
  f2d_dot_reduce<<<nv, 256, 0, h->stream>>>(h->partial, out, kDotBlocks, accumulate);
}

static void vnorm(wg2d_problem* h, const double2* w) {
  dots(h, w, 1, w, h->hp, 0);
  f2d_sqrt_real<<<1, 1, 0, h->stream>>>(h->hp, h->nrm);
}

}  // extern "C"

template <typename VB>
static void dots32(wg2d_problem* h, const VB* V, int nv, const float2* w, double2* out, int accumulate) {
  f2d_dot_partial32<VB><<<dim3(kDotBlocks, nv), 256, 0, h->stream>>>(V, h->n, w, h->partial, h->n);
  f2d_dot_reduce<<<nv, 256, 0, h->stream>>>(h->partial, out, kDotBlocks, accumulate);
}

extern "C" {

static void vnorm32(wg2d_problem* h, const float2* w) {
  dots32(h, w, 1, w, h->hp, 0);
  f2d_sqrt_real<<<1, 1, 0, h->stream>>>(h->hp, h->nrm);
}

static void free_solver(wg2d_problem* h) {
  void* ptrs[] = {h->V, h->Zb, h->r, h->w, h->z, h->b, h->xs, h->H, h->g, h->sn, h->hc, h->hp, h->yc, h->cs,
                  h->partial, h->nrm, h->bc_rt, h->bc_p, h->bc_ph, h->bc_sh};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h->bc_rt = h->bc_p = h->bc_ph = h->bc_sh = nullptr;
  h->V = h->Zb = h->r = h->w = h->z = h->b = h->xs = h->H = h->g = h->sn = h->hc = h->hp = h->yc = nullptr;
  h->cs = h->partial = h->nrm = nullptr;
  h->vm = 0;
}

static void free_preconditioner(wg2d_problem* h) {
  wg::ozaki_free(h->UH);
  wg::ozaki_free(h->Us);
  void* ptrs[] = {h->UHd, h->Usd, h->xinv, h->xcpl, h->fwd, h->tinv, h->pa, h->pb, h->UH32, h->Us32, h->xinv32,
                  h->xcpl32, h->tinv32, h->pa32, h->pb32, h->xmaps};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h->xmaps = nullptr;
  h->x_chunks = 1;
  h->UHd = h->Usd = h->xinv = h->xcpl = h->tinv = h->pa = h->pb = nullptr;
  h->UH32 = h->Us32 = h->xinv32 = h->xcpl32 = h->tinv32 = h->pa32 = h->pb32 = nullptr;
  h->fwd = nullptr;
  h->pre32 = false;
  h->pre_ready = false;
}

int wg2d_set_transport_masks(wg2d_problem* h, int axis, int n_terms, const unsigned char* masks) {
  if (!h) return WG_ERR_ARG;
  if (axis != 0) return fail(h, WG_ERR_ARG, "wg2d_set_transport_masks: only the rho_x axis (0) takes Y masks");
  wg2d_problem::Axis& a = h->ax[0];
  if (n_terms != a.T) return fail(h, WG_ERR_ARG, "wg2d_set_transport_masks: n_terms must equal the terms set");
  cudaStreamSynchronize(h->stream);
  cudaFree(a.ymask);
  a.ymask = nullptr;
  if (!masks) return WG_OK;
  const size_t nm = (size_t)n_terms * h->nY;
  F2_CK(cudaMalloc(&a.ymask, nm));
  F2_CK(cudaMemcpy(a.ymask, masks, nm, cudaMemcpyHostToDevice));
  // a masked term leaves the dense tensor-core path (which applies a term on every column)
  for (int t = 0; t < n_terms; ++t) {
    bool all = true;
    for (int i = 0; i < h->nY; ++i) all = all && masks[(size_t)t * h->nY + i];
    if (!all && ((a.dense_mask >> t) & 1u)) {
      wg::ozaki_free(a.dense[t]);
      a.dense_mask &= ~(1u << t);
    }
  }
  return WG_OK;
}

int wg2d_set_hard_wall(wg2d_problem* h, const unsigned char* active, const double* projection, double scale) {
  if (!h) return WG_ERR_ARG;
  cudaStreamSynchronize(h->stream);
  void* old[] = {h->wall_act, h->wall_T, h->wall_T32, h->wall_u, h->wall_u32};
  for (void* p : old)
    if (p) cudaFree(p);
  h->wall_act = nullptr;
  h->wall_T = nullptr;
  h->wall_T32 = nullptr;
  h->wall_u = nullptr;
  h->wall_u32 = nullptr;
  h->wall = false;
  if (!active) return WG_OK;
  if (!projection || !(scale > 0) || !std::isfinite(scale))
    return fail(h, WG_ERR_ARG, "wg2d_set_hard_wall: projection required and scale positive and finite");
  if (h->s.periodic_y) return fail(h, WG_ERR_ARG, "wg2d_set_hard_wall: the Y axis is periodic");
  const long long na = (long long)h->nY * h->nry;
  const long long nt = (long long)h->s.n_el_y * h->nry * h->s.nk_y * h->s.nk_y;
  std::vector<float> t32(projection, projection + nt);
  F2_CK(cudaMalloc(&h->wall_act, na));
  F2_CK(dalloc(&h->wall_T, nt));
  F2_CK(dalloc(&h->wall_T32, nt));
  F2_CK(dalloc(&h->wall_u, h->n));
  F2_CK(dalloc(&h->wall_u32, h->n));
  F2_CK(cudaMemcpy(h->wall_act, active, na, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(h->wall_T, projection, sizeof(double) * nt, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(h->wall_T32, t32.data(), sizeof(float) * nt, cudaMemcpyHostToDevice));
  h->wall_scale = scale;
  h->wall = true;
  return WG_OK;
}

int wg2d_apply(wg2d_problem* h, const double* x, double* y) {
  if (!h || !x || !y) return h ? fail(h, WG_ERR_ARG, "wg2d_apply: null argument") : WG_ERR_ARG;
  F2_CK(cudaMemcpyAsync(h->x, x, sizeof(double2) * h->n, cudaMemcpyHostToDevice, h->stream));
  const int rc = apply_device(h);
  if (rc) return rc;
  F2_CK(cudaMemcpyAsync(y, h->y, sizeof(double2) * h->n, cudaMemcpyDeviceToHost, h->stream));
  int flag = 0;
  F2_CK(cudaMemcpyAsync(&flag, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  if (flag) return fail(h, WG_ERR_TIMEOUT, "tensor-core GEMM: bounded barrier wait timed out");
  return WG_OK;
}

int wg2d_apply_repeat(wg2d_problem* h, int n, double* ms, double* parts_ms) {
  if (!h || n < 1 || !ms) return h ? fail(h, WG_ERR_ARG, "wg2d_apply_repeat: n >= 1 and ms required") : WG_ERR_ARG;
  int rc = apply_device(h);      // warm-up
  if (rc) return rc;
  F2_CK(cudaEventRecord(h->ev[0], h->stream));
  for (int i = 0; i < n && !rc; ++i) rc = apply_device(h);
  if (rc) return rc;
  F2_CK(cudaEventRecord(h->ev[1], h->stream));
  F2_CK(cudaEventSynchronize(h->ev[1]));
  float t = 0.f;
  F2_CK(cudaEventElapsedTime(&t, h->ev[0], h->ev[1]));
  *ms = t / n;
  int flag = 0;
  F2_CK(cudaMemcpy(&flag, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) return fail(h, WG_ERR_TIMEOUT, "tensor-core GEMM: bounded barrier wait timed out");
  if (parts_ms) {
    F2_CK(cudaEventRecord(h->ev[0], h->stream));
    rc = apply_drift(h);
    F2_CK(cudaEventRecord(h->ev[1], h->stream));
    if (!rc) rc = apply_transport(h, 0);
    if (!rc) rc = apply_transport(h, 1);
    F2_CK(cudaEventRecord(h->ev[2], h->stream));
    if (rc) return rc;
    F2_CK(cudaEventSynchronize(h->ev[2]));
    float a = 0.f, b = 0.f;
    F2_CK(cudaEventElapsedTime(&a, h->ev[0], h->ev[1]));
    F2_CK(cudaEventElapsedTime(&b, h->ev[1], h->ev[2]));
    parts_ms[0] = b;
    parts_ms[1] = a;
  }
  return WG_OK;
}


static void free32(wg2d_problem* h) {
  void* ptrs[] = {h->blocks32[0], h->blocks32[1], h->coef32[0], h->coef32[1], h->val32[0], h->val32[1], h->interp32,
                  h->proj32, h->cap32, h->dV32, h->Uq32, h->Rq32, h->G32, h->V32, h->Z32, h->w32, h->Vh32, h->vj32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h->blocks32[0] = h->blocks32[1] = h->coef32[0] = h->coef32[1] = nullptr;
  h->val32[0] = h->val32[1] = nullptr;
  h->interp32 = h->proj32 = h->cap32 = h->dV32 = nullptr;
  h->Uq32 = h->Rq32 = h->G32 = h->V32 = h->Z32 = h->w32 = h->vj32 = nullptr;
  h->Vh32 = nullptr;
  h->vm32 = 0;
  h->d32_ready = false;
}

// FP32 copies of the operator (rebuilt after any change of its factors or of the potential)
static int ensure32(wg2d_problem* h) {
  if (h->d32_ready) return WG_OK;
  const int vm = h->vm32;
  float2 *V = h->V32, *Z = h->Z32, *w = h->w32, *vj = h->vj32;
  __half2* Vh = h->Vh32;
  h->V32 = h->Z32 = h->w32 = h->vj32 = nullptr;
  h->Vh32 = nullptr;
  free32(h);
  h->V32 = V;
  h->Z32 = Z;
  h->w32 = w;
  h->vj32 = vj;
  h->Vh32 = Vh;
  h->vm32 = vm;
  auto conv = [&](float** dst, const double* src, long long count) -> int {
    F2_CK(dalloc(dst, count));
    f2d_d2f<<<(unsigned)((count + 255) / 256), 256, 0, h->stream>>>(src, *dst, count);
    return WG_OK;
  };
  for (int a = 0; a < 2; ++a) {
    wg2d_problem::Axis& ax = h->ax[a];
    if (!ax.T) continue;
    const int nk = a == 0 ? h->s.nk_x : h->s.nk_y, ne = a == 0 ? h->s.n_el_x : h->s.n_el_y;
    const int nr = a == 0 ? h->nrx : h->nry;
    int nnz = 0;
    std::vector<int> rp((size_t)ax.T * (nr + 1));
    F2_CK(cudaMemcpy(rp.data(), ax.rp, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost));
    for (int t = 0; t < ax.T; ++t) nnz += rp[(size_t)t * (nr + 1) + nr];
    int rc = conv(&h->blocks32[a], ax.blocks, (long long)ax.T * ne * 3 * nk * nk);
    if (!rc) rc = conv(&h->coef32[a], ax.dcoef, ax.T);
    if (!rc) rc = conv(reinterpret_cast<float**>(&h->val32[a]), reinterpret_cast<const double*>(ax.val), 2LL * nnz);
    if (rc) return rc;
  }
  const long long slab = (long long)h->nel * h->nq;
  int rc = conv(&h->interp32, h->interp, (long long)h->nq * h->nloc);
  if (!rc) rc = conv(&h->proj32, h->proj, (long long)h->nq * h->nloc);
  if (!rc) rc = conv(&h->cap32, h->cap, h->nrel);
  if (!rc) rc = conv(&h->dV32, h->dV, slab * h->nvert);
  if (rc) return rc;
  F2_CK(dalloc(&h->Uq32, slab * h->nrel));
  F2_CK(dalloc(&h->Rq32, slab * h->nrel));
  F2_CK(dalloc(&h->G32, (size_t)std::max(1, std::max(h->ax[0].T, h->ax[1].T)) * h->n));
  if (h->nrx * kRelxCols * sizeof(float2) > 48 * 1024)
    F2_CK(cudaFuncSetAttribute(f2d_relx_kernel<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(h->nrx * kRelxCols * sizeof(float2))));
  F2_CK(cudaStreamSynchronize(h->stream));
  h->d32_ready = true;
  return WG_OK;
}

}  // extern "C"

OpData<float2, float> op32(wg2d_problem* h) {
  OpData<float2, float> d;
  for (int a = 0; a < 2; ++a) {
    d.blocks[a] = h->blocks32[a];
    d.val[a] = h->val32[a];
    d.coef[a] = h->coef32[a];
  }
  d.interp = h->interp32;
  d.proj = h->proj32;
  d.cap = h->cap32;
  d.dV = h->dV32;
  d.Uq = h->Uq32;
  d.Rq = h->Rq32;
  d.G = h->G32;
  d.pot16 = make_float2((float)(h->pot.x / 16.0), (float)(h->pot.y / 16.0));
  d.capc = (float)h->capc;
  return d;
}

extern "C" {

// out = A in in FP32 (every term on the CUDA cores, the dense abs(A_x) factor included)
static int apply32(wg2d_problem* h, const float2* in, float2* out) {
  const OpData<float2, float> d = op32(h);
  const float2* src = in;
  if (h->wall) {
    f2d_wall_mask_kernel<float2><<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(in, h->wall_u32,
                                                                                    h->wall_act, h->nrx, h->nry,
                                                                                    h->nX, h->n);
    src = h->wall_u32;
  }
  drift_terms<float2, float>(h, d, src, out);
  for (int a = 0; a < 2; ++a)
    if (h->ax[a].T) transport_terms<float2, float>(h, a, d, src, out, 0u);
  F2_CK(cudaGetLastError());
  if (h->wall) return wall_project<float2, float>(h, out, in, h->wall_T32);
  return WG_OK;
}

// real embedding of a complex row-major n x n matrix scaled by a: [[re, -im], [im, re]] per entry
static std::vector<double> embed(const double* A, int n, double a, bool conj_transpose) {
  std::vector<double> E((size_t)4 * n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const size_t src = conj_transpose ? ((size_t)j * n + i) : ((size_t)i * n + j);
      const double re = a * A[2 * src], im = (conj_transpose ? -a : a) * A[2 * src + 1];
      E[(size_t)(2 * i) * 2 * n + 2 * j] = re;
      E[(size_t)(2 * i) * 2 * n + 2 * j + 1] = -im;
      E[(size_t)(2 * i + 1) * 2 * n + 2 * j] = im;
      E[(size_t)(2 * i + 1) * 2 * n + 2 * j + 1] = re;
    }
  return E;
}

int wg2d_set_preconditioner(wg2d_problem* h, const double* U, double sigma, const double* x_inverse,
                            const double* x_coupling, const int* forward, const double* t_inverse, int fp32) {
  if (!h) return WG_ERR_ARG;
  if (!U || !x_inverse || !x_coupling || !forward || !t_inverse || !(sigma > 0) || !std::isfinite(sigma))
    return fail(h, WG_ERR_ARG, "wg2d_set_preconditioner: null argument or sigma not positive and finite");
  const int nT = h->nry * h->nY;
  const size_t tsm64 = sizeof(double2) * ((size_t)nT * nT + (size_t)nT * kTxTile);
  const size_t tsm = fp32 ? tsm64 / 2 : tsm64;
  if (tsm > 220 * 1024)
    return fail(h, WG_ERR_ARG, "wg2d_set_preconditioner: transverse block n_rho_y * n_Y too large");
  cudaStreamSynchronize(h->stream);
  free_preconditioner(h);
  h->nT = nT;
  h->sigma = sigma;
  const int nr = h->nrx, nk = h->s.nk_x, ne = h->s.n_el_x;
  const size_t nx = (size_t)nr * ne * nk * nk, nt = (size_t)nr * nT * nT;
  // X-line sweep in chunks of L elements (about 16 chunks, at least 4 elements each);
  // WG_XLINE_CHUNKS=<n> sets the chunk count, 0 or 1 keeps one sequential sweep per line
  {
    int C = ne >= 8 ? std::min(16, ne / 4) : 1;
    if (const char* env = getenv("WG_XLINE_CHUNKS")) C = std::max(1, std::min(atoi(env), ne));
    const int L = (ne + C - 1) / std::max(1, C);
    h->x_chunk_len = L;
    h->x_chunks = C > 1 ? (ne + L - 1) / L : 1;
    if (h->x_chunks > 1)
      F2_CK(dalloc(&h->xmaps, (size_t)h->x_chunks * (nk * nk + nk) * ((size_t)nr * h->nry * h->nY)));
  }
  F2_CK(dalloc(&h->fwd, nr));
  F2_CK(cudaMemcpy(h->fwd, forward, sizeof(int) * nr, cudaMemcpyHostToDevice));
  // U^H and U / sigma as complex [nr][nr] row-major
  std::vector<double> uh((size_t)2 * nr * nr), us((size_t)2 * nr * nr);
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nr; ++j) {
      uh[2 * ((size_t)i * nr + j)] = U[2 * ((size_t)j * nr + i)];
      uh[2 * ((size_t)i * nr + j) + 1] = -U[2 * ((size_t)j * nr + i) + 1];
      us[2 * ((size_t)i * nr + j)] = U[2 * ((size_t)i * nr + j)] / sigma;
      us[2 * ((size_t)i * nr + j) + 1] = U[2 * ((size_t)i * nr + j) + 1] / sigma;
    }
  if (fp32) {
    auto up32 = [&](float2** dst, const double* src, size_t count) -> int {
      std::vector<float> f(2 * count);
      for (size_t i = 0; i < 2 * count; ++i) f[i] = (float)src[i];
      F2_CK(dalloc(dst, count));
      F2_CK(cudaMemcpy(*dst, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
      return WG_OK;
    };
    int rc = up32(&h->xinv32, x_inverse, nx);
    if (!rc) rc = up32(&h->xcpl32, x_coupling, nx);
    if (!rc) rc = up32(&h->tinv32, t_inverse, nt);
    if (!rc) rc = up32(&h->UH32, uh.data(), (size_t)nr * nr);
    if (!rc) rc = up32(&h->Us32, us.data(), (size_t)nr * nr);
    if (rc) return rc;
    F2_CK(dalloc(&h->pa32, h->n));
    F2_CK(dalloc(&h->pb32, h->n));
    F2_CK(cudaFuncSetAttribute(f2d_transverse_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    if (h->nrx * kRelxCols * sizeof(float2) > 48 * 1024)
      F2_CK(cudaFuncSetAttribute(f2d_dense_rx_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(h->nrx * kRelxCols * sizeof(float2))));
    h->pre32 = true;
    h->pre_ready = true;
    return WG_OK;
  }
  F2_CK(dalloc(&h->xinv, nx));
  F2_CK(dalloc(&h->xcpl, nx));
  F2_CK(dalloc(&h->tinv, nt));
  F2_CK(dalloc(&h->pa, h->n));
  F2_CK(dalloc(&h->pb, h->n));
  F2_CK(cudaMemcpy(h->xinv, x_inverse, sizeof(double2) * nx, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(h->xcpl, x_coupling, sizeof(double2) * nx, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(h->tinv, t_inverse, sizeof(double2) * nt, cudaMemcpyHostToDevice));
  F2_CK(cudaFuncSetAttribute(f2d_transverse_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
  if (h->nrx * kRelxCols * sizeof(double2) > 48 * 1024)
    F2_CK(cudaFuncSetAttribute(f2d_dense_rx_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(h->nrx * kRelxCols * sizeof(double2))));
  if (h->s.tensor_cores) {
    int rc = wg::ozaki_rows_upload(embed(U, nr, 1.0, true), 2 * nr, 2 * nr, h->UH, h->err);
    if (!rc) rc = wg::ozaki_rows_upload(embed(U, nr, 1.0 / sigma, false), 2 * nr, 2 * nr, h->Us, h->err);
    if (!rc && !h->cols.dig) rc = wg::ozaki_cols_alloc(h->n / nr, 2 * nr, h->cols, h->err);
    if (rc) return rc;
  } else {
    F2_CK(dalloc(&h->UHd, (size_t)nr * nr));
    F2_CK(dalloc(&h->Usd, (size_t)nr * nr));
    F2_CK(cudaMemcpy(h->UHd, uh.data(), sizeof(double) * uh.size(), cudaMemcpyHostToDevice));
    F2_CK(cudaMemcpy(h->Usd, us.data(), sizeof(double) * us.size(), cudaMemcpyHostToDevice));
  }
  h->pre_ready = true;
  return WG_OK;
}

int wg2d_precondition(wg2d_problem* h, const double* r, double* z) {
  if (!h || !r || !z) return h ? fail(h, WG_ERR_ARG, "wg2d_precondition: null argument") : WG_ERR_ARG;
  F2_CK(cudaMemcpyAsync(h->x, r, sizeof(double2) * h->n, cudaMemcpyHostToDevice, h->stream));
  const int rc = precondition_device(h, h->x, h->y);
  if (rc) return rc;
  F2_CK(cudaMemcpyAsync(z, h->y, sizeof(double2) * h->n, cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  return WG_OK;
}

// Restarted flexible GMRES(m) (Saad's FGMRES: the preconditioned vectors are kept, so an FP32
// preconditioner does not limit the FP64 accuracy), right-preconditioned with the line-transverse
// preconditioner, classical Gram-Schmidt with a DGKS-gated second pass, FP64 (runGmresWithProgress of solve_transport_DG_full2D.m:422-506
// with MATLAB's gmres semantics: relative residual of the original system, warm start as x0).
int wg2d_solve(wg2d_problem* h, const double* rhs, double* x, const wg2d_solve_opts* opts, wg2d_solve_info* info) {
  if (!h) return WG_ERR_ARG;
  if (!opts || !info) return fail(h, WG_ERR_ARG, "wg2d_solve: null argument");
  const int m = opts->restart > 0 ? opts->restart : 40;
  const int maxit = opts->maxit > 0 ? opts->maxit : 50;
  const double tol = opts->tol > 0 ? opts->tol : 1e-8;
  if (m > 256) return fail(h, WG_ERR_ARG, "wg2d_solve: restart at most 256");
  if (!h->potential_ready) return fail(h, WG_ERR_ARG, "wg2d_solve: set the potential first");
  const long long n = h->n;
  if (!rhs && !h->b_ready) return fail(h, WG_ERR_ARG, "wg2d_solve: rhs = NULL needs the right-hand side of a previous solve");
  if (!x && opts->use_x0 && !h->xs_ready)
    return fail(h, WG_ERR_ARG, "wg2d_solve: x = NULL with use_x0 needs the resident solution of a previous solve");
  if (h->vm < m + 1) {
    // the right-hand side and the solution stay resident across a change of the restart length
    double2* keep_b = h->b;
    double2* keep_xs = h->xs;
    h->b = h->xs = nullptr;
    free_solver(h);
    h->b = keep_b;
    h->xs = keep_xs;
    const size_t need = (size_t)(2 * m + 1) * n * sizeof(double2);
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    if (need + 6 * n * sizeof(double2) > freeb) return fail(h, WG_ERR_OOM, "wg2d_solve: Krylov basis does not fit");
    F2_CK(dalloc(&h->V, (size_t)(m + 1) * n));
    F2_CK(dalloc(&h->Zb, (size_t)m * n));
    F2_CK(dalloc(&h->r, n));
    F2_CK(dalloc(&h->w, n));
    F2_CK(dalloc(&h->z, n));
    if (!h->b) F2_CK(dalloc(&h->b, n));
    if (!h->xs) F2_CK(dalloc(&h->xs, n));
    F2_CK(dalloc(&h->H, (size_t)(m + 1) * m));
    F2_CK(dalloc(&h->g, m + 1));
    F2_CK(dalloc(&h->sn, m));
    F2_CK(dalloc(&h->hc, m + 1));
    F2_CK(dalloc(&h->hp, m + 1));
    F2_CK(dalloc(&h->yc, m));
    F2_CK(dalloc(&h->cs, m));
    F2_CK(dalloc(&h->partial, (size_t)2 * kDotBlocks * (m + 1)));
    F2_CK(dalloc(&h->nrm, 1));
    h->vm = m + 1;
  }
  std::memset(info, 0, sizeof(*info));
  h->resvec.clear();
  if (rhs) {
    h->b_ready = false;
    F2_CK(cudaMemcpyAsync(h->b, rhs, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
    h->b_ready = true;
  }
  h->xs_ready = false;
  if (opts->use_x0) {
    if (x) F2_CK(cudaMemcpyAsync(h->xs, x, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
  } else {
    F2_CK(cudaMemsetAsync(h->xs, 0, sizeof(double2) * n, h->stream));
  }
  double bnorm = 0, beta = 0;
  vnorm(h, h->b);
  F2_CK(cudaMemcpyAsync(&bnorm, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  auto true_residual = [&]() -> int {
    int rc = apply_op(h, h->xs, h->r);
    if (rc) return rc;
    f2d_sub<<<blocks256(n), 256, 0, h->stream>>>(h->b, h->r, n);
    vnorm(h, h->r);
    F2_CK(cudaMemcpyAsync(&beta, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    F2_CK(cudaStreamSynchronize(h->stream));
    return WG_OK;
  };
  int rc = true_residual();
  if (rc) return rc;
  h->resvec.push_back(beta);
  info->rhs_norm = bnorm;
  const double bn = bnorm > 0 ? bnorm : 1.0;
  info->initial_relres = beta / bn;
  const double target = tol * bn;
  const int ldh = m + 1;
  int info_reorth = 0;
  if (opts->mixed) {
    // FP64 iterative refinement around an FP32 flexible GMRES on the FP32 operator: the FP64
    // residual r = b - A x decides convergence, each refinement solves A d = r / |r| in FP32 to
    // max(inner_tol, 0.5 target / |r|) and adds |r| d in FP64.
    if (!h->pre32) return fail(h, WG_ERR_ARG, "wg2d_solve: the mixed form needs the FP32 preconditioner");
    rc = ensure32(h);
    if (rc) return rc;
    const int mi = m;
    // the inner basis in FP32 (default) or FP16 storage with FP32 arithmetic (inner_basis_fp16)
    const bool b16 = opts->inner_basis_fp16 != 0;
    if (h->vm32 < mi + 1 || h->vbasis16 != b16) {
      for (void* p : {(void*)h->V32, (void*)h->Vh32, (void*)h->vj32, (void*)h->Z32, (void*)h->w32})
        if (p) cudaFree(p);
      h->V32 = h->Z32 = h->w32 = h->vj32 = nullptr;
      h->Vh32 = nullptr;
      h->vm32 = 0;
      if (b16) {
        F2_CK(dalloc(&h->Vh32, (size_t)(mi + 1) * n));
        F2_CK(dalloc(&h->vj32, n));
      } else {
        F2_CK(dalloc(&h->V32, (size_t)(mi + 1) * n));
      }
      F2_CK(dalloc(&h->Z32, (size_t)mi * n));
      F2_CK(dalloc(&h->w32, n));
      h->vm32 = mi + 1;
      h->vbasis16 = b16;
    }
    const double inner_tol = opts->inner_tol > 0 ? opts->inner_tol : 1e-3;
    while (info->cycles < maxit && beta > target && std::isfinite(beta)) {
      if (b16) f2d_to16_scaled<<<blocks256(n), 256, 0, h->stream>>>(h->r, h->Vh32, h->vj32, h->nrm, n);
      else f2d_to32_scaled<<<blocks256(n), 256, 0, h->stream>>>(h->r, h->V32, h->nrm, n);
      const double2 one = make_double2(1.0, 0.0);
      F2_CK(cudaMemsetAsync(h->g, 0, sizeof(double2) * (m + 1), h->stream));
      F2_CK(cudaMemcpyAsync(h->g, &one, sizeof(double2), cudaMemcpyHostToDevice, h->stream));
      const double itgt = std::max(inner_tol, 0.5 * target / beta);
      int k = 0, j_cur = 0;
      // the basis as the Gram-Schmidt kernels read it
      auto gs_dots = [&](double2* out) {
        if (b16) dots32(h, h->Vh32, j_cur + 1, h->w32, out, 0);
        else dots32(h, h->V32, j_cur + 1, h->w32, out, 0);
      };
      auto gs_update = [&](const double2* coef) {
        if (b16) f2d_gs_update32<<<blocks256(n), 256, 0, h->stream>>>(h->Vh32, n, h->w32, coef, j_cur + 1, n);
        else f2d_gs_update32<<<blocks256(n), 256, 0, h->stream>>>(h->V32, n, h->w32, coef, j_cur + 1, n);
      };
      for (int j = 0; j < mi; ++j) {
        j_cur = j;
        // the preconditioner works on the basis vector as stored (its FP32 copy with an FP16 basis)
        const float2* Vj = b16 ? h->vj32 : h->V32 + (long long)j * n;
        float2* Zj = h->Z32 + (long long)j * n;
        precond_stages<float2>(h, h->UH32, h->Us32, h->xinv32, h->xcpl32, h->tinv32, Vj, h->pa32, h->pb32, Zj);
        rc = apply32(h, Zj, h->w32);
        if (rc) return rc;
        gs_dots(h->hc);
        gs_update(h->hc);
        vnorm32(h, h->w32);
        std::vector<double2> hh(j + 1);
        double w1 = 0;
        F2_CK(cudaMemcpyAsync(hh.data(), h->hc, sizeof(double2) * (j + 1), cudaMemcpyDeviceToHost, h->stream));
        F2_CK(cudaMemcpyAsync(&w1, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        F2_CK(cudaStreamSynchronize(h->stream));
        double h2 = 0;
        for (const double2& c : hh) h2 += c.x * c.x + c.y * c.y;
        if (w1 * w1 < 0.5 * (w1 * w1 + h2)) {
          gs_dots(h->hp);
          f2d_dot_reduce<<<j + 1, 256, 0, h->stream>>>(h->partial, h->hc, kDotBlocks, 1);
          gs_update(h->hp);
          vnorm32(h, h->w32);
        }
        f2d_givens<<<1, 1, 0, h->stream>>>(h->H, h->hc, h->nrm, h->cs, h->sn, h->g, j, ldh);
        if (b16)
          f2d_scale16<<<blocks256(n), 256, 0, h->stream>>>(h->w32, h->Vh32 + (long long)(j + 1) * n, h->vj32,
                                                           h->nrm, n);
        else
          f2d_scale32<<<blocks256(n), 256, 0, h->stream>>>(h->w32, h->V32 + (long long)(j + 1) * n, h->nrm, n);
        double2 gj;
        F2_CK(cudaMemcpyAsync(&gj, h->g + j + 1, sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
        F2_CK(cudaStreamSynchronize(h->stream));
        k = j + 1;
        info->iterations += 1;
        h->resvec.push_back(beta * std::hypot(gj.x, gj.y));
        if (!(std::hypot(gj.x, gj.y) > itgt)) break;
      }
      f2d_backsolve<<<1, 1, 0, h->stream>>>(h->H, h->g, h->yc, k, ldh);
      F2_CK(cudaMemcpyAsync(h->nrm, &beta, sizeof(double), cudaMemcpyHostToDevice, h->stream));
      f2d_correct32<<<blocks256(n), 256, 0, h->stream>>>(h->xs, h->Z32, n, h->yc, k, h->nrm, n);
      info->cycles += 1;
      rc = true_residual();
      if (rc) return rc;
    }
  }
  while (!opts->mixed && info->cycles < maxit && beta > target && std::isfinite(beta)) {
    f2d_scale<<<blocks256(n), 256, 0, h->stream>>>(h->r, h->V, h->nrm, n);
    const double2 g0 = make_double2(beta, 0.0);
    F2_CK(cudaMemsetAsync(h->g, 0, sizeof(double2) * (m + 1), h->stream));
    F2_CK(cudaMemcpyAsync(h->g, &g0, sizeof(double2), cudaMemcpyHostToDevice, h->stream));
    int k = 0;
    for (int j = 0; j < m; ++j) {
      double2* Vj = h->V + (long long)j * n;
      double2* Zj = h->Zb + (long long)j * n;      // flexible GMRES: keep z_j = M^-1 v_j
      if (h->pre_ready) rc = precondition_device(h, Vj, Zj);      // no preconditioner set: identity
      else F2_CK(cudaMemcpyAsync(Zj, Vj, sizeof(double2) * n, cudaMemcpyDeviceToDevice, h->stream));
      if (!rc) rc = apply_op(h, Zj, h->w);
      if (rc) return rc;
      // classical Gram-Schmidt; a second pass only when the first lost more than half of |w|^2
      // (Daniel-Gragg-Kaufman-Stewart: |w'|^2 < eta^2 (|w'|^2 + |h|^2), eta = 1/sqrt(2))
      dots(h, h->V, j + 1, h->w, h->hc, 0);
      f2d_gs_update<<<blocks256(n), 256, 0, h->stream>>>(h->V, n, h->w, h->hc, j + 1, n);
      vnorm(h, h->w);
      std::vector<double2> hh(j + 1);
      double w1 = 0;
      F2_CK(cudaMemcpyAsync(hh.data(), h->hc, sizeof(double2) * (j + 1), cudaMemcpyDeviceToHost, h->stream));
      F2_CK(cudaMemcpyAsync(&w1, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      F2_CK(cudaStreamSynchronize(h->stream));
      double h2 = 0;
      for (const double2& c : hh) h2 += c.x * c.x + c.y * c.y;
      if (w1 * w1 < 0.5 * (w1 * w1 + h2)) {
        dots(h, h->V, j + 1, h->w, h->hp, 0);    // second pass
        f2d_dot_reduce<<<j + 1, 256, 0, h->stream>>>(h->partial, h->hc, kDotBlocks, 1);   // hc += hp
        f2d_gs_update<<<blocks256(n), 256, 0, h->stream>>>(h->V, n, h->w, h->hp, j + 1, n);
        vnorm(h, h->w);
        info_reorth += 1;
      }
      f2d_givens<<<1, 1, 0, h->stream>>>(h->H, h->hc, h->nrm, h->cs, h->sn, h->g, j, ldh);
      f2d_scale<<<blocks256(n), 256, 0, h->stream>>>(h->w, h->V + (long long)(j + 1) * n, h->nrm, n);
      double2 gj;
      F2_CK(cudaMemcpyAsync(&gj, h->g + j + 1, sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
      F2_CK(cudaStreamSynchronize(h->stream));
      k = j + 1;
      info->iterations += 1;
      const double est = std::hypot(gj.x, gj.y);
      h->resvec.push_back(est);
      if (!(est > target)) break;
    }
    f2d_backsolve<<<1, 1, 0, h->stream>>>(h->H, h->g, h->yc, k, ldh);
    f2d_combine<<<blocks256(n), 256, 0, h->stream>>>(h->Zb, n, h->yc, h->z, k, n);   // x += Z y
    f2d_axpy<<<blocks256(n), 256, 0, h->stream>>>(h->xs, h->z, n);
    info->cycles += 1;
    rc = true_residual();
    if (rc) return rc;
  }
  int flag = 0;
  if (x) F2_CK(cudaMemcpyAsync(x, h->xs, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaMemcpyAsync(&flag, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  if (flag) return fail(h, WG_ERR_TIMEOUT, "tensor-core GEMM: bounded barrier wait timed out");
  h->xs_ready = true;
  info->relres = beta / bn;
  if (!std::isfinite(beta)) return fail(h, WG_ERR_NUMERIC, "wg2d_solve: non-finite residual");
  info->flag = beta <= target ? 0 : 1;
  return info->flag ? WG_NOT_CONVERGED : WG_OK;
}

// Preconditioned BiCGSTAB (van der Vorst), right-preconditioned as MATLAB's bicgstab(A, b, tol, maxit, M)
// that runBicgstabWithProgress calls (solve_transport_DG_full2D.m:248-272, 367-420): M^-1 is the
// line-transverse preconditioner when one is set, the identity otherwise.  maxit counts full iterations;
// convergence is tested after each half step on |s| and |r| against tol |b|, and the final true residual
// b - A x decides the flag.  info->cycles: half steps done (MATLAB's iter = cycles / 2); info->iterations:
// full iterations begun.  The resvec holds the initial residual and the norm after every half step.
int wg2d_solve_bicgstab(wg2d_problem* h, const double* rhs, double* x, const wg2d_solve_opts* opts,
                        wg2d_solve_info* info) {
  if (!h) return WG_ERR_ARG;
  if (!opts || !info) return fail(h, WG_ERR_ARG, "wg2d_solve_bicgstab: null argument");
  if (!h->potential_ready) return fail(h, WG_ERR_ARG, "wg2d_solve_bicgstab: set the potential first");
  const int maxit = opts->maxit > 0 ? opts->maxit : 50;
  const double tol = opts->tol > 0 ? opts->tol : 1e-8;
  const long long n = h->n;
  if (!rhs && !h->b_ready) return fail(h, WG_ERR_ARG, "wg2d_solve_bicgstab: rhs = NULL needs a previous right-hand side");
  if (!x && opts->use_x0 && !h->xs_ready)
    return fail(h, WG_ERR_ARG, "wg2d_solve_bicgstab: x = NULL with use_x0 needs a resident solution");
  {
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    int missing = 0;
    for (double2* p : {h->r, h->w, h->z, h->b, h->xs, h->bc_rt, h->bc_p, h->bc_ph, h->bc_sh}) missing += p ? 0 : 1;
    if ((size_t)missing * n * sizeof(double2) > freeb)
      return fail(h, WG_ERR_OOM, "wg2d_solve_bicgstab: BiCGSTAB vectors do not fit");
  }
  for (double2** p : {&h->r, &h->w, &h->z, &h->b, &h->xs, &h->bc_rt, &h->bc_p, &h->bc_ph, &h->bc_sh})
    if (!*p) F2_CK(dalloc(p, n));
  if (!h->hc) F2_CK(dalloc(&h->hc, 2));
  if (!h->hp) F2_CK(dalloc(&h->hp, 2));
  if (!h->partial) F2_CK(dalloc(&h->partial, (size_t)2 * kDotBlocks * 2));
  if (!h->nrm) F2_CK(dalloc(&h->nrm, 1));
  std::memset(info, 0, sizeof(*info));
  h->resvec.clear();
  if (rhs) {
    h->b_ready = false;
    F2_CK(cudaMemcpyAsync(h->b, rhs, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
    h->b_ready = true;
  }
  h->xs_ready = false;
  if (opts->use_x0) {
    if (x) F2_CK(cudaMemcpyAsync(h->xs, x, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
  } else {
    F2_CK(cudaMemsetAsync(h->xs, 0, sizeof(double2) * n, h->stream));
  }
  const unsigned nb = blocks256(n);
  auto read_dot = [&](const double2* a, const double2* b, double2* out) -> int {
    dots(h, a, 1, b, h->hc, 0);
    F2_CK(cudaMemcpyAsync(out, h->hc, sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    F2_CK(cudaStreamSynchronize(h->stream));
    return WG_OK;
  };
  auto norm_of = [&](const double2* v, double* out) -> int {
    vnorm(h, v);
    F2_CK(cudaMemcpyAsync(out, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    F2_CK(cudaStreamSynchronize(h->stream));
    return WG_OK;
  };
  auto prec = [&](const double2* in, double2* out) -> int {
    if (h->pre_ready) return precondition_device(h, in, out);
    F2_CK(cudaMemcpyAsync(out, in, sizeof(double2) * n, cudaMemcpyDeviceToDevice, h->stream));
    return WG_OK;
  };
  double bnorm = 0, beta = 0;
  int rc = norm_of(h->b, &bnorm);
  if (rc) return rc;
  auto true_residual = [&]() -> int {
    int e = apply_op(h, h->xs, h->r);
    if (e) return e;
    f2d_sub<<<nb, 256, 0, h->stream>>>(h->b, h->r, n);
    return norm_of(h->r, &beta);
  };
  // the iteration runs on the system scaled by 1/|b| (the FP32 preconditioner would overflow on
  // the physical magnitudes, cf. the RHS normalisation of solveStationarySystem :299-304); the
  // resident b and x are scaled back afterwards
  const double bn = bnorm > 0 ? bnorm : 1.0;
  f2d_rscale<<<nb, 256, 0, h->stream>>>(h->b, 1.0 / bn, n);
  f2d_rscale<<<nb, 256, 0, h->stream>>>(h->xs, 1.0 / bn, n);
  struct Unscale {
    wg2d_problem* h;
    double bn;
    unsigned nb;
    ~Unscale() {
      f2d_rscale<<<nb, 256, 0, h->stream>>>(h->b, bn, h->n);
      f2d_rscale<<<nb, 256, 0, h->stream>>>(h->xs, bn, h->n);
    }
  };
  rc = true_residual();
  if (rc) return rc;
  h->resvec.push_back(beta * bn);
  info->rhs_norm = bnorm;
  info->initial_relres = beta;
  const double target = tol;
  {
  Unscale unscale{h, bn, nb};
  if (beta > target && std::isfinite(beta)) {
    auto cdiv = [](double2 a, double2 b) {
      const double d = b.x * b.x + b.y * b.y;
      return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
    };
    auto cmulh = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    F2_CK(cudaMemcpyAsync(h->bc_rt, h->r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, h->stream));
    double2 rho = make_double2(1, 0), alpha = make_double2(1, 0), omega = make_double2(1, 0);
    for (int it = 1; it <= maxit; ++it) {
      info->iterations = it;
      double2 rho1;
      if ((rc = read_dot(h->bc_rt, h->r, &rho1))) return rc;
      if (rho1.x == 0.0 && rho1.y == 0.0) break;                     // breakdown: flag stays 1
      if (it == 1) {
        F2_CK(cudaMemcpyAsync(h->bc_p, h->r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, h->stream));
      } else {
        const double2 bta = cmulh(cdiv(rho1, rho), cdiv(alpha, omega));
        f2d_bicg_p<<<nb, 256, 0, h->stream>>>(h->bc_p, h->r, h->w, bta, omega, n);
      }
      if ((rc = prec(h->bc_p, h->bc_ph))) return rc;
      if ((rc = apply_op(h, h->bc_ph, h->w))) return rc;              // v
      double2 rtv;
      if ((rc = read_dot(h->bc_rt, h->w, &rtv))) return rc;
      if (rtv.x == 0.0 && rtv.y == 0.0) break;
      alpha = cdiv(rho1, rtv);
      f2d_caxpy<<<nb, 256, 0, h->stream>>>(h->r, h->w, make_double2(-alpha.x, -alpha.y), n);   // s = r - alpha v
      double sn = 0;
      if ((rc = norm_of(h->r, &sn))) return rc;
      h->resvec.push_back(sn * bn);
      info->cycles += 1;
      if (!(sn > target) || !std::isfinite(sn)) {
        f2d_caxpy<<<nb, 256, 0, h->stream>>>(h->xs, h->bc_ph, alpha, n);
        break;
      }
      if ((rc = prec(h->r, h->bc_sh))) return rc;
      if ((rc = apply_op(h, h->bc_sh, h->z))) return rc;             // t
      double2 tt, ts;
      if ((rc = read_dot(h->z, h->z, &tt))) return rc;
      if ((rc = read_dot(h->z, h->r, &ts))) return rc;
      if (tt.x == 0.0) break;
      omega = make_double2(ts.x / tt.x, ts.y / tt.x);
      f2d_caxpy<<<nb, 256, 0, h->stream>>>(h->xs, h->bc_ph, alpha, n);
      f2d_caxpy<<<nb, 256, 0, h->stream>>>(h->xs, h->bc_sh, omega, n);
      f2d_caxpy<<<nb, 256, 0, h->stream>>>(h->r, h->z, make_double2(-omega.x, -omega.y), n);   // r = s - omega t
      double rn = 0;
      if ((rc = norm_of(h->r, &rn))) return rc;
      h->resvec.push_back(rn * bn);
      info->cycles += 1;
      if (!(rn > target) || !std::isfinite(rn)) break;
      if (omega.x == 0.0 && omega.y == 0.0) break;
      rho = rho1;
    }
    rc = true_residual();
    if (rc) return rc;
  }
  }   // b and x scaled back
  int flag = 0;
  if (x) F2_CK(cudaMemcpyAsync(x, h->xs, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaMemcpyAsync(&flag, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  if (flag) return fail(h, WG_ERR_TIMEOUT, "tensor-core GEMM: bounded barrier wait timed out");
  h->xs_ready = true;
  info->relres = beta;
  if (!std::isfinite(beta)) return fail(h, WG_ERR_NUMERIC, "wg2d_solve_bicgstab: non-finite residual");
  info->flag = beta <= target ? 0 : 1;
  return info->flag ? WG_NOT_CONVERGED : WG_OK;
}

int wg2d_get_state(wg2d_problem* h, double* x) {
  if (!h || !x) return h ? fail(h, WG_ERR_ARG, "wg2d_get_state: null argument") : WG_ERR_ARG;
  if (!h->xs_ready) return fail(h, WG_ERR_ARG, "wg2d_get_state: no resident solution");
  F2_CK(cudaMemcpyAsync(x, h->xs, sizeof(double2) * h->n, cudaMemcpyDeviceToHost, h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  return WG_OK;
}

int wg2d_solve_resvec(wg2d_problem* h, double* out, int cap, int* count) {
  if (!h || !count) return h ? fail(h, WG_ERR_ARG, "wg2d_solve_resvec: null count") : WG_ERR_ARG;
  *count = (int)h->resvec.size();
  if (out)
    for (int i = 0; i < cap && i < *count; ++i) out[i] = h->resvec[i];
  return WG_OK;
}

int wg2d_set_observables(wg2d_problem* h, const wg2d_observables_desc* d, const double* W, const double* wj) {
  if (!h) return WG_ERR_ARG;
  if (!d || !W || !wj) return fail(h, WG_ERR_ARG, "wg2d_set_observables: null argument");
  bool ok = d->n_zero_x >= 1 && d->n_zero_x <= 2 && d->n_zero_y >= 1 && d->n_zero_y <= 2 && d->n_dx >= 0 &&
            d->n_dx <= 8 && d->n_dy >= 0 && d->n_dy <= 8 && d->n_target_y >= 1;
  for (int i = 0; ok && i < d->n_zero_x; ++i) ok = d->zero_x[i] >= 0 && d->zero_x[i] < h->nrx;
  for (int i = 0; ok && i < d->n_zero_y; ++i) ok = d->zero_y[i] >= 0 && d->zero_y[i] < h->nry;
  for (int i = 0; ok && i < d->n_dx; ++i) ok = d->dx_idx[i] >= 0 && d->dx_idx[i] < h->nrx;
  for (int i = 0; ok && i < d->n_dy; ++i) ok = d->dy_idx[i] >= 0 && d->dy_idx[i] < h->nry;
  if (!ok) return fail(h, WG_ERR_ARG, "wg2d_set_observables: zero cells or derivative rows out of range");
  cudaStreamSynchronize(h->stream);
  void* old[] = {h->obs_W, h->obs_wj, h->obs_out};
  for (void* p : old)
    if (p) cudaFree(p);
  h->obs_W = h->obs_wj = h->obs_out = nullptr;
  h->obs_ready = false;
  const size_t nty = d->n_target_y;
  F2_CK(dalloc(&h->obs_W, nty * h->nY));
  F2_CK(dalloc(&h->obs_wj, nty));
  F2_CK(dalloc(&h->obs_out, (size_t)3 * h->nX * h->nY + (size_t)3 * h->nX * nty + h->nX));
  F2_CK(cudaMemcpy(h->obs_W, W, sizeof(double) * nty * h->nY, cudaMemcpyHostToDevice));
  F2_CK(cudaMemcpy(h->obs_wj, wj, sizeof(double) * nty, cudaMemcpyHostToDevice));
  h->obs = *d;
  h->obs_ready = true;
  return WG_OK;
}

int wg2d_observables(wg2d_problem* h, const double* rho, double* nDG, double* jxDG, double* jyDG, double* n,
                     double* jx, double* jy, double* j) {
  if (!h) return WG_ERR_ARG;
  if (!h->obs_ready) return fail(h, WG_ERR_ARG, "wg2d_observables: wg2d_set_observables was not called");
  const double2* F = h->xs;
  if (rho) {
    F2_CK(cudaMemcpyAsync(h->x, rho, sizeof(double2) * h->n, cudaMemcpyHostToDevice, h->stream));
    F = h->x;
  } else if (!h->xs_ready) {
    return fail(h, WG_ERR_ARG, "wg2d_observables: no resident solution (pass rho)");
  }
  f2d_observables_kernel<<<(h->nX + 127) / 128, 128, 0, h->stream>>>(F, h->obs, h->obs_W, h->obs_wj, h->nX, h->nY,
                                                                      h->nrx, h->nry, h->obs_out);
  F2_CK(cudaGetLastError());
  const size_t g = (size_t)h->nX * h->nY, t = (size_t)h->nX * h->obs.n_target_y;
  double* outs[] = {nDG, jxDG, jyDG, n, jx, jy, j};
  const size_t offs[] = {0, g, 2 * g, 3 * g, 3 * g + t, 3 * g + 2 * t, 3 * g + 3 * t};
  const size_t cnt[] = {g, g, g, t, t, t, (size_t)h->nX};
  for (int i = 0; i < 7; ++i)
    if (outs[i])
      F2_CK(cudaMemcpyAsync(outs[i], h->obs_out + offs[i], sizeof(double) * cnt[i], cudaMemcpyDeviceToHost,
                            h->stream));
  F2_CK(cudaStreamSynchronize(h->stream));
  return WG_OK;
}

}  // extern "C"
