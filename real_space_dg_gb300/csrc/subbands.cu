// Transverse subband eigensolve (mode space) on the device (sm_103a).
//
// For every valley v and x slice the reference builds the Ny x Ny finite-difference
// Hamiltonian of the confinement direction (eval_transversal_Hamiltonian.m:20-37) and asks
// eigs for the n_of_modes eigenpairs of smallest magnitude (solve_bandstructure.m:17-33),
// then fixes the signs of valley 1 against its first slice (solve_subbands.m:22-40).
//
// Ht is tridiagonal and symmetric except for its copied end rows; with positive
// off-diagonal products T = D^-1 Ht D is symmetric tridiagonal for a diagonal D
// (d_{i+1} / d_i = sqrt(Ht(i+1,i) / Ht(i,i+1))), with the same eigenvalues and the
// eigenvectors v = D w.  Per slice:
//   subband_slice_kernel    one warp per slice (problem, valley, x):
//     1. Ht's diagonal a, T's off-diagonal b, b^2 and the ratios of D in shared memory;
//     2. Sturm counts (signs of the LDL^T pivots of T - x) locate the eigenvalues with
//        index in [n0 - nm, n0 + nm), n0 = #(< 0), by multisection: the nc candidates
//        share the 32 lanes, g = 32 / nc lanes per candidate each counting at one of g
//        interior points, so an interval shrinks (g + 1)-fold per step;
//     3. the nm of smallest magnitude, a contiguous run around zero, ascending;
//     4. one lane per mode: the eigenvector of T from the twisted factorisation of
//        T - lambda (Dhillon and Parlett, "Orthogonal eigenvectors and relative gaps",
//        SIAM J. Matrix Anal. Appl. 25 (2004) 858-899): top-down pivots D+, bottom-up
//        pivots D-, the twist index r of smallest |gamma_r| = |D+_r + D-_r - (a_r - lambda)|,
//        then w_r = 1 and the one-term recurrences out of r; v = D w normalised in the
//        2-norm and signed by its last entry (solve_bandstructure.m:28-30).
//   subband_cleanup_kernel  one warp per (problem, x >= 1, mode) of valley 1: v -> -v when
//                           its overlap with the same mode of slice 1 is below -1/2.
// A handle solves a batch of independent problems (gate or bias points) in one launch.
// The pivots live in a scratch [slice][i][mode] (lanes = modes, coalesced).  All FP64.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <string>

#include "wigner_gb300.h"

namespace {

constexpr int kMaxModes = 32;
constexpr int kMaxNy = 1024;

struct SliceShared {
  double *a, *b, *b2, *rr, *lam;
  float *af, *b2f;   // FP32 copies of a and b^2 for the coarse bisection
};

// per warp: a, b, b2, rr [ny] doubles, lam [2 kMaxModes] doubles, af, b2f [ny] floats
__host__ __device__ constexpr int slice_doubles(int ny) { return 5 * ny + 2 * kMaxModes; }

__device__ __forceinline__ SliceShared slice_shared(double* base, int ny) {
  SliceShared s;
  s.a = base;
  s.b = base + ny;
  s.b2 = base + 2 * ny;
  s.rr = base + 3 * ny;
  s.lam = base + 4 * ny;
  s.af = reinterpret_cast<float*>(base + 4 * ny + 2 * kMaxModes);
  s.b2f = s.af + ny;
  return s;
}

__device__ __forceinline__ double guard(double q, double pivmin) { return fabs(q) < pivmin ? -pivmin : q; }

// Number of eigenvalues of T below x: negative pivots of T - x = L D L^T.
__device__ int sturm_count(const SliceShared& s, int n, double x, double pivmin) {
  double q = guard(s.a[0] - x, pivmin);
  int c = q < 0.0;
  for (int i = 1; i < n; ++i) {
    q = guard(s.a[i] - x - s.b2[i - 1] / q, pivmin);
    c += q < 0.0;
  }
  return c;
}

// The same count in FP32 (coarse: wrong only within ~ny FP32 ulps of an eigenvalue).
__device__ int sturm_count32(const SliceShared& s, int n, float x, float pivmin) {
  float q = s.af[0] - x;
  q = fabsf(q) < pivmin ? -pivmin : q;
  int c = q < 0.f;
  for (int i = 1; i < n; ++i) {
    q = s.af[i] - x - s.b2f[i - 1] / q;
    q = fabsf(q) < pivmin ? -pivmin : q;
    c += q < 0.f;
  }
  return c;
}

__device__ __forceinline__ double hop(double t0, double ma, double mb) { return -2.0 * t0 / (ma + mb); }

__global__ void __launch_bounds__(128) subband_slice_kernel(const double* __restrict__ me_y, const double* __restrict__ pot,
                                                            double t0, int nslice, int nv, int nx, int ny, int nm,
                                                            double* __restrict__ E, double* __restrict__ Vsub,
                                                            double* __restrict__ dplus, double* __restrict__ dminus,
                                                            int* __restrict__ err) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slice = blockIdx.x * (blockDim.x >> 5) + warp;   // slice = (problem * nv + v) * nx + x
  if (slice >= nslice) return;
  SliceShared s = slice_shared(smem + (size_t)warp * slice_doubles(ny), ny);
  const double* m = me_y + (size_t)slice * ny;
  const double* V = pot + ((size_t)(slice / (nv * nx)) * nx + slice % nx) * ny;

  // 1. Ht's diagonal (rows 0 and ny-1 copy rows 1 and ny-2) and the symmetrised pairs.
  int bad = 0;
  for (int i = lane; i < ny; i += 32) {
    const int r = i == 0 ? 1 : (i == ny - 1 ? ny - 2 : i);
    const double lo = hop(t0, m[r - 1], m[r]), up = hop(t0, m[r + 1], m[r]);
    s.a[i] = -(lo + up) + V[r];
    if (!isfinite(s.a[i])) bad = 1;
    if (i < ny - 1) {
      const double U = i == 0 ? hop(t0, m[2], m[1]) : hop(t0, m[i + 1], m[i]);              // Ht(i, i+1)
      const double L = i + 1 == ny - 1 ? hop(t0, m[ny - 3], m[ny - 2]) : hop(t0, m[i], m[i + 1]);  // Ht(i+1, i)
      const double p = U * L;
      if (!(p > 0.0) || !isfinite(p)) bad = 1;
      s.b2[i] = p;
      s.b[i] = U < 0.0 ? -sqrt(p) : sqrt(p);
      s.rr[i] = sqrt(L / U);
    } else {
      s.b2[i] = 0.0;
      s.b[i] = 0.0;
      s.rr[i] = 1.0;
    }
    s.af[i] = (float)s.a[i];
    s.b2f[i] = (float)s.b2[i];
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicOr(err, 1);
    for (int k = lane; k < nm; k += 32) E[(size_t)slice * nm + k] = NAN;
    return;
  }
  __syncwarp();

  // Gershgorin interval of T and the pivot floor (LAPACK's dstebz convention).
  double glo = INFINITY, ghi = -INFINITY, bmax = 0.0;
  for (int i = lane; i < ny; i += 32) {
    const double rad = fabs(s.b[i]) + (i > 0 ? fabs(s.b[i - 1]) : 0.0);
    glo = fmin(glo, s.a[i] - rad);
    ghi = fmax(ghi, s.a[i] + rad);
    bmax = fmax(bmax, s.b2[i]);
  }
  for (int o = 16; o; o >>= 1) {
    glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
  }
  const double gnorm = fmax(fabs(glo), fabs(ghi));
  const double pivmin = DBL_MIN * fmax(1.0, bmax);
  glo -= 2.0 * DBL_EPSILON * gnorm + 2.0 * pivmin;
  ghi += 2.0 * DBL_EPSILON * gnorm + 2.0 * pivmin;
  const double atol = DBL_EPSILON * gnorm;

  // 2. bisection of the candidates around zero
  const int n0 = __shfl_sync(0xffffffffu, lane == 0 ? sturm_count(s, ny, 0.0, pivmin) : 0, 0);
  const int c0 = max(0, n0 - nm), c1 = min(ny, n0 + nm), nc = c1 - c0;
  if (nc <= 16) {
    // multisection: candidate c on lanes [c g, c g + g); every lane of the warp takes part in
    // each step (the ballot), lanes past nc g and converged groups only vote 0
    const int g = 32 / nc, c = lane / g, j = lane % g;
    const bool mine = c < nc;
    const int k = c0 + (mine ? c : 0);
    const unsigned gmask = (g == 32 ? 0xffffffffu : ((1u << g) - 1u)) << (mine ? c * g : 0);
    // coarse FP32 multisection to ~1e-5 of the spectral radius (FP32 divisions are cheap)
    const float pivf = FLT_MIN * fmaxf(1.f, (float)bmax), ctol = 1e-5f * (float)gnorm;
    float flo = (float)glo, fhi = (float)ghi;
    for (int it = 0; it < 64; ++it) {
      const bool open = mine && fhi - flo > ctol;
      if (!__any_sync(0xffffffffu, open)) break;
      const float step = (fhi - flo) / (g + 1);
      const float p = flo + (j + 1) * step;
      const bool above = open && (p >= fhi || (p > flo && sturm_count32(s, ny, p, pivf) > k));
      const unsigned vote = __ballot_sync(0xffffffffu, above) & gmask;
      if (open) {
        const int jf = vote ? __ffs(vote) - 1 - c * g : g;
        const float nlo = jf == 0 ? flo : fmaxf(flo, flo + jf * step);
        const float nhi = jf == g ? fhi : fminf(fhi, flo + (jf + 1) * step);
        if (!(nlo > flo || nhi < fhi)) break;
        flo = nlo;
        fhi = nhi;
      }
    }
    // widen by a margin and confirm the bracket with FP64 counts (count(lo) <= k < count(hi)); a
    // bracket the FP32 counts got wrong falls back to the Gershgorin interval
    double lo = fmax(glo, (double)flo - 2e-5 * gnorm), hi = fmin(ghi, (double)fhi + 2e-5 * gnorm);
    {
      const bool chk = mine && j < 2;
      const int cnt = chk ? sturm_count(s, ny, j == 0 ? lo : hi, pivmin) : 0;
      const bool bad = chk && (j == 0 ? cnt > k : cnt <= k);
      if (__ballot_sync(0xffffffffu, bad) & gmask) {
        lo = glo;
        hi = ghi;
      }
    }
    for (int it = 0; it < 256; ++it) {
      const bool open = mine && hi - lo > atol + 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi));
      if (!__any_sync(0xffffffffu, open)) break;
      // lane j counts at p_j = lo + (j + 1) (hi - lo) / (g + 1); a point rounded onto or past an
      // end of the interval takes that end's known side (count(lo) <= k < count(hi))
      const double step = (hi - lo) / (g + 1);
      const double p = lo + (j + 1) * step;
      const bool above = open && (p >= hi || (p > lo && sturm_count(s, ny, p, pivmin) > k));
      const unsigned vote = __ballot_sync(0xffffffffu, above) & gmask;
      if (open) {
        // the first point of the group with more than k eigenvalues below it bounds from above
        const int jf = vote ? __ffs(vote) - 1 - c * g : g;
        const double nlo = jf == 0 ? lo : fmax(lo, lo + jf * step);
        const double nhi = jf == g ? hi : fmin(hi, lo + (jf + 1) * step);
        if (!(nlo > lo || nhi < hi)) {   // no progress at this resolution: the interval is final
          lo = hi = 0.5 * (lo + hi);
        } else {
          lo = nlo;
          hi = nhi;
        }
      }
    }
    if (mine && j == 0) s.lam[c] = 0.5 * (lo + hi);
  } else {
    for (int c = lane; c < nc; c += 32) {
      const int k = c0 + c;
      double lo = glo, hi = ghi;
      for (int it = 0; it < 256; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (!(hi - lo > atol + 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) || mid <= lo || mid >= hi) break;
        if (sturm_count(s, ny, mid, pivmin) > k) hi = mid;
        else lo = mid;
      }
      s.lam[c] = 0.5 * (lo + hi);
    }
  }
  __syncwarp();

  // 3. the nm of smallest magnitude: grow a window outwards from the sign change
  int lo = n0 - c0 - 1, hi = n0 - c0;
  for (int t = 0; t < nm; ++t) {
    if (hi < nc && (lo < 0 || fabs(s.lam[hi]) <= fabs(s.lam[lo]))) ++hi;
    else --lo;
  }
  const int first = lo + 1;

  // 4. eigenvectors, one lane per mode
  for (int k = lane; k < nm; k += 32) {
    const double lam = s.lam[first + k];
    E[(size_t)slice * nm + k] = lam;
    double* dp = dplus + (size_t)slice * ny * nm + k;    // [i][mode]
    double* dm = dminus + (size_t)slice * ny * nm + k;
    double q = guard(s.a[0] - lam, pivmin);
    dp[0] = q;
    for (int i = 1; i < ny; ++i) {
      q = guard(s.a[i] - lam - s.b2[i - 1] / q, pivmin);
      dp[(size_t)i * nm] = q;
    }
    double g = guard(s.a[ny - 1] - lam, pivmin);
    dm[(size_t)(ny - 1) * nm] = g;
    int r = ny - 1;
    double best = fabs(dp[(size_t)(ny - 1) * nm]);
    for (int i = ny - 2; i >= 0; --i) {
      g = guard(s.a[i] - lam - s.b2[i] / g, pivmin);
      dm[(size_t)i * nm] = g;
      const double gam = fabs(dp[(size_t)i * nm] + g - (s.a[i] - lam));
      if (gam < best) {
        best = gam;
        r = i;
      }
    }
    // w overwrites the top-down pivots: below r they are read just before being replaced
    dp[(size_t)r * nm] = 1.0;
    double w = 1.0;
    for (int i = r - 1; i >= 0; --i) {
      w = -(s.b[i] / dp[(size_t)i * nm]) * w;
      dp[(size_t)i * nm] = w;
    }
    w = 1.0;
    for (int i = r + 1; i < ny; ++i) {
      w = -(s.b[i - 1] / dm[(size_t)i * nm]) * w;
      dp[(size_t)i * nm] = w;
    }
    // v = D w, its norm and the sign of its last entry
    double d = 1.0, nrm = 0.0, last = 0.0;
    for (int i = 0; i < ny; ++i) {
      const double v = d * dp[(size_t)i * nm];
      nrm += v * v;
      last = v;
      d *= s.rr[i];
    }
    const double sc = (last > 0.0 ? 1.0 : (last < 0.0 ? -1.0 : 0.0)) / sqrt(nrm);
    if (!isfinite(sc)) atomicOr(err, 2);
    double* out = Vsub + ((size_t)slice * nm + k) * ny;
    d = 1.0;
    for (int i = 0; i < ny; ++i) {
      out[i] = sc * d * dp[(size_t)i * nm];
      d *= s.rr[i];
    }
  }
}

__global__ void __launch_bounds__(256) subband_cleanup_kernel(double* __restrict__ Vsub, int batch, int nv, int nx,
                                                              int ny, int nm) {
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (long long)batch * (nx - 1) * nm) return;
  const int b = (int)(warp / ((long long)(nx - 1) * nm));
  const int rem = (int)(warp % ((long long)(nx - 1) * nm));
  const int x = 1 + rem / nm, k = rem % nm;
  const size_t base = (size_t)b * nv * nx;                   // problem b, valley 1
  const double* v0 = Vsub + ((base + 0) * nm + k) * ny;      // slice 1
  double* v = Vsub + ((base + x) * nm + k) * ny;
  double dot = 0.0;
  for (int i = lane; i < ny; i += 32) dot += v0[i] * v[i];
  for (int o = 16; o; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
  if (dot < -0.5)
    for (int i = lane; i < ny; i += 32) v[i] = -v[i];
}

size_t slice_smem(int ny) { return (size_t)slice_doubles(ny) * sizeof(double); }

int warps_per_block(int ny) {
  int w = 4;
  while (w > 1 && (size_t)w * slice_smem(ny) > 160 * 1024) --w;
  return w;
}

}  // namespace

struct wg_subbands {
  int batch = 0, nv = 0, nx = 0, ny = 0, nm = 0;
  cudaStream_t stream = nullptr;
  double *me_y = nullptr, *V = nullptr, *E = nullptr, *Vsub = nullptr, *dp = nullptr, *dm = nullptr;
  int* err = nullptr;
  std::string msg;
};

extern "C" {

int wg_subbands_create(int batch, int n_valleys, int nx, int ny, int n_modes, wg_subbands** out) {
  if (!out) return WG_ERR_ARG;
  *out = nullptr;
  if (batch < 1 || n_valleys < 1 || nx < 1 || ny < 3 || ny > kMaxNy || n_modes < 1 || n_modes > kMaxModes ||
      n_modes > ny || (long long)batch * n_valleys * nx > (1LL << 30))
    return WG_ERR_ARG;
  wg_subbands* h = new wg_subbands;
  h->batch = batch;
  h->nv = n_valleys;
  h->nx = nx;
  h->ny = ny;
  h->nm = n_modes;
  const size_t slices = (size_t)batch * n_valleys * nx;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&h->me_y, slices * ny * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->V, (size_t)batch * nx * ny * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->E, slices * n_modes * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->Vsub, slices * n_modes * ny * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->dp, slices * n_modes * ny * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->dm, slices * n_modes * ny * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->err, 0, sizeof(int));
  if (e == cudaSuccess && warps_per_block(ny) * slice_smem(ny) > 48 * 1024)
    e = cudaFuncSetAttribute(subband_slice_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(warps_per_block(ny) * slice_smem(ny)));
  if (e != cudaSuccess) {
    wg_subbands_destroy(h);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  *out = h;
  return WG_OK;
}

int wg_subbands_destroy(wg_subbands* h) {
  if (!h) return WG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (double* p : {h->me_y, h->V, h->E, h->Vsub, h->dp, h->dm})
    if (p) cudaFree(p);
  if (h->err) cudaFree(h->err);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return WG_OK;
}

const char* wg_subbands_last_error(const wg_subbands* h) { return h ? h->msg.c_str() : "null handle"; }

int wg_subbands_solve_device(wg_subbands* h, double dy_nm, const double* me_y, const double* V, double* E,
                             double* Vsub, void* stream) {
  if (!h || !me_y || !V || !E || !Vsub || !(dy_nm > 0.0)) return WG_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  const double hb = 6.626e-34 / 2 / M_PI;
  const double t0 = hb * hb / 2 / (9.109e-31 * dy_nm * dy_nm * 1.602e-19 * 1e-18);   // eval_transversal_Hamiltonian.m:20
  const int slices = h->batch * h->nv * h->nx, wpb = warps_per_block(h->ny);
  subband_slice_kernel<<<(slices + wpb - 1) / wpb, 32 * wpb, wpb * slice_smem(h->ny), st>>>(
      me_y, V, t0, slices, h->nv, h->nx, h->ny, h->nm, E, Vsub, h->dp, h->dm, h->err);
  if (h->nx > 1) {
    const long long warps = (long long)h->batch * (h->nx - 1) * h->nm;
    subband_cleanup_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(Vsub, h->batch, h->nv, h->nx,
                                                                                  h->ny, h->nm);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->msg = cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  return WG_OK;
}

int wg_subbands_status(wg_subbands* h, void* stream) {
  if (!h) return WG_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    h->msg = cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  if (flag & 1) {
    h->msg = "non-finite Hamiltonian entry or non-positive off-diagonal product (masses must be positive)";
    return WG_ERR_NUMERIC;
  }
  if (flag & 2) {
    h->msg = "eigenvector with a zero or non-finite last entry";
    return WG_ERR_NUMERIC;
  }
  return WG_OK;
}

int wg_subbands_solve(wg_subbands* h, double dy_nm, const double* me_y, const double* V, double* E, double* Vsub) {
  if (!h || !me_y || !V || !E || !Vsub || !(dy_nm > 0.0)) return WG_ERR_ARG;
  const size_t slices = (size_t)h->batch * h->nv * h->nx;
  for (size_t i = 0; i < slices * h->ny; ++i)
    if (!(me_y[i] > 0.0) || !std::isfinite(me_y[i])) {
      h->msg = "effective masses must be positive and finite";
      return WG_ERR_ARG;
    }
  for (size_t i = 0; i < (size_t)h->batch * h->nx * h->ny; ++i)
    if (!std::isfinite(V[i])) {
      h->msg = "potential must be finite";
      return WG_ERR_ARG;
    }
  cudaError_t e = cudaMemcpyAsync(h->me_y, me_y, slices * h->ny * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->V, V, (size_t)h->batch * h->nx * h->ny * sizeof(double), cudaMemcpyHostToDevice,
                        h->stream);
  if (e != cudaSuccess) {
    h->msg = cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  int rc = wg_subbands_solve_device(h, dy_nm, h->me_y, h->V, h->E, h->Vsub, h->stream);
  if (rc != WG_OK) return rc;
  e = cudaMemcpyAsync(E, h->E, slices * h->nm * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(Vsub, h->Vsub, slices * h->nm * h->ny * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) {
    h->msg = cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  return wg_subbands_status(h, h->stream);
}

int wg_subbands_buffers(wg_subbands* h, double** me_y, double** V, double** E, double** Vsub) {
  if (!h) return WG_ERR_ARG;
  if (me_y) *me_y = h->me_y;
  if (V) *V = h->V;
  if (E) *E = h->E;
  if (Vsub) *Vsub = h->Vsub;
  return WG_OK;
}

}  // extern "C"
