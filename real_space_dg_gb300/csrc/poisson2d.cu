// 2D Poisson step of the Full-2D Gummel loop on the device (sm_103a).
//
// The reference's electrostatic step (RTD/make_RTD_poisson_step.m:44-54):
//   n   = project_DG_density_RTD(nDG)         exact DG integrals over the dual volumes
//                                             (RTD/project_DG_density_RTD.m:16-31)
//   phi = solve_Poisson2D_rtd(M, n, phi0)     the direct or approximate-Newton update on the
//                                             unique nodes (RTD/solve_Poisson2D_rtd.m:64-131)
// with M the 5-point div(eps grad) operator of RTD/eval_Poisson2D_rtd.m:107-188 (harmonic-mean
// faces, half control volumes at free X ends and non-periodic Y ends, Dirichlet identity rows,
// Y endpoints identified when periodic).
//
// Unique nodes k = ix + iy nx (x fastest, MATLAB's order), iy < nu (nu = Ny - 1 when periodic).
// The update solves J d = -F(free) with J = A_ff (direct) or A_ff - diag(q^2 n / (kB T)) (Newton),
// ordered by x columns: J is block tridiagonal, the column blocks D_ix (the Y stencil, a ring
// when periodic, plus the diagonal) coupled to the neighbour columns by diagonal matrices
// L_ix, U_ix (the X faces).  Block LU without pivoting (J is diagonally dominant; Dirichlet
// nodes stay in as identity rows with a zero right-hand side):
//   S_0 = D_0,  S_ix = D_ix - L_ix S_{ix-1}^-1 U_{ix-1},  g_ix = S_ix^-1 (r_ix - L_ix g_{ix-1}),
//   d_{nx-1} = g_{nx-1},  d_ix = g_ix - S_ix^-1 U_ix d_{ix+1}.
// Row a of S_ix needs row a of S_{ix-1}^-1 only, so one warp runs the sweep with lane a holding
// row a in registers (NU = 4/8/12/16/24/32, padded with identity rows); the Gauss-Jordan inversion of
// each S_ix broadcasts the pivot row by shuffles.  The inverses go to a scratch [nx][NU][NU]
// for the backward sweep.  One warp per problem (a batch of bias points runs as a grid);
// projection, residuals and diagnostics run in the same warp with fixed-order reductions.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

#include "wigner_gb300.h"

namespace {

constexpr double kQ = 1.602176634e-19;
constexpr double kKB = 1.380649e-23;
constexpr double kEps0 = 8.8541878128e-12;

struct P2Dev {
  int nx, ny, nu, periodic, batch;
  const unsigned char* fixed;     // [nu nx]
  const double *cxm, *cxp, *cym, *cyp, *diag;   // stencil of the free rows (0 on fixed rows)
  const double* net;              // Nd - Na [nu nx]
  const double *vx, *vy;          // control-volume widths for the charge diagnostics [nx], [nu]
  // projection (optional)
  int ndx, ndy;
  const int *tx_rp, *tx_col, *ty_rp, *ty_col;
  const double *tx_val, *ty_val, *wx, *wy, *srcx, *srcy;
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// (A u)_k on the unique nodes: free rows the stencil (periodic Y ring), fixed rows the identity.
__device__ __forceinline__ double stencil(const P2Dev& P, const double* u, int ix, int iy) {
  const int k = ix + iy * P.nx;
  if (P.fixed[k]) return u[k];
  double s = P.diag[k] * u[k];
  if (ix > 0) s += P.cxm[k] * u[k - 1];
  if (ix < P.nx - 1) s += P.cxp[k] * u[k + 1];
  if (iy > 0 || P.periodic) s += P.cym[k] * u[(iy > 0 ? iy - 1 : P.nu - 1) * P.nx + ix];
  if (iy < P.nu - 1 || P.periodic) s += P.cyp[k] * u[(iy < P.nu - 1 ? iy + 1 : 0) * P.nx + ix];
  return s;
}

template <int NU>
__global__ void __launch_bounds__(32) poisson2d_step_kernel(
    P2Dev P, const double* __restrict__ src, int src_is_dg, const double* __restrict__ phi0,
    const double* __restrict__ bc, int newton, double q_kt, double alpha, double* __restrict__ phi,
    double* __restrict__ density, double* __restrict__ work, double* __restrict__ sinv_all,
    wg_poisson2d_info* __restrict__ info) {
  const int b = blockIdx.x, lane = threadIdx.x;
  const int nx = P.nx, ny = P.ny, nu = P.nu, nun = nu * nx;
  const size_t full = (size_t)nx * ny;
  src += (size_t)b * (src_is_dg ? (size_t)P.ndx * P.ndy : full);
  phi0 += (size_t)b * full;
  bc += (size_t)b * nun;
  phi += (size_t)b * full;
  density += (size_t)b * full;
  double* n = work + (size_t)b * 6 * nun;      // density on the unique nodes
  double* v = n + nun;                          // v = phi0, contacts set
  double* F = v + nun;                          // A v - charge
  double* g = F + nun;                          // forward-sweep vectors, then the update d
  double* r = g + nun;                          // -F on free nodes
  double* t = r + nun;                          // scratch
  double* Sinv = sinv_all + (size_t)b * nx * NU * NU;

  // 1. the density on the unique nodes: DG integrals over the dual volumes, or given
  double src_int = 0.0, tgt_int = 0.0;
  if (src_is_dg) {
    for (int k = lane; k < nun; k += 32) {
      const int ix = k % nx, iy = k / nx;
      double acc = 0.0;
      for (int p = P.tx_rp[ix]; p < P.tx_rp[ix + 1]; ++p) {
        const double tx = P.tx_val[p];
        const double* row = src + P.tx_col[p];
        double s = 0.0;
        for (int q = P.ty_rp[iy]; q < P.ty_rp[iy + 1]; ++q) s += P.ty_val[q] * row[(size_t)P.ty_col[q] * P.ndx];
        acc += tx * s;
      }
      tgt_int += acc;
      n[k] = acc / (P.wx[ix] * P.wy[iy]);
    }
    for (int e = lane; e < P.ndx * P.ndy; e += 32) src_int += P.srcx[e % P.ndx] * src[e] * P.srcy[e / P.ndx];
    src_int = warp_sum(src_int);
    tgt_int = warp_sum(tgt_int);
  } else {
    for (int k = lane; k < nun; k += 32) n[k] = src[(size_t)(k / nx) * nx + k % nx];
  }
  // 2. v, A v, F = A v - charge and the residual scale (free nodes)
  for (int k = lane; k < nun; k += 32) v[k] = P.fixed[k] ? bc[k] : phi0[k];
  __syncwarp();
  double m_qn = 0.0, m_qnet = 0.0, m_av = 0.0, m_f = 0.0;
  for (int k = lane; k < nun; k += 32) {
    const double av = stencil(P, v, k % nx, k / nx);
    const double ch = kQ * (n[k] - P.net[k]);
    F[k] = av - ch;
    if (!P.fixed[k]) {
      m_qn = fmax(m_qn, fabs(kQ * n[k]));
      m_qnet = fmax(m_qnet, fabs(kQ * P.net[k]));
      m_av = fmax(m_av, fabs(av));
      m_f = fmax(m_f, fabs(F[k]));
    }
    r[k] = P.fixed[k] ? 0.0 : -F[k];
  }
  m_qn = warp_max(m_qn);
  m_qnet = warp_max(m_qnet);
  m_av = warp_max(m_av);
  m_f = warp_max(m_f);
  const double scale = fmax(fmax(m_qn, m_qnet), fmax(m_av, kQ));
  __syncwarp();

  // 3. forward block sweep: lane a holds row a of S_ix and then of S_ix^-1 (rows nu..NU-1
  //    are identity padding; lanes NU..31 carry zero rows and store nothing)
  const bool live = lane < nu;
  double row[NU];
#pragma unroll
  for (int j = 0; j < NU; ++j) row[j] = 0.0;
  double uprev = 0.0, gprev = 0.0;   // u_{ix-1} and g_{ix-1} of this lane's row
  for (int ix = 0; ix < nx; ++ix) {
    const int k = ix + lane * nx;
    const bool fx = !live || P.fixed[k];
    const double l = fx ? 0.0 : P.cxm[k];
    const double u = fx ? 0.0 : P.cxp[k];
    // S row a = D row a - l_a Sinv_prev[a][j] u_prev[j], built in place over Sinv_prev's row
    const double dg = fx ? 1.0 : P.diag[k] - (newton ? q_kt * n[k] : 0.0);
    const int jm = fx ? -1 : (lane > 0 ? lane - 1 : (P.periodic ? nu - 1 : -1));
    const int jp = fx ? -1 : (lane < nu - 1 ? lane + 1 : (P.periodic ? 0 : -1));
    const double cm = fx ? 0.0 : P.cym[k], cp = fx ? 0.0 : P.cyp[k];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      const double uj = __shfl_sync(0xffffffffu, uprev, j);
      const double dj = (j == lane && lane < NU ? dg : 0.0) + (j == jm ? cm : 0.0) + (j == jp ? cp : 0.0);
      row[j] = dj - (ix > 0 ? l * row[j] * uj : 0.0);
    }
    // t = r_ix - L_ix g_{ix-1}
    const double tk = (live ? r[k] : 0.0) - l * gprev;
    // Gauss-Jordan inversion in place (no pivoting: S is diagonally dominant)
#pragma unroll
    for (int p = 0; p < NU; ++p) {
      const double pinv = 1.0 / __shfl_sync(0xffffffffu, row[p], p);
      if (lane == p) {
        row[p] = 1.0;
#pragma unroll
        for (int j = 0; j < NU; ++j) row[j] *= pinv;
      }
      const double f = row[p];
#pragma unroll
      for (int j = 0; j < NU; ++j) {
        const double pj = __shfl_sync(0xffffffffu, row[j], p);
        if (lane != p) row[j] = j == p ? -f * pj : row[j] - f * pj;
      }
    }
    // g_ix = S^-1 t
    double gk = 0.0;
#pragma unroll
    for (int j = 0; j < NU; ++j) gk += row[j] * __shfl_sync(0xffffffffu, tk, j);
    if (lane < NU) {
      double* so = Sinv + ((size_t)ix * NU + lane) * NU;
#pragma unroll
      for (int j = 0; j < NU; ++j) so[j] = row[j];
    }
    if (live) g[k] = gk;
    gprev = gk;
    uprev = u;
  }
  __syncwarp();
  // 4. backward sweep: d_ix = g_ix - S_ix^-1 U_ix d_{ix+1}
  double dnext = 0.0;
  for (int ix = nx - 1; ix >= 0; --ix) {
    const int k = ix + lane * nx;
    const bool fx = !live || P.fixed[k];
    const double u = fx ? 0.0 : P.cxp[k];
    const double w = u * dnext;
    const double* so = Sinv + ((size_t)ix * NU + (lane < NU ? lane : 0)) * NU;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NU; ++j) s += (lane < NU ? so[j] : 0.0) * __shfl_sync(0xffffffffu, w, j);
    const double d = (live ? g[k] : 0.0) - (ix < nx - 1 ? s : 0.0);
    if (live) g[k] = d;
    dnext = d;
  }
  __syncwarp();
  // 5. the linear residual J d + F, the update, iter_err, the step size
  double m_lin = 0.0, e2 = 0.0, m_d = 0.0;
  for (int k = lane; k < nun; k += 32) {
    t[k] = P.fixed[k] ? 0.0 : g[k];
  }
  __syncwarp();
  for (int k = lane; k < nun; k += 32) {
    if (P.fixed[k]) continue;
    const double jd = stencil(P, t, k % nx, k / nx) - (newton ? q_kt * n[k] * t[k] : 0.0);
    m_lin = fmax(m_lin, fabs(jd + F[k]));
    m_d = fmax(m_d, fabs(t[k]));
  }
  __syncwarp();
  for (int k = lane; k < nun; k += 32) {
    const double up = P.fixed[k] ? v[k] : v[k] + alpha * t[k];
    if (!P.fixed[k]) {
      const double dd = up - phi0[k];
      e2 += dd * dd;
    }
    r[k] = up;   // updated
  }
  __syncwarp();
  // 6. the residual after the update and the charge diagnostics
  double m_after = 0.0, qnet = 0.0, qabs_net = 0.0, qabs_n = 0.0;
  bool finite = true;
  for (int k = lane; k < nun; k += 32) {
    const int ix = k % nx, iy = k / nx;
    const double ch = kQ * (n[k] - P.net[k]);
    if (!P.fixed[k]) m_after = fmax(m_after, fabs(stencil(P, r, ix, iy) - ch));
    const double vol = P.vx[ix] * P.vy[iy];
    qnet += vol * ch;
    qabs_net += vol * fabs(P.net[k]);
    qabs_n += vol * fabs(n[k]);
    if (!isfinite(r[k])) finite = false;
  }
  m_lin = warp_max(m_lin);
  m_d = warp_max(m_d);
  e2 = warp_sum(e2);
  m_after = warp_max(m_after);
  qnet = warp_sum(qnet);
  qabs_net = warp_sum(qabs_net);
  qabs_n = warp_sum(qabs_n);
  finite = __all_sync(0xffffffffu, finite);
  // 7. phi and the density on the full grid (the duplicate Y column when periodic)
  for (size_t k = lane; k < full; k += 32) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    const int ku = (iy < nu ? iy : 0) * nx + ix;
    phi[k] = r[ku];
    density[k] = n[ku];
  }
  if (lane == 0) {
    wg_poisson2d_info& o = info[b];
    const double lin = m_lin / fmax(m_f, kQ);
    o.converged = finite && isfinite(lin) && lin < 1e-8;
    o.linear_relres = lin;
    o.physical_relres_before = m_f / scale;
    o.physical_relres_after = m_after / scale;
    o.physical_residual_before = m_f;
    o.residual_scale = scale;
    o.unmixed_step = m_d;
    o.iter_err = sqrt(e2);
    o.net_charge_per_length = -qnet;
    o.relative_charge_imbalance = fabs(qnet) / fmax(kQ * fmax(qabs_net, qabs_n), DBL_MIN);
    o.source_integral = src_int;
    o.target_integral = tgt_int;
  }
}

// M u on the full grid: the reference's operator with every row (free stencil rows, Dirichlet
// identity rows, phi(:,end) - phi(:,1) rows for the periodic duplicate).
__global__ void poisson2d_apply_kernel(P2Dev P, const double* __restrict__ u, double* __restrict__ y) {
  const size_t full = (size_t)P.nx * P.ny;
  const int b = blockIdx.y;
  u += b * full;
  y += b * full;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < full; k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % P.nx), iy = (int)(k / P.nx);
    if (P.periodic && iy == P.ny - 1) {
      y[k] = u[k] - u[ix];
      continue;
    }
    // unique-node stencil; a Y neighbour on the duplicate column reads column 0 (expand)
    const int ku = ix + iy * P.nx;
    if (P.fixed[ku]) {
      y[k] = u[k];
      continue;
    }
    double s = P.diag[ku] * u[k];
    if (ix > 0) s += P.cxm[ku] * u[k - 1];
    if (ix < P.nx - 1) s += P.cxp[ku] * u[k + 1];
    if (iy > 0) s += P.cym[ku] * u[k - P.nx];
    else if (P.periodic) s += P.cym[ku] * u[(size_t)(P.ny - 2) * P.nx + ix];
    if (iy < P.ny - 1) {
      const int jp = P.periodic && iy + 1 == P.ny - 1 ? 0 : iy + 1;
      s += P.cyp[ku] * u[(size_t)jp * P.nx + ix];
    }
    y[k] = s;
  }
}

template <typename T>
cudaError_t upload(T** d, const std::vector<T>& h) {
  cudaError_t e = cudaMalloc(d, std::max<size_t>(1, h.size()) * sizeof(T));
  if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

}  // namespace

struct wg_poisson2d {
  wg_poisson2d_desc d{};
  int nu = 0, NU = 0;
  P2Dev P{};
  cudaStream_t stream = nullptr;
  std::vector<void*> owned;
  double *src = nullptr, *phi0 = nullptr, *bc = nullptr, *phi = nullptr, *dens = nullptr, *work = nullptr,
         *sinv = nullptr;
  wg_poisson2d_info* info = nullptr;
  bool projection = false;
  std::string msg;
};

namespace {

int fail(wg_poisson2d* h, int rc, const char* m) {
  if (h) h->msg = m;
  return rc;
}

template <typename T>
cudaError_t keep(wg_poisson2d* h, T** d, const std::vector<T>& v) {
  cudaError_t e = upload(d, v);
  if (e == cudaSuccess) h->owned.push_back((void*)*d);
  return e;
}

cudaError_t launch_step(wg_poisson2d* h, const double* src, int is_dg, const double* phi0, const double* bc,
                        int newton, double alpha, double* phi, double* dens, cudaStream_t st) {
  const double q_kt = kQ * kQ / (kKB * h->d.temp);
  const int B = h->d.batch;
  double* work = h->work;
#define WG_P2_CASE(NU_)                                                                                      \
  case NU_:                                                                                                  \
    poisson2d_step_kernel<NU_><<<B, 32, 0, st>>>(h->P, src, is_dg, phi0, bc, newton, q_kt, alpha, phi, dens, \
                                                 work, h->sinv, h->info);                                    \
    break;
  switch (h->NU) {
    WG_P2_CASE(4)
    WG_P2_CASE(8)
    WG_P2_CASE(12)
    WG_P2_CASE(16)
    WG_P2_CASE(24)
    WG_P2_CASE(32)
    default:
      return cudaErrorInvalidValue;
  }
#undef WG_P2_CASE
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int wg_poisson2d_create(const wg_poisson2d_desc* d, const double* eps_r, const unsigned char* boundary,
                        const double* nd_m3, const double* na_m3, wg_poisson2d** out) {
  if (!d || !eps_r || !nd_m3 || !out) return WG_ERR_ARG;
  *out = nullptr;
  const int nx = d->nx, ny = d->ny, B = d->batch;
  if (nx < 2 || ny < 1 || B < 1 || !(d->dx_nm > 0) || !(d->dy_nm > 0) || !std::isfinite(d->dx_nm) ||
      !std::isfinite(d->dy_nm) || !(d->temp > 0))
    return WG_ERR_ARG;
  const int periodic = d->periodic_y ? 1 : 0;
  if (periodic && ny < 3) return WG_ERR_ARG;                       // RTD:PoissonPeriodicMaterial
  const int nu = ny - periodic;
  if (nu > 32) return WG_ERR_ARG;                                   // the warp-row block sweep
  const size_t full = (size_t)nx * ny;
  double emax = 0.0;
  for (size_t k = 0; k < full; ++k) {
    if (!(eps_r[k] > 0) || !std::isfinite(eps_r[k])) return WG_ERR_ARG;
    emax = std::max(emax, eps_r[k]);
    if (!(nd_m3[k] >= 0) || !std::isfinite(nd_m3[k]) || (na_m3 && (!(na_m3[k] >= 0) || !std::isfinite(na_m3[k]))))
      return WG_ERR_ARG;
  }
  auto at = [&](const double* a, int ix, int iy) { return a[(size_t)iy * nx + ix]; };
  if (periodic)
    for (int ix = 0; ix < nx; ++ix)
      if (std::fabs(at(eps_r, ix, ny - 1) - at(eps_r, ix, 0)) > 1e-12 * emax) return WG_ERR_ARG;
  std::vector<unsigned char> fixedf(full, 0);
  if (boundary) {
    for (size_t k = 0; k < full; ++k) fixedf[k] = boundary[k] ? 1 : 0;
  } else if (!d->neumann_x) {
    for (int iy = 0; iy < ny; ++iy) fixedf[(size_t)iy * nx] = fixedf[(size_t)iy * nx + nx - 1] = 1;
  }
  bool any = false;
  for (unsigned char f : fixedf) any = any || f;
  if (d->neumann_x && any) return WG_ERR_ARG;                       // RTD:PoissonBoundaryConflict
  if (!d->neumann_x && !any) return WG_ERR_ARG;                     // Dirichlet needs a fixed node
  if (periodic)
    for (int ix = 0; ix < nx; ++ix)
      if (fixedf[(size_t)(ny - 1) * nx + ix] != fixedf[ix]) return WG_ERR_ARG;   // RTD:PoissonPeriodicBoundary

  // the stencil of the unique rows (eval_Poisson2D_rtd.m:118-185)
  const int nun = nu * nx;
  std::vector<unsigned char> fx(nun);
  std::vector<double> cxm(nun, 0.0), cxp(nun, 0.0), cym(nun, 0.0), cyp(nun, 0.0), dg(nun, 0.0), net(nun);
  const double cx = kEps0 * 1e18 / (d->dx_nm * d->dx_nm), cy = kEps0 * 1e18 / (d->dy_nm * d->dy_nm);
  auto hm = [](double a, double b) { return 2 * a * b / (a + b); };
  for (int iy = 0; iy < nu; ++iy)
    for (int ix = 0; ix < nx; ++ix) {
      const int k = ix + iy * nx;
      fx[k] = fixedf[(size_t)iy * nx + ix];
      net[k] = at(nd_m3, ix, iy) - (na_m3 ? at(na_m3, ix, iy) : 0.0);
      if (fx[k]) continue;
      const double e0 = at(eps_r, ix, iy);
      double diag = 0.0;
      if (ix > 0) {
        double c = cx * hm(e0, at(eps_r, ix - 1, iy));
        if (ix == nx - 1) c *= 2;
        cxm[k] = c;
        diag -= c;
      }
      if (ix < nx - 1) {
        double c = cx * hm(e0, at(eps_r, ix + 1, iy));
        if (ix == 0) c *= 2;
        cxp[k] = c;
        diag -= c;
      }
      if (iy > 0 || periodic) {
        const int jm = iy > 0 ? iy - 1 : ny - 2;
        double c = cy * hm(e0, at(eps_r, ix, jm));
        if (!periodic && iy == ny - 1) c *= 2;
        cym[k] = c;
        diag -= c;
      }
      if (iy < ny - 1) {
        int jp = iy + 1;
        if (periodic && jp == ny - 1) jp = 0;
        double c = cy * hm(e0, at(eps_r, ix, jp));
        if (!periodic && iy == 0) c *= 2;
        cyp[k] = c;
        diag -= c;
      }
      dg[k] = diag;
    }
  // control-volume widths of the charge diagnostics (solve_Poisson2D_rtd.m:115-118)
  std::vector<double> vx(nx, d->dx_nm * 1e-9), vy(nu, d->dy_nm * 1e-9);
  vx[0] /= 2;
  vx[nx - 1] /= 2;
  if (!periodic && nu > 1) {
    vy[0] /= 2;
    vy[nu - 1] /= 2;
  }
  wg_poisson2d* h = new wg_poisson2d;
  h->d = *d;
  h->d.periodic_y = periodic;
  h->nu = nu;
  h->NU = nu <= 4 ? 4 : nu <= 8 ? 8 : nu <= 12 ? 12 : nu <= 16 ? 16 : nu <= 24 ? 24 : 32;
  P2Dev& P = h->P;
  P.nx = nx;
  P.ny = ny;
  P.nu = nu;
  P.periodic = periodic;
  P.batch = B;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  unsigned char* dfx = nullptr;
  double *dcxm = nullptr, *dcxp = nullptr, *dcym = nullptr, *dcyp = nullptr, *ddg = nullptr, *dnet = nullptr,
         *dvx = nullptr, *dvy = nullptr;
  if (e == cudaSuccess) e = keep(h, &dfx, fx);
  if (e == cudaSuccess) e = keep(h, &dcxm, cxm);
  if (e == cudaSuccess) e = keep(h, &dcxp, cxp);
  if (e == cudaSuccess) e = keep(h, &dcym, cym);
  if (e == cudaSuccess) e = keep(h, &dcyp, cyp);
  if (e == cudaSuccess) e = keep(h, &ddg, dg);
  if (e == cudaSuccess) e = keep(h, &dnet, net);
  if (e == cudaSuccess) e = keep(h, &dvx, vx);
  if (e == cudaSuccess) e = keep(h, &dvy, vy);
  P.fixed = dfx;
  P.cxm = dcxm;
  P.cxp = dcxp;
  P.cym = dcym;
  P.cyp = dcyp;
  P.diag = ddg;
  P.net = dnet;
  P.vx = dvx;
  P.vy = dvy;
  const size_t sz = (size_t)B * full * sizeof(double);
  if (e == cudaSuccess) e = cudaMalloc(&h->src, sz);
  if (e == cudaSuccess) e = cudaMalloc(&h->phi0, sz);
  if (e == cudaSuccess) e = cudaMalloc(&h->bc, (size_t)B * nun * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->phi, sz);
  if (e == cudaSuccess) e = cudaMalloc(&h->dens, sz);
  if (e == cudaSuccess) e = cudaMalloc(&h->work, (size_t)B * 6 * nun * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->sinv, (size_t)B * nx * h->NU * h->NU * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->info, (size_t)B * sizeof(wg_poisson2d_info));
  if (e != cudaSuccess) {
    wg_poisson2d_destroy(h);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA;
  }
  *out = h;
  return WG_OK;
}

int wg_poisson2d_destroy(wg_poisson2d* h) {
  if (!h) return WG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->owned) cudaFree(p);
  for (void* p : {(void*)h->src, (void*)h->phi0, (void*)h->bc, (void*)h->phi, (void*)h->dens, (void*)h->work,
                  (void*)h->sinv, (void*)h->info})
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return WG_OK;
}

const char* wg_poisson2d_last_error(const wg_poisson2d* h) { return h ? h->msg.c_str() : "null handle"; }

int wg_poisson2d_set_projection(wg_poisson2d* h, int ndof_x, const int* tx_rp, const int* tx_col, const double* tx_val,
                                int ndof_y, const int* ty_rp, const int* ty_col, const double* ty_val,
                                const double* wx, const double* wy, const double* src_x, const double* src_y) {
  if (!h || ndof_x < 1 || ndof_y < 1 || !tx_rp || !tx_col || !tx_val || !ty_rp || !ty_col || !ty_val || !wx || !wy ||
      !src_x || !src_y)
    return WG_ERR_ARG;
  const int nx = h->d.nx, nu = h->nu;
  if (tx_rp[0] != 0 || ty_rp[0] != 0) return fail(h, WG_ERR_ARG, "CSR row pointers must start at 0");
  for (int i = 0; i < nx; ++i)
    if (tx_rp[i + 1] < tx_rp[i]) return fail(h, WG_ERR_ARG, "Tx row pointers must not decrease");
  for (int i = 0; i < nu; ++i)
    if (ty_rp[i + 1] < ty_rp[i]) return fail(h, WG_ERR_ARG, "Ty row pointers must not decrease");
  for (int p = 0; p < tx_rp[nx]; ++p)
    if (tx_col[p] < 0 || tx_col[p] >= ndof_x) return fail(h, WG_ERR_ARG, "Tx column out of range");
  for (int p = 0; p < ty_rp[nu]; ++p)
    if (ty_col[p] < 0 || ty_col[p] >= ndof_y) return fail(h, WG_ERR_ARG, "Ty column out of range");
  for (int i = 0; i < nx; ++i)
    if (!(wx[i] > 0)) return fail(h, WG_ERR_ARG, "dual-volume widths must be positive");
  for (int i = 0; i < nu; ++i)
    if (!(wy[i] > 0)) return fail(h, WG_ERR_ARG, "dual-volume widths must be positive");
  std::vector<int> vtr(tx_rp, tx_rp + nx + 1), vtc(tx_col, tx_col + tx_rp[nx]), vyr(ty_rp, ty_rp + nu + 1),
      vyc(ty_col, ty_col + ty_rp[nu]);
  std::vector<double> vtv(tx_val, tx_val + tx_rp[nx]), vyv(ty_val, ty_val + ty_rp[nu]), vwx(wx, wx + nx),
      vwy(wy, wy + nu), vsx(src_x, src_x + ndof_x), vsy(src_y, src_y + ndof_y);
  P2Dev& P = h->P;
  int *a = nullptr, *b = nullptr, *c = nullptr, *dd = nullptr;
  double *e1 = nullptr, *e2 = nullptr, *e3 = nullptr, *e4 = nullptr, *e5 = nullptr, *e6 = nullptr;
  cudaError_t e = keep(h, &a, vtr);
  if (e == cudaSuccess) e = keep(h, &b, vtc);
  if (e == cudaSuccess) e = keep(h, &c, vyr);
  if (e == cudaSuccess) e = keep(h, &dd, vyc);
  if (e == cudaSuccess) e = keep(h, &e1, vtv);
  if (e == cudaSuccess) e = keep(h, &e2, vyv);
  if (e == cudaSuccess) e = keep(h, &e3, vwx);
  if (e == cudaSuccess) e = keep(h, &e4, vwy);
  if (e == cudaSuccess) e = keep(h, &e5, vsx);
  if (e == cudaSuccess) e = keep(h, &e6, vsy);
  if (e != cudaSuccess) return fail(h, WG_ERR_CUDA, cudaGetErrorString(e));
  if ((size_t)ndof_x * ndof_y > (size_t)h->d.nx * h->d.ny) {
    // the source buffer holds nDG for the host entry points
    cudaFree(h->src);
    h->src = nullptr;
    e = cudaMalloc(&h->src, (size_t)h->d.batch * ndof_x * ndof_y * sizeof(double));
    if (e != cudaSuccess) return fail(h, WG_ERR_OOM, "source buffer");
  }
  P.ndx = ndof_x;
  P.ndy = ndof_y;
  P.tx_rp = a;
  P.tx_col = b;
  P.ty_rp = c;
  P.ty_col = dd;
  P.tx_val = e1;
  P.ty_val = e2;
  P.wx = e3;
  P.wy = e4;
  P.srcx = e5;
  P.srcy = e6;
  h->projection = true;
  return WG_OK;
}

int wg_poisson2d_apply(wg_poisson2d* h, const double* phi, double* out) {
  if (!h || !phi || !out) return WG_ERR_ARG;
  const size_t sz = (size_t)h->d.batch * h->d.nx * h->d.ny * sizeof(double);
  cudaError_t e = cudaMemcpyAsync(h->phi0, phi, sz, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    dim3 grid((unsigned)std::min<size_t>(1024, ((size_t)h->d.nx * h->d.ny + 255) / 256), h->d.batch);
    poisson2d_apply_kernel<<<grid, 256, 0, h->stream>>>(h->P, h->phi0, h->phi);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, h->phi, sz, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  return e == cudaSuccess ? WG_OK : fail(h, WG_ERR_CUDA, cudaGetErrorString(e));
}

int wg_poisson2d_contacts(wg_poisson2d* h, const double* bias, const double* vbc, double* bc_out) {
  // solve_Poisson2D_rtd.m:50-52: bc(end,:) = bias unless mat.Vbc gives the contact potential
  if (!h || !bc_out || (!bias && !vbc)) return WG_ERR_ARG;
  const int nx = h->d.nx, nu = h->nu, B = h->d.batch;
  for (int b = 0; b < B; ++b)
    for (int iy = 0; iy < nu; ++iy)
      for (int ix = 0; ix < nx; ++ix) {
        const size_t k = (size_t)b * nu * nx + (size_t)iy * nx + ix;
        bc_out[k] = vbc ? vbc[(size_t)b * nx * h->d.ny + (size_t)iy * nx + ix] : (ix == nx - 1 ? bias[b] : 0.0);
      }
  return WG_OK;
}

int wg_poisson2d_solve_device(wg_poisson2d* h, const double* src, int src_is_dg, const double* phi0,
                              const double* bc, int newton, double alpha, double* phi, double* density, void* stream) {
  if (!h || !src || !phi0 || !bc || !phi || !density || !(alpha > 0 && alpha <= 1)) return WG_ERR_ARG;
  if (src_is_dg && !h->projection) return fail(h, WG_ERR_ARG, "wg_poisson2d_set_projection first");
  if (!newton && h->d.neumann_x) return fail(h, WG_ERR_ARG, "RTD:NeumannNeedsNewton");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  const cudaError_t e = launch_step(h, src, src_is_dg, phi0, bc, newton, alpha, phi, density, st);
  return e == cudaSuccess ? WG_OK : fail(h, WG_ERR_CUDA, cudaGetErrorString(e));
}

int wg_poisson2d_info_get(wg_poisson2d* h, void* stream, wg_poisson2d_info* info) {
  if (!h || !info) return WG_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  cudaError_t e = cudaMemcpyAsync(info, h->info, (size_t)h->d.batch * sizeof(wg_poisson2d_info),
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? WG_OK : fail(h, WG_ERR_CUDA, cudaGetErrorString(e));
}

int wg_poisson2d_solve(wg_poisson2d* h, const double* src, int src_is_dg, const double* phi0, const double* bias,
                       const double* vbc, int newton, double alpha, double* phi, double* density,
                       wg_poisson2d_info* info) {
  if (!h || !src || !phi0 || !phi || !density || !info || (!bias && !vbc)) return WG_ERR_ARG;
  const int nx = h->d.nx, ny = h->d.ny, B = h->d.batch;
  const size_t full = (size_t)nx * ny;
  if (src_is_dg && !h->projection) return fail(h, WG_ERR_ARG, "wg_poisson2d_set_projection first");
  if (h->d.neumann_x && !newton) return fail(h, WG_ERR_ARG, "RTD:NeumannNeedsNewton");
  if (h->d.neumann_x && vbc) return fail(h, WG_ERR_ARG, "RTD:PoissonBoundaryConflict");
  const size_t nsrc = src_is_dg ? (size_t)h->P.ndx * h->P.ndy : full;
  for (size_t k = 0; k < (size_t)B * nsrc; ++k)
    if (!std::isfinite(src[k])) return fail(h, WG_ERR_ARG, "density must be finite");
  for (size_t k = 0; k < (size_t)B * full; ++k)
    if (!std::isfinite(phi0[k])) return fail(h, WG_ERR_ARG, "phi0 must be finite");
  if (!src_is_dg && h->d.neumann_x) {
    // solve_Poisson2D_rtd.m:97-100: Newton screening needs a non-negative, non-zero density
    for (int b = 0; b < B; ++b) {
      bool pos = false;
      for (size_t k = 0; k < full; ++k) {
        if (src[b * full + k] < 0) return fail(h, WG_ERR_ARG, "RTD:NeumannDensityResponse");
        pos = pos || src[b * full + k] > 0;
      }
      if (!pos) return fail(h, WG_ERR_ARG, "RTD:NeumannDensityResponse");
    }
  }
  if (h->d.periodic_y) {
    // solve_Poisson2D_rtd.m:53-57 and 133-137: the included Y endpoints must agree
    auto periodic_ok = [&](const double* a) {
      for (int b = 0; b < B; ++b) {
        double mx = 1.0;
        for (size_t k = 0; k < full; ++k) mx = std::max(mx, std::fabs(a[b * full + k]));
        for (int ix = 0; ix < nx; ++ix)
          if (std::fabs(a[b * full + ix] - a[b * full + (size_t)(ny - 1) * nx + ix]) > 1e-10 * mx) return false;
      }
      return true;
    };
    if ((!src_is_dg && !periodic_ok(src)) || !periodic_ok(phi0) || (vbc && !periodic_ok(vbc)))
      return fail(h, WG_ERR_ARG, "RTD:NonperiodicPoissonData");
  }
  std::vector<double> bc((size_t)B * h->nu * nx);
  int rc = wg_poisson2d_contacts(h, bias, vbc, bc.data());
  if (rc != WG_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(h->src, src, (size_t)B * nsrc * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->phi0, phi0, (size_t)B * full * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->bc, bc.data(), bc.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_step(h, h->src, src_is_dg, h->phi0, h->bc, newton, alpha, h->phi, h->dens, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(phi, h->phi, (size_t)B * full * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(density, h->dens, (size_t)B * full * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return fail(h, WG_ERR_CUDA, cudaGetErrorString(e));
  rc = wg_poisson2d_info_get(h, h->stream, info);
  if (rc != WG_OK) return rc;
  return WG_OK;
}

int wg_poisson2d_buffers(wg_poisson2d* h, double** src, double** phi0, double** bc, double** phi, double** density) {
  if (!h) return WG_ERR_ARG;
  if (src) *src = h->src;
  if (phi0) *phi0 = h->phi0;
  if (bc) *bc = h->bc;
  if (phi) *phi = h->phi;
  if (density) *density = h->dens;
  return WG_OK;
}

}  // extern "C"
