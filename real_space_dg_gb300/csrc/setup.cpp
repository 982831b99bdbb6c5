// Host-side discretisation set-up of the 1D Wigner operator.
//
// Restates, from the mathematics, the set-up steps of the reference's 1D path:
//   JacobiGQ/JacobiGL/JacobiP/Vandermonde1D/Dmatrix1D   DG_code/core/*.m
//   grids, mass matrix, constants                      DG_code/initParams.m:58-221
//   plane-wave k basis                                 DG_code/core/Basisfunktionen_Q_m.m:22-33
//   flux blocks K1..K6 and the Delta-xi mass scaling   DG_code/core/get_Diff.m:22-45
//   CAP profile                                        DG_code/core/get_CAP.m:1-12
//   quadrature points, interpolation W = V~/V          get_Drift_accel_trial_permutedShell.m:15-55,183
//   contact occupation f(k) -> xi -> k                 DG_code/core/verteilung.m:118-170
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>

namespace wg {

namespace {

std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> v(n);
  if (n == 1) { v[0] = b; return v; }
  const double step = (b - a) / (n - 1);
  for (int i = 0; i < n; ++i) v[i] = a + i * step;
  v[n - 1] = b;
  return v;
}

// Eigenvalues of a small symmetric matrix by cyclic Jacobi rotations (ascending).
std::vector<double> sym_eigvals(std::vector<double> A, int n) {
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (A[q * n + q] - A[p * n + p]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
      }
  }
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = A[i * n + i];
  std::sort(d.begin(), d.end());
  return d;
}

// Gauss nodes of the Jacobi weight (JacobiGQ.m): eigenvalues of the recurrence matrix.
std::vector<double> jacobi_gq_nodes(double alpha, double beta, int n) {
  if (n == 0) return {-(alpha - beta) / (alpha + beta + 2)};
  const int m = n + 1;
  std::vector<double> J(m * m, 0.0);
  for (int i = 0; i < m; ++i) {
    const double h1 = 2.0 * i + alpha + beta;
    J[i * m + i] = -0.5 * (alpha * alpha - beta * beta) / (h1 + 2) / h1;
  }
  if (alpha + beta < 10 * 2.220446049250313e-16) J[0] = 0.0;
  for (int i = 1; i <= n; ++i) {
    const double h1 = 2.0 * (i - 1) + alpha + beta;
    const double v = 2.0 / (h1 + 2) *
                     std::sqrt(i * (i + alpha + beta) * (i + alpha) * (i + beta) / (h1 + 1) / (h1 + 3));
    J[(i - 1) * m + i] = v;
    J[i * m + (i - 1)] = v;
  }
  return sym_eigvals(J, m);
}

double legendre(int n, double x) {
  double p0 = 1.0, p1 = x;
  if (n == 0) return p0;
  for (int k = 1; k < n; ++k) {
    const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// Gauss-Lobatto nodes/weights (JacobiGL.m), alpha = beta = 0.
void jacobi_gl(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n + 1, 0.0);
  w.assign(n + 1, 0.0);
  if (n == 0) { x[0] = 0; w[0] = 2; return; }
  if (n == 1) { x = {-1, 1}; w = {1, 1}; return; }
  std::vector<double> xi = jacobi_gq_nodes(1, 1, n - 2);
  x[0] = -1;
  for (int i = 0; i < n - 1; ++i) x[i + 1] = xi[i];
  x[n] = 1;
  const int m = n + 1;
  for (int i = 0; i < (m + 1) / 2; ++i) {
    const double P = legendre(m - 1, x[i]);
    w[i] = 2.0 / (m * (m - 1)) / (P * P);
    w[m - 1 - i] = w[i];
  }
}

// Orthonormal Jacobi polynomial of order n (JacobiP.m), alpha, beta integers here.
double jacobi_p(double x, double alpha, double beta, int n) {
  const double gamma0 = std::pow(2.0, alpha + beta + 1) / (alpha + beta + 1) * std::tgamma(alpha + 1) *
                        std::tgamma(beta + 1) / std::tgamma(alpha + beta + 1);
  double pm1 = 1.0 / std::sqrt(gamma0);
  if (n == 0) return pm1;
  const double gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0;
  double p = ((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / std::sqrt(gamma1);
  if (n == 1) return p;
  double aold = 2 / (2 + alpha + beta) * std::sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3));
  for (int i = 1; i < n; ++i) {
    const double h1 = 2 * i + alpha + beta;
    const double anew = 2 / (h1 + 2) *
                        std::sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) * (i + 1 + beta) /
                                  (h1 + 1) / (h1 + 3));
    const double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
    const double pn = 1 / anew * (-aold * pm1 + (x - bnew) * p);
    pm1 = p;
    p = pn;
    aold = anew;
  }
  return p;
}

double grad_jacobi_p(double r, int n) {
  if (n == 0) return 0.0;
  return std::sqrt(n * (n + 1.0)) * jacobi_p(r, 1, 1, n - 1);
}

// Dense inverse by Gauss-Jordan with partial pivoting (row-major, small n).
std::vector<double> inverse(const std::vector<double>& A, int n) {
  std::vector<double> a = A, inv(n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[piv * n + k]);
        std::swap(inv[c * n + k], inv[piv * n + k]);
      }
    const double d = a[c * n + c];
    for (int k = 0; k < n; ++k) { a[c * n + k] /= d; inv[c * n + k] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
  return inv;
}

std::vector<double> matmul(const std::vector<double>& A, const std::vector<double>& B, int m, int k, int n) {
  std::vector<double> C(m * n, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0;
      for (int l = 0; l < k; ++l) s += A[i * k + l] * B[l * n + j];
      C[i * n + j] = s;
    }
  return C;
}

double cap_profile(double q, double l_xi, double delta_xi) {
  const double W0 = 1.0, n = 1.0;
  const double L0 = l_xi / 2 - delta_xi;
  const double weite = l_xi * 0.40;
  double v = 0.0;
  if (q >= L0 - weite) v += std::pow(W0 / weite * (q - L0 + weite), 2 * n);
  if (q <= -L0 + weite) v += std::pow(W0 / weite * (q + L0 - weite), 2 * n);
  return v;
}

// Householder QR of a (m x n, row-major, m >= n) in place.
void householder_qr(std::vector<cplx>& a, std::vector<cplx>& tau, int m, int n) {
  tau.assign(n, cplx(0));
  for (int j = 0; j < n; ++j) {
    double nrm2 = 0;
    for (int i = j; i < m; ++i) nrm2 += std::norm(a[i * n + j]);
    const double nrm = std::sqrt(nrm2);
    if (nrm == 0) continue;
    const cplx x0 = a[j * n + j];
    const cplx phase = std::abs(x0) > 0 ? x0 / std::abs(x0) : cplx(1);
    const cplx alpha = -phase * nrm;
    // v = x - alpha e1, stored in column j below and at the diagonal; normalise so v0 = 1
    const cplx v0 = x0 - alpha;
    for (int i = j + 1; i < m; ++i) a[i * n + j] /= v0;
    // tau = (v^H v)^{-1} * 2 with v0 = 1
    double vnorm2 = 1.0;
    for (int i = j + 1; i < m; ++i) vnorm2 += std::norm(a[i * n + j]);
    const double t = 2.0 / vnorm2;
    tau[j] = t;
    a[j * n + j] = alpha;
    for (int c = j + 1; c < n; ++c) {
      cplx s = a[j * n + c];
      for (int i = j + 1; i < m; ++i) s += std::conj(a[i * n + j]) * a[i * n + c];
      s *= t;
      a[j * n + c] -= s;
      for (int i = j + 1; i < m; ++i) a[i * n + c] -= s * a[i * n + j];
    }
  }
}

}  // namespace

std::string build_shape_light(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff,
                              double mpc) {
  if (n_el < 2) return "n_el must be >= 2";
  if (nK < 2 || nK > kMaxLocal) return "n_local must be 2..4 (DG order 1..3)";
  if (nk < 2) return "nk must be >= 2";
  if (nxi < nk) return "n_xi must be >= nk (least-squares contact projection)";
  if (!(l_xi > 0)) return "l_xi must be positive";
  s.n_el = n_el; s.nK = nK; s.nk = nk; s.nxi = nxi; s.l_xi = l_xi;
  s.m_diff = m_diff > 0 ? m_diff : kMElektronRef;
  s.q_diff = kHquer / s.m_diff;
  s.q_drift = kQ / kHquer;
  s.mpc = mpc != 0 ? mpc : 1.0;
  // xi grids (initParams.m:178-182, permutedShell.m:27-28)
  std::vector<double> xi = linspace(-l_xi / 2, l_xi / 2, nxi);
  s.delta_xi = xi[1] - xi[0];
  s.xi_elem = linspace(-(l_xi - s.delta_xi) / 2, (l_xi - s.delta_xi) / 2, nxi);
  s.xi_edge = linspace(-l_xi / 2, l_xi / 2, nxi + 1);
  s.cap.resize(nxi + 1);
  for (int i = 0; i <= nxi; ++i) s.cap[i] = cap_profile(s.xi_edge[i], l_xi, s.delta_xi);
  // DG reference element (initParams.m:186-191)
  jacobi_gl(kNqx - 1, s.gl_x, s.gl_w);
  std::vector<double> rw;
  jacobi_gl(nK - 1, s.r, rw);
  std::vector<double> V(nK * nK), Vt(kNqx * nK), Vr(nK * nK);
  for (int i = 0; i < nK; ++i)
    for (int j = 0; j < nK; ++j) {
      V[i * nK + j] = jacobi_p(s.r[i], 0, 0, j);
      Vr[i * nK + j] = grad_jacobi_p(s.r[i], j);
    }
  for (int i = 0; i < kNqx; ++i)
    for (int j = 0; j < nK; ++j) Vt[i * nK + j] = jacobi_p(s.gl_x[i], 0, 0, j);
  const std::vector<double> invV = inverse(V, nK);
  std::vector<double> invVt(nK * nK);
  for (int i = 0; i < nK; ++i)
    for (int j = 0; j < nK; ++j) invVt[i * nK + j] = invV[j * nK + i];
  s.M = matmul(invVt, invV, nK, nK, nK);
  // Flux blocks (get_Diff.m:22-45)
  std::vector<double> Dm = matmul(Vr, invV, nK, nK, nK);
  std::vector<double> Dr = matmul(s.M, Dm, nK, nK, nK);
  for (double& d : Dr)
    if (std::fabs(d) < 1e-15) d = 0.0;
  std::vector<double> Ms(nK * nK);
  for (int i = 0; i < nK * nK; ++i) Ms[i] = s.delta_xi / 2 * s.M[i];
  s.invM = inverse(Ms, nK);
  std::vector<double> T1 = Dr;
  T1[0] += 0.5;
  T1[(nK - 1) * nK + (nK - 1)] -= 0.5;
  s.K1 = matmul(s.invM, T1, nK, nK, nK);
  s.K2.assign(nK * nK, 0.0);
  s.K3.assign(nK * nK, 0.0);
  s.K5.assign(nK * nK, 0.0);
  for (int a = 0; a < nK; ++a) {
    s.K2[a * nK + 0] += s.invM[a * nK + 0] * 0.5;
    s.K2[a * nK + nK - 1] += s.invM[a * nK + nK - 1] * 0.5;
    s.K3[a * nK + nK - 1] = -0.5 * s.invM[a * nK + 0];
    s.K5[a * nK + 0] = 0.5 * s.invM[a * nK + nK - 1];
  }
  // Interpolation to the quadrature points and drift weights
  s.W = matmul(Vt, invV, kNqx, nK, nK);
  s.kap.assign(nK * nK * kNqx, 0.0);
  s.kap_sum.assign(nK * nK, 0.0);
  for (int a = 0; a < nK; ++a)
    for (int b = 0; b < nK; ++b)
      for (int q = 0; q < kNqx; ++q) {
        const double v = s.q_drift * s.invM[a * nK + b] * s.gl_w[q] * s.W[q * nK + a] * s.W[q * nK + b];
        s.kap[(a * nK + b) * kNqx + q] = v;
        s.kap_sum[a * nK + b] += v;
      }
  // Plane-wave basis (Basisfunktionen_Q_m.m:22-33)
  s.k.resize(nk);
  for (int j = 0; j < nk; ++j) s.k[j] = -2 * M_PI / l_xi * ((j + 1) - 0.5 * (nk + 1));
  s.phi.resize((size_t)nxi * nk);
  const double sc = std::sqrt(l_xi);
  for (int i = 0; i < nxi; ++i)
    for (int j = 0; j < nk; ++j) {
      const double th = s.xi_elem[i] * s.k[j];
      s.phi[(size_t)i * nk + j] = cplx(std::cos(th), std::sin(th)) / sc;
    }
  s.cosm.resize((size_t)nxi * nk);
  for (int i = 0; i < nxi; ++i)
    for (int j = 0; j < nk; ++j) s.cosm[(size_t)i * nk + j] = std::cos(s.xi_elem[i] * s.k[j]);
  return "";
}

std::string build_shape(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff, double mpc) {
  std::string e = build_shape_light(s, n_el, nK, nk, nxi, l_xi, m_diff, mpc);
  if (!e.empty()) return e;
  s.qr = s.phi;
  householder_qr(s.qr, s.tau, nxi, nk);
  // Phi^+ column by column: z = argmin |Phi z - e_i|
  s.pinv.assign((size_t)nk * nxi, cplx(0));
  std::vector<cplx> unit(nxi), z;
  for (int i = 0; i < nxi; ++i) {
    std::fill(unit.begin(), unit.end(), cplx(0));
    unit[i] = 1.0;
    phi_lstsq(s, unit, z);
    for (int j = 0; j < nk; ++j) s.pinv[(size_t)j * nxi + i] = z[j];
  }
  return "";
}

std::string build_shape_cached(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff,
                               double mpc) {
  // The expensive part (QR and pseudo-inverse of Phi) depends only on (nk, nxi, l_xi).
  struct Key {
    int nk, nxi;
    double l_xi;
    bool operator<(const Key& o) const {
      if (nk != o.nk) return nk < o.nk;
      if (nxi != o.nxi) return nxi < o.nxi;
      return l_xi < o.l_xi;
    }
  };
  static std::mutex mu;
  static std::map<Key, std::shared_ptr<const Shape>> cache;
  const Key key{nk, nxi, l_xi};
  std::shared_ptr<const Shape> hit;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) hit = it->second;
  }
  if (hit && hit->n_el == n_el && hit->nK == nK && hit->m_diff == (m_diff > 0 ? m_diff : kMElektronRef) &&
      hit->mpc == (mpc != 0 ? mpc : 1.0)) {
    s = *hit;
    return "";
  }
  if (hit) {
    // same xi/k basis, different element data: rebuild the cheap part, reuse QR and Phi^+
    Shape t;
    std::vector<cplx> qr = hit->qr, tau = hit->tau, pinv = hit->pinv;
    std::string e = build_shape_light(t, n_el, nK, nk, nxi, l_xi, m_diff, mpc);
    if (!e.empty()) return e;
    t.qr = std::move(qr);
    t.tau = std::move(tau);
    t.pinv = std::move(pinv);
    s = t;
    return "";
  }
  std::string e = build_shape(s, n_el, nK, nk, nxi, l_xi, m_diff, mpc);
  if (!e.empty()) return e;
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = std::make_shared<const Shape>(s);
  return "";
}

void phi_lstsq(const Shape& s, const std::vector<cplx>& f, std::vector<cplx>& z) {
  const int m = s.nxi, n = s.nk;
  std::vector<cplx> y = f;
  for (int j = 0; j < n; ++j) {
    if (s.tau[j] == cplx(0)) continue;
    cplx t = y[j];
    for (int i = j + 1; i < m; ++i) t += std::conj(s.qr[(size_t)i * n + j]) * y[i];
    t *= s.tau[j];
    y[j] -= t;
    for (int i = j + 1; i < m; ++i) y[i] -= t * s.qr[(size_t)i * n + j];
  }
  z.assign(n, cplx(0));
  for (int i = n - 1; i >= 0; --i) {
    cplx acc = y[i];
    for (int c = i + 1; c < n; ++c) acc -= s.qr[(size_t)i * n + c] * z[c];
    z[i] = acc / s.qr[(size_t)i * n + i];
  }
}

void quad_points(const Shape& s, double l_chi, std::vector<double>& xq) {
  const double dchi = l_chi / s.n_el;
  std::vector<double> disk = linspace(0.0, l_chi, s.n_el + 1);
  double chi_gl[kNqx];
  chi_gl[0] = 0.0;
  for (int i = 0; i < kNqx - 1; ++i) chi_gl[i + 1] = chi_gl[i] + (s.gl_x[i + 1] - s.gl_x[i]) / 2 * dchi;
  xq.resize((size_t)s.n_el * kNqx);
  for (int e = 0; e < s.n_el; ++e)
    for (int q = 0; q < kNqx; ++q) xq[(size_t)e * kNqx + q] = disk[e] + chi_gl[q];
}

}  // namespace wg
