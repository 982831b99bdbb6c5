// Host-side discretisation set-up of the 1D Wigner operator (internal header).
#pragma once
#include <complex>
#include <string>
#include <vector>

namespace wg {

using cplx = std::complex<double>;

constexpr int kNqx = 10;          // Gauss-Lobatto points per element (initParams.m:61)
constexpr int kNkz = 1001;        // kz samples of the contact integral (verteilung.m:142)
constexpr int kMaxLocal = 4;      // N_K_chi <= 4 (DG order p <= 3)

// Constants of initParams.m:101-107.
constexpr double kHquer = 1.054571817e-34;
constexpr double kQ = 1.602176634e-19;
constexpr double kMElektronRef = 0.041 * 9.1094e-31;
// Constants of verteilung.m:161-165 and solve_transport_DG_2D.m:6-8.
constexpr double kHV = 6.626e-34;
constexpr double kM0V = 9.109e-31;
constexpr double kKBV = 1.38e-23;
constexpr double kQV = 1.602e-19;

// Shape-dependent constants shared by every problem of a handle.
struct Shape {
  int n_el = 0, nK = 0, nk = 0, nxi = 0;
  double l_xi = 0, delta_xi = 0, m_diff = 0, q_diff = 0, q_drift = 0, mpc = 1;
  std::vector<double> gl_x, gl_w;       // 10 GL points/weights on [-1,1]
  std::vector<double> r;                // nK GL nodes
  std::vector<double> M;                // nK x nK reference mass (row-major)
  std::vector<double> invM;             // inv(delta_xi/2 * M)
  std::vector<double> K1, K2, K3, K5;   // flux blocks (K4 = K3, K6 = -K5), row-major
  std::vector<double> W;                // 10 x nK interpolation DG nodes -> GL points
  std::vector<double> kap;              // [nK*nK][10]: Q_drift invM(a,b) w_q W(q,a) W(q,b)
  std::vector<double> kap_sum;          // [nK*nK]: sum_q kap
  std::vector<double> k;                // nk wave numbers
  std::vector<double> xi_elem;          // nxi cell centres (rows of Phi)
  std::vector<double> xi_edge;          // nxi+1 edges used by the drift
  std::vector<double> cap;              // CAP(xi_edge)
  std::vector<cplx> phi;                // nxi x nk, row-major (s, j)
  // Householder QR of Phi for the least-squares contact projection
  std::vector<cplx> qr;                 // nxi x nk packed reflectors + R (row-major)
  std::vector<cplx> tau;
  std::vector<cplx> pinv;               // nk x nxi: Phi^+ = R^-1 Q^H (row-major)
  std::vector<double> cosm;             // nxi x nk: cos(xi_s k_j) (verteilung.m:158-161)
};

// Shape constants are pure functions of (n_el, nK, nk, nxi, l_xi, m_diff, mpc);
// the QR and pseudo-inverse of Phi are shared through a process-wide cache.
std::string build_shape_cached(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff,
                               double mpc);

// Build every shape constant.  Returns an empty string on success.
std::string build_shape(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff,
                        double mpc);

// The element/xi constants without the QR and pseudo-inverse of Phi.
std::string build_shape_light(Shape& s, int n_el, int nK, int nk, int nxi, double l_xi, double m_diff,
                              double mpc);

// Quadrature x coordinates (n_el*10) for an element length delta_chi, built as
// cumulative GL spacings (get_Drift_accel_trial_permutedShell.m:16-55).
void quad_points(const Shape& s, double l_chi, std::vector<double>& xq);

// Least-squares solve Phi z = f using the stored QR.
void phi_lstsq(const Shape& s, const std::vector<cplx>& f, std::vector<cplx>& z);

}  // namespace wg
