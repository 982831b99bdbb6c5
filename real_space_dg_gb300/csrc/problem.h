// Device-side state of a wg_problem handle (internal header).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>
#include <array>
#include <vector>

#include "setup.h"
#include "wigner_gb300.h"

namespace wg {

// Small constant blocks passed by value to kernels (fits the parameter space).
struct FluxBlocks {
  int nK;
  int single;        // 1: K3 couples only the last node of the left element, K5 only the first of the right
  double K1[kMaxLocal * kMaxLocal];
  double K2[kMaxLocal * kMaxLocal];
  double K3[kMaxLocal * kMaxLocal];
  double K5[kMaxLocal * kMaxLocal];
  double invM[kMaxLocal * kMaxLocal];
  double Kp[kMaxLocal * kMaxLocal];   // K1 + K2: k K1 + |k| K2 = k Kp for k > 0
  double Km[kMaxLocal * kMaxLocal];   // K1 - K2: ... = k Km for k < 0
  double K3c[kMaxLocal];              // 2 K3[a][nK-1]: (k + |k|) K3 x_left = k K3c x_left[nK-1]
  double K5c[kMaxLocal];              // 2 K5[a][0]:    (k - |k|) K5 x_right = k K5c x_right[0]
};

// FP32 copies of the flux blocks for the mixed form (no FP64 instruction per element).
struct FluxBlocks32 {
  int nK;
  float Kp[kMaxLocal * kMaxLocal];
  float Km[kMaxLocal * kMaxLocal];
  float K3c[kMaxLocal];
  float K5c[kMaxLocal];
};

// Fill the derived blocks (Kp, Km, K3c, K5c, single) from K1, K2, K3, K5.
inline void finish_flux_blocks(FluxBlocks& fb) {
  const int n = fb.nK;
  bool single = true;
  for (int a = 0; a < n; ++a)
    for (int c = 0; c < n; ++c) {
      fb.Kp[a * n + c] = fb.K1[a * n + c] + fb.K2[a * n + c];
      fb.Km[a * n + c] = fb.K1[a * n + c] - fb.K2[a * n + c];
      if (c != n - 1 && fb.K3[a * n + c] != 0.0) single = false;
      if (c != 0 && fb.K5[a * n + c] != 0.0) single = false;
    }
  for (int a = 0; a < n; ++a) {
    fb.K3c[a] = 2.0 * fb.K3[a * n + n - 1];
    fb.K5c[a] = 2.0 * fb.K5[a * n + 0];
  }
  fb.single = single ? 1 : 0;
}

// Per-problem scalar parameters on the device: pp[b * kPP + PP_*].
constexpr int kPP = 10;
enum { PP_LX = 0, PP_QD, PP_M0, PP_M1, PP_MEZ, PP_TEMP, PP_EFL, PP_EFR, PP_VMIN, PP_VMAX };

// Per-problem host copy of the set-up that stays fixed until the next set_potential.
struct HostProblem {
  bool ready = false;
  double l_chi = 0;                 // device length [m]
  double qd = 0;                    // Q_diff * mpc / detJ
  double ef_l = 0, ef_r = 0;        // contact Fermi levels [eV]
  std::vector<double> m_nodes;      // mass at the DG nodes [kg]
};

// Device buffers of the mixed-precision inner solver (allocated only for WG_PREC_MIXED).
struct MixedBuffers {
  __nv_bfloat16* phi1 = nullptr;     // [2 N_xi][2 Nk]  real embedding of Phi (GEMM 1 A operand)
  __nv_bfloat16* phi2 = nullptr;     // [2 Nk][2 N_xi]  real embedding of i Phi^H (GEMM 2 A operand)
  __nv_bfloat162* xin16 = nullptr;   // [B*N] bf16 staging of a GEMM 1 B operand
  __nv_bfloat162* zb16 = nullptr;    // [B*N] bf16 copy of the preconditioned vector
  __nv_bfloat162* yh16 = nullptr;    // [ncols][N_xi] bf16 stencil output (GEMM 2 B operand)
  float2* xh = nullptr;              // [ncols][N_xi] fp32 GEMM 1 output
  float2* V = nullptr;               // [B][m_inner+1][N] fp32 Krylov basis
  __half2* Vh = nullptr;             // the same basis stored in FP16 (basis16; V is then unused)
  bool basis16 = false;              // inner basis stored in FP16, arithmetic in FP32
  float2* w = nullptr;               // [B*N]
  float2* z = nullptr;               // [B*N]
  float2* r = nullptr;               // [B*N] normalised outer residual
  float2* d = nullptr;               // [B*N] inner correction
  // fp32 copies of the potential weights, rows padded to ne4 = (nxi + 1) rounded up to 4:
  // beta [B][n_el][nK(nK+1)/2][ne4] holds the pairs a <= c only (the weights are symmetric),
  // betai [nK*nK][ne4] the CAP part
  float* beta = nullptr;
  float* betai = nullptr;
  int ne4 = 0;
  float* kvec = nullptr;             // [nk]
  float* qd = nullptr;               // [B]
  float* dinv = nullptr;             // [nk][nK*nK]
  float* h = nullptr;                // [nk][nK]
  float2* hcol = nullptr;            // [B][m+1] Gram-Schmidt coefficients in FP32
  float2* y = nullptr;               // [B][m] Hessenberg solution in FP32
  float* inv = nullptr;              // [B] 1/|w| in FP32
  FluxBlocks32 fb;
  int* err = nullptr;                // raised by a GEMM whose barrier wait timed out
  CUtensorMap tmA1, tmB1, tmB1z, tmA2, tmB2;
  CUtensorMap tmB1n, tmB1zn;          // the GEMM 1 B operands in 64-column boxes (fused GEMM 1 + stencil)
  bool fused = false;                // the apply runs as GEMM 1 + stencil and GEMM 2 + flux (two launches)
  // FP64 outer residual on the tensor cores (digit slices, see ozaki.cuh)
  bool ozaki = false;
  __nv_bfloat16* oa1 = nullptr;      // [S][2 N_xi][2 Nk] digits of Phi'
  __nv_bfloat16* oa2 = nullptr;      // [S][2 Nk][2 N_xi] digits of (i Phi^H)'
  int* ea1 = nullptr;                // [2 N_xi] row exponents
  int* ea2 = nullptr;                // [2 Nk]
  __nv_bfloat16* ob = nullptr;       // [S][ncols][max(2 Nk, 2 N_xi)] digits of the B operand
  int* eb = nullptr;                 // [ncols] column exponents
  CUtensorMap tmOA1, tmOA2, tmOB1, tmOB2;
};

// Kernel classes timed and counted by the profiler.
enum ProfClass { PROF_FLUX = 0, PROF_GEMM_F64, PROF_GEMM_BF16, PROF_STENCIL, PROF_PRECOND, PROF_MULTIDOT,
                 PROF_GSUPDATE, PROF_KRYLOV, PROF_OTHER, PROF_GEMM_F64TC, PROF_FLUX64, PROF_STENCIL64, PROF_GEMM_STENCIL,
                 PROF_GEMM_FLUX, PROF_N };

// CUDA-event timing of kernel classes on the handle's stream (off by default;
// launch counts are kept always).
struct Profiler {
  bool on = false;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> pending;
  double ms[PROF_N] = {};
  long long timed[PROF_N] = {};
  long long launches[PROF_N] = {};
  double bytes[PROF_N] = {};   // algorithmic bytes of the timed launches
  double flops[PROF_N] = {};   // algorithmic flops of the timed launches
  std::vector<double> pend_bytes, pend_flops;
  // Work actually done by a masked launch: a one-warp kernel enqueued just before the
  // launch's start event writes, into slot i, the fraction of the batch the launch's
  // mask lets through and the digit-weighted fraction of an emulated FP64 GEMM (see
  // prof_begin); the pending bytes / flops (given for the whole batch) are scaled by
  // them when collected.  Slot -1: an unmasked launch that processes every problem.
  std::vector<int> pend_slot;
  double* d_frac = nullptr;    // [kProfSlots][2] on the device (allocated on first use)
  static constexpr int kProfSlots = 8192 + 16;
};

// CUDA graphs of the Arnoldi steps: the launches of each chunk of steps (steps 0, 1, 2-3,
// then 4 at a time) of one restart cycle are captured once (on the chunk's second use, after the launch
// helpers' one-time set-up ran eagerly) and replayed in later cycles and refinements.
// Every kernel argument of a chunk is a device pointer or a per-handle constant except
// the flux shift, so the graphs are rebuilt when the shift (or the restart length)
// changes.  Disabled by WG_CUDA_GRAPHS=0 and while the per-launch profiler is on.
struct ArnoldiGraphs {
  std::vector<cudaGraphExec_t> exec;               // per chunk, nullptr until captured
  std::vector<std::array<long long, PROF_N>> launches;   // profiler launch counts of one replay
  std::vector<int> eager;                          // eager runs of the chunk so far
  double shift = 0;
  int m = -1;
  int kline_L = -1, st_cells = -1;                 // launch shapes the graphs were captured with
  bool disabled = false;
  long long replays = 0;
};

// Device arrays of the Gummel loop (allocated on the first wg_gummel_set).
struct GummelDev {
  double* vc = nullptr;      // [B][nx] band edge
  double* nd = nullptr;      // [B][nx] donors
  double* phi = nullptr;     // [B][nx] electrostatic potential
  double* phi0 = nullptr;    // [B][nx] initial potential of wg_gummel_set
  double* cand = nullptr;    // [B][nx] Poisson candidate
  double* ncv = nullptr;     // [B][nx] control-volume density
  double* tri = nullptr;     // [B][3][nx] Poisson stencil (lower, diagonal, upper)
  double* work = nullptr;    // [B][2][nx] Thomas scratch
  double* projc = nullptr;   // [B][nx][2][kMaxLocal] projection weights
  int* proje = nullptr;      // [B][nx][2] projection element indices (-1: none)
  double* ndg = nullptr;     // [B][ncol] density at the DG nodes [m^-3]
  double* jdg = nullptr;     // [B][ncol] current density at the DG nodes
  double* nprev = nullptr;   // [B][ncol] previous iteration's density
  double* diag = nullptr;    // [B][8] Poisson-step diagnostics
  double* bias = nullptr;    // [B]
  double* temp = nullptr;    // [B]
  double* scale = nullptr;   // [B] |Vsub|^2 / dy
  int* active = nullptr;     // [B]
  int* mix = nullptr;        // [B]
};

struct GummelHost {
  bool ready = false;
  double bias = 0;
  bool step_pending = false;   // a transient bias step waits for its potential re-solve
  // state of the problem's Gummel loop
  int running = 0;             // 1 while the loop iterates
  int it = 0;                  // iterations done
  double tol = 0;              // transport tolerance of the next solve
  double t0 = 0;               // start of the loop [s, steady clock]
  int waiting = -1;            // >= 0: iterations spent waiting for the batched final re-solve
  wg_gummel_info info{};
};

struct Problem {
  // shape
  Shape s;
  int batch = 0;
  int precision = WG_PREC_FP64;
  int restart = 50;
  int restart_inner = 40;   // inner GMRES length of the mixed form
  int restart_max = 50;     // sizes the Hessenberg storage: max(restart, restart_inner)
  double inner_tol = 1e-3;  // floor of the inner relative tolerance of the mixed form
  double reorth_eta = 0.7071067811865476;        // DGKS threshold of the FP64 Arnoldi (>= 1 always, < 0 never)
  double inner_reorth_eta = -1.0;                // the same for the mixed form's inner FP32 Arnoldi
  long long N = 0;          // complex entries per problem
  long long ncols = 0;      // DG nodes in the batch = batch * n_el * nK
  double device_bytes = 0;
  double mem_budget = 0;
  FluxBlocks fb{};
  double shift = 0;         // sigma of the shifted operator A + sigma I (0: the stationary A)
  bool fp64_tc = false;     // FP64 handle whose transforms run as FP64 emulated on the tensor cores
  bool inner_basis16 = true;  // mixed form: the inner Krylov basis stored in FP16
  std::string err;

  std::vector<HostProblem> hp;

  cudaStream_t stream = nullptr;
  // constant device data
  double2* phi = nullptr;        // nxi x nk row-major
  double* kvec = nullptr;        // nk
  double* xi_edge = nullptr;     // nxi + 1
  double* kap = nullptr;         // nK*nK*10
  double* betai = nullptr;       // [nK*nK][nxi+1] CAP part of the potential weights (imaginary)
  double* pre_dinv = nullptr;    // [B][nk][nK*nK] inverse of k K1 + |k| K2 + shift/qd_b
  double* pre_h = nullptr;       // [B][nk][nK] that inverse times the coupling column
  void* kmap_a = nullptr;        // [B][n_chunks][nk] k-line chunk maps: factor (double or float)
  void* kmap_s = nullptr;        // [B][n_chunks][nk] k-line chunk maps: offset (double2 or float2)
  double* cosm = nullptr;        // [nxi][nk] cos(xi_s k_j)
  double2* pinv = nullptr;       // [nk][nxi] pseudo-inverse of Phi
  // per-problem device data
  double* qd = nullptr;          // [B]
  double* pp = nullptr;          // [B][kPP] per-problem scalars
  double* flr = nullptr;         // [B][2][nk] contact occupations f_L, f_R
  double* fxi = nullptr;         // [B][2][nxi] their cosine transforms to the xi cells
  double* beta = nullptr;        // [B][n_el][nK*nK][nxi+1] real potential weights
  double* xq = nullptr;          // [B][n_el*10] quadrature x [m]
  double* pot_x = nullptr;       // [B][nx] material grid [m]
  double* pot_v = nullptr;       // [B][nx] potential [eV]
  double* vslope = nullptr;      // [B][nx] slopes of its linear interpolation
  double* m_nodes = nullptr;     // [B][n_el*nK] masses at DG nodes [kg]
  int nx = 0;
  // vectors
  double2* rhs = nullptr;        // [B*N]
  double2* tr_b = nullptr;       // [B*N] Crank-Nicolson right-hand side (allocated by the first transient)
  double2* x = nullptr;          // [B*N] solution (resident across solves)
  double2* w = nullptr;          // [B*N] work
  double2* z = nullptr;          // [B*N] work
  double2* r = nullptr;          // [B*N] work
  double2* V = nullptr;          // [B][m+1][N] Krylov basis
  double2* xh = nullptr;         // [nxi][ncols] transformed state
  double2* yh = nullptr;         // [nxi][ncols]
  // GMRES small data
  double2* H = nullptr;          // [B][m+1][m] column-major per problem: H[b][col*(m+1)+row]
  double2* cs = nullptr;         // [B][m]
  double2* sn = nullptr;         // [B][m]
  double2* g = nullptr;          // [B][m+1]
  double2* hcol = nullptr;       // [B][m+1] current column partial results
  double2* ycoef = nullptr;      // [B][m]
  double2* partial = nullptr;    // [B][m+1][nchunk]
  double* nrm_partial = nullptr; // [B][nchunk]
  double* nrm = nullptr;         // [B]
  double* nrm_keep = nullptr;    // [B] outer residual norms of the mixed refinement
  double* inv64 = nullptr;       // [B] inverse basis-vector norms
  double* target = nullptr;      // [B] absolute residual targets
  int* active = nullptr;         // [B] 1 while iterating in this cycle
  int* reorth = nullptr;         // [B] 1 where the current Arnoldi step re-orthogonalises
  int* res_mask = nullptr;       // [B] problems whose true residual is evaluated
  int* res_digits = nullptr;     // [B] digits of the emulated FP64 transforms per problem
  std::vector<int> h_res_digits;
  ArnoldiGraphs graphs[2];       // [0] FP64 basis, [1] the mixed form's FP32 inner basis
  // launch shapes picked by the autotuner (tune.cu) on the first solve of a shape
  int kline_L = 4;               // elements per k-line chunk
  int st_cells = 4;              // xi cells per thread of the FP32 stencil
  bool tuned = false;
  std::vector<int> h_res_mask;
  int* md_count = nullptr;       // [B] last-block tickets of the multi-dot (zero between launches)
  int* gs_count = nullptr;       // [B] last-block tickets of the Gram-Schmidt update
  int* kused = nullptr;          // [B] iterations used in this cycle
  int* any_active = nullptr;     // [1]
  int nchunk = 0;  // 2048-element chunks of one problem vector (multi-dot partials)
  int nblk = 0;    // 256-element blocks of one problem vector (norm partials)
  // host mirrors
  std::vector<double> h_nrm;
  std::vector<int> h_active, h_kused;

  MixedBuffers mx;
  Profiler prof;
  GummelDev gd;
  std::vector<GummelHost> gh;
  cudaEvent_t ev[16] = {};       // user event slots (wg_event_record)
  std::vector<double> tol_pp;    // per-problem relative tolerances for the next solve (empty: opts.tol)
};

// Profiler helpers (operator.cu).  prof_begin counts `n` launches of class cls
// and, when timing is on, records a start event; prof_end records the stop event.
// bytes / flops are the algorithmic work of the launch for all `batch` problems.
// When the launch skips problems (mask: problems b with mask[b] == 0 do nothing) the
// work is credited only for the problems it processes; an emulated FP64 GEMM with
// nd > 0 leading digits (per problem nd_pp[b] when given) is credited with
// nd (nd + 1) / 2 digit-slice products per problem, `flops` being one product.
cudaEvent_t prof_begin(Problem& P, int cls, int n = 1, double bytes = 0, double flops = 0,
                       const int* mask = nullptr, int nd = 0, const int* nd_pp = nullptr);
void prof_end(Problem& P, int cls, cudaEvent_t a);
cudaError_t prof_collect(Problem& P);
void prof_release(Problem& P);

// Kernel launchers (operator.cu)
cudaError_t launch_apply(Problem& P, const double2* x, double2* y);
// rscale (device, optional): r enters scaled by rscale[b]; rout (optional): the scaled r is written there
// (per-problem stride rout_stride), the Arnoldi step's next basis vector.
cudaError_t launch_precondition(Problem& P, const double2* r, long long r_stride, double2* z,
                                const double* rscale = nullptr, double2* rout = nullptr, long long rout_stride = 0);
// k-line factors of A + sigma I for every problem (sigma = P.shift), uploaded to pre_dinv / pre_h.
int set_kline_factors(Problem& P);
// Device bytes of a handle before allocation (the admission estimate of wg_problem_create).
double estimate_bytes(const Shape& s, int batch, int restart, int restart_inner, int precision, bool fp64_tc = false,
                      bool basis16 = true);
cudaError_t launch_flux_f64(Problem& P, const double2* x, double2* y, const int* mask = nullptr);
cudaError_t launch_stencil_f64(Problem& P, const double2* xh, double2* yh, const int* mask = nullptr);
// FP64 operator apply with the transforms emulated on the tensor cores (mixed form only).
// nd: leading digits of the emulated FP64 transforms (8: ~1e-14 of |Phi||x|; fewer for a
// residual that only has to resolve a loose tolerance, ~2^(-6 nd)).
cudaError_t launch_apply_f64_tc(Problem& P, const double2* x, double2* y, const int* mask = nullptr, int nd = 8,
                                const int* nd_pp = nullptr);
int debug_gemm_f64_tc(const double* A, const double* B, double* C, int M, int N, int K, std::string& err, int nd = 8);
// Rebuild potential-dependent data (Vw weights, contact inflow rhs) of problems [b0, b1).
// mask (device, optional): problems b with mask[b] == 0 are left untouched.
cudaError_t launch_potential_update(Problem& P, int b0, int b1, const int* mask = nullptr);
cudaError_t launch_observables(Problem& P, int b, double* n_dg, double* j);
cudaError_t launch_rho_xi(Problem& P, int b, double2* out);
// Allocation-free operator apply on caller-owned device buffers (operator.cu).
int apply_noalloc(const wg_operator_view& v, const double* x, double* y, void* stream, std::string& err);
// Krylov (gmres.cu)
int gmres_solve_fp64(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info);
// Mixed form (mixed.cu)
std::string mixed_check_shape(const Shape& s);
double mixed_bytes(const Shape& s, int batch, int restart, bool basis16);
int mixed_alloc(Problem& P);
// Digit slices of Phi, state slice buffer and tensor maps of the FP64 emulation (any precision).
int ozaki_alloc(Problem& P);
void mixed_free(Problem& P);
cudaError_t mixed_sync_weights(Problem& P);
// mask (device, optional): problems b with mask[b] == 0 are skipped (their output is left as is).
cudaError_t launch_apply_mixed(Problem& P, const float2* x, const __nv_bfloat162* xb, float2* y,
                               const int* mask = nullptr);
cudaError_t launch_precondition_mixed(Problem& P, const float2* r, long long r_stride, float2* z,
                                      __nv_bfloat162* zb, const int* mask = nullptr, const float* rscale = nullptr,
                                      float2* rout = nullptr, long long rout_stride = 0);
// The same with the (scaled) input rounded to FP16 first and written to rout, an FP16 basis
// vector: the preconditioner works on exactly the vector the basis stores.
cudaError_t launch_precondition_mixed_h(Problem& P, const float2* r, long long r_stride, float2* z,
                                        __nv_bfloat162* zb, const int* mask, const float* rscale, __half2* rout,
                                        long long rout_stride);
// The FP32 xi stencil alone (M.xh -> M.yh16, every problem), for the autotuner.
cudaError_t launch_stencil_mixed(Problem& P);
cudaError_t apply_mixed_f64(Problem& P, const double2* x, double2* y);
cudaError_t apply_mixed_repeat(Problem& P, const double2* x, int n_apply);
int debug_gemm_bf16(const float* A, const float* B, float* C, int M, int N, int K, std::string& err);
int debug_wait_timeout(long long limit, std::string& err);
int gmres_solve_mixed(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info);
// FP64 GMRES or the mixed-precision refinement, by P.precision.
int solve_dispatch(Problem& P, const wg_solve_opts& o, bool warm, wg_solve_info* info);
// Picks the handle's launch shapes (k-line chunk length, FP32 stencil cells per thread)
// by timing the candidates on the handle's own buffers; the choice is cached per shape
// (n_el, N_K, Nk, N_xi, precision) for the process.  WG_AUTOTUNE=0 keeps the defaults.
int autotune(Problem& P);
// Gummel loop (gummel.cu)
int gummel_set(Problem& P, int b, const wg_device& dev, const wg_rtd_1d& rtd);
int gummel_run(Problem& P, const wg_gummel_opts& o, wg_gummel_info* info);
// Problem b's loop from its current state: warm keeps its Wigner function, from_phi0
// resets the potential to the phi0 of wg_gummel_set.
int gummel_start(Problem& P, int b, const wg_gummel_opts& o, bool warm, bool from_phi0);
// One iteration of every running loop (the others keep their state untouched).
int gummel_iterate(Problem& P, const wg_gummel_opts& o, int* still_running);
int gummel_get(Problem& P, int b, double* phi, double* n_dg, double* j);
cudaError_t gummel_observables(Problem& P);                               // ndg, jdg of every problem from x
cudaError_t gummel_poisson(Problem& P, const int* active_dev, bool linear);  // cand, diag
cudaError_t gummel_potential(Problem& P, const int* active_dev);          // pot_v = Vc - phi
cudaError_t gummel_mix(Problem& P, const int* mix_dev, double alpha);
int transient_set_bias(Problem& P, int b, double bias);
int transient_run(Problem& P, const wg_transient_opts& o, double* n_hist, double* j_hist, wg_transient_info* info);
void gummel_free(Problem& P);

}  // namespace wg

// The opaque handle of the C ABI.
struct wg_problem {
  wg::Problem P;
};
