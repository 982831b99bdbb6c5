/*
 * wigner_gb300.h - C ABI of the GB300-native Wigner-transport solve.
 *
 * Drop-in boundary for the 1D phase-space (x, xi->k) Wigner solve of the
 * reference MATLAB simulator jonasneu1207/real_space_DG.  One handle owns the
 * device state of a BATCH of problems that share the discretisation shape
 * (N_el, N_K, Nk, N_xi, L_xi) but carry their own potential, masses, contact
 * Fermi levels and device length.  Valleys x modes of one
 * solve_transport_DG_2D call, bias points of a sweep or gate voltages map to
 * batch entries.
 *
 * Conventions
 *  - Plain C types only.  Complex vectors are interleaved (re, im) doubles,
 *    the layout of MATLAB's interleaved-complex MEX API.
 *  - State vector order (permute_shell = true, DG_code/core/get_Diff.m:66-84):
 *    k fastest, then the local DG node, then the x element:
 *    idx = (e*N_K + a)*Nk + j.  A batch stores problem b at offset b*N.
 *  - Every call returns an int status (WG_OK ...).  The library never calls
 *    exit/abort; wg_last_error(h) describes the last failure on a handle.
 *  - A handle is thread-compatible: one host thread per handle at a time.
 *
 * Reference interfaces replaced (file:line in the reference project):
 *  - solve_transport_DG_2D(mat,Esub,Vsub,EfL,EfR)   DG_code/solve_transport_DG_2D.m:1
 *    -> wg_problem_create + wg_set_potential + wg_solve + wg_get_observables
 *  - [A,rhs] = get_SysM(mat,p,EM)                    DG_code/core/get_SysM.m:1
 *    -> wg_set_potential (operator data resident on the device) + wg_apply / wg_get_rhs
 *  - rho = A\rhs                                     DG_code/solve_transport_DG_2D.m:101
 *    -> wg_solve (restarted right-preconditioned GMRES + k-line preconditioner)
 *  - preconditioner.apply(r)                         DG_code/core/get_LineTransversePreconditioner_full2D.m:199
 *    -> wg_precondition
 *  - DG.info.solve.{flag,relres,iterations,...}      DG_code/solve_transport_DG_full2D.m:279-334
 *    -> wg_solve_info
 *  - Gummel loop of RTD/solve2D_rtd_self_consistent.m:88-205 with the Poisson
 *    step of RTD/solve_Poisson2D_rtd.m:56-186 (1D, Ny = 1)
 *    -> wg_gummel_set / wg_gummel_run / wg_gummel_get
 *  - RK4 loop of DG_code/solve_transport_DG_2D_transient_SC_new.m:124-212
 *    (RK4 kept, Crank-Nicolson added)                -> wg_transient_set_bias / wg_transient_run
 *  - the bias loop of RTD/solve2D_rtd_self_consistent.m, served: requests of
 *    mixed shapes admitted under a device-memory budget -> wg_server_*
 *  - sysInfo.makeGPUApply() and the Krylov solve of the Full-2D solver
 *    (DG_code/core/get_SysM_full2D.m:81, DG_code/solve_transport_DG_full2D.m:132-346,
 *    get_LineTransversePreconditioner_full2D.m)       -> wg2d_*
 *  - [M,node_num,node_type] = eval_Poisson2D_rtd(mat), project_DG_density_RTD and
 *    solve_Poisson2D_rtd (RTD directory; the poissonStep of make_RTD_poisson_step.m)
 *                                                     -> wg_poisson2d_*
 *  - [E,V] = solve_subbands(mat)                      solve_subbands.m:1 -> wg_subbands_*
 */
#ifndef WIGNER_GB300_H
#define WIGNER_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (error identifiers of the reference: DG:Full2D:*, RTD:*). */
enum {
  WG_OK = 0,
  WG_NOT_CONVERGED = 1,   /* iterative solve stopped above tolerance: a status, not an error */
  WG_ERR_ARG = 2,         /* invalid argument or size */
  WG_ERR_OOM = 3,         /* device memory budget exceeded (DG:Full2D:GmresMemoryLimit) */
  WG_ERR_TIMEOUT = 4,     /* bounded device wait ran out */
  WG_ERR_CUDA = 5,        /* CUDA runtime error */
  WG_ERR_NUMERIC = 6      /* NaN/Inf met in a reduction */
};

enum { WG_PREC_FP64 = 0, WG_PREC_MIXED = 1 };

/* Discretisation shared by all problems of a handle (initParams.m:58-221). */
typedef struct {
  int n_el;          /* N_chi: x elements                          (initParams.m:59)  */
  int n_local;       /* N_K_chi: DG nodes per element, 2..4        (initParams.m:58)  */
  int nk;            /* Nk = mat.dg.params.N: k points             (initParams.m:62)  */
  int n_xi;          /* N_xi: FV xi cells, >= nk                   (initParams.m:60)  */
  double l_xi;       /* Ly: xi interval length [m]                 (initParams.m:110) */
  double m_diff;     /* mass in Q_diff = hbar/m [kg]; <= 0 selects the reference's 0.041*m0 (initParams.m:102) */
  double mpc;        /* MPC prefactor of A and rhs (solve_transport_DG_2D.m:95-98); 0 -> 1 */
  int precision;     /* WG_PREC_FP64 (drop-in) or WG_PREC_MIXED */
  int restart;       /* GMRES restart length m (basis m+1 vectors); 0 -> 50 */
  double mem_budget_bytes; /* admission budget for this handle; 0 -> no limit */
  int inner_restart; /* mixed form: inner FP32 GMRES length; 0 -> 40 */
  double inner_tol;  /* mixed form: floor of the inner relative tolerance; 0 -> 1e-3 */
  double reorth;     /* Gram-Schmidt: a second classical pass when |w1| < reorth |w| (Daniel-Gragg-
                        Kaufman-Stewart test); 0 -> 1/sqrt(2); >= 1: always (CGS2); < 0: never (CGS) */
  double inner_reorth; /* the same for the mixed form's inner FP32 solve; 0 -> never (one classical pass:
                          the inner solve only has to reduce the residual by inner_tol, and the FP64
                          refinement keeps the accuracy; a second pass measured 25% slower, same iterations) */
  int fp64_tc;       /* FP64 handles: 1 = the two Phi transforms as FP64 products emulated on the tensor cores
                        (8-digit slices, ~1e-14 of |Phi| |x|, 2 Nk and 2 N_xi <= 1024); 0 = native FP64 (default) */
  int inner_basis_fp32; /* mixed form: 1 keeps the inner Krylov basis in FP32; 0 (default) stores it in FP16
                           with FP32 arithmetic (the preconditioner works on the stored FP16 vector; the FP64
                           refinement keeps the accuracy; C2: the same inner iteration counts, half the basis
                           traffic of the Gram-Schmidt kernels) */
} wg_params;

/* One problem's device/material data on the material grid (mat.x, nm). */
typedef struct {
  int nx;              /* mat.Nx = n_el*(n_local-1)+1 */
  const double* x_nm;  /* [nx] material grid in nm, x_nm[0] = 0, x_nm[nx-1] = L_x */
  const double* m_kg;  /* [nx] effective mass along x [kg] (mat.me_x(IV,:,mid)*m0) */
  double me_z;         /* transverse mass, units of m0 (mat.me_z_ch) */
  double temp;         /* mat.Temp [K] */
} wg_device;

typedef struct {
  double tol;          /* relative residual target; 0 -> 1e-10 */
  int maxit;           /* restart cycles; 0 -> 50 */
  int use_rho0;        /* 1: warm start from the rho0 argument / the resident state */
} wg_solve_opts;

typedef struct {
  int flag;            /* 0 converged, 1 not converged (iterativeStatus) */
  int iterations;      /* inner Krylov iterations (all cycles) */
  int cycles;          /* restart cycles run */
  int refinements;     /* outer FP64 refinement steps (mixed form; 0 for FP64) */
  double relres;       /* true relative residual |b - A x| / |b| in FP64 */
  double initial_relres; /* |b - A x0| / |b| (1 without warm start) */
  double rhs_norm;     /* |b| */
} wg_solve_info;

typedef struct wg_problem wg_problem;

/* Create a handle for `batch` problems.  Allocates all device memory. */
int wg_problem_create(const wg_params* prm, int batch, wg_problem** out);
int wg_problem_destroy(wg_problem* h);
/* Device bytes a handle of `batch` problems would allocate (the admission estimate
 * of wg_problem_create, GmresMemoryLimit analogue of solve_transport_DG_full2D.m:198). */
int wg_problem_bytes(const wg_params* prm, int batch, double* bytes);
const char* wg_last_error(const wg_problem* h);
/* Library-level last error (for failures before a handle exists). */
const char* wg_global_error(void);

/* Sizes: N per problem (complex entries), batch, bytes of device memory held. */
int wg_problem_sizes(const wg_problem* h, long long* n_per_problem, int* batch, double* device_bytes);

/* Runtime state of a handle: the CUDA graphs of its Arnoldi steps (chunks of 4
 * steps captured once and replayed; WG_CUDA_GRAPHS=0 disables them) and the launch
 * shapes the autotuner picked on its first solve (WG_AUTOTUNE=0 keeps the defaults).
 * No reference counterpart (MATLAB's gmres has neither). */
typedef struct {
  long long graph_replays;  /* Arnoldi chunks replayed from graphs so far */
  int graphs_captured;      /* chunk graphs instantiated (both bases) */
  int graphs_disabled;      /* 1 when a capture failed and the handle launches eagerly */
  int tuned;                /* 1 once the autotuner ran (or found the shape cached) */
  int kline_chunk;          /* elements per k-line chunk in use */
  int stencil_cells;        /* xi cells per thread of the FP32 stencil (mixed form) */
} wg_runtime_stats;
int wg_runtime_stats_get(const wg_problem* h, wg_runtime_stats* out);
/* Pin the launch shapes instead of tuning them (e.g. for results reproducible across
 * processes): kline_chunk elements per k-line chunk (1 .. n_el, at most 64 chunks),
 * stencil_cells 2 or 4 (ignored by FP64 handles); 0 keeps the current value. */
int wg_set_launch_shapes(wg_problem* h, int kline_chunk, int stencil_cells);

/* Set problem b's potential (Esub [eV] on the material grid), masses and the
 * contact Fermi levels.  Rebuilds on the device: the Wigner-potential kernel
 * data Vw(x,k) (get_Drift_accel_trial_permutedShell.m:64-147), the contact
 * inflow (verteilung.m:118-170, get_Diff.m:77-83) and the line factors. */
int wg_set_potential(wg_problem* h, int b, const wg_device* dev, const double* esub_ev,
                     double ef_l, double ef_r);

/* Solve A rho = rhs for every problem of the batch.  rho0 (nullable, batch*N
 * complex) is a physical warm start; with opts->use_rho0 and rho0 == NULL the
 * resident solution of the previous solve is the warm start.  info has batch
 * entries.  Returns WG_OK when every problem converged, WG_NOT_CONVERGED when
 * at least one did not (see info[b].flag). */
int wg_solve(wg_problem* h, const wg_solve_opts* opts, const double* rho0, wg_solve_info* info);

/* Copy problem b's solution (N complex) to the host. */
int wg_get_rho(wg_problem* h, int b, double* rho);

/* Problem b's charge and current density at the DG nodes (n_el*n_local each):
 * n_dg = Re of the centre-xi value of Phi*rho, j = q hbar/m Im(d rho_u/d xi)
 * (solve_transport_DG_2D.m:114-156). */
int wg_get_observables(wg_problem* h, int b, double* n_dg, double* j);
/* Overwrite problem b's resident Wigner function (N complex values, the rho of
 * wg_get_rho; the INIT.rho of solve_transport_DG_2D_transient_SC_new.m:22) or its
 * right-hand side (INIT.rhs, :21).  A later wg_set_potential or operator refresh
 * rebuilds the right-hand side unless the transient keeps it (fixed_rhs). */
int wg_set_rho(wg_problem* h, int b, const double* rho);
int wg_set_rhs(wg_problem* h, int b, const double* rhs);

/* Problem b's Wigner function on the xi grid, rho_u = Phi * rho per DG node
 * (solve_transport_DG_2D.m:118, DG.RHO(IV,IM,:,:)): n_el*n_local rows of
 * n_xi complex values (row = DG node, xi fastest). */
int wg_get_rho_xi(wg_problem* h, int b, double* rho_u);

/* y = A x for the whole batch (host buffers, batch*N complex each).  FP64 handles
 * use native FP64 arithmetic; mixed handles apply the operator of their FP64
 * refinement residual, whose transforms are FP64 products emulated on the tensor
 * cores (about 1e-14 relative to |Phi| |x|) when 2 N_k and 2 N_xi are at most 1024. */
int wg_apply(wg_problem* h, const double* x, double* y);
/* y = A_lo x with the operator of the mixed form's inner solve (BF16 tensor-core
 * transforms, FP32 flux and stencil); mixed handles only.  Host FP64 buffers. */
int wg_apply_lowprec(wg_problem* h, const double* x, double* y);
/* z = M^-1 r with the k-line preconditioner (host buffers). */
int wg_precondition(wg_problem* h, const double* r, double* z);
/* The batch's right-hand sides (batch*N complex). */
int wg_get_rhs(wg_problem* h, double* rhs);

/* ---- Gummel self-consistency (1D RTD, Dirichlet contacts) ----------------
 * RTD/solve2D_rtd_self_consistent.m:88-205 with the approximate-Newton
 * Poisson step of RTD/solve_Poisson2D_rtd.m:56-186 and the DG -> control
 * volume projection of RTD/project_DG_density_RTD.m, for Ny = 1. */
typedef struct {
  const double* vc_ev;  /* [nx] conduction band edge (mat.Vc) [eV]; V = Vc - phi */
  const double* nd_m3;  /* [nx] ionised donors (mat.Nd) [m^-3] */
  const double* eps_r;  /* [nx] relative permittivity (mat.eps) */
  const double* phi0;   /* [nx] initial electrostatic potential [V], phi(0)=0, phi(end)=bias */
  double bias;          /* drain bias [V] */
  double ef_offset;     /* E_F - Vc at both contacts [eV] (0.05 in solve2D_rtd_self_consistent.m:110) */
  double dy_nm;         /* density normalisation: n = n_DG |Vsub|^2 / dy (solve_transport_DG_2D.m:204) */
} wg_rtd_1d;

typedef struct {
  int max_iterations;          /* 0 -> 100 */
  double mixing;               /* alpha in (0,1]; 0 -> 0.1 */
  double potential_tol;        /* max |phi* - phi| [V]; 0 -> 5e-4 */
  double density_tol;          /* relative density change; 0 -> 5e-4 */
  double poisson_residual_tol; /* |F|_inf / scale before the step; 0 -> 8e-2 */
  double transport_tol;        /* GMRES relative residual; 0 -> 1e-8 */
  int transport_maxit;         /* GMRES restart cycles; 0 -> 50 */
  int warm_start;              /* 1: first transport solve starts from the resident rho */
  int restart_from_phi0;       /* 1: reset phi to the phi0 of wg_gummel_set (device copy) */
  double inexact_factor;       /* > 0: inexact Gummel, transport tol = clamp(factor * defect[V], transport_tol,
                                  inexact_cap) per problem; convergence is only accepted after a solve at
                                  transport_tol with the same potential.  0: fixed transport_tol (reference) */
  double inexact_cap;          /* loosest transport tolerance of the inexact mode; 0 -> 1e-4 */
  int defer_final;             /* inexact mode: a problem whose loop converged on a loose solve waits, frozen,
                                  for its re-solve at transport_tol until no problem of the handle is in its
                                  loose phase (or at most defer_final iterations), so that the long final
                                  solves of a batch run together instead of one after another in lockstep
                                  with the others' short ones.  Every problem's own sequence of iterates is
                                  unchanged.  0 -> 64; < 0: no waiting */
} wg_gummel_opts;

enum { WG_GUMMEL_CONVERGED = 0, WG_GUMMEL_ITERATION_LIMIT = 1, WG_GUMMEL_TRANSPORT_FAILED = 2,
       WG_GUMMEL_POISSON_FAILED = 3 };

typedef struct {
  int status;                  /* WG_GUMMEL_* (sweep.status of the reference) */
  int iterations;              /* Gummel iterations run */
  int gmres_iterations;        /* inner Krylov iterations over all transport solves */
  double potential_defect;     /* last max |phi* - phi| [V] */
  double density_change;       /* last relative density change */
  double poisson_relres;       /* last Poisson residual before the step */
  double transport_relres;     /* last transport true relative residual */
  double seconds;              /* wall time from the start of wg_gummel_run to this problem's exit */
} wg_gummel_info;

/* Problem b: device/material data, RTD electrostatics and initial potential.
 * Sets the transport data for V = Vc - phi0 (calls wg_set_potential). */
int wg_gummel_set(wg_problem* h, int b, const wg_device* dev, const wg_rtd_1d* rtd);
/* Run every problem's Gummel loop to convergence (or a limit).  info has batch entries.
 * Returns WG_OK when all converged, WG_NOT_CONVERGED otherwise. */
int wg_gummel_run(wg_problem* h, const wg_gummel_opts* opts, wg_gummel_info* info);
/* Problem b's potential phi [nx], density n [n_el*n_local] in m^-3 and current density j. */
int wg_gummel_get(wg_problem* h, int b, double* phi, double* n_dg, double* j);

/* ---- Transient self-consistent solve (1D RTD) -------------------------------
 * DG_code/solve_transport_DG_2D_transient_SC_new.m:124-212 on the state of a
 * Gummel handle: d rho/dt = scale_rhs * rhs - scale_a * A rho, the operator and
 * the inflow rebuilt from the potential before step t when (t-1) % E == 0 or
 * t < F (:131-149), the linear Poisson problem of solve_Poisson2D_transient.m
 * solved for the current density after step t when t % E == 0 or t < F
 * (:204-211), n and j after every step (:161-185).  Integrators: the
 * reference's RK4 (:153-158) or Crank-Nicolson,
 * (A + s I) rho' = (s I - A) rho + 2 scale_rhs/scale_a rhs with s = 2/(dt scale_a),
 * one restarted-GMRES solve per step with the shifted k-line preconditioner,
 * warm-started from the previous step (the plain or the mixed form of the handle). */
enum { WG_TRANSIENT_CN = 0, WG_TRANSIENT_RK4 = 1 };

typedef struct {
  double dt;            /* time step [s] (mat.dt) */
  int nsteps;           /* steps of this call (mat.Nt) */
  int method;           /* WG_TRANSIENT_CN or WG_TRANSIENT_RK4 */
  double scale_a;       /* operator scale; 0 -> 2e-10 (solve_transport_DG_2D_transient_SC_new.m:148) */
  double scale_rhs;     /* inflow scale; 0 -> scale_a, so the stationary state is A^-1 rhs */
  int refresh_every;    /* E; 0 -> 20; < 0: potential and operator fixed after the first step */
  int refresh_first;    /* F; 0 -> 50; < 0 -> none */
  double tol;           /* Crank-Nicolson GMRES relative residual per step; 0 -> 1e-10 */
  int maxit;            /* restart cycles per step; 0 -> 20 */
  int record_every;     /* store n and j after every record_every-th step; 0: none */
  int fixed_rhs;        /* 1: keep the resident right-hand side (the reference's rhs_INIT, never refreshed,
                           :153-156) and rebuild only the operator at a refresh; 0: rebuild both */
} wg_transient_opts;

typedef struct {
  int status;                  /* 0: every step solved to tol; 1: some step stopped above tol */
  int steps;                   /* steps taken */
  long long gmres_iterations;  /* inner Krylov iterations over all steps */
  double max_relres;           /* largest final relative residual of the step solves */
  int refreshes;               /* operator and inflow rebuilds */
  int poisson_solves;          /* potential re-solves (incl. the one of a bias step) */
  double seconds;              /* wall time of the call */
} wg_transient_info;

/* Step problem b's drain bias at t = 0 of the next wg_transient_run: the right
 * contact's Fermi level and the Poisson boundary value change now; the potential
 * is re-solved for the current density before the first step. */
int wg_transient_set_bias(wg_problem* h, int b, double bias);
/* Advance every problem of the handle by nsteps from its resident state (the
 * Wigner function and the potential of wg_gummel_run or of a previous call).
 * n_hist, j_hist (either may be NULL): [nsteps / record_every][batch][n_el*n_local],
 * n in m^-3 as wg_gummel_get.  info has batch entries. */
int wg_transient_run(wg_problem* h, const wg_transient_opts* opts, double* n_hist, double* j_hist,
                     wg_transient_info* info);

/* ---- Serving: continuous batching of self-consistent bias points -----------
 * A request is one point of an I-V sweep (the bias loop of
 * RTD/solve2D_rtd_self_consistent.m run through wg_gummel_*).  Requests of equal
 * shape (n_el, n_local, nk, n_xi, l_xi) share a handle of max_slots problems; a
 * worker thread per handle admits queued requests into free slots between Gummel
 * iterations while the other slots keep iterating, and retires each slot the
 * moment its own loop ends.  Handles of different shapes run on their own
 * streams, so their work overlaps on the device.  A handle is created only when
 * its estimated bytes fit the device-memory budget next to the live handles, and
 * released when it has been idle for idle_release_s while others wait for memory.
 * Warm start: a request is seeded from the nearest finished bias with the same
 * device_key and shape -- in the same slot when free (Wigner function and
 * potential resident on the device), else from that bias' potential. */
typedef struct {
  double mem_budget_bytes;     /* device bytes for all handles; 0 -> 150e9 */
  int max_slots;               /* problems per handle; 0 -> 8 */
  int precision;               /* WG_PREC_FP64 or WG_PREC_MIXED */
  int restart, inner_restart;  /* 0 -> 50, 40 */
  double inner_tol;            /* 0 -> 1e-3 */
  double reorth, inner_reorth; /* Gram-Schmidt thresholds as in wg_params */
  wg_gummel_opts gummel;       /* loop options of every request (warm_start, restart_from_phi0 unused) */
  int warm_start;              /* 1: seed requests from neighbouring biases */
  double idle_release_s;       /* 0 -> 0.5 */
} wg_server_opts;

typedef struct {
  int n_el, n_local, nk, n_xi;  /* shape (wg_params) */
  double l_xi, m_diff, mpc;     /* as in wg_params (0 -> the reference's defaults) */
  wg_device dev;                /* copied at submission */
  wg_rtd_1d rtd;                /* copied at submission (phi0 = the cold-start potential) */
  long long device_key;         /* requests of one device share warm starts */
} wg_request;

enum { WG_REQ_QUEUED = 0, WG_REQ_RUNNING = 1, WG_REQ_DONE = 2, WG_REQ_FAILED = 3 };

typedef struct {
  int state;                   /* WG_REQ_* */
  wg_gummel_info info;         /* the request's Gummel loop (status WG_GUMMEL_*) */
  double t_submit, t_admit, t_done;  /* seconds since wg_server_create */
  int handle, slot;            /* where it ran */
  int warm;                    /* 0 cold, 1 potential seeded, 2 potential and Wigner function resident */
  char error[192];             /* why a request failed (WG_REQ_FAILED), else empty */
} wg_request_status;

typedef struct {
  int handles;                 /* live handles */
  int queued, running;         /* requests */
  long long done, failed;
  double device_bytes, device_bytes_peak;  /* estimated bytes of the live handles */
} wg_server_stats;

typedef struct wg_server wg_server;
int wg_server_create(const wg_server_opts* opts, wg_server** out);
/* Queue a request (all inputs are copied); *id identifies it. */
int wg_server_submit(wg_server* s, const wg_request* req, long long* id);
/* Wait up to timeout_s (< 0: no limit) for the request to finish.  WG_OK with st
 * filled once it is done or failed; WG_ERR_TIMEOUT (st filled) otherwise. */
int wg_server_wait(wg_server* s, long long id, double timeout_s, wg_request_status* st);
/* Results of a finished request: phi [nx], n_dg and j [n_el*n_local] (any may be NULL). */
int wg_server_result(wg_server* s, long long id, double* phi, double* n_dg, double* j);
/* Forget a finished request (its stored results). */
int wg_server_release(wg_server* s, long long id);
int wg_server_stats_get(wg_server* s, wg_server_stats* st);
/* Finish the queued and running requests, stop the workers, free every handle. */
int wg_server_destroy(wg_server* s);

/* ---- Allocation-free operator apply ----------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they call in: applications that own all device memory through their
 * own allocator (a MEX gateway on gpuArray storage, a framework pool with a
 * hard budget, an embedding that reserved the whole device up front), where a
 * library allocation would fail or break the owner's accounting.  y = A x (the
 * FP64 operator of wg_apply) on caller-owned DEVICE buffers; the library
 * allocates nothing.  The transform scratch is a fixed file-scope device array
 * of 2^20 complex doubles (16 MiB) that every GPU loading the library keeps
 * until exit; problems with n_xi*batch*n_el*n_local > 2^19 are rejected with
 * WG_ERR_ARG.  All calls share that array: calls whose kernels overlap on the
 * GPU race and must be serialised by the caller.  The first call on a device
 * (and the first after a device reset replaced its context) looks up the
 * array's device address; make it before any stream capture.  Kernels are
 * enqueued on `stream` (NULL: the default stream) and the call does not
 * synchronise. */
typedef struct {
  int n_el, n_local, nk, n_xi, batch;
  const double* phi;    /* device: n_xi x nk complex, row-major (xi row s, k column j), exp(i k_j xi_s)/sqrt(Ly) */
  const double* kvec;   /* device: nk wave numbers */
  const double* qd;     /* device: batch values Q_diff * MPC / detJ (detJ = L_x / n_el / 2) */
  const double* beta;   /* device: [batch][n_el][n_local^2][n_xi+1] real xi-stencil weights of the potential */
  const double* betai;  /* device: [n_local^2][n_xi+1] imaginary (CAP) xi-stencil weights */
  double K1[16], K2[16], K3[16], K5[16];  /* host: element flux blocks, row-major n_local x n_local */
} wg_operator_view;
int wg_apply_noalloc(const wg_operator_view* op, const double* x, double* y, void* stream);

/* Diagnostic: C = bf16(A) * bf16(B) on the tcgen05 tensor-core GEMM of the mixed
 * form, FP32 accumulation.  A row-major M x K, B column-major K x N, C column-major
 * M x N, host buffers; K >= 64 and K % 8 == 0.  No counterpart in the reference. */
int wg_debug_gemm_bf16(const float* A, const float* B, float* C, int M, int N, int K);
/* Diagnostic of the failure path of the tensor-core kernels: one thread waits on an mbarrier that
 * nothing arrives at, with the bounded wait of those kernels limited to spin_limit polls (1 .. 2^24).
 * Returns WG_ERR_TIMEOUT with "bounded barrier wait timed out" when the wait gave up and raised its
 * error flag, as a GEMM whose copies never land would; the context stays usable.  No counterpart in
 * the reference. */
int wg_debug_wait_timeout(long long spin_limit);
/* Diagnostic: C = A * B in FP64 emulated on the tensor cores (6-bit digit slices,
 * exact BF16 products, grouped FP32 accumulation, recombination in 64-bit integer
 * fixed point, one rounding to FP64), the
 * GEMM of the mixed form's FP64 outer residual.  A row-major M x K, B column-major
 * K x N, C column-major M x N, host buffers; 64 <= K <= 1024, K % 8 == 0.  No
 * counterpart in the reference. */
int wg_debug_gemm_f64_tc(const double* A, const double* B, double* C, int M, int N, int K);
/* The same with only the nd (1 .. 8) leading digits of each operand (error ~2^(-6 nd) of |A||B|),
 * as the mixed form's residual uses for loose tolerances. */
int wg_debug_gemm_f64_tc_digits(const double* A, const double* B, double* C, int M, int N, int K, int nd);

/* Diagnostic: apply the operator n times to the resident state on the device and
 * return the mean time of one apply in *ms.  which = 0: the FP64 operator;
 * 1: the mixed form's low-precision operator (BF16 transforms, FP32 flux and
 * stencil); 2: the mixed form's FP64 operator (transforms emulated on the tensor
 * cores).  No counterpart in the reference (operator applies/s). */
int wg_apply_repeat(wg_problem* h, int which, int n, double* ms);

/* Kernel-class profiler (the reference's tic/toc solveInfo timings,
 * solve_transport_DG_full2D.m:182-233, as CUDA events on the handle's stream).
 * Classes: FP32 upwind flux (mixed form), FP64 transform GEMMs on the FP64 pipe,
 * BF16 tensor-core GEMMs, FP32 xi stencil, k-line preconditioner, Gram-Schmidt
 * multi-dot, Gram-Schmidt update, small Krylov kernels (reductions, normalisation,
 * Givens), other, FP64 transform GEMMs emulated on the tensor cores (digit slicing +
 * slice products), FP64 upwind flux, FP64 xi stencil, the fused mixed apply's GEMM 1 with the
 * xi stencil in its epilogue and GEMM 2 with the FP32 flux in its epilogue. */
enum { WG_PROF_FLUX = 0, WG_PROF_GEMM_F64, WG_PROF_GEMM_BF16, WG_PROF_STENCIL, WG_PROF_PRECOND, WG_PROF_MULTIDOT,
       WG_PROF_GSUPDATE, WG_PROF_KRYLOV, WG_PROF_OTHER, WG_PROF_GEMM_F64TC, WG_PROF_FLUX64, WG_PROF_STENCIL64,
       WG_PROF_GEMM_STENCIL, WG_PROF_GEMM_FLUX, WG_PROF_N };
int wg_profile_enable(wg_problem* h, int on);
/* Arrays of WG_PROF_N entries.  ms[i]: summed event time of class i; timed[i]:
 * timed launches; launches[i]: kernel launches of class i since the last reset
 * (always counted); bytes[i] and flops[i]: algorithmic bytes and flops of the
 * timed launches (any may be NULL), credited only for the problems each launch
 * processed (launches skip converged or masked problems); for WG_PROF_GEMM_F64TC
 * flops count the BF16 digit-slice products the chosen digit counts need. */
int wg_profile_read(wg_problem* h, double* ms, long long* timed, long long* launches, double* bytes, double* flops,
                    int reset);

/* CUDA events on the handle's stream (16 slots): device-side timing of any
 * sequence of calls.  wg_event_elapsed waits for slot b. */
int wg_event_record(wg_problem* h, int slot);
int wg_event_elapsed(wg_problem* h, int a, int b, double* ms);
/* The waiter's stream waits (on the device, the host does not block) for event
 * `slot` last recorded on the signaler's stream: brackets work that several
 * handles run concurrently on their own streams with one pair of events. */
int wg_event_wait(wg_problem* waiter, wg_problem* signaler, int slot);

/* ------------------------------------------------------------------------------------------------
 * Full-2D (X, Y, rho_x, rho_y) matrix-free operator: the device-resident apply that
 * sysInfo.makeGPUApply() returns (DG_code/core/get_SysM_full2D.m:81, 124-139):
 *   y = sum_parts c (R U) C^T           (applyKronOperator, get_Diff_full2D.m:618-639)
 *     + CAP + FV-consistent potential   (applyFVConsistentDrift, get_Drift_full2D.m:331-364).
 * State order F(i_rho_x, i_rho_y, i_X, i_Y), rho_x fastest (complex interleaved FP64).
 * The host builds the one-dimensional factors once (as the reference does before
 * makeGPUApply) and hands them over; every apply runs on the device.
 * ------------------------------------------------------------------------------------------------ */
typedef struct wg2d_problem wg2d_problem;

typedef struct {
  int n_el_x, nk_x;         /* centre DG along X: elements, local nodes */
  int n_el_y, nk_y;         /* centre DG along Y */
  int n_rho_x, n_rho_y;     /* relative FV cells */
  int periodic_y;           /* 1: the Y element chain is closed (core/close_PeriodicDGAxis_full2D.m) */
  int n_quad;               /* potential quadrature points per centre element */
  int tensor_cores;         /* 1: dense rho_x factors (the characteristic |A_x|) as FP64 GEMMs emulated
                               on the tensor cores (~1e-14 of |R||G|); 0: FP64 CUDA-core kernels */
} wg2d_shape;

int wg2d_create(const wg2d_shape* s, wg2d_problem** out);
int wg2d_destroy(wg2d_problem* h);
const char* wg2d_last_error(const wg2d_problem* h);

/* Transport terms of one axis (0: X with rho_x, 1: Y with rho_y): y += sum_t coef[t] (C_t along the
 * centre axis) (R_t along the relative axis), i.e. the parts kron(I_Y, C_X) x kron(I_rho_y, R_x) and
 * kron(C_Y, I_X) x kron(R_y, I_rho_x) of get_Diff_full2D.m:76-146.  C_t: element blocks
 * [n_el][3][nk][nk] (coupling to element e-1, e, e+1; row-major nk x nk; the neighbours of the first
 * and last element wrap when the axis is periodic and are ignored otherwise).  R_t: CSR
 * (row_ptr [n_rho+1], col [nnz_t], complex values [nnz_t]) for each term, concatenated.
 * Replaces the terms of that axis. */
int wg2d_set_transport(wg2d_problem* h, int axis, int n_terms, const double* coef, const double* center_blocks,
                       const int* row_ptr, const int* col, const double* val);

/* Potential and CAP (get_Drift_full2D.m:133-300): interp [n_quad][n_local] (DG values at the
 * element quadrature points), proj [n_quad][n_local] (quadrature weights times the inverse local mass),
 * the quadrature coordinates xq, yq [n_elements][n_quad] (m), the relative vertex coordinates
 * vx, vy [n_vert] (m; n_vert = (n_rho_x+1)(n_rho_y+1), or (n_rho_x+1) n_rho_y when periodic),
 * the complex potential coefficient pot (i Q_drift scale), the real CAP coefficient and profile
 * cap [n_rho_x n_rho_y]. */
int wg2d_set_drift(wg2d_problem* h, const double* interp, const double* proj, const double* xq, const double* yq,
                   const double* vx, const double* vy, const double* pot, double cap_coef, const double* cap);

/* Potential V on the material grid gx [nx] x gy [ny] (m, ascending; V column-major, x fastest):
 * rebuilds the vertex potential differences V(X + rho/2) - V(X - rho/2) on the device with X clamped
 * and Y clamped or wrapped (get_Drift_full2D.m:620-666). */
int wg2d_set_potential(wg2d_problem* h, int nx, int ny, const double* gx, const double* gy, const double* V);

/* Y masks of the rho_x-axis transport terms set by wg2d_set_transport (axis 0): masks[t][iY] = 1 where
 * term t acts.  The closed (masked-off) pieces of the outer X faces take the rho_x-reflected interior
 * state as their incoming characteristics (get_Diff_full2D.m:393-423, with centre factor
 * kron(diag(closed), leftBoundary / rightBoundary) and relative factor A+- R_x); the caller sets those
 * corrections as terms with their closed Y dofs as mask.  masks = NULL: every term acts everywhere.
 * Must follow wg2d_set_transport (which clears the masks). */
int wg2d_set_transport_masks(wg2d_problem* h, int axis, int n_terms, const unsigned char* masks);

/* Hard-wall Y boundary (full2D_Y_boundary = 'hard-wall'; replaces constrain_HardWall_full2D.m:1-44 with
 * get_HardWallGeometry_full2D.m:15-48): every apply becomes T A (mask u) + scale (u - mask u).
 * active [nY][n_rho_y] (1: the sample's two particle coordinates Y +- rho_y/2 lie inside the Y
 * interval); projection [n_el_y][n_rho_y][nk_y][nk_y] row-major: per Y element and rho_y cell the
 * exact-DG-mass projection M(keep,keep)^-1 M(keep,:) on the element's nodes (zero rows for inactive
 * nodes); scale: the weight of the constraint rows.  The transport terms must not carry the Y
 * boundary penalty (the reference drops it for hard walls).  active = NULL removes the wall. */
int wg2d_set_hard_wall(wg2d_problem* h, const unsigned char* active, const double* projection, double scale);

/* y = A x on host buffers (n = n_rho_x n_rho_y n_X n_Y complex entries). */
int wg2d_apply(wg2d_problem* h, const double* x, double* y);

/* Line-transverse preconditioner M = (sigma I + X_ref)(sigma I + T_ref) / sigma
 * (get_LineTransversePreconditioner_full2D.m:17-238), factors built on the host as the reference
 * does: U [n_rho_x][n_rho_x] complex row-major (column k = eigenmode k of -i D_rho_x), the shift
 * sigma, the X-line factors x_inverse and x_coupling [n_rho_x][n_el_x][nk_x][nk_x] complex
 * (row-major blocks), forward [n_rho_x] (1: sweep towards +X), and the inverses of the transverse
 * blocks t_inverse [n_rho_x][nT][nT] complex with nT = n_rho_y n_Y (t = i_rho_y + n_rho_y i_Y).
 * fp32 = 1: the preconditioner runs in FP32 (an approximate inverse; wg2d_solve is a flexible GMRES,
 * so the solve keeps its FP64 accuracy); 0: FP64 (mode transforms on the tensor cores when the
 * handle was created with tensor_cores). */
int wg2d_set_preconditioner(wg2d_problem* h, const double* U, double sigma, const double* x_inverse,
                            const double* x_coupling, const int* forward, const double* t_inverse, int fp32);
int wg2d_precondition(wg2d_problem* h, const double* r, double* z);

/* A rho = rhs by restarted GMRES(restart), right-preconditioned (the identity when no preconditioner
 * was set; the mixed form needs the FP32 preconditioner), to tol relative to |rhs|, at most
 * maxit restart cycles (solveStationarySystem / runGmresWithProgress,
 * solve_transport_DG_full2D.m:132-346, 422-506).  x: the warm start when use_x0 (a correction about
 * x0, the tolerance still relative to |rhs|), the solution on return.  WG_NOT_CONVERGED is a status. */
typedef struct {
  double tol;
  int maxit;                /* restart cycles (plain) or refinements (mixed) */
  int restart;
  int use_x0;
  int mixed;                /* 1: FP64 refinement around FP32 flexible GMRES on the FP32 operator
                               (needs the FP32 preconditioner); 0: FP64 flexible GMRES */
  double inner_tol;         /* mixed: floor of each refinement's relative inner tolerance (default 1e-3) */
  int inner_basis_fp16;     /* mixed: 1 stores the inner basis in FP16 with FP32 arithmetic (the preconditioner
                               works on the stored vector); 0 (default) keeps it in FP32.  At the recorded run's
                               shape and 5e-6 target FP16 needed 9% more inner iterations for a 1% faster one */
} wg2d_solve_opts;
typedef struct {
  int flag;                 /* 0 converged, 1 not */
  int iterations;           /* inner iterations */
  int cycles;
  double relres;            /* true relative residual at exit */
  double initial_relres;
  double rhs_norm;
} wg2d_solve_info;
int wg2d_solve(wg2d_problem* h, const double* rhs, double* x, const wg2d_solve_opts* opts, wg2d_solve_info* info);
/* Resident forms of wg2d_solve (the device keeps the right-hand side and the solution between calls, as
 * the reference keeps DG.rho for the next warm start, solve2D_rtd_self_consistent.m:185,204): rhs = NULL
 * reuses the right-hand side of the previous solve; x = NULL takes the warm start (when use_x0) from the
 * resident solution and leaves the result on the device only.  wg2d_get_state copies the resident
 * solution out (n complex values). */
int wg2d_get_state(wg2d_problem* h, double* x);
/* A rho = rhs by preconditioned BiCGSTAB (the full2D_solver = 'bicgstab' branch of solveStationarySystem,
 * solve_transport_DG_full2D.m:248-272: MATLAB's bicgstab with the preconditioner as M), with the
 * line-transverse preconditioner when one is set and none otherwise.  opts: tol (relative to |rhs|),
 * maxit (full iterations), use_x0; restart, mixed and inner_tol are ignored.  rhs / x = NULL as for
 * wg2d_solve.  info: flag from the final true residual, relres, iterations (full iterations begun),
 * cycles (half steps done; MATLAB's iter = cycles / 2); wg2d_solve_resvec gives the initial residual
 * and the norm after every half step.  WG_NOT_CONVERGED (also after a breakdown) is a status. */
int wg2d_solve_bicgstab(wg2d_problem* h, const double* rhs, double* x, const wg2d_solve_opts* opts,
                        wg2d_solve_info* info);
/* Residual history of the last solve (DG.info.solve.resvec of solveStationarySystem,
 * solve_transport_DG_full2D.m:317-326): the initial true residual norm, then the GMRES estimate
 * |b - A x_j| after every inner iteration (absolute, in the units of rhs).  Copies
 * min(cap, count) values to out (out may be NULL) and the count to *count. */
int wg2d_solve_resvec(wg2d_problem* h, double* out, int cap, int* count);

/* Observables at zero relative separation on the device (get_Observables_full2D.m:19-79):
 * nDG = real rho(0,0,X,Y), jxDG = scale_x imag(d rho/d rho_x)(0,0,X,Y), jyDG = scale_y
 * imag(d rho/d rho_y)(0,0,X,Y); n, jx, jy their projections onto the material Y grid (duplicate DG Y
 * nodes averaged, linear interpolation with extrapolation); j = jx integrated over Y (trapezoid).
 * The zero of an axis is one cell (weight 1) or two bracketing cells (linear weights), its derivative
 * row at most 8 nonzeros (zeroInterpolationWeights / derivativeRowAtZero of the same file). */
typedef struct {
  int n_zero_x, n_zero_y;          /* 1 or 2 */
  int zero_x[2], zero_y[2];        /* rho_x / rho_y cell indices (0-based) */
  double w_zero_x[2], w_zero_y[2];
  int n_dx, n_dy;                  /* nonzeros of the derivative rows, <= 8 */
  int dx_idx[8], dy_idx[8];
  double dx_val[8], dy_val[8];     /* [1/m] */
  double scale_x, scale_y;         /* q hbar / m_x, q hbar / m_y */
  int n_target_y;                  /* material Y points */
} wg2d_observables_desc;
/* W: [n_target_y][nY] projection weights from the DG Y dofs to the material Y points; wj: [n_target_y]
 * integration weights over them.  Kept by the handle. */
int wg2d_set_observables(wg2d_problem* h, const wg2d_observables_desc* d, const double* W, const double* wj);
/* rho: a host state (n complex values) or NULL for the resident solution.  Outputs (any may be NULL),
 * row-major with X (the DG X dof) slowest: nDG, jxDG, jyDG [nX][nY]; n, jx, jy [nX][n_target_y]; j [nX]. */
int wg2d_observables(wg2d_problem* h, const double* rho, double* nDG, double* jxDG, double* jyDG, double* n,
                     double* jx, double* jy, double* j);
/* Diagnostic: n applies to the resident device state; mean time of one apply in *ms, with the time
 * of its transport and potential kernels in parts_ms[0..1] (may be NULL). */
int wg2d_apply_repeat(wg2d_problem* h, int n, double* ms, double* parts_ms);

/* ------------------------------------------------------------------------------------------------
 * Transverse subband eigensolve in mode space: replaces [E, V] = solve_subbands(mat)
 * (solve_subbands.m:1-40 with solve_bandstructure.m:1-33 and eval_transversal_Hamiltonian.m:1-37).
 * Per valley and x slice: the n_of_modes eigenpairs of smallest magnitude of the Ny x Ny
 * transverse Hamiltonian, ascending, vectors 2-norm normalised with a positive last entry, then
 * valley 1's vectors sign-aligned with its first slice.  A handle solves `batch` independent
 * problems (gate or bias points) at once.  C-order arrays, problem index outermost:
 *   me_y [batch][nv][nx][ny] (mat.me_y), V [batch][nx][ny] eV (mat.V), dy in nm (mat.dy),
 *   E [batch][nv][nx][nm] eV, Vsub [batch][nv][nx][nm][ny] -- the Esub / Vsub of solve_transport_DG_2D.
 * ny in 3..1024, n_modes in 1..min(32, ny).
 * ------------------------------------------------------------------------------------------------ */
typedef struct wg_subbands wg_subbands;

int wg_subbands_create(int batch, int n_valleys, int nx, int ny, int n_modes, wg_subbands** out);
int wg_subbands_destroy(wg_subbands* h);
const char* wg_subbands_last_error(const wg_subbands* h);
/* Host buffers in and out; validates the masses (positive) and the potential (finite). */
int wg_subbands_solve(wg_subbands* h, double dy_nm, const double* me_y, const double* V, double* E, double* Vsub);
/* Device pointers; enqueued on `stream` (NULL: the handle's), no allocation, no synchronisation. */
int wg_subbands_solve_device(wg_subbands* h, double dy_nm, const double* me_y, const double* V, double* E,
                             double* Vsub, void* stream);
/* Synchronise `stream` (NULL: the handle's) and report a numeric failure of any device solve since
 * the previous status call (the flag is cleared). */
int wg_subbands_status(wg_subbands* h, void* stream);
/* The handle's device buffers for me_y, V, E and Vsub (any pointer may be NULL). */
int wg_subbands_buffers(wg_subbands* h, double** me_y, double** V, double** E, double** Vsub);

/* ------------------------------------------------------------------------------------------------
 * 2D Poisson step of the Full-2D Gummel loop: replaces
 *   [M, node_num, node_type] = eval_Poisson2D_rtd(mat)          (RTD/eval_Poisson2D_rtd.m:1-196)
 *   n = project_DG_density_RTD(nDG, p, mat, periodicY)          (RTD/project_DG_density_RTD.m:1-37)
 *   [phi, iter_err, info] = solve_Poisson2D_rtd(M, ..., n, mat, phi0, bias)  (RTD/solve_Poisson2D_rtd.m)
 * i.e. poissonStep of RTD/make_RTD_poisson_step.m:44-54, for a batch of bias points.  Grid arrays are
 * [ny][nx] with x fastest (MATLAB's column-major [Nx, Ny], node k = ix + iy nx), in SI units as in the
 * reference (densities m^-3, potentials V); nDG is [ndof_y][ndof_x] (X fastest).
 * ------------------------------------------------------------------------------------------------ */
typedef struct wg_poisson2d wg_poisson2d;

typedef struct {
  int nx, ny;          /* mat.Nx, mat.Ny (ny - periodic_y <= 32) */
  double dx_nm, dy_nm; /* mat.dx, mat.dy */
  int periodic_y;      /* 1: Y endpoints identified (full2D_Y_boundary 'periodic' / mat.poisson.yBoundary) */
  int neumann_x;       /* 1: mat.poisson.xBoundary = 'neumann' (no Dirichlet nodes; Newton only) */
  double temp;         /* mat.Temp [K] (Newton screening q^2 n / (kB T)) */
  int batch;           /* bias points solved per call */
} wg_poisson2d_desc;

typedef struct {
  int converged;                     /* the linear update solved to 1e-8 (not self-consistency) */
  double linear_relres, physical_relres_before, physical_relres_after, physical_residual_before;
  double residual_scale, unmixed_step, iter_err;
  double net_charge_per_length, relative_charge_imbalance;
  double source_integral, target_integral;   /* the projection's conservation check (0 without nDG) */
} wg_poisson2d_info;

/* eps_r, nd_m3 (mat.Nd), na_m3 (mat.Na, may be NULL) [ny][nx]; boundary [ny][nx] 1 = Dirichlet
 * (mat.boundary) or NULL for the default (x = first/last column unless neumann_x). */
int wg_poisson2d_create(const wg_poisson2d_desc* d, const double* eps_r, const unsigned char* boundary,
                        const double* nd_m3, const double* na_m3, wg_poisson2d** out);
int wg_poisson2d_destroy(wg_poisson2d* h);
const char* wg_poisson2d_last_error(const wg_poisson2d* h);
/* The DG -> dual-volume integration maps (CSR, built by the caller as project_DG_density_RTD.m:39-69
 * does): Tx [nx x ndof_x], Ty [nu x ndof_y] with the periodic endpoint rows merged, the dual widths
 * wx [nx], wy [nu] and the element-integral weights src_x [ndof_x], src_y [ndof_y]. */
int wg_poisson2d_set_projection(wg_poisson2d* h, int ndof_x, const int* tx_rp, const int* tx_col, const double* tx_val,
                                int ndof_y, const int* ty_rp, const int* ty_col, const double* ty_val,
                                const double* wx, const double* wy, const double* src_x, const double* src_y);
/* out = M phi for every problem of the batch (host [batch][ny][nx]). */
int wg_poisson2d_apply(wg_poisson2d* h, const double* phi, double* out);
/* Host entry: src = nDG [batch][ndof_y][ndof_x] (src_is_dg = 1) or n [batch][ny][nx] (m^-3);
 * phi0 [batch][ny][nx]; bias [batch] (bc(end,:) = bias) or vbc [batch][ny][nx] (mat.Vbc);
 * newton 0 = 'direct', 1 = 'newton-raphson'; alpha in (0, 1].  Out: phi, density [batch][ny][nx],
 * info [batch]. */
int wg_poisson2d_solve(wg_poisson2d* h, const double* src, int src_is_dg, const double* phi0, const double* bias,
                       const double* vbc, int newton, double alpha, double* phi, double* density,
                       wg_poisson2d_info* info);
/* Contact potentials on the unique nodes [batch][nu][nx] for the device entry (host arrays). */
int wg_poisson2d_contacts(wg_poisson2d* h, const double* bias, const double* vbc, double* bc_out);
/* Device entry: pointers on the device, enqueued on `stream` (NULL: the handle's), no allocation. */
int wg_poisson2d_solve_device(wg_poisson2d* h, const double* src, int src_is_dg, const double* phi0,
                              const double* bc, int newton, double alpha, double* phi, double* density, void* stream);
/* Synchronise `stream` and copy the batch's info to the host. */
int wg_poisson2d_info_get(wg_poisson2d* h, void* stream, wg_poisson2d_info* info);
/* The handle's device buffers (src sized for nDG once a projection is set). */
int wg_poisson2d_buffers(wg_poisson2d* h, double** src, double** phi0, double** bc, double** phi, double** density);

#ifdef __cplusplus
}
#endif
#endif /* WIGNER_GB300_H */
