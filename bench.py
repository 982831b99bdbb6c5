#!/usr/bin/env python
"""Benchmark: converged self-consistent RTD bias points per second on one GB300.

Workload (the configuration the headline metric is quoted on): a self-consistent
RTD, GaAs, 80 nm device with 20 nm contacts at 1e18 cm^-3, Al0.3Ga0.7As double
barrier 0.27 eV x 3 nm around a 5 nm well; DG p=3, 240 elements, Nk=256 (245,760
complex unknowns per bias point); Gummel mixing 0.3, potential tolerance 1e-6 V;
every transport solve to a 1e-8 relative residual.  One step = one batch of
`--batch` (16) bias points (0.2 V * (1..B)/B) solved from a cold start to the Gummel
fixed point, all points advancing together in one handle.  Default form: mixed
precision (BF16 tensor-core transforms inside FP64 refinement) with the inexact
Gummel schedule (transport tolerance 0.3 x the potential defect in V, at most
1e-3; every accepted state re-solved at 1e-8); ``--precision fp64 --inexact 0``
is the plain drop-in form.

Arms: default (ours, this library on the GPU) and ``--impl reference`` (the CPU
restatement of the reference algorithm, timed on a bounded sample).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged self-consistent bias points/s at 1e-8 transport residual (C2 RTD, batched)"
UNIT = "bias_points/s"

SPEC = dict(length_nm=80.0, contact_nm=20.0, barrier_ev=0.27, barrier_nm=3.0, well_nm=5.0, doping_m3=1e24,
            m_rel=0.067, temp_k=300.0, order=3, n_el=240, nk=256, l_xi_m=30e-9)
GUMMEL = dict(mixing=0.3, potentialTolerance=1e-6, densityTolerance=5e-4, poissonResidualTolerance=8e-2,
              maxIterations=200, transportTolerance=1e-8, transportMaxCycles=60)
# Krylov iterations per converged bias point of this workload with the reference's
# loop (FP64 GMRES(50), mixing 0.3, every transport solve at 1e-8), measured on the
# plain FP64 GPU path, which runs the same algorithm as the CPU restatement; used to
# extrapolate the CPU sample.  A plain-form run replaces it by its live count.
ITERS_PER_POINT_FALLBACK = 9229.0
E2E_STEPS = 5            # timed public calls of the e2e line (after one untimed call)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if r[0] == str(PHYS_GPU)] or self.rows
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


PHYS_GPU = 0   # index (nvidia-smi numbering) of this rank's GPU


def select_device():
    """One GPU per rank: LOCAL_RANK picks an entry of CUDA_VISIBLE_DEVICES (or that index when
    unset) and narrows the visible devices to it before the library initialises CUDA, so
    every rank's handles, streams and server threads run on device 0 of their own view."""
    global PHYS_GPU
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if int(os.environ.get("WORLD_SIZE", "1")) <= 1:
        return
    vis = [v for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    pick = vis[local % len(vis)] if vis else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = pick
    PHYS_GPU = int(pick) if pick.isdigit() else local


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    select_device()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(v, dist):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, dist):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def make_workload(batch):
    from real_space_dg_gb300 import devices
    spec = devices.RTDSpec(**SPEC)
    mat = devices.make_mat(spec)
    mat["dy_norm_nm"] = devices.density_normalisation_nm(mat)
    biases = 0.2 * np.arange(1, batch + 1) / batch
    return spec, mat, biases


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one timed gemm_f64_tc event of the mixed form (digit
# slicing + emulated GEMM; the mean of the C = AB and C += AB launches) per state column (element x node), from
# ncu captures of residuals at 5 digits (profiles/gemm_ozaki_c2_batch8_mixed.md): the GEMMs at batch 8 (7,680
# columns) 44.5 and 75.8 MB, the slicing at a 2-problem handle (1,920 columns) 7.9 MB (its digit writes stay in
# L2).  The traffic grows with the columns, so a launch of the bench's batch scales by its columns.
OZAKI_TRAFFIC_PER_COLUMN = 7.89e6 / 1920 + 0.5 * (44.53e6 + 75.75e6) / 7680
FP64_NOMINAL_TFLOPS = 1.25   # no FP64 peak is measured on this machine: nominal GB300 FP64 (CUDA cores)


def rooflines(prof, precision):
    """Achieved rate per kernel class from the library's CUDA-event timings and the
    algorithmic bytes/flops it attributed to each timed launch (credited only for the
    problems a launch processed; the emulated FP64 GEMM's flops count the BF16
    digit-slice products its digit counts need).  A fraction above 1.05 of a measured
    peak is flagged: it means the class's operands were served from L2 (129 MB) or
    that the attribution is wrong, never that the peak was beaten."""
    hbm, bf16, src = read_peaks()
    out = {}
    total = sum(v[0] for v in prof.values() if v[1] > 0) or 1.0
    for cls, (ms, n_t, n_l, by, fl) in prof.items():
        if n_t == 0 or ms <= 0:
            continue
        sec = ms / 1000.0
        if cls in ("gemm_stencil", "gemm_flux") and by > 0:
            # the fused apply kernels stream their operands: HBM-bound by design
            ach, peak, bound, unit, psrc = by / sec / 1e9, hbm, "hbm", "GB/s", "hbm_gbs (%s)" % src
        elif cls == "gemm_bf16":
            ach, peak, bound, unit, psrc = fl / sec / 1e12, bf16, "tensor", "TFLOP/s", "bf16_tflops (%s)" % src
        elif cls == "gemm_f64_tc":
            ach, peak, bound, unit = fl / sec / 1e12, bf16, "tensor", "TFLOP/s"
            psrc = "bf16_tflops (%s); achieved counts the BF16 digit-slice products of FP64 emulated on the " \
                   "tensor cores" % src
        elif cls in ("gemm_f64", "flux_f64", "stencil_f64") and fl > 0:
            # FP64 arithmetic on the CUDA cores: the FP64 pipe bounds these on GB300 (1/64 of FP32)
            ach, peak, bound, unit = fl / sec / 1e12, FP64_NOMINAL_TFLOPS, "fp64", "TFLOP/s"
            psrc = "nominal GB300 FP64 %.2f TFLOP/s (no measured FP64 peak)" % FP64_NOMINAL_TFLOPS
        elif by > 0:
            ach, peak, bound, unit, psrc = by / sec / 1e9, hbm, "hbm", "GB/s", "hbm_gbs (%s)" % src
        else:
            continue
        r = {"kernel": cls, "bound": bound, "achieved": round(ach, 3), "peak": peak, "unit": unit,
             "frac": round(ach / peak, 4), "traffic": None, "peak_source": psrc,
             "avg_launch_us": round(1000.0 * ms / n_t, 2), "launches": int(n_t), "share": round(ms / total, 4),
             "per_launch": {"bytes": by / n_t, "flops": fl / n_t}}
        if bound == "fp64" and by > 0:
            r["hbm_frac"] = round(by / sec / 1e9 / hbm, 4)
        if cls in ("gemm_stencil", "gemm_flux"):
            r["tensor_frac"] = round(fl / sec / 1e12 / bf16, 4)
        if ach / peak > 1.05:
            r["flag"] = ("above 1.05 of the peak: operands served from L2 (the class's working set of the "
                         "remaining active problems fits the 129 MB L2) or misattributed work; not an HBM rate")
        out[cls] = r
    return out


def run_ours(args, rank, world, dist):
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import _lib
    from real_space_dg_gb300.rtd import RTDSweep, release_handles, run_concurrent, solve_rtd_self_consistent

    spec, mat, biases = make_workload(args.batch)
    opts = dict(GUMMEL, precision=args.precision, restart=args.restart, innerRestart=args.inner_restart,
                innerTol=args.inner_tol, inexactFactor=args.inexact, inexactCap=args.inexact_cap, reorth=args.reorth,
                innerReorth=args.inner_reorth, fp64TensorCores=args.fp64_tc,
                innerBasisFP32=args.inner_basis_fp32, deferFinal=args.defer_final)
    if args.max_gummel:
        opts["maxIterations"] = args.max_gummel      # profiling runs only: points need not converge
    K = max(1, min(args.handles, args.batch))
    sweeps = [RTDSweep(mat, len(range(k, args.batch, K)), opts) for k in range(K)]
    for i, v in enumerate(biases):
        sweeps[i % K].set(i // K, v)
    H0 = sweeps[0].P
    if args.launch_shapes:
        kl, cells = (int(t) for t in args.launch_shapes.split(","))
        for sw in sweeps:
            sw.P.set_launch_shapes(kl, cells)

    def step(concurrent=True):
        """One step: every handle's Gummel loops from phi0, the handles concurrently on their own
        streams; device-timed by a pair of events on handle 0's stream that the other streams are
        fenced against (they start after the first event, the second waits for all of them).
        concurrent=False runs the handles one after another (the per-launch profile, whose event
        times would otherwise include the other streams' kernels)."""
        H0.event(0)
        for sw in sweeps[1:]:
            sw.P.wait_event(H0, 0)
        if concurrent:
            outs = run_concurrent(sweeps, restart_from_phi0=True)
        else:
            outs = [sw.run(restart_from_phi0=True) for sw in sweeps]
        for sw in sweeps[1:]:
            sw.P.event(15)
            H0.wait_event(sw.P, 15)
        H0.event(1)
        info = [outs[i % K][1][i // K] for i in range(args.batch)]
        return H0.elapsed_ms(0, 1), info

    def profile(on):
        merged = {}
        for sw in sweeps:
            for cls, v in sw.P.profile(on=on, reset=True).items():
                a = merged.get(cls, (0.0, 0, 0, 0.0, 0.0))
                merged[cls] = tuple(x + y for x, y in zip(a, v))
        return merged

    concurrent = not args.serial_handles
    for _ in range(args.warmup):
        step(concurrent)
    # the timed region runs without the per-launch event profiler (launches are still counted)
    profile(False)
    clocks = ClockSampler()
    clocks.start()
    barrier(dist)
    lat, pts, its, gummel_its, statuses = [], 0, 0, 0, []
    total_ms = 0.0
    for _ in range(args.steps):
        ms, info = step(concurrent)
        total_ms += ms
        for i in info:
            statuses.append(i["status"])
            if i["status"] == 0:
                pts += 1
                lat.append(i["seconds"])
            its += i["gmres_iterations"]
            gummel_its += i["iterations"]
    clk = clocks.stop()
    rs = H0.runtime_stats
    shapes = {"kline_chunk": rs["kline_chunk"], "stencil_cells": rs["stencil_cells"],
              "source": "pinned (--launch-shapes)" if args.launch_shapes else "autotuned"}
    counted = profile(False)
    launches = sum(v[2] for v in counted.values())
    t_max = max_over_ranks(total_ms / 1000.0, dist)
    pts_all = sum_over_ranks(pts, dist)
    value = pts_all / t_max if t_max > 0 else 0.0
    # one more step, untimed, with CUDA events around every launch and the handles run one after
    # another: per-class rooflines of the kernels the timed steps run, free of the other streams
    profile(True)
    step(concurrent=False)
    prof = profile(False)
    roofs = rooflines(prof, args.precision)
    if "gemm_f64_tc" in roofs:
        ncols = len(range(0, args.batch, K)) * SPEC["n_el"] * (SPEC["order"] + 1)
        roofs["gemm_f64_tc"]["traffic"] = round(OZAKI_TRAFFIC_PER_COLUMN * ncols)
        roofs["gemm_f64_tc"]["traffic_source"] = ("ncu dram bytes of one slicing + emulated GEMM event at batch 8, "
                                                  "scaled by columns to a handle of %d problems"
                                                  % len(range(0, args.batch, K)))
    roof = max(roofs.values(), key=lambda r: r["share"]) if roofs else None
    # e2e: the public call with host inputs and outputs, every step
    e2e = None
    if not args.no_e2e and rank == 0:
        # the public call, host arrays in and out; one untimed call opens the handles it keeps
        # for the next calls of the same shape (keepHandles), then E2E_STEPS timed calls
        t0 = time.perf_counter()
        solve_rtd_self_consistent(mat, biases, opts, mode="batched", handles=K)
        first_s = time.perf_counter() - t0
        n_e2e = max(1, min(args.steps, E2E_STEPS))
        conv, t0 = 0, time.perf_counter()
        for _ in range(n_e2e):
            r = solve_rtd_self_consistent(mat, biases, opts, mode="batched", handles=K)
            conv += sum(r["sweep"]["converged"])
        e2e_s = time.perf_counter() - t0
        release_handles()
        nx = int(mat["Nx"])
        ncol = spec.n_el * (spec.order + 1)
        e2e = {"value": round(conv / e2e_s, 5), "unit": UNIT,
               "h2d_bytes_per_step": int(args.batch * 6 * nx * 8),
               "d2h_bytes_per_step": int(args.batch * (nx + 2 * ncol) * 8),
               "seconds": round(e2e_s / n_e2e, 3), "steps": n_e2e,
               "first_call_seconds": round(first_s, 3),
               "definition": "solve_rtd_self_consistent(mat, biases, options, handles=%d) per step, host "
                             "arrays in and out; the handles kept from the untimed first call (which opens "
                             "them, first_call_seconds) serve the timed calls" % K}
    apply = whole_apply(mat, args) if rank == 0 else None
    # the timed form's converged state (the profiled step ran the same form from the same start)
    ours_res = [sweeps[i % K].get(i // K) for i in range(args.batch)]
    ours_info = info
    for sw in sweeps:
        sw.close()
    plain = mixed_exact = accuracy = None
    if not args.no_plain and rank == 0:
        plain, mixed_exact, accuracy = other_forms(args, mat, biases, opts, ours_res, ours_info)
    lat_sorted = sorted(lat)
    p50 = float(np.percentile(lat_sorted, 50)) if lat else None
    p99 = float(np.percentile(lat_sorted, 99)) if lat else None
    iters_per_point = its / max(1, len(statuses))
    cpu = None
    if rank == 0 and not args.no_cpu:
        # the CPU port runs the plain algorithm: extrapolate with the plain form's live count
        is_plain = args.precision == "fp64" and args.inexact == 0
        ipp = iters_per_point if is_plain else (plain["gmres_iterations_per_point"] if plain else args.iters_per_point)
        cpu = cpu_baseline(args, ipp)
    out = {
        "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000.0 * t_max / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "bf16/f32 in f64 refinement",
        "data": "synthetic RTD device of the named shape (seeded, deterministic)",
        "config": {"workload": "C2 self-consistent RTD 80 nm, p=3, N_el=240, Nk=256, 245760 unknowns/point",
                   "batch_bias_points": args.batch, "biases_v": [round(float(b), 4) for b in biases],
                   "handles": K, "handles_run": "one after another" if args.serial_handles else "concurrently",
                   "launch_shapes": shapes,
                   "defer_final": "none" if args.defer_final < 0 else
                   "%d Gummel iterations (inexact mode)" % (args.defer_final or 64),
                   "profile": "rooflines from one extra step with per-launch CUDA events, handles run one after another",
                   "precision": args.precision, "gmres_restart": args.restart,
                   "inner_restart": args.inner_restart, "inner_tol": args.inner_tol,
                   "inexact_gummel_factor": args.inexact, "inexact_cap": args.inexact_cap, "gummel_mixing": 0.3,
                   "reorth": args.reorth, "inner_reorth": args.inner_reorth, "fp64_tensor_cores": args.fp64_tc,
                   "inner_basis": "fp32" if args.inner_basis_fp32 else "fp16 storage, fp32 arithmetic",
                   "potential_tol_v": 1e-6, "transport_rtol": 1e-8,
                   "l2": "inputs larger than L2 (Krylov basis %.2f GB)" %
                         (16.0 * (args.restart + 1) * args.batch * spec.n_el * (spec.order + 1) * spec.nk / 1e9)},
        "latency_s": {"p50": p50, "p99": p99, "definition": "time from step start to each point's Gummel exit"},
        "converged_points": int(pts_all), "points_attempted": len(statuses) * world,
        "gmres_iterations_per_point": round(iters_per_point, 1),
        "gummel_iterations_per_point": round(gummel_its / max(1, len(statuses)), 2),
        "roofline": roof, "rooflines": roofs, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
        "gpu_launches_by_class": {c: int(v[2]) for c, v in counted.items() if v[2]}, "clocks": clk,
        "plain": plain, "mixed_exact_gummel": mixed_exact, "accuracy": accuracy, "apply": apply,
        "parity_note": "1D oracle parity unpinned against the reference itself (MATLAB/Octave absent, no 1D golden "
                       "vectors in the reference); pinned to the oracle restatement; the Full-2D path is pinned to "
                       "the reference's recorded Sim_Res.mat run",
    }
    return out


def apply_bytes(batch, n_el, n_local, nk, nxi, mixed=True):
    """Algorithmic bytes of one operator apply: read x and write y (complex, 8 B in FP32 / 16 B
    in FP64), the potential coefficients B(x_q, xi_e) at the N_el x 10 quadrature points and N_xi + 1
    cells (4 B BF16 complex / 16 B), and Phi (N_xi x Nk, 4 B / 16 B)."""
    s_vec, s_coef = (8.0, 4.0) if mixed else (16.0, 16.0)
    N = n_el * n_local * nk
    return batch * (2.0 * N * s_vec + n_el * 10 * (nxi + 1) * s_coef) + nxi * nk * s_coef


def whole_apply(mat, args, n_apply=50):
    """The mixed form's inner operator apply on the full batch (all problems active), in the form
    the Arnoldi step runs it (BF16 copy of x from the preconditioner), against the algorithmic
    bytes of one apply."""
    from real_space_dg_gb300.rtd import RTDSweep
    hbm, _, src = read_peaks()
    S = RTDSweep(mat, args.batch, dict(GUMMEL, precision="mixed"))
    try:
        for b, v in enumerate(0.2 * np.arange(1, args.batch + 1) / args.batch):
            S.set(b, v)
        S.P.apply_time("lowprec", 5)
        ms = S.P.apply_time("lowprec", n_apply)
        S.P.profile(on=True, reset=True)
        S.P.apply_time("lowprec", 5)
        prof = S.P.profile(on=False, reset=True)
    finally:
        S.close()
    by = apply_bytes(args.batch, SPEC["n_el"], SPEC["order"] + 1, SPEC["nk"], SPEC["nk"])
    launches = {k: int(v[2]) for k, v in prof.items() if v[2]}
    return {"form": "mixed inner operator: BF16 tensor-core transforms, FP32 flux and xi stencil", "batch": args.batch,
            "us_per_apply": round(1000.0 * ms, 2), "algorithmic_bytes": round(by),
            "achieved_gbs": round(by / (ms / 1000.0) / 1e9, 1), "peak_gbs": hbm,
            "frac": round(by / (ms / 1000.0) / 1e9 / hbm, 4), "peak_source": "hbm_gbs (%s)" % src,
            "launches_per_apply": round(sum(launches.values()) / 5.0, 2),
            "bytes_definition": "per problem 2 N x 8 B (x in, y out, FP32 complex) + N_el x 10 x (N_xi + 1) x 4 B "
                                "(BF16 complex potential coefficients); + N_xi x Nk x 4 B (Phi)"}


def _run_form(mat, batch, biases, opts, phi0=None, handles=1):
    """One device-timed Gummel step of `batch` bias points in fresh handles (the batch dealt
    round-robin to `handles` concurrent handles, as the headline); untimed by the headline.
    Returns (ms, info, [(phi, n, j)] per point)."""
    from real_space_dg_gb300.rtd import RTDSweep, run_concurrent
    K = max(1, min(handles, batch))
    sweeps = [RTDSweep(mat, len(range(k, batch, K)), opts) for k in range(K)]
    try:
        for i, v in enumerate(biases):
            sweeps[i % K].set(i // K, v, phi0=None if phi0 is None else phi0[i])
        H0 = sweeps[0].P
        H0.event(0)
        for sw in sweeps[1:]:
            sw.P.wait_event(H0, 0)
        outs = run_concurrent(sweeps, restart_from_phi0=True)
        for sw in sweeps[1:]:
            sw.P.event(15)
            H0.wait_event(sw.P, 15)
        H0.event(1)
        ms = H0.elapsed_ms(0, 1)
        info = [outs[i % K][1][i // K] for i in range(batch)]
        res = [sweeps[i % K].get(i // K) for i in range(batch)]
    finally:
        for sw in sweeps:
            sw.close()
    return ms, info, res


def _rel(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / nb) if nb > 0 else float(np.linalg.norm(a))


def _compare(res, ref):
    """Errors of a result set against a reference set: terminal current (the mean of j over
    the DG nodes, the reference's Id), the current and density profiles (relative L2) and
    the potential (max abs, V); each the max over the bias points."""
    cur = max(abs(np.mean(r[2]) - np.mean(q[2])) / abs(np.mean(q[2])) for r, q in zip(res, ref))
    return {"terminal_current_rel": cur,
            "current_profile_rel_l2": max(_rel(r[2], q[2]) for r, q in zip(res, ref)),
            "density_rel_l2": max(_rel(r[1], q[1]) for r, q in zip(res, ref)),
            "potential_max_abs_v": max(float(np.max(np.abs(r[0] - q[0]))) for r, q in zip(res, ref))}


def other_forms(args, mat, biases, opts, ours_res, ours_info):
    """The two other arms of the same C2 step, run untimed by the headline after it:
    - plain: the drop-in FP64 form (FP64 GMRES(50), every transport solve at 1e-8, fixed
      schedule; the two Phi transforms as FP64 emulated on the tensor cores, 8 digits);
    - mixed_exact: the mixed form with the fixed schedule (no inexact Gummel), so that the
      precision gain and the schedule gain are reported apart;
    and the accuracy of the headline's result against plain FP64, in two parts: the fixed
    points of the two loops (bounded by the 1e-6 V Gummel tolerance), and the transport alone
    at the headline's converged potential (one FP64 solve at 1e-8 of that very potential:
    the error the mixed transport itself leaves)."""
    batch = len(biases)
    fixed = dict(opts, inexactFactor=0.0)
    plain_opts = dict(fixed, precision="fp64", fp64TensorCores=True)
    K = args.handles
    ms_p, info_p, res_p = _run_form(mat, batch, biases, plain_opts, handles=K)
    ms_m, info_m, res_m = _run_form(mat, batch, biases, dict(fixed, precision="mixed"), handles=K)
    # FP64 transport at the headline's final potential: one Gummel iteration from phi0 = that
    # potential hands back the FP64 density and current of that potential, phi unchanged; solved
    # to 1e-12 (the reference solution) and to the same 1e-8 as the headline (the plain form's own
    # error at that residual)
    phis = [r[0] for r in ours_res]
    _, _, res_t = _run_form(mat, batch, biases, dict(plain_opts, maxIterations=1, transportTolerance=1e-12,
                                                     transportMaxCycles=200), phi0=phis, handles=K)
    _, _, res_t8 = _run_form(mat, batch, biases, dict(plain_opts, maxIterations=1), phi0=phis, handles=K)
    # the mixed transport at a 1e-10 residual at the same potential, and the headline form with its final
    # re-solves at 1e-10: what the benchmark spec's 1e-7 current bar costs at C2's conditioning
    _, _, res_m10 = _run_form(mat, batch, biases, dict(opts, maxIterations=1, transportTolerance=1e-10,
                                                       inexactFactor=0.0, transportMaxCycles=200),
                              phi0=phis, handles=K)
    ms_10, info_10, res_10 = _run_form(mat, batch, biases, dict(opts, transportTolerance=1e-10,
                                                                transportMaxCycles=200), handles=K)

    def arm(ms, info, form):
        conv = sum(i["status"] == 0 for i in info)
        return {"value": round(conv / (ms / 1000.0), 6), "unit": UNIT, "ms_per_step": round(ms, 3),
                "converged_points": int(conv), "points": len(info), "form": form,
                "gmres_iterations_per_point": round(float(np.mean([i["gmres_iterations"] for i in info])), 1),
                "gummel_iterations_per_point": round(float(np.mean([i["iterations"] for i in info])), 2),
                "timing": "one step, CUDA events on the library stream, same batch and biases as the headline"}

    plain = arm(ms_p, info_p, "FP64 GMRES(%d), k-line preconditioner, fixed 1e-8 transport schedule, Phi transforms "
                              "as FP64 emulated on the tensor cores" % args.restart)
    mixed_exact = arm(ms_m, info_m, "mixed (BF16 transforms, FP32 flux/preconditioner, FP64 refinement), fixed 1e-8 "
                                    "transport schedule")
    tight = arm(ms_10, info_10, "the headline form with every accepted transport solve at 1e-10 (inexact "
                                "Gummel, final re-solves at 1e-10)")
    acc = {"reference": "plain FP64 GPU form (above), same biases",
           "headline_vs_plain_fixed_point": _compare(ours_res, res_p),
           "mixed_exact_vs_plain_fixed_point": _compare(res_m, res_p),
           "headline_transport_vs_fp64_1e-12_at_same_potential": _compare(ours_res, res_t),
           "plain_fp64_1e-8_transport_vs_fp64_1e-12_at_same_potential": _compare(res_t8, res_t),
           "mixed_1e-10_transport_vs_fp64_1e-12_at_same_potential": _compare(res_m10, res_t),
           "headline_at_1e-10": dict(tight, vs_plain_fixed_point=_compare(res_10, res_p)),
           "targets": {"terminal_current_rel_transport": 1e-7,
                       "fixed_point": "set by the Gummel potential tolerance 1e-6 V, the same for both loops",
                       "note": "a 1e-8 relative residual bounds the current error only to ~cond * 1e-8; the plain "
                               "FP64 form at 1e-8 is listed beside the headline for that reason"}}
    return plain, mixed_exact, acc


def cpu_baseline(args, iters_per_point):
    """Oracle (CPU restatement) GMRES iterations on the same C2 operator, timed on a
    bounded sample and extrapolated with the measured iterations per bias point."""
    from oracle import dg1d, krylov
    from real_space_dg_gb300 import devices
    spec, mat, biases = make_workload(1)
    bias = 0.2
    V = devices.flatband_potential(mat, bias)
    efl, efr = devices.contact_fermi_levels(mat, bias)
    m = np.full(mat["Nx"], spec.m_rel * dg1d.M0_V)
    p = dg1d.init_params(mat, efl, efr, V, m)
    op = krylov.Operator1D(mat, p, V)
    pre = krylov.KLinePreconditioner(op, use_drift_diag=False)
    _, rhs = dg1d.get_diff(p)
    n_it = args.cpu_iters
    t0 = time.perf_counter()
    krylov.gmres_right(op.apply, pre.apply, rhs, restart=n_it, tol=1e-30, maxit=1)
    dt = time.perf_counter() - t0
    t_iter = dt / n_it
    value = 1.0 / (t_iter * iters_per_point)
    return {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d oracle GMRES(right, k-line) iterations on the C2 operator in %.2f s (%.3f s/iteration, "
                      "NumPy/BLAS on all host cores), extrapolated with %.0f iterations per converged bias point"
                      % (n_it, dt, t_iter, iters_per_point)}


def run_reference(args, rank, world, dist):
    if rank != 0:
        return None
    # warm-up: import and operator set-up are outside the timed samples
    vals = []
    for i in range(args.warmup + args.steps):
        cpu = cpu_baseline(args, args.iters_per_point)
        if i >= args.warmup:
            vals.append(cpu["value"])
    value = float(np.median(vals))
    cpu["value"] = value
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic RTD device of the named shape",
            "config": {"workload": "C2 self-consistent RTD 80 nm, p=3, N_el=240, Nk=256, 245760 unknowns/point",
                       "sample": cpu["sample"]},
            "cpu_baseline": cpu, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}


SERVED = dict(devices=12, biases_per_device=8, rate_hz=20.0, budget_bytes=150e9, max_slots=8, seed=2026,
              max_gummel=500)


def served_requests(seed):
    """The mixed-shape I-V workload: devices with seeded random barrier height
    U(0.20, 0.35) eV, barrier width U(2, 4) nm and well width U(4, 6) nm, each on a
    grid drawn from Nk in {128, 256, 512}, N_el in {120, 240, 480}, p in {1, 2, 3},
    swept over biases drawn from U(0, 0.6) V; requests arrive as a Poisson process."""
    from real_space_dg_gb300 import devices
    rng = np.random.default_rng(seed)
    jobs, shapes = [], []
    for d in range(SERVED["devices"]):
        spec = devices.RTDSpec(**dict(SPEC, barrier_ev=rng.uniform(0.20, 0.35), barrier_nm=rng.uniform(2, 4),
                                      well_nm=rng.uniform(4, 6), nk=int(rng.choice([128, 256, 512])),
                                      n_el=int(rng.choice([120, 240, 480])), order=int(rng.choice([1, 2, 3]))))
        mat = devices.make_mat(spec)
        mat["dy_norm_nm"] = devices.density_normalisation_nm(mat)
        shapes.append((spec.n_el, spec.order, spec.nk))
        for v in rng.uniform(0.0, 0.6, SERVED["biases_per_device"]):
            jobs.append((mat, float(v), d))
    order = rng.permutation(len(jobs))
    jobs = [jobs[i] for i in order]
    arrivals = np.cumsum(rng.exponential(1.0 / SERVED["rate_hz"], len(jobs)))
    arrivals -= arrivals[0]
    return jobs, arrivals, shapes


def run_served(args):
    """Continuous-batching server on the mixed-shape I-V workload: throughput and latency."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300.serve import Server, serve_sweep
    jobs, arrivals, shapes = served_requests(SERVED["seed"])
    # the C2 loop settings; high-bias points of the stiffer devices need more than 200 damped iterations
    opts = dict(GUMMEL, maxIterations=SERVED["max_gummel"], precision=args.precision, restart=args.restart,
                innerRestart=args.inner_restart, innerTol=args.inner_tol, inexactFactor=args.inexact,
                inexactCap=args.inexact_cap,
                reorth=args.reorth, innerReorth=args.inner_reorth)
    clocks = ClockSampler()
    clocks.start()
    with Server(opts, mem_budget_bytes=SERVED["budget_bytes"], max_slots=SERVED["max_slots"], warm_start=True) as S:
        res, wall = serve_sweep(S, jobs, arrivals)
        stats = S.stats()
    clk = clocks.stop()
    lat = np.array([r["latency"] for r in res if r["state"] == "done"])
    conv = sum(r["status"] == "fixed-point-converged" for r in res)
    unknowns = sum(n_el * (p + 1) * nk for (mat, v, d) in jobs for (n_el, p, nk) in [shapes[d]])
    return {
        "metric": "served converged bias points/s (mixed-shape I-V sweep, continuous batching)",
        "value": round(conv / wall, 4), "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
        "dtype": "f64" if args.precision == "fp64" else "bf16/f32 in f64 refinement",
        "data": "synthetic RTD devices, seeded random barriers and grids, Poisson arrivals",
        "config": {"workload": "%d devices x %d biases U(0,0.6) V, Nk {128,256,512}, N_el {120,240,480}, "
                               "p {1,2,3}, %g req/s, %g GB budget" % (SERVED["devices"], SERVED["biases_per_device"],
                                                                       SERVED["rate_hz"], SERVED["budget_bytes"] / 1e9),
                   "shapes": shapes, "precision": args.precision, "inexact_gummel_factor": args.inexact,
                   "max_slots": SERVED["max_slots"], "unknowns_per_point_mean": unknowns / len(jobs)},
        "wall_s": round(wall, 3), "requests": len(jobs), "converged_points": int(conv),
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "definition": "request arrival to result"},
        "warm_started": int(sum(r["warm"] > 0 for r in res)),
        "statuses": {k: int(sum(r["status"] == k for r in res)) for k in sorted({r["status"] for r in res})},
        "gummel_iterations_per_point": float(np.mean([r["info"]["iterations"] for r in res])),
        "server": stats, "clocks": clk,
    }


TRANSIENT = dict(batch=16, order=2, n_el=240, nk=512, dt=1e-15, seed=2027)


def run_transient(args):
    """Crank-Nicolson bias-step transients of the C5 RTD, batched; every step one
    shifted GMRES solve per transient and a Poisson re-solve (refresh every step)."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.rtd import RTDSweep
    rng = np.random.default_rng(TRANSIENT["seed"])
    B = TRANSIENT["batch"]
    widths = rng.uniform(2.0, 4.0, B)
    steps_v = rng.uniform(0.1, 0.4, B)
    base = dict(SPEC, order=TRANSIENT["order"], n_el=TRANSIENT["n_el"], nk=TRANSIENT["nk"])
    opts = dict(GUMMEL, precision=args.precision, restart=args.restart, innerRestart=args.inner_restart,
                innerTol=args.inner_tol, inexactFactor=args.inexact, inexactCap=args.inexact_cap, reorth=args.reorth,
                innerReorth=args.inner_reorth)
    # one handle; the problems differ in their barrier width (device data per problem)
    mats = []
    for w in widths:
        spec = devices.RTDSpec(**dict(base, barrier_nm=float(w)))
        mat = devices.make_mat(spec)
        mat["dy_norm_nm"] = devices.density_normalisation_nm(mat)
        mats.append(mat)
    S = RTDSweep(mats[0], B, opts)
    for b in range(B):
        S.set(b, 0.0, mat=mats[b])
    st, info = S.run()                                   # stationary state at 0 V (INIT)
    for b in range(B):
        S.step_bias(b, float(steps_v[b]))
    kw = dict(refresh_every=1, refresh_first=1, tol=1e-8, maxit=20, record_every=0)
    S.transient(TRANSIENT["dt"], args.warmup, "cn", **kw)          # untimed
    clocks = ClockSampler()
    clocks.start()
    S.P.profile(on=False, reset=True)
    S.P.event(0)
    st, tinfo, _, _ = S.transient(TRANSIENT["dt"], args.steps, "cn", **kw)
    S.P.event(1)
    ms = S.P.elapsed_ms(0, 1)
    counted = S.P.profile(on=False, reset=True)
    clk = clocks.stop()
    S.close()
    n = TRANSIENT["n_el"] * (TRANSIENT["order"] + 1) * TRANSIENT["nk"]
    return {
        "metric": "Crank-Nicolson transient steps/s (C5 RTD, %d transients batched)" % B,
        "value": round(B * args.steps / (ms / 1000.0), 3), "unit": "problem_steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "bf16/f32 in f64 refinement",
        "data": "synthetic RTD devices (seeded barrier widths and bias steps)",
        "config": {"workload": "C5 transient RTD p=2, N_el=240, Nk=512, %d unknowns per transient, dt=1 fs, "
                               "Poisson every step" % n, "batch": B, "stationary_status": int(st),
                   "step_tolerance": 1e-8, "precision": args.precision},
        "gmres_iterations_per_step": float(np.mean([t["gmres_iterations"] for t in tinfo])) / max(1, args.steps),
        "max_step_relres": float(max(t["max_relres"] for t in tinfo)),
        "gpu_launches": int(sum(v[2] for v in counted.values())), "clocks": clk,
    }


C1 = dict(length_nm=60.0, contact_nm=15.0, barrier_ev=0.27, barrier_nm=3.0, well_nm=5.0, doping_m3=1e24, m_rel=0.067,
          temp_k=300.0, order=2, n_el=120, nk=128, l_xi_m=30e-9, bias=0.1, tol=1e-10, restart=50, batch=64)


def run_c1(args):
    """C1: the reference's CPU-runnable case -- the stationary flat-band RTD (60 nm, p=2, N_el=120,
    Nk=128, 46,080 unknowns, 0.1 V linear drop, no Poisson), plain FP64, GMRES(50) with the
    k-line preconditioner to a 1e-10 relative residual, n(x) and J out.  One step solves a batch of
    64 such problems (the same device at 64 biases in 0..0.1 V) from a zero start; e2e is one solve
    through solve_transport_DG_2D; the CPU line is the reference's own method, the sparse LU of
    the assembled system (A\\rhs), in the oracle port on the host cores."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.transport import Problem1D, shape_from_mat, solve_transport_DG_2D
    spec = devices.RTDSpec(**{k: v for k, v in C1.items() if k not in ("bias", "tol", "restart", "batch")})
    mat = devices.make_mat(spec)
    B = C1["batch"]
    biases = C1["bias"] * np.arange(1, B + 1) / B
    m = np.full(mat["Nx"], spec.m_rel * 9.109e-31)
    P = Problem1D(batch=B, precision="fp64", restart=C1["restart"], **shape_from_mat(mat))
    for b, v in enumerate(biases):
        E = devices.flatband_potential(mat, v)
        efl, efr = devices.contact_fermi_levels(mat, v)
        P.set_potential(b, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
    for _ in range(args.warmup):
        P.solve(tol=C1["tol"], maxit=100)
    clocks = ClockSampler()
    clocks.start()
    P.profile(on=False, reset=True)
    P.event(0)
    infos = []
    for _ in range(args.steps):
        st, info = P.solve(tol=C1["tol"], maxit=100)
        infos.append(info)
    P.event(1)
    ms = P.elapsed_ms(0, 1)
    counted = P.profile(on=False, reset=True)
    clk = clocks.stop()
    conv = sum(1 for i in infos[-1] if i["flag"] == 0)
    iters = float(np.mean([i["iterations"] for i in infos[-1]]))
    P.close()
    E = devices.flatband_potential(mat, C1["bias"])
    efl, efr = devices.contact_fermi_levels(mat, C1["bias"])
    solve_transport_DG_2D(mat, E, np.ones(mat["Nx"]), efl, efr, tol=C1["tol"], maxit=100)   # warm-up
    t0 = time.perf_counter()
    ne = 5
    for _ in range(ne):
        DG = solve_transport_DG_2D(mat, E, np.ones(mat["Nx"]), efl, efr, tol=C1["tol"], maxit=100)
    e2e_s = (time.perf_counter() - t0) / ne
    out = {"metric": "stationary flat-band RTD solves/s at 1e-10 relative residual (C1, plain FP64)",
           "value": round(B * args.steps / (ms / 1000.0), 3), "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic RTD of the named shape (C1), 64 biases in 0..0.1 V",
           "config": {"workload": "C1 flat-band RTD 60 nm, p=2, N_el=120, Nk=128, 46,080 unknowns, GMRES(50), "
                                  "rtol 1e-10, k-line preconditioner", "batch": B},
           "solves_converged": conv, "gmres_iterations_per_solve": iters,
           "e2e": {"value": round(1.0 / e2e_s, 3), "unit": "solves/s", "path": "solve_transport_DG_2D, one problem",
                   "h2d_bytes_per_step": int(8 * 3 * mat["Nx"]),
                   "d2h_bytes_per_step": int(DG["RHO"].nbytes + DG["n"].nbytes + DG["j"].nbytes)},
           "gpu_launches": int(sum(v[2] for v in counted.values())), "clocks": clk}
    if not args.no_cpu:
        from oracle import dg1d
        t0 = time.perf_counter()
        dg1d.solve_transport_dg_2d(mat, E, np.ones(mat["Nx"]), efl, efr)
        t1 = time.perf_counter()
        out["cpu_baseline"] = {"value": round(1.0 / (t1 - t0), 4), "unit": "solves/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "one oracle solve_transport_DG_2D with sparse LU "
                               "(the reference's A\\rhs) at the C1 size, %.2f s including assembly" % (t1 - t0)}
    return out


FET = dict(n_gates=32, vg_max=0.6, v_drain=0.4, tol=1e-8, maxit=60)


def run_fet(args):
    """C4: multi-subband FET transport at 32 gate voltages in 0..0.6 V, V_d = 0.4 V.  A gate
    point is the 8 subband solves (2 valley types x 4 cross-section modes) of
    solve_transport_DG_2D at a 1e-8 relative residual plus the summed n and j.  One step sets
    the potentials of every gate point and solves them all from a zero start as one batch
    (gates x subbands problems in one handle); e2e runs the same sweep through
    solve_transport_DG_2D one gate point per call (host arrays in, n and j out)."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.transport import M0, Problem1D, shape_from_mat, solve_transport_DG_2D
    spec = devices.FETSpec()
    vgs = np.linspace(0.0, FET["vg_max"], FET["n_gates"])
    utb = args.workload == "c4_utb"
    sub = None
    if utb:
        # the confinement direction resolved on a grid (5 nm body between 1 nm oxides, dy = 0.1 nm): every
        # step solves the subbands of all gate points on the GPU (one batched call) before the transport
        from real_space_dg_gb300.subbands import SubbandSolver
        secs = [devices.utb_cross_section(spec, float(vg), FET["v_drain"]) for vg in vgs]
        me_all = np.stack([c[2] for c in secs])
        V_all = np.stack([c[3] for c in secs])
        sub = SubbandSolver(me_all.shape[1], me_all.shape[2], me_all.shape[3], spec.n_modes, batch=len(vgs))
        E0, _ = sub.solve(me_all, V_all, 0.1)
        pts = []
        for gi, vg in enumerate(vgs):
            mat, _, _, _, _ = devices.make_fet(spec, float(vg), FET["v_drain"])
            efl = float(E0[gi][:, 0, :].min()) + spec.fermi_offset_ev
            pts.append((mat, E0[gi], None, efl, efl - FET["v_drain"]))
    else:
        pts = [devices.make_fet(spec, float(vg), FET["v_drain"]) for vg in vgs]
    mat0 = pts[0][0]
    shp = shape_from_mat(mat0)
    nv, nm = int(mat0["n_of_valleys"]), int(mat0["n_of_modes"])
    nsub = nv * nm
    B = len(pts) * nsub
    kw = dict(precision=args.precision, restart=args.restart, inner_restart=args.inner_restart,
              inner_tol=args.inner_tol, reorth=args.reorth, inner_reorth=args.inner_reorth)
    P = Problem1D(batch=B, **kw, **shp)
    x_nm = np.asarray(mat0["x"], dtype=float)

    def step():
        if utb:
            E, _ = sub.solve(me_all, V_all, 0.1)
            for gi in range(len(pts)):
                mat, _, _, efl, efr = pts[gi]
                pts[gi] = (mat, E[gi], None, efl, efr)
        for gi, (mat, esub, _, efl, efr) in enumerate(pts):
            for iv in range(nv):
                m = np.asarray(mat["me_x"], dtype=float)[iv, :, 0] * M0
                for im in range(nm):
                    P.set_potential(gi * nsub + iv * nm + im, x_nm, esub[iv, :, im], m, float(mat["me_z_ch"]),
                                    float(mat["Temp"]), efl, efr)
        return P.solve(tol=FET["tol"], maxit=FET["maxit"])

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler()
    clocks.start()
    P.profile(on=False, reset=True)
    t0 = time.perf_counter()
    infos = []
    for _ in range(args.steps):
        st, info = step()
        infos.append(info)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    counted = P.profile(on=False, reset=True)
    conv = sum(1 for i in infos[-1] if i["relres"] <= FET["tol"])
    iters = float(np.mean([i["iterations"] for i in infos[-1]]))
    dev_bytes = P.device_bytes
    P.close()
    if sub is not None:
        sub.close()
    n_pts = len(pts) * args.steps
    out = {
        "metric": "converged gate points/s at 1e-8 transport residual (C4 multi-subband FET, %d subbands per point)"
                  % nsub,
        "value": round(n_pts / wall, 4), "unit": "gate_points/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * wall / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "bf16/f32 in f64 refinement",
        "data": ("synthetic double-gate UTB Si FET: subbands from the GPU transverse eigensolve of the resolved "
                 "5 nm body between 1 nm oxides (solved inside every step), compact gate-controlled band profile "
                 "(not self-consistent)" if utb else
                 "synthetic UTB Si FET: subbands of a 5 x 5 nm box, compact gate-controlled band profile "
                 "(not self-consistent)"),
        "config": {"workload": "C4 FET 50 nm (15 nm S/D at 1e20 cm^-3), p=2, N_el=200, Nk=256, "
                               "%d unknowns per subband, %d gate points x %d subbands in one handle"
                               % (shp["n_el"] * shp["n_local"] * shp["nk"], len(pts), nsub),
                   "v_drain": FET["v_drain"], "v_gate": [0.0, FET["vg_max"]], "precision": args.precision,
                   "device_bytes": dev_bytes, "timing": "wall clock, potentials set from the host every step"},
        "subband_solves_converged": conv, "subband_solves": B, "gmres_iterations_per_subband": iters,
        "gpu_launches": int(sum(v[2] for v in counted.values())) if counted else None, "clocks": clk,
    }
    if utb:
        out["metric"] = out["metric"].replace("C4 multi-subband FET", "C4 FET with GPU subband eigensolve")
        out["config"]["subbands"] = "32 gates x 2 valleys x 401 slices, Ny = 71, 4 modes: one batched device call per step"
    if not args.no_e2e and not utb:
        Pe = Problem1D(batch=nsub, **kw, **shp)
        t0 = time.perf_counter()
        cur = []
        for mat, esub, vsub, efl, efr in pts:
            DG = solve_transport_DG_2D(mat, esub, vsub, efl, efr, tol=FET["tol"], maxit=FET["maxit"],
                                       restart=args.restart, problem=Pe, return_info=False)
            cur.append(float(np.mean(DG["j"])))          # mean j of the reference's units
        we = time.perf_counter() - t0
        Pe.close()
        nb = pts[0][0]["Nx"] * 8 * (2 + nsub) * len(pts)
        out["e2e"] = {"value": round(len(pts) / we, 4), "unit": "gate_points/s",
                      "h2d_bytes_per_step": int(nb), "d2h_bytes_per_step": int(len(pts) * 2 * 8 * shp["n_el"]
                                                                                  * shp["n_local"] * nsub),
                      "path": "solve_transport_DG_2D per gate point (batch of its 8 subbands)",
                      "mean_j_first_last_gate": [cur[0], cur[-1]]}
    return out


FULL2D = dict(length_nm=90.0, width_nm=3.0, nx=361, ny=13, n_el_x=120, nk_x=3, n_el_y=2, nk_y=3, n_rho_x=121,
              n_rho_y=12, l_rho_x=1e-7, me_x_ch=0.063, quad=5)


def full2d_case(cfg=FULL2D):
    """The Full-2D operator of the shape of the reference's recorded run (2026-10-28_08-47:
    90 nm x 3 nm RTD, p=2 in X and Y, 120 x 2 elements, 121 x 12 relative cells, periodic Y,
    upwind fluxes, FV-consistent potential; 3,136,320 complex unknowns) on a seeded synthetic
    double-barrier potential (0.3 eV barriers, a linear 0.2 V drop, a weak Y modulation)."""
    x = np.linspace(0.0, cfg["length_nm"], cfg["nx"])
    y = np.linspace(0.0, cfg["width_nm"], cfg["ny"])
    prm = dict(N_K_X=cfg["nk_x"], N_K_Y=cfg["nk_y"], N_el_X=cfg["n_el_x"], N_el_Y=cfg["n_el_y"],
               N_rho_x=cfg["n_rho_x"], N_rho_y=cfg["n_rho_y"], L_rho_x=cfg["l_rho_x"], full2D_X_flux="upwind",
               full2D_Y_flux="upwind", full2D_Y_boundary="periodic", full2D_potentialQuadratureOrder=cfg["quad"])
    mat = dict(x=x, y=y, Nx=len(x), Ny=len(y), me_x_ch=cfg["me_x_ch"], dg=dict(params=prm))
    X, Y = np.meshgrid(x, y, indexing="ij")
    c = cfg["length_nm"] / 2
    barrier = 0.3 * (((X > c - 6.5) & (X < c - 2.5)) | ((X > c + 2.5) & (X < c + 6.5)))
    V = barrier - 0.2 * np.clip((X - 20.0) / (cfg["length_nm"] - 40.0), 0, 1) \
        + 0.005 * np.cos(2 * np.pi * Y / cfg["width_nm"])
    return mat, V


def full2d_recorded_case():
    """The system of the reference's recorded run at its last bias point (0.6 V): the stored
    potential on the 361 x 13 material grid, the run's DG parameters and its contact-mode
    reservoirs (E_F,L = 1.474 eV, E_F,R = 0.874 eV inputs; contact-neutrality Fermi levels),
    from the fixture tests/golden/full2d_reservoir_golden.npz."""
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                             "full2d_reservoir_golden.npz"))
    prm = {k[4:]: float(g[k]) for k in g.files if k.startswith("prm_")}
    for k in ("N_K_X", "N_K_Y", "N_el_X", "N_el_Y", "N_rho_x", "N_rho_y", "full2D_contactMode_Nkx",
              "full2D_contactMode_Nkz"):
        prm[k] = int(prm[k])
    prm.update(full2D_Y_boundary="periodic", full2D_reservoirModel="contact-modes", full2D_X_flux="upwind",
               full2D_Y_flux="upwind", full2D_contactModeFermiModel="contact-neutrality",
               full2D_potentialQuadratureOrder=5)
    mat = dict(x=g["x"], y=g["y"], Nx=int(g["Nx"]), Ny=int(g["Ny"]), me_x_ch=float(g["me_x_ch"]),
               me_y_ch=float(g["me_y_ch"]), me_z_ch=float(g["me_z_ch"]), deg_factor=float(g["deg_factor"]),
               Temp=float(g["Temp"]), dg=dict(params=prm))
    return mat, np.asarray(g["potential"]), float(g["ef_input_source"]), float(g["ef_input_drain"])


def full2d_flops(f, n):
    """Algorithmic FP64 flops of one apply from the host factors (complex MAC = 8 flops,
    real x complex = 4), as (transport, potential): centre factors 3 nk per entry and term,
    relative factors nnz per row; potential interpolation + projection 2 nq n_local per
    element entry and the vertex stencil."""
    s = f["shape"]
    tr = 0.0
    for axis, nk, nr in ((0, s["nk_x"], s["n_rho_x"]), (1, s["nk_y"], s["n_rho_y"])):
        for _, _, R in f["terms"][axis]:
            tr += n * (3 * nk * 4 + 8 * np.count_nonzero(R) / nr)
    nloc = s["nk_x"] * s["nk_y"]
    return tr, n / nloc * f["nq"] * (2 * nloc * 4 + 4 * 2 + 16 * 2)


def run_full2d(args):
    """Full-2D operator applies/s (a9: applyKronOperator + FV-consistent potential + CAP, FP64;
    the dense characteristic |A_x| factor as FP64 emulated on the tensor cores, and without)."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = full2d_case()
    hbm, bf16, src = read_peaks()
    res = {}
    for tc in (True, False):
        op = Full2DOperator(mat, V, tensor_cores=tc)
        for _ in range(args.warmup):
            op.apply_time(1)
        clocks = ClockSampler()
        clocks.start()
        steps = max(10, args.steps)
        ms, parts = op.apply_time(steps)
        clk = clocks.stop()
        res[tc] = (ms, parts, clk, op)
    n = res[True][3].n
    ms, parts, clk, op = res[True]
    fl_tr, fl_pot = full2d_flops(op.factors, n)
    u = (np.sin(np.arange(n) * 1.3) + 1j * np.cos(np.arange(n) * 0.7)).astype(complex)
    op.apply(u)
    t0 = time.perf_counter()
    ne = 3
    for _ in range(ne):
        op.apply(u)
    e2e_s = (time.perf_counter() - t0) / ne
    peak = 1.25
    pot = {"kernel": "full2d_potential", "bound": "fp64", "achieved": round(fl_pot / parts[1] / 1e9, 3),
           "peak": peak, "unit": "TFLOP/s", "frac": round(fl_pot / parts[1] / 1e9 / peak, 4), "traffic": None,
           "peak_source": "nominal GB300 FP64 1.25 TFLOP/s (no measured FP64 peak)", "ms": round(float(parts[1]), 4)}
    # transport: the dense rho_x factor on the tensor cores counts its 36 BF16 digit products
    nrx = op.shape["n_rho_x"]
    dense_fl = sum(2 * (2 * nrx) * (2 * nrx) * (n / nrx) for _, _, R in op.terms[0] if np.count_nonzero(R) * 4 > nrx * nrx)
    tr = {"kernel": "full2d_transport", "bound": "tensor+fp64", "achieved_fp64_equivalent": round(fl_tr / parts[0] / 1e9, 3),
          "tensor_tflops_of_digit_products": round(36 * dense_fl / parts[0] / 1e9, 3), "peak": bf16, "unit": "TFLOP/s",
          "frac": round(36 * dense_fl / parts[0] / 1e9 / bf16, 4), "traffic": None,
          "peak_source": "bf16_tflops (%s); the whole transport time counted against the digit products" % src,
          "ms": round(float(parts[0]), 4)}
    roof = pot if parts[1] >= parts[0] else tr
    out = {"metric": "Full-2D operator applies/s (3,136,320 complex unknowns, FP64)", "value": round(1000.0 / ms, 3),
           "unit": "applies/s", "n_gpus": 1, "steps": max(10, args.steps), "warmup": args.warmup,
           "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic double-barrier potential on the grid of the reference's recorded Full-2D run",
           "config": {"workload": "Full-2D apply: X 120 el x p=2, Y 2 el x p=2 periodic, rho 121 x 12, upwind, "
                                  "FV-consistent potential (5 x 5 quadrature), CAP", "unknowns": n,
                      "dense_rho_x_factor": "FP64 emulated on the tensor cores (8 digits, 36 products)",
                      "l2": "state 50 MB and intermediates 0.4 GB, larger than L2"},
           "roofline": roof, "rooflines": {"potential": pot, "transport": tr},
           "flops_per_apply_fp64": fl_tr + fl_pot,
           "fp64_cuda_cores": {"applies_per_s": round(1000.0 / res[False][0], 3), "ms": round(res[False][0], 4),
                               "transport_ms": round(float(res[False][1][0]), 4),
                               "fp64_tflops": round((fl_tr + fl_pot) / res[False][0] / 1e9, 3)},
           "e2e": {"value": round(1.0 / e2e_s, 3), "unit": "applies/s", "h2d_bytes_per_step": 16 * n,
                   "d2h_bytes_per_step": 16 * n},
           "gpu_launches": 11, "clocks": clk}
    # the Full-2D solve (solve_transport_DG_full2D: GMRES(40), tol 5e-6, at most 150 cycles as in the
    # recorded run) with the line-transverse preconditioner, on the recorded run's own system at its
    # last bias point: stored potential, contact-mode reservoir right-hand side
    for _, (_, _, _, o) in res.items():
        o.close()
    mat_r, V_r, efl_r, efr_r = full2d_recorded_case()
    op = Full2DOperator(mat_r, V_r)
    t0 = time.perf_counter()
    rhs, inflow = op.reservoir_rhs(efl_r, efr_r)
    rhs_s = time.perf_counter() - t0
    op.set_preconditioner()
    t0 = time.perf_counter()
    st, sinfo, xs = op.solve(rhs, tol=5e-6, maxit=args.solve_maxit, restart=40) if args.solve_maxit > 0 else \
        (0, dict(iterations=0, cycles=0, relres=None), None)
    solve_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    stm, minfo, xm = op.solve(rhs, tol=5e-6, maxit=max(args.solve_maxit, 1) * 4, restart=40, mixed=True) \
        if args.solve_maxit > 0 else (0, dict(iterations=0, cycles=0, relres=None), None)
    mixed_s = time.perf_counter() - t0
    recorded = {}
    if xm is not None:
        # the reference's own transport output for this system (sweep.density / sweep.current of the
        # recorded run at 0.6 V, solved there to a 4.96e-6 relative residual)
        g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                 "full2d_reservoir_golden.npz"))
        for name, x in (("mixed", xm), ("fp64", xs)):
            if x is None:
                continue
            n_o, j_o, _, _ = op.observables(x)
            recorded[name] = {"density_max_rel_diff": float(np.abs(n_o - g["density"]).max() / np.abs(g["density"]).max()),
                              "current_max_rel_diff": float(np.abs(j_o - g["current"]).max() / np.abs(g["current"]).max()),
                              "mean_current": float(np.mean(j_o)), "recorded_mean_current": float(np.mean(g["current"]))}
    pre_ms = None
    try:
        r = rhs.copy()
        op.precondition(r)
        t1 = time.perf_counter()
        for _ in range(3):
            op.precondition(r)
        pre_ms = (time.perf_counter() - t1) / 3 * 1000.0
    except Exception:
        pass
    out["vs_recorded_run"] = recorded
    out["solve_mixed"] = {"status": int(stm), "seconds": round(mixed_s, 3), "inner_iterations": minfo["iterations"],
                          "refinements": minfo["cycles"], "relres": minfo["relres"], "tol": 5e-6,
                          "ms_per_iteration": round(1000.0 * mixed_s / max(1, minfo["iterations"]), 3),
                          "form": "FP64 refinement around FP32 flexible GMRES(40) on the FP32 operator"}
    out["solve"] = {"status": int(st), "seconds": round(solve_s, 3), "gmres_iterations": sinfo["iterations"],
                    "cycles": sinfo["cycles"], "relres": sinfo["relres"], "tol": 5e-6, "restart": 40,
                    "ms_per_iteration": round(1000.0 * solve_s / max(1, sinfo["iterations"]), 3),
                    "precondition_host_call_ms": None if pre_ms is None else round(pre_ms, 3),
                    "rhs": "the recorded run's system at 0.6 V: stored potential, contact-mode reservoirs "
                           "(contact-neutrality E_F %.6f / %.6f eV), right-hand side built in %.3f s on the host"
                           % (inflow["source"][1]["fermiLevelUsed"], inflow["drain"][1]["fermiLevelUsed"], rhs_s)}
    op.close()
    if not args.no_cpu:
        from oracle import full2d as F2
        t0 = time.perf_counter()
        p, partsk, dd = F2.system(mat, V)
        t1 = time.perf_counter()
        F2.apply_system(p, partsk, dd, u)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": round(1.0 / (t2 - t1), 5), "unit": "applies/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "one oracle apply (scipy.sparse Kronecker parts + the "
                               "element loop of the FV potential) at the full size, %.1f s; set-up %.1f s"
                               % (t2 - t1, t1 - t0)}
    return out


SUBBANDS = dict(n_gates=32, vg_max=0.6, v_drain=0.4, n_modes=8, dy_nm=0.1)


def run_subbands(args):
    """f4: the transverse subband eigensolve of the mode-space set-up (solve_subbands.m) for the
    C4 gate sweep with the confinement direction resolved: per gate point 2 valleys x 401
    slices of the 5 nm body between 1 nm oxides (Ny = 71, dy = 0.1 nm), the 8 eigenpairs of
    smallest magnitude per slice.  One step solves all 32 gate points as one batch (one
    launch of the slice kernel and one of the sign clean-up) from potentials resident on the
    device; e2e runs the same batch through SubbandSolver.solve with host arrays (copies in
    and out timed)."""
    import torch
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.subbands import SubbandSolver
    spec = devices.FETSpec(n_modes=SUBBANDS["n_modes"])
    vgs = np.linspace(0.0, SUBBANDS["vg_max"], SUBBANDS["n_gates"])
    secs = [devices.utb_cross_section(spec, float(vg), SUBBANDS["v_drain"], dy_nm=SUBBANDS["dy_nm"]) for vg in vgs]
    me = secs[0][2]
    nv, nx, ny = me.shape
    nm = SUBBANDS["n_modes"]
    G = len(vgs)
    dev = torch.device("cuda:0")
    me_all = np.ascontiguousarray(np.broadcast_to(me[None], (G, nv, nx, ny)))
    V_all = np.stack([s_[3] for s_ in secs])
    me_d = torch.tensor(me_all, device=dev)
    V_d = torch.tensor(V_all, device=dev)
    E_d = torch.empty((G, nv, nx, nm), dtype=torch.float64, device=dev)
    Vs_d = torch.empty((G, nv, nx, nm, ny), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sol = SubbandSolver(nv, nx, ny, nm, batch=G)

    def step():
        sol.solve_device(SUBBANDS["dy_nm"], me_d.data_ptr(), V_d.data_ptr(), E_d.data_ptr(), Vs_d.data_ptr(),
                         stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        sol.status(stream.cuda_stream)
        clocks = ClockSampler()
        clocks.start()
        ms = 0.0
        for _ in range(args.steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        clk = clocks.stop()
        sol.status(stream.cuda_stream)
    slices = G * nv * nx
    value = slices * args.steps / (ms / 1000.0)
    # per slice, FP64 only: Sturm counts of ny entries (2 subtractions, 1 division, 1 compare) -- 1 + the
    # 2 bracket checks + 32 / nm lanes per candidate x the multisection steps from the FP32 bracket
    # (4e-5 of the spectral radius) down to eps x nm candidates (all eigenvalues positive here) -- and
    # the 5 passes of the twisted factorisation per mode (~14 flops per entry); the coarse FP32
    # multisection runs on the FP32 pipe and is not counted
    g = 32 // nm
    steps64 = int(np.ceil(np.log(4e-5 / 2.2e-16) / np.log(g + 1)))
    flops_slice = ((3 + steps64 * g * nm) * 4 + 14 * nm) * ny
    achieved = flops_slice * value / 1e12
    out = {"metric": "transverse subband eigensolves (slices/s, %d eigenpairs of smallest magnitude per slice)" % nm,
           "value": round(value, 1), "unit": "slices/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic double-gate UTB Si FET cross-sections",
           "config": {"workload": "f4 subbands: %d gate points x %d valleys x %d slices, Ny = %d (5 nm body + 2 x 1 nm "
                                  "oxide, dy = 0.1 nm), %d modes" % (G, nv, nx, ny, nm),
                      "l2": "256 MB buffer written between timed steps"},
           "gpu_launches": 2 * args.steps,
           "roofline": {"bound": "fp64", "achieved": round(achieved, 4), "peak": 1.25, "unit": "TFLOP/s",
                        "frac": round(achieved / 1.25, 4), "traffic": None,
                        "peak_source": "nominal GB300 FP64 1.25 TFLOP/s (no measured FP64 peak); flops estimated "
                                       "from the Sturm counts and eigenvector passes, a division counted as "
                                       "one (it is ~10 FP64 instructions)"},
           "clocks": clk}
    if not args.no_e2e:
        sol.solve(me_all, V_all, SUBBANDS["dy_nm"])
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sol.solve(me_all, V_all, SUBBANDS["dy_nm"])
        we = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": round(slices / we, 1), "unit": "slices/s",
                      "h2d_bytes_per_step": int(G * 8 * (nv * nx * ny + nx * ny)),
                      "d2h_bytes_per_step": int(G * 8 * nv * nx * nm * (1 + ny)),
                      "path": "SubbandSolver.solve (wg_subbands_solve) of the 32-point batch, host arrays in and out"}
    sol.close()
    if not args.no_cpu:
        from oracle import subbands as S
        mat = dict(n_of_modes=nm, n_of_valleys=nv, Nx=nx, Ny=ny, dy=SUBBANDS["dy_nm"], me_y=me, V=secs[0][3])
        t0 = time.perf_counter()
        S.solve_subbands(mat)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(nv * nx / tc, 2), "unit": "slices/s", "cores": os.cpu_count(),
                               "kind": "port",
                               "sample": "one gate point (%d slices) through the oracle: a dense eigensolve of each "
                                         "slice's Hamiltonian, %.1f s" % (nv * nx, tc)}
    return out


POISSON2D = dict(nx=361, ny=13, dx_nm=0.25, dy_nm=0.25, batch=16, nex=120, ney=2, nk=3)


def poisson2d_case(cfg=POISSON2D):
    """The material grid of the reference's recorded Full-2D run (90 nm x 3 nm: 361 x 13 nodes,
    periodic Y, Dirichlet source/drain columns) with a seeded double-barrier permittivity and
    doping layout, and the DG axes of that run (120 x 2 elements, p = 2) for the projection."""
    nx, ny = cfg["nx"], cfg["ny"]
    x = np.arange(nx) * cfg["dx_nm"]
    y = np.arange(ny) * cfg["dy_nm"]
    eps = np.where(((x > 35) & (x < 40)) | ((x > 50) & (x < 55)), 12.9 * 0.9, 12.9)[:, None] * np.ones((1, ny))
    nd = np.where((x < 25) | (x > 65), 1e24, 1e21)[:, None] * np.ones((1, ny))
    prm = dict(N_K_X=cfg["nk"], N_K_Y=cfg["nk"], N_el_X=cfg["nex"], N_el_Y=cfg["ney"], N_rho_x=8, N_rho_y=4,
               L_rho_x=8e-9, full2D_Y_boundary="periodic")
    mat = dict(Nx=nx, Ny=ny, dx=cfg["dx_nm"], dy=cfg["dy_nm"], x=x, y=y, eps=eps, Nd=nd, Temp=300.0,
               dg=dict(params=prm))
    return mat


def run_full2d_solve(args):
    """The mixed Full-2D solve alone on the recorded run's 0.6 V system (stored potential, contact-mode
    reservoirs, line-transverse preconditioner, flexible GMRES(40) with FP64 refinement), to a 1e-12
    residual for at most --solve-maxit refinements: a fixed amount of inner iterations for timing
    and for the per-kernel launch list.  value = inner iterations/s."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300.full2d import Full2DOperator
    mat_r, V_r, efl_r, efr_r = full2d_recorded_case()
    with Full2DOperator(mat_r, V_r) as op:
        rhs, _ = op.reservoir_rhs(efl_r, efr_r)
        op.set_preconditioner()
        clocks = ClockSampler()
        clocks.start()
        t0 = time.perf_counter()
        st, info, _ = op.solve(rhs, tol=1e-12, maxit=args.solve_maxit, restart=40, mixed=True)
        wall = time.perf_counter() - t0
        clk = clocks.stop()
    its = info["iterations"]
    return {"metric": "Full-2D mixed solve inner iterations/s (3,136,320 unknowns)", "value": round(its / wall, 2),
            "unit": "iterations/s", "n_gpus": 1, "steps": its, "warmup": 0,
            "ms_per_step": round(1000 * wall / max(1, its), 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 inner, f64 refinement", "data": "the recorded run's 0.6 V system",
            "config": {"workload": "Full-2D mixed FGMRES(40), %d refinements, line-transverse preconditioner"
                                   % info["cycles"]}, "relres": info["relres"], "clocks": clk}


def run_poisson2d(args):
    """f3: the Poisson step of the Full-2D Gummel loop (project_DG_density_RTD + the approximate
    Newton update of solve_Poisson2D_rtd) for 16 bias points on the material grid of the
    reference's recorded run, one device call per step from nDG resident on the device; e2e
    through Poisson2D.solve with host arrays; the oracle (scipy sparse LU) as CPU baseline."""
    import ctypes
    import torch
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300 import full2d as host2d
    from real_space_dg_gb300.poisson2d import Poisson2D
    cfg = POISSON2D
    mat = poisson2d_case(cfg)
    B, nx, ny = cfg["batch"], cfg["nx"], cfg["ny"]
    X = host2d.dg_axis(np.asarray(mat["x"]) * 1e-9, cfg["nk"], cfg["nex"])
    Y = host2d.dg_axis(np.asarray(mat["y"]) * 1e-9, cfg["nk"], cfg["ney"])
    p = {"X": X, "Y": Y, "coordinateScale": 1e-9}
    rng = np.random.default_rng(0)
    ndx, ndy = X["nd"], Y["nd"]
    prof = np.where((X["verts"][:-1] < 25e-9) | (X["verts"][:-1] > 65e-9), 1e24, 3e22)
    nDG = np.repeat(prof, cfg["nk"])[None, :, None] * rng.uniform(0.8, 1.2, (B, ndx, ndy))
    bias = np.linspace(0.0, 0.3, B)
    phi0 = np.zeros((B, nx, ny))
    op = Poisson2D(mat, batch=B)
    op.set_projection(p, mat)
    dev = torch.device("cuda:0")
    src_d = torch.tensor(np.ascontiguousarray(np.swapaxes(nDG, -1, -2)), device=dev)
    phi0_d = torch.zeros((B, ny, nx), dtype=torch.float64, device=dev)
    bc = np.empty(B * (ny - 1) * nx)
    bias_c = np.ascontiguousarray(bias)
    op.lib.wg_poisson2d_contacts(op.h, bias_c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None,
                                 bc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    bc_d = torch.tensor(bc, device=dev)
    phi_d = torch.empty((B, ny, nx), dtype=torch.float64, device=dev)
    n_d = torch.empty((B, ny, nx), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        op.lib.wg_poisson2d_solve_device(op.h, src_d.data_ptr(), 1, phi0_d.data_ptr(), bc_d.data_ptr(), 1, 1.0,
                                         phi_d.data_ptr(), n_d.data_ptr(), stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        clocks = ClockSampler()
        clocks.start()
        ms = 0.0
        for _ in range(args.steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        clk = clocks.stop()
    value = B * args.steps / (ms / 1000.0)
    nu = ny - 1
    # per bias point: the block sweep (nx Gauss-Jordan inversions of 16 x 16 padded blocks, 2 NU^3
    # flops each, plus the Schur updates and the two block matvecs) and ~60 flops per node for the
    # projection, residuals and diagnostics
    NU = 16
    flops = nx * (2 * NU ** 3 + 4 * NU * NU) + 60 * nx * ny
    out = {"metric": "2D Poisson steps/s (DG density projection + approximate-Newton update, %d x %d grid)" % (nx, ny),
           "value": round(value, 2), "unit": "bias_point_steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic double-barrier permittivity and doping, seeded nDG",
           "config": {"workload": "f3 Poisson step: %d bias points per call, material grid %d x %d (periodic Y, %d "
                                  "unique rows), DG axes 120 x 2 elements p=2" % (B, nx, ny, nu),
                      "l2": "256 MB buffer written between timed steps"},
           "gpu_launches": args.steps,
           "roofline": {"bound": "latency", "achieved": round(flops * value / 1e12, 5), "peak": 1.25,
                        "unit": "TFLOP/s", "frac": round(flops * value / 1e12 / 1.25, 5), "traffic": None,
                        "peak_source": "nominal GB300 FP64 1.25 TFLOP/s; one warp per bias point runs the "
                                       "sequential block sweep (latency-bound by construction)"},
           "clocks": clk}
    if not args.no_e2e:
        op.solve(nDG, phi0, bias, method="newton-raphson", dg=True)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            op.solve(nDG, phi0, bias, method="newton-raphson", dg=True)
        we = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": round(B / we, 2), "unit": "bias_point_steps/s",
                      "h2d_bytes_per_step": int(8 * B * (ndx * ndy + nx * ny + nu * nx)),
                      "d2h_bytes_per_step": int(8 * B * 2 * nx * ny),
                      "path": "Poisson2D.solve(nDG, ..., dg=True) (wg_poisson2d_solve) for the 16 points"}
    op.close()
    if not args.no_cpu:
        from oracle import poisson2d as P2
        mat_n = dict(mat, poisson=dict(opt=dict(solve="newton-raphson")))
        pax = {"X": dict(nLocal=X["nl"], nElements=X["ne"], nDof=X["nd"], r=X["r"], M=X["M"], vertices=X["verts"],
                         jacobian=X["jac"]),
               "Y": dict(nLocal=Y["nl"], nElements=Y["ne"], nDof=Y["nd"], r=Y["r"], M=Y["M"], vertices=Y["verts"],
                         jacobian=Y["jac"]), "coordinateScale": 1e-9}
        t0 = time.perf_counter()
        M, num, typ, _ = P2.eval_poisson2d(mat_n)
        t1 = time.perf_counter()
        for b in range(4):
            d, _ = P2.project_dg_density(nDG[b], pax, mat_n, True)
            P2.solve_poisson2d(M, typ, num, d, mat_n, phi0[b], bias[b])
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": round(4 / (t2 - t1), 3), "unit": "bias_point_steps/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "4 bias points through the oracle (projection + scipy "
                               "sparse LU of the Newton system), %.2f s; operator assembly %.2f s once"
                               % (t2 - t1, t1 - t0)}
    return out


def run_full2d_sc(args):
    """The Full-2D self-consistent loop (solve2D_rtd_self_consistent.m) over the first --biases bias
    points of the reference's recorded sweep (0, 0.02, ... V; 31 in the run) on the 90 nm x 3 nm
    periodic RTD (3,136,320 unknowns): contact-mode reservoirs, approximate-Newton Poisson step,
    mixing 0.3 (main2D_rtd.m), transport by mixed flexible GMRES(40) to 5e-6, warm-started, each
    bias continued from the previous one; compared with the run's stored trajectory, potential,
    density (0 V) and mean current and Gummel iterations (every bias).
    value = self-consistent bias points/s."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300.full2d_sc import solve2D_rtd_self_consistent
    mat, _, _, _ = full2d_recorded_case()
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                "full2d_reservoir_golden.npz"))
    mat.update(Vc=gold["Vc"], eps=gold["eps"], Nd=gold["Nd"], Lc1=float(gold["Lc1"]), Lc2=float(gold["Lc2"]),
               dx=float(gold["dx"]), dy=float(gold["dy"]), Vdd=np.asarray(gold["sweep_bias"])[:max(1, args.biases)],
               poisson=dict(opt=dict(solve="newton-raphson")))
    mat["dg"]["params"].update(full2D_solverTol=5e-6, full2D_gmresRestart=40, full2D_solverMaxIt=150)
    nb = len(mat["Vdd"])
    hist = []
    clocks = ClockSampler()
    clocks.start()
    t0 = time.perf_counter()
    res = solve2D_rtd_self_consistent("DG", mat, {"mixing": 0.3},
                                      callback=lambda ib, it, h: hist.append(h) if ib == 0 else None)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    sw = res["sweep"]
    rec = gold["history0"]
    m = min(len(hist), rec.shape[0])
    defect_rel = [abs(hist[i]["potentialDefect"] - rec[i, 1]) / rec[i, 1] for i in range(m)]
    its = sum(sum(h["gmresIterations"] for h in hb) for hb in res["histories"])
    done = int(np.sum(sw["converged"]))
    ids = np.mean(sw["current"][:, :done], axis=0) if done else np.array([])
    rid = np.asarray(gold["sweep_id"])[:done]
    out = {"metric": "Full-2D self-consistent bias points/s (transport + Poisson Gummel loop to the recorded run's "
                     "tolerances)", "value": round(done / wall, 5), "unit": "bias_points/s", "n_gpus": 1, "steps": nb,
           "warmup": 0, "ms_per_step": round(1000 * wall / max(1, nb), 1), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "bf16/f32 in f64 refinement (transport), f64 (Poisson)",
           "data": "the reference's recorded run (Sim_Res.mat fixture): device fields, reservoirs, bias 0 V",
           "config": {"workload": "Full-2D RTD 90 x 3 nm, 120 x 2 elements p=2, 121 x 12 relative cells, periodic Y, "
                                  "3,136,320 unknowns; %d bias points from 0 V in 0.02 V steps; mixing 0.3, Newton "
                                  "Poisson, GMRES(40) 5e-6" % nb, "wall_s": round(wall, 2),
                      "timing": "wall clock of the whole sweep (host set-up of reservoirs and observables included)"},
           "converged_bias_points": done, "phase_seconds": res.get("timing"),
           "gummel_iterations": [int(v) for v in sw["iterations"][:done]],
           "recorded_gummel_iterations": [int(v) for v in np.asarray(gold["sweep_iterations"])[:done]],
           "gmres_iterations_total": int(its),
           "recorded_gmres_iterations_total": int(np.asarray(gold["sweep_gmres"])[:done].sum()),
           "mean_current": [round(float(v), 6) for v in ids],
           "mean_current_max_diff_vs_recorded_rel_to_max": float(np.max(np.abs(ids - rid)) / max(np.abs(rid).max(), 1e-30))
           if done else None,
           "status": res["status"],
           "vs_recorded_run": {
               "potential_max_abs_diff_V": float(np.abs(sw["potential"][:, :, 0] - gold["potential0"]).max()),
               "density_max_rel_diff": float(np.abs(sw["density"][:, :, 0] - gold["density0"]).max() /
                                             np.abs(gold["density0"]).max()),
               "first_defect_rel_diff": float(defect_rel[0]) if defect_rel else None,
               "max_defect_rel_diff": float(max(defect_rel)) if defect_rel else None},
           "clocks": clk}
    return out


def run_apply(args):
    """Operator applies/s on the C2 batch: the FP64 operator (plain form), the mixed form's
    low-precision inner operator and its tensor-core FP64 operator, with per-kernel rooflines."""
    import __graft_entry__ as g
    g.build()
    from real_space_dg_gb300.rtd import RTDSweep
    spec, mat, biases = make_workload(args.batch)
    S = RTDSweep(mat, args.batch, dict(GUMMEL, precision="mixed"))
    for b, v in enumerate(biases):
        S.set(b, v)
    out = {"metric": "operator applies/s (C2 RTD, batch %d)" % args.batch, "unit": "applies/s",
           "config": {"workload": "C2 operator, %d problems x 245760 unknowns" % args.batch}, "forms": {}}
    for which in ("fp64", "lowprec", "fp64_tc"):
        S.P.apply_time(which, 3)                                    # warm-up
        ms = S.P.apply_time(which, max(10, args.steps))
        S.P.profile(on=True, reset=True)
        S.P.apply_time(which, 5)
        prof = S.P.profile(on=False, reset=True)
        roofs = rooflines(prof, "mixed" if which != "fp64" else "fp64")
        out["forms"][which] = {"ms_per_apply": round(ms, 4), "applies_per_s": round(args.batch * 1000.0 / ms, 1),
                               "rooflines": roofs}
    S.close()
    out["value"] = out["forms"]["lowprec"]["applies_per_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "served", "transient", "apply", "c1", "c4", "full2d",
                                                   "full2d_sc", "full2d_solve", "subbands", "poisson2d", "c4_utb"],
                    help="c2: the headline batched C2 sweep; served: mixed-shape requests through the server; "
                         "transient: batched Crank-Nicolson steps of the C5 RTD; apply: operator applies/s; "
                         "c1: the flat-band C1 solve (plain FP64); c4: multi-subband FET gate sweep; "
                         "full2d: Full-2D operator applies/s; subbands: transverse subband eigensolves/s; "
                         "poisson2d: Full-2D Poisson steps/s; full2d_sc: the Full-2D self-consistent loop at 0 V; "
                         "full2d_solve: the mixed Full-2D solve alone (--solve-maxit refinements); "
                         "c4_utb: the C4 sweep with its subbands from the GPU eigensolve in every step")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--handles", type=int, default=8,
                    help="c2: the batch dealt round-robin to this many handles run concurrently on their own streams")
    ap.add_argument("--serial-handles", action="store_true",
                    help="c2: every step runs the handles one after another from one host thread (launch lists "
                         "under a profiler, which serialises the launches of all threads anyway)")
    ap.add_argument("--launch-shapes", default="",
                    help="c2: 'L,C' pins the k-line chunk length and the FP32 stencil's cells per thread on every "
                         "handle instead of the autotuner's choice (launch lists under a profiler, whose "
                         "serialised launches would mislead the tuner)")
    ap.add_argument("--restart", type=int, default=50)
    ap.add_argument("--inner-restart", type=int, default=40)
    ap.add_argument("--inner-tol", type=float, default=1e-3)
    ap.add_argument("--max-gummel", type=int, default=0,
                    help="cap on Gummel iterations for profiling runs (0: run to convergence)")
    ap.add_argument("--inexact", type=float, default=0.5,
                    help="inexact Gummel factor (transport tol = factor * potential defect); 0 = fixed 1e-8 "
                         "(C2 sweep, points/s: 0.1 23.4, 0.3 31.3, 0.5 37.5-38.0, 0.7 41.8, 1.0 45.5 at cap 1e-2; "
                         "3.0 and 10.0 do not converge)")
    ap.add_argument("--inexact-cap", type=float, default=1e-2,
                    help="loosest transport tolerance of the inexact Gummel schedule")
    ap.add_argument("--reorth", type=float, default=0.0,
                    help="DGKS re-orthogonalisation threshold of the FP64 Arnoldi (0: 1/sqrt(2), <0 never, >=1 always)")
    ap.add_argument("--inner-reorth", type=float, default=0.0,
                    help="the same for the mixed form's inner FP32 Arnoldi (0: never, one classical pass)")
    ap.add_argument("--defer-final", type=int, default=0,
                    help="Gummel iterations a loosely converged point may wait for the batched final re-solve "
                         "(0: the library's 64; -1: none)")
    ap.add_argument("--inner-basis-fp32", action="store_true",
                    help="mixed form: keep the inner Krylov basis in FP32 (default: FP16 storage, FP32 arithmetic)")
    ap.add_argument("--fp64-tc", action="store_true",
                    help="plain FP64 form with its two transforms as FP64 emulated on the tensor cores")
    ap.add_argument("--cpu-iters", type=int, default=8)
    ap.add_argument("--iters-per-point", type=float, default=ITERS_PER_POINT_FALLBACK)
    ap.add_argument("--solve-maxit", type=int, default=150,
                    help="full2d: restart cycles of the timed Full-2D solve (0: skip the solve)")
    ap.add_argument("--biases", type=int, default=1,
                    help="full2d_sc: bias points of the recorded sweep to run (31 = the whole sweep)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="c2: skip the untimed plain-FP64 and fixed-schedule mixed arms and the accuracy fields")
    args = ap.parse_args()
    rank, world, dist = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, rank, world, dist)
    elif args.workload == "served":
        out = run_served(args) if rank == 0 else None
    elif args.workload == "transient":
        out = run_transient(args) if rank == 0 else None
    elif args.workload == "apply":
        out = run_apply(args) if rank == 0 else None
    elif args.workload in ("c4", "c4_utb"):
        out = run_fet(args) if rank == 0 else None
    elif args.workload == "c1":
        out = run_c1(args) if rank == 0 else None
    elif args.workload == "full2d":
        out = run_full2d(args) if rank == 0 else None
    elif args.workload == "subbands":
        out = run_subbands(args) if rank == 0 else None
    elif args.workload == "poisson2d":
        out = run_poisson2d(args) if rank == 0 else None
    elif args.workload == "full2d_sc":
        out = run_full2d_sc(args) if rank == 0 else None
    elif args.workload == "full2d_solve":
        out = run_full2d_solve(args) if rank == 0 else None
    else:
        out = run_ours(args, rank, world, dist)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
