"""Serving of self-consistent bias points (continuous batching), Python side.

``Server`` wraps the native request loop of libwigner_gb300.so (wg_server_*):
requests are I-V points of RTD devices (``mat`` dicts as for
``rtd.solve_rtd_self_consistent``), admitted into free slots of per-shape
handles under a device-memory budget while other requests are iterating, and
seeded from the nearest finished bias of the same device.  ``serve_sweep``
replays an arrival schedule (e.g. a Poisson process) against a server and
reports latencies and throughput.
"""
import ctypes as C
import threading
import time

import numpy as np

from . import _lib, devices
from ._lib import WignerError
from .rtd import DEFAULTS
from .transport import M0, shape_from_mat


def _gummel_opts(o):
    return _lib.WgGummelOpts(int(o["maxIterations"]), float(o["mixing"]), float(o["potentialTolerance"]),
                             float(o["densityTolerance"]), float(o["poissonResidualTolerance"]),
                             float(o["transportTolerance"]), int(o["transportMaxCycles"]), 0, 0,
                             float(o["inexactFactor"]), float(o["inexactCap"]), int(o["deferFinal"]))


class Server:
    """Continuous-batching server of self-consistent RTD bias points."""

    def __init__(self, options=None, mem_budget_bytes=150e9, max_slots=8, warm_start=True, idle_release_s=0.5):
        # a served request waits at most 8 Gummel iterations for its batched final re-solve (latency)
        o = dict(DEFAULTS, deferFinal=8)
        for k, v in (options or {}).items():
            if k not in o:
                raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownSelfConsistencyOption %s" % k)
            o[k] = v
        self.o = o
        self.lib = _lib.load()
        so = _lib.WgServerOpts(float(mem_budget_bytes), int(max_slots),
                               _lib.WG_PREC_MIXED if o["precision"] == "mixed" else _lib.WG_PREC_FP64,
                               int(o["restart"]), int(o["innerRestart"]), float(o["innerTol"]), float(o["reorth"]),
                               float(o["innerReorth"]), _gummel_opts(o),
                               1 if warm_start else 0, float(idle_release_s))
        self.h = C.c_void_p()
        st = self.lib.wg_server_create(C.byref(so), C.byref(self.h))
        if st != _lib.WG_OK:
            raise WignerError(st, "wg_server_create failed")
        self._shapes = {}

    def close(self):
        if self.h:
            self.lib.wg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, mat, bias, device_key=0, phi0=None):
        """Queue the self-consistent point of ``mat`` at ``bias``; returns its id."""
        shp = shape_from_mat(mat)
        nx = int(mat["Nx"])
        x = np.ascontiguousarray(mat["x"], dtype=float)
        m = np.ascontiguousarray(np.asarray(mat["me_x"], dtype=float).reshape(-1, nx, int(mat["Ny"]))[0, :, 0] * M0)
        vc = np.ascontiguousarray(mat["Vc"], dtype=float)
        nd = np.ascontiguousarray(mat["Nd"], dtype=float)
        eps = np.ascontiguousarray(mat["eps"], dtype=float)
        phi0 = np.ascontiguousarray(bias * np.asarray(mat["ramp"], dtype=float) if phi0 is None else phi0,
                                    dtype=float)
        dy = float(mat.get("dy_norm_nm") or devices.density_normalisation_nm(mat, self.o["fermiOffset"]))
        req = _lib.WgRequest(shp["n_el"], shp["n_local"], shp["nk"], shp["n_xi"] or 0, shp["l_xi"], shp["m_diff"],
                             shp["mpc"],
                             _lib.WgDevice(nx, _lib.dptr(x), _lib.dptr(m), float(mat["me_z_ch"]), float(mat["Temp"])),
                             _lib.WgRtd1D(_lib.dptr(vc), _lib.dptr(nd), _lib.dptr(eps), _lib.dptr(phi0), float(bias),
                                          float(self.o["fermiOffset"]), dy),
                             int(device_key))
        rid = C.c_longlong()
        st = self.lib.wg_server_submit(self.h, C.byref(req), C.byref(rid))
        if st != _lib.WG_OK:
            raise WignerError(st, "wg_server_submit rejected the request")
        self._shapes[rid.value] = (nx, shp["n_el"] * shp["n_local"])
        return rid.value

    def wait(self, rid, timeout=None, release=True):
        """Block until request ``rid`` ends; returns a dict with its status, timings and results."""
        st = _lib.WgRequestStatus()
        rc = self.lib.wg_server_wait(self.h, int(rid), -1.0 if timeout is None else float(timeout), C.byref(st))
        if rc == _lib.WG_ERR_TIMEOUT:
            raise TimeoutError("request %d still %s" % (rid, _lib.REQUEST_STATES[st.state]))
        if rc != _lib.WG_OK:
            raise WignerError(rc, "wg_server_wait failed")
        out = {"id": rid, "state": _lib.REQUEST_STATES[st.state], "info": st.info.as_dict(),
               "status": _lib.GUMMEL_STATUS.get(st.info.status, str(st.info.status)),
               "t_submit": st.t_submit, "t_admit": st.t_admit, "t_done": st.t_done,
               "latency": st.t_done - st.t_submit, "handle": st.handle, "slot": st.slot, "warm": st.warm,
               "error": st.error.decode(errors="replace")}
        if st.state == 2:
            nx, ncol = self._shapes[rid]
            phi, n, j = np.empty(nx), np.empty(ncol), np.empty(ncol)
            rc = self.lib.wg_server_result(self.h, int(rid), _lib.dptr(phi), _lib.dptr(n), _lib.dptr(j))
            if rc != _lib.WG_OK:
                raise WignerError(rc, "wg_server_result failed")
            out.update(phi=phi, n=n, j=j)
        if release:
            self.lib.wg_server_release(self.h, int(rid))
            self._shapes.pop(rid, None)
        return out

    def stats(self):
        st = _lib.WgServerStats()
        self.lib.wg_server_stats_get(self.h, C.byref(st))
        return st.as_dict()


def serve_sweep(server, jobs, arrivals=None):
    """Submit ``jobs`` [(mat, bias, device_key), ...] at the offsets ``arrivals`` [s]
    (all at once if None) from a feeder thread; returns (results in job order,
    wall seconds from the first arrival to the last completion)."""
    n = len(jobs)
    arrivals = np.zeros(n) if arrivals is None else np.asarray(arrivals, dtype=float)
    ids = [None] * n
    errors = []
    t0 = time.perf_counter()

    def feeder():
        try:
            for i in np.argsort(arrivals, kind="stable"):
                delay = arrivals[i] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                mat, bias, key = jobs[i]
                ids[i] = server.submit(mat, bias, key)
        except Exception as e:          # surfaced to the caller below
            errors.append(e)

    th = threading.Thread(target=feeder)
    th.start()
    results = [None] * n
    for i in np.argsort(arrivals, kind="stable"):
        while ids[i] is None and not errors:
            time.sleep(0.001)
        if errors:
            break
        results[i] = server.wait(ids[i])
    th.join()
    if errors:
        raise errors[0]
    return results, time.perf_counter() - t0
