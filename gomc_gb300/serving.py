"""Continuous-batching job server over the C ABI (gb_server_* in
include/gomc_gb300.h).

The scheduler is native (gomc_gb300/csrc/gb_serve.cu); this module packs
jobs into the C structures and unpacks results.  The reference has no
serving layer: it runs one simulation per process (src/Simulation.cpp).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GB_MIXED, GbError, lib
from .engine import config_struct, mc_params, system_desc

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3
STATUS_NAMES = {QUEUED: "queued", RUNNING: "running", DONE: "done",
                FAILED: "failed"}
STATS_KEYS = ["jobs_done", "moves", "wall_s", "moves_per_s",
              "sweep_p50_ms", "sweep_p99_ms", "job_p50_s", "job_p99_s",
              "rounds", "mean_resident", "helper_busy_s", "round_busy_s"]
OCCUPANCY_KEYS = ["mean_admitted", "mean_in_round", "cta_slot_frac",
                  "smem_frac", "mean_queued", "stops_mem", "stops_smem",
                  "stops_ctas", "launch_balance", "round_gap_s"]


class Server:
    """Resident simulation jobs on one GPU, batched per round."""

    def __init__(self, device: int = 0, quantum: int = 1000,
                 mem_budget: int = 0, max_resident: int = 0):
        c = _lib.ServerConfig()
        c.device, c.quantum = int(device), int(quantum)
        c.mem_budget, c.max_resident = int(mem_budget), int(max_resident)
        h = C.c_void_p()
        rc = lib().gb_server_create(C.byref(c), C.byref(h))
        if rc:
            raise GbError(rc, "gb_server_create failed")
        self.h = h
        self.device = int(device)
        self._sizes = {}

    def _chk(self, rc: int) -> None:
        if rc:
            msg = lib().gb_server_error(self.h)
            raise GbError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, sysm, cfg, seed: int, nsteps: int,
               move_frac: Sequence[float] = (0.5, 0.5, 0.0),
               adj_steps: int = 1000,
               scales: Optional[Sequence[float]] = None,
               recompute_freq: int = 10000, cluster_size: int = 0,
               sweep_moves: int = 0) -> int:
        d, keep = system_desc(sysm)
        c = config_struct(cfg, GB_MIXED, self.device)
        p = mc_params(seed, move_frac, adj_steps, scales, recompute_freq,
                      cluster_size)
        jid = C.c_int64()
        self._chk(lib().gb_server_submit(self.h, C.byref(d), C.byref(c),
                                         C.byref(p), int(nsteps),
                                         int(sweep_moves), C.byref(jid)))
        del keep  # the server copied the inputs
        self._sizes[jid.value] = (sysm.n_atoms, sysm.n_mol)
        return jid.value

    def estimate(self, sysm, cfg, cluster_size: int = 0) -> dict:
        """Device bytes the server reserves for such a job at admission,
        and the CTAs per chain it would run it with."""
        d, keep = system_desc(sysm)
        c = config_struct(cfg, GB_MIXED, self.device)
        p = mc_params(0, (0.5, 0.5, 0.0), 1000, cluster_size=cluster_size)
        b, cs = C.c_int64(), C.c_int32()
        self._chk(lib().gb_server_estimate(self.h, C.byref(d), C.byref(c),
                                           C.byref(p), C.byref(b),
                                           C.byref(cs)))
        del keep
        return dict(bytes=b.value, ctas_per_chain=cs.value)

    def step(self) -> int:
        n = C.c_int32()
        self._chk(lib().gb_server_step(self.h, C.byref(n)))
        return n.value

    def run_until_idle(self) -> None:
        while self.step():
            pass

    def start(self) -> None:
        self._chk(lib().gb_server_start(self.h))

    def drain(self, timeout_s: float = 0.0) -> None:
        self._chk(lib().gb_server_drain(self.h, float(timeout_s)))

    def job(self, jid: int) -> dict:
        st, n = C.c_int32(), C.c_int64()
        t = np.zeros(3)
        self._chk(lib().gb_server_job(self.h, int(jid), C.byref(st),
                                      C.byref(n),
                                      t.ctypes.data_as(C.POINTER(C.c_double))))
        return dict(status=STATUS_NAMES[st.value], steps_done=n.value,
                    t_submit=t[0], t_admit=t[1], t_done=t[2])

    def result(self, jid: int) -> dict:
        na, nm = self._sizes[jid]
        xyz = np.empty((na, 3))
        com = np.empty((nm, 3))
        e = np.empty(5)
        dp = C.POINTER(C.c_double)
        self._chk(lib().gb_server_result(self.h, int(jid),
                                         xyz.ctypes.data_as(dp),
                                         com.ctypes.data_as(dp),
                                         e.ctypes.data_as(dp)))
        return dict(xyz=xyz, com=com, energy=e)

    def stats(self) -> dict:
        o = np.zeros(12)
        self._chk(lib().gb_server_stats(self.h,
                                        o.ctypes.data_as(C.POINTER(C.c_double))))
        d = dict(zip(STATS_KEYS, o.tolist()))
        occ = np.zeros(10)
        self._chk(lib().gb_server_occupancy(
            self.h, occ.ctypes.data_as(C.POINTER(C.c_double))))
        d.update(zip(OCCUPANCY_KEYS, occ.tolist()))
        return d
