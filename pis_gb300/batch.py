"""Batched replicas and served jobs over the C ABI (pis_batch_*, pis_serve_run).

A ``Batch`` is one device pool of independent LJ systems advanced together: one launch per kernel
per step over every slot, 50-step CUDA graphs, slots admitted and released between advances.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _ffi
from ._ffi import PisError


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def lj_job(k, rho, t_star, steps, seed, rcut=2.5, skin=0.3, dt=0.005) -> _ffi.LJJob:
    """Synthetic LJ-liquid job: 4 k^3 atoms on an FCC lattice at density rho, T* from seed."""
    return _ffi.LJJob(int(k), float(rho), float(t_star), float(rcut), float(skin), float(dt), int(steps), int(seed))


def lj_pool_cells(k, rho, rlist=2.8) -> int:
    """Cell entries a job occupies in the pool (cells at rcut + skin, plus one sentinel)."""
    L = (4.0 / rho) ** (1.0 / 3.0) * k
    n = max(1, math.floor(L / rlist))
    return n ** 3 + 1


class Batch:
    def __init__(self, max_atoms, max_slots, max_cells=0, precision="mixed", fp64_fast=False, mixed_kahan=False,
                 lanes=0, batch=0, tma=False, cluster=0, scan=0, tiles=False,
                 plain_graphs=False, unfused=False):
        self._lib = _ffi.lib()
        flags = _ffi.option_flags(fp64_fast, mixed_kahan, lanes, batch, tma, cluster, scan, tiles,
                                  plain_graphs, unfused)
        h = C.c_void_p()
        st = self._lib.pis_batch_create(int(max_atoms), int(max_slots), int(max_cells), _ffi.PRECISION[precision],
                                        flags, C.byref(h))
        if st != 0:
            raise PisError(st, "pis_batch_create failed")
        self._h = h

    def _check(self, st):
        if st != 0:
            msg = self._lib.pis_batch_last_error(self._h)
            raise PisError(st, msg.decode() if msg else "")

    def admit_lj(self, job: _ffi.LJJob) -> int:
        slot = C.c_int32(-1)
        self._check(self._lib.pis_batch_admit_lj(self._h, C.byref(job), C.byref(slot)))
        return slot.value

    def admit(self, positions, type_ids, masses, h, table, steps, velocities=None, skin=0.3, dt=0.005) -> int:
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        t = np.ascontiguousarray(type_ids, dtype=np.int32)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64).reshape(n, 3)
        hc = np.ascontiguousarray(np.asarray(h, dtype=np.float64).reshape(3, 3).T)
        pairs = (_ffi.LJPair * len(table))()
        for k, ((ti, tj), (e, s, rc)) in enumerate(table.items()):
            pairs[k] = _ffi.LJPair(int(ti), int(tj), float(e), float(s), float(rc), 1)
        job = _ffi.Job(n, len(m), t.ctypes.data_as(C.POINTER(C.c_int32)), _dp(m), _dp(pos), _dp(vel), _dp(hc), pairs,
                       len(table), float(skin), float(dt), int(steps))
        slot = C.c_int32(-1)
        self._check(self._lib.pis_batch_admit(self._h, C.byref(job), C.byref(slot)))
        return slot.value

    def fits_lj(self, job) -> bool:
        return bool(self._lib.pis_batch_fits_lj(self._h, C.byref(job)))

    def advance(self, k):
        self._check(self._lib.pis_batch_advance(self._h, int(k)))

    def run_timed(self, k) -> float:
        ms = C.c_double()
        self._check(self._lib.pis_batch_run_timed(self._h, int(k), C.byref(ms)))
        return ms.value

    def poll(self, cap=4096):
        done = (C.c_int32 * cap)()
        nd = C.c_int32()
        self._check(self._lib.pis_batch_poll(self._h, done, cap, C.byref(nd)))
        return [done[q] for q in range(min(nd.value, cap))]

    def result(self, slot, n=None, state=True):
        pe, ke, steps = C.c_double(), C.c_double(), C.c_int64()
        pos = vel = frc = None
        if state:
            pos, vel, frc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        self._check(self._lib.pis_batch_result(self._h, int(slot), _dp(pos), _dp(vel), _dp(frc), C.byref(pe),
                                               C.byref(ke), C.byref(steps)))
        return {"pe": pe.value, "ke": ke.value, "steps": steps.value, "pos": pos, "vel": vel, "force": frc}

    def pe_history(self, slot, n):
        out = np.zeros(n)
        self._check(self._lib.pis_batch_pe_history(self._h, int(slot), int(n), _dp(out)))
        return out

    def release(self, slot):
        self._check(self._lib.pis_batch_release(self._h, int(slot)))

    @property
    def atoms(self) -> int:
        return int(self._lib.pis_batch_atoms(self._h))

    def serve(self, requests, graph_steps=50):
        """requests: list of (arrival_s, LJJob). Returns (list of result dicts, wall seconds)."""
        n = len(requests)
        reqs = (_ffi.Request * max(n, 1))()
        for q, (t, job) in enumerate(requests):
            reqs[q] = _ffi.Request(float(t), job)
        out = (_ffi.RequestResult * max(n, 1))()
        wall = C.c_double()
        self._check(self._lib.pis_serve_run(self._h, reqs, n, int(graph_steps), out, C.byref(wall)))
        res = [{"arrival_s": requests[q][0], "admitted_s": out[q].admitted_s, "finished_s": out[q].finished_s,
                "atoms": out[q].atoms, "steps": out[q].steps, "pe": out[q].pe, "ke": out[q].ke,
                "status": out[q].status} for q in range(n)]
        return res, wall.value

    def serve_stats(self) -> dict:
        """Per-graph accounting of the last serve(): atom-steps and device seconds, over all graphs
        and over the saturated ones (queued while a request waited for pool space)."""
        st = _ffi.ServeStats()
        self._check(self._lib.pis_serve_last_stats(self._h, C.byref(st)))
        out = {f: getattr(st, f) for f, _ in _ffi.ServeStats._fields_}
        out["atom_steps_per_device_s"] = st.atom_steps / st.device_s if st.device_s > 0 else None
        out["saturated_atom_steps_per_device_s"] = (st.saturated_atom_steps / st.saturated_device_s
                                                    if st.saturated_device_s > 0 else None)
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pis_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
