"""Python mirror of the reference's potential-manager interface over the CUDA C ABI.

``GpuContext`` wraps one ``pis_gpu_ctx`` (include/pis_gpu.h). ``LJGpuManager`` presents the
reference's ``PotentialManager`` contract (src/potentials/potential.rs:12-136) on ``Atoms``
objects: ``compute_potential(atoms)`` zeroes and fills ``atoms.forces`` and returns the
potential energy; ``verlet_step_nve(atoms, dt)`` advances the state one step and returns the
energy of the new configuration. The device keeps the state resident between calls and only
re-uploads when the host arrays were changed behind its back.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import PisError


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class GpuContext:
    """One device-resident LJ system (the C-ABI context)."""

    def __init__(self, table, n_types, skin=0.3, precision="fp64", list_kind="default", shift=True,
                 fp64_fast=False, mixed_kahan=False, lanes=0, batch=0, tma=False, cluster=0, scan=0, tiles=False,
                 plain_graphs=False, unfused=False, ref_order=False, list_capacity=0, auto_grow=True,
                 wait_limit=None):
        self._lib = _ffi.lib()
        self.n_types = int(n_types)
        pairs = (_ffi.LJPair * len(table))()
        for k, ((ti, tj), (eps, sigma, rc)) in enumerate(table.items()):
            pairs[k] = _ffi.LJPair(int(ti), int(tj), float(eps), float(sigma), float(rc), int(bool(shift)))
        h = C.c_void_p()
        st = self._lib.pis_gpu_create(pairs, len(table), self.n_types, float(skin),
                                      _ffi.PRECISION[precision], C.byref(h))
        if st != 0:
            raise PisError(st, "pis_gpu_create failed")
        self._h = h
        self.n = 0
        self.precision = precision
        flags = _ffi.option_flags(fp64_fast, mixed_kahan, lanes, batch, tma, cluster, scan, tiles,
                                  plain_graphs, unfused, ref_order)
        if list_kind != "default" or flags:
            self._check(self._lib.pis_gpu_set_options(self._h, _ffi.LIST_KIND[list_kind], flags))
        if list_capacity or not auto_grow:
            self._check(self._lib.pis_gpu_set_list_capacity(self._h, int(list_capacity), int(bool(auto_grow))))
        if wait_limit is not None:
            self._check(self._lib.pis_gpu_set_wait_limit(self._h, int(wait_limit)))

    def _check(self, st):
        if st != 0:
            msg = self._lib.pis_gpu_last_error(self._h)
            raise PisError(st, msg.decode() if msg else "")

    def set_state(self, positions, type_ids, masses, h, velocities=None, forces=None):
        """Upload an Atoms state. ``h`` is the 3x3 box matrix (row/column form irrelevant for
        the orthorhombic boxes supported)."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        t = np.ascontiguousarray(type_ids, dtype=np.int32).reshape(n)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64).reshape(n, 3)
        frc = None if forces is None else np.ascontiguousarray(forces, dtype=np.float64).reshape(n, 3)
        hc = np.ascontiguousarray(np.asarray(h, dtype=np.float64).reshape(3, 3).T)  # column-major storage
        pbc = (C.c_uint8 * 3)(1, 1, 1)
        self._check(self._lib.pis_gpu_set_state(self._h, n, t.ctypes.data_as(C.POINTER(C.c_int32)), _dp(m),
                                                 _dp(pos), _dp(vel), _dp(frc), _dp(hc), pbc))
        self.n = n

    def compute_potential(self, want_forces=True):
        pe = C.c_double()
        f = np.zeros((self.n, 3)) if want_forces else None
        self._check(self._lib.pis_gpu_compute_potential(self._h, C.byref(pe), _dp(f)))
        return pe.value, f

    def verlet_step_nve(self, dt, n_steps=1, want_pe=True):
        pe = np.zeros(n_steps) if want_pe else None
        self._check(self._lib.pis_gpu_verlet_step_nve(self._h, float(dt), int(n_steps), _dp(pe)))
        return pe

    def verlet_step_nve_thermo(self, dt, n_steps):
        """n_steps NVE steps with every step's (PE, KE, virial trace) recorded on the device and
        read back once: three arrays of n_steps values."""
        pe, ke, tr = np.zeros(n_steps), np.zeros(n_steps), np.zeros(n_steps)
        self._check(self._lib.pis_gpu_verlet_step_nve_thermo(self._h, float(dt), int(n_steps), _dp(pe), _dp(ke),
                                                             _dp(tr)))
        return pe, ke, tr

    def run_timed(self, dt, n_steps, stages=False):
        """Measurement hook: (device milliseconds, per-stage milliseconds or None)."""
        ms = C.c_double()
        st = np.zeros(5) if stages else None
        self._check(self._lib.pis_gpu_run_timed(self._h, float(dt), int(n_steps), C.byref(ms), _dp(st)))
        return ms.value, st

    def get_state(self, out=None):
        """(positions, velocities, forces) as (n, 3) arrays; ``out`` may supply three C-contiguous
        float64 (n, 3) arrays to fill (e.g. in pinned host memory)."""
        if out is None:
            out = (np.zeros((self.n, 3)), np.zeros((self.n, 3)), np.zeros((self.n, 3)))
        for a in out:
            if a.dtype != np.float64 or a.shape != (self.n, 3) or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("output arrays must be C-contiguous float64 of shape (n, 3)")
        pos, vel, frc = out
        self._check(self._lib.pis_gpu_get_state(self._h, _dp(pos), _dp(vel), _dp(frc)))
        return pos, vel, frc

    def reductions(self):
        ke = C.c_double()
        w = np.zeros(9)
        self._check(self._lib.pis_gpu_reductions(self._h, C.byref(ke), _dp(w)))
        return ke.value, w.reshape(3, 3)

    def neighbour_list(self):
        off = np.zeros(self.n + 1, dtype=np.int64)
        total = C.c_int64()
        self._check(self._lib.pis_gpu_neighbour_list(self._h, off.ctypes.data_as(C.POINTER(C.c_int64)), None, 0,
                                                      C.byref(total)))
        idx = np.zeros(max(total.value, 1), dtype=np.int32)
        self._check(self._lib.pis_gpu_neighbour_list(self._h, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                                      idx.ctypes.data_as(C.POINTER(C.c_int32)), total.value,
                                                      C.byref(total)))
        return off, idx[: total.value]

    def scale_velocities(self, m):
        mm = np.ascontiguousarray(m, dtype=np.float64).reshape(9)
        self._check(self._lib.pis_gpu_scale_velocities(self._h, _dp(mm)))

    def scale_box(self, m):
        mm = np.ascontiguousarray(m, dtype=np.float64).reshape(9)
        self._check(self._lib.pis_gpu_scale_box(self._h, _dp(mm)))

    def pressure_tensor(self) -> np.ndarray:
        """Atoms::pressure_tensor: (sum v v^T + sum r F^T) / volume (3x3)."""
        p = np.zeros(9)
        self._check(self._lib.pis_gpu_pressure_tensor(self._h, _dp(p)))
        return p.reshape(3, 3)

    def box(self) -> np.ndarray:
        """The current box matrix h (3x3, columns = box vectors)."""
        hc = np.zeros(9)
        self._check(self._lib.pis_gpu_get_box(self._h, _dp(hc)))
        return hc.reshape(3, 3).T.copy()

    def stats(self) -> dict:
        s = _ffi.Stats()
        self._check(self._lib.pis_gpu_get_stats(self._h, C.byref(s)))
        return {"n_atoms": s.n_atoms, "steps": s.steps, "rebuilds": s.rebuilds, "list_entries": s.list_entries,
                "list_capacity": s.list_capacity, "cells": tuple(s.cells), "pe": s.pe, "ke": s.ke,
                "virial": np.array(s.virial).reshape(3, 3), "fused_step": bool(s.fused_step)}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pis_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launches() -> int:
    return int(_ffi.lib().pis_gpu_kernel_launches())


class LJGpuManager:
    """GPU ``PotentialManager`` (the would-be ``PotentialManagerKind::LJGpu`` variant).

    ``table`` maps (ti, tj) -> (epsilon, sigma, rcut) exactly like the reference's pair Table
    (src/potentials/potential.rs:143-144); energies are shifted (src/system.rs:161)."""

    def __init__(self, table, n_types=None, skin=0.3, precision="fp64", list_kind="default"):
        self.table = dict(table)
        self.n_types = n_types or max(max(k) for k in self.table)
        self.ctx = GpuContext(self.table, self.n_types, skin=skin, precision=precision, list_kind=list_kind)
        self._synced = None

    def _sync_in(self, atoms):
        key = (id(atoms), atoms.version)
        if self._synced != key:
            self.ctx.set_state(atoms.positions, atoms.type_ids, atoms.masses, atoms.sim_box.h,
                               velocities=atoms.velocities, forces=atoms.forces)
            self._synced = key

    def compute_potential(self, atoms) -> float:
        """PotentialManager::compute_potential with zeroed forces (src/potentials/potential.rs:24-26)."""
        self._sync_in(atoms)
        pe, f = self.ctx.compute_potential()
        atoms.forces[:] = f
        self._synced = (id(atoms), atoms.touch())
        return pe

    def verlet_step_nve(self, atoms, dt) -> float:
        """PotentialManager::verlet_step_nve (src/potentials/potential.rs:15-33)."""
        self._sync_in(atoms)
        pe = self.ctx.verlet_step_nve(dt, 1)
        pos, vel, frc = self.ctx.get_state()
        atoms.positions[:] = pos
        atoms.velocities[:] = vel
        atoms.forces[:] = frc
        self._synced = (id(atoms), atoms.touch())
        return float(pe[0])

    def verlet_step_nvt_nhc(self, atoms, dt, chain) -> float:
        """PotentialManager::verlet_step_nvt_nhc (src/potentials/potential.rs:35-58): thermostat
        half step, velocities scaled by exp(-dt xi_0 / 2), the NVE step, the same scale, and the
        thermostat half step on the new kinetic energy. ``chain`` is a
        pis_gb300.ensemble.NHThermostatChain; the kinetic energies come from the device."""
        import math
        self._sync_in(atoms)
        n = atoms.n_atoms
        ke, _ = self.ctx.reductions()
        chain.compute_forces(ke, n)
        chain.propagate_half_step(dt)
        scale = math.exp(-0.5 * dt * chain.xi[0])
        m = np.diag([scale, scale, scale])
        self.ctx.scale_velocities(m)
        pe = self.ctx.verlet_step_nve(dt, 1)
        self.ctx.scale_velocities(m)
        ke, _ = self.ctx.reductions()
        chain.compute_forces(ke, n)
        chain.propagate_half_step(dt)
        pos, vel, frc = self.ctx.get_state()
        atoms.positions[:] = pos
        atoms.velocities[:] = vel
        atoms.forces[:] = frc
        self._synced = (id(atoms), atoms.touch())
        return float(pe[0])

    def run_nve(self, atoms, dt, steps):
        """``steps`` NVE steps with the state resident on the device; returns per-step PE."""
        self._sync_in(atoms)
        pe = self.ctx.verlet_step_nve(dt, steps)
        pos, vel, frc = self.ctx.get_state()
        atoms.positions[:] = pos
        atoms.velocities[:] = vel
        atoms.forces[:] = frc
        self._synced = (id(atoms), atoms.touch())
        return pe
