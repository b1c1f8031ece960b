"""CPU oracle for the PIS Lennard-Jones MD step - TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import this package, and only as the checker. The product (``pis_gb300``) never
imports, loads or executes anything from here.

It wraps ``oracle/pis_oracle.cpp`` (a C++ restatement of the reference's FP64 arithmetic,
built by ``oracle/Makefile`` into ``oracle/_build/liboracle.so``) and
``oracle/data_file.py`` (a restatement of the reference's data-file reader).

Parity status: "parity unpinned" against reference outputs - the reference is a Rust
crate that cannot be built here and its tests pin no physics. The oracle is anchored on
known-answer tests derived from the reference's example inputs instead, and its answers on
three seeded states and on those inputs are committed under tests/golden (written by
tests/golden/make_golden.py, which checks the known answers first).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from .data_file import read_data  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

OFFSET, ALLPAIRS, VERLET27, PARALLEL, FULLLIST = 0, 1, 2, 3, 4
KB = 0.0083144621  # src/constants.rs:3


def build() -> str:
    """Compile the oracle library (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _System(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("n_types", C.c_int32),
        ("pbc", C.c_int32 * 3),
        ("type_ids", C.POINTER(C.c_int32)),
        ("masses", C.POINTER(C.c_double)),
        ("pos", C.POINTER(C.c_double)),
        ("vel", C.POINTER(C.c_double)),
        ("force", C.POINTER(C.c_double)),
        ("h", C.c_double * 9),
        ("hinv", C.c_double * 9),
        ("eps", C.POINTER(C.c_double)),
        ("sigma", C.POINTER(C.c_double)),
        ("rcut", C.POINTER(C.c_double)),
        ("present", C.POINTER(C.c_int32)),
        ("shift", C.c_int32),
    ]


class _Nhc(C.Structure):
    _fields_ = [("m", C.c_int32), ("t_start", C.c_double), ("t_end", C.c_double), ("t_target", C.c_double),
                ("xi", C.c_double * 3), ("eta", C.c_double * 3), ("g", C.c_double * 3), ("q", C.c_double * 3)]


class _Mtk(C.Structure):
    _fields_ = [("p_target", C.c_double * 9), ("momentum", C.c_double * 9), ("w", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER
        S = P(_System)
        d = C.c_double
        L.or_inverse3.argtypes = [P(d), P(d)]
        L.or_determinant3.argtypes = [P(d)]
        L.or_determinant3.restype = d
        L.or_min_image.argtypes = [S, P(d)]
        L.or_wrap.argtypes = [S, P(d)]
        L.or_lj_pair.argtypes = [d, d, d, C.c_int32, P(d), P(d), P(d)]
        L.or_max_rcut.argtypes = [S]
        L.or_max_rcut.restype = d
        L.or_divide_into_cells.argtypes = [S, d, P(C.c_int64)]
        for name in ("or_compute_allpairs", "or_compute_verlet27", "or_compute_offset", "or_compute_full_list"):
            getattr(L, name).argtypes = [S]
            getattr(L, name).restype = d
        L.or_compute_parallel.argtypes = [S, C.c_int32]
        L.or_compute_parallel.restype = d
        L.or_compute_potential.argtypes = [S, C.c_int32, C.c_int32]
        L.or_compute_potential.restype = d
        L.or_build_full_list.argtypes = [S, P(C.c_int64), P(C.c_int32), C.c_int64]
        L.or_build_full_list.restype = C.c_int64
        L.or_verlet_step_nve.argtypes = [S, d, C.c_int32, C.c_int32]
        L.or_verlet_step_nve.restype = d
        L.or_kinetic_energy.argtypes = [S]
        L.or_kinetic_energy.restype = d
        L.or_virial_tensor.argtypes = [S, P(d)]
        L.or_pressure.argtypes = [S, d]
        L.or_pressure.restype = d
        L.or_temperature.argtypes = [S, d]
        L.or_temperature.restype = d
        L.or_run_nve.argtypes = [S, d, C.c_int64, C.c_int32, C.c_int32, P(d), P(d)]
        L.or_xsum_array.argtypes = [P(d), C.c_int64]
        L.or_xsum_array.restype = d
        L.or_exact_kinetic_energy.argtypes = [S]
        L.or_exact_kinetic_energy.restype = d
        L.or_exact_virial_tensor.argtypes = [S, P(d)]
        L.or_compute_offset_exact.argtypes = [S, P(d)]
        L.or_compute_offset_exact.restype = d
        L.or_run_nve_exact.argtypes = [S, d, C.c_int64, P(d), P(d), P(d)]
        L.or_fcc_lattice.argtypes = [d, C.c_int64, C.c_int64, C.c_int64, P(d)]
        L.or_remove_drift_and_rescale.argtypes = [S, d]
        L.or_gaussian_velocities.argtypes = [C.c_int64, P(d), d, C.c_uint64, P(d)]
        L.or_num_threads_available.restype = C.c_int32
        N = P(_Nhc)
        L.or_nhc_init.argtypes = [N, d, d, d]
        L.or_nhc_compute_forces.argtypes = [N, d, C.c_int64]
        L.or_nhc_propagate_half_step.argtypes = [N, d]
        L.or_nhc_kinetic_energy.argtypes = [N]
        L.or_nhc_kinetic_energy.restype = d
        L.or_nhc_potential_energy.argtypes = [N, C.c_int64]
        L.or_nhc_potential_energy.restype = d
        L.or_nhc_target.argtypes = [N, C.c_int64, C.c_int64]
        L.or_verlet_step_nvt_nhc.argtypes = [S, d, N, C.c_int32, C.c_int32]
        L.or_verlet_step_nvt_nhc.restype = d
        L.or_run_nvt.argtypes = [S, d, C.c_int64, d, d, d, C.c_int32, C.c_int32, P(d), P(d), P(d), N]
        B = P(_Mtk)
        L.or_expm3.argtypes = [P(d), P(d)]
        L.or_mtk_init.argtypes = [B, d, d, C.c_int64, d]
        L.or_pressure_tensor.argtypes = [S, P(d)]
        L.or_mtk_delta_momentum.argtypes = [B, S, d, P(d)]
        L.or_mtk_scale.argtypes = [B, d, C.c_int32, P(d)]
        L.or_mtk_kinetic_energy.argtypes = [B]
        L.or_mtk_kinetic_energy.restype = d
        L.or_mtk_potential_energy.argtypes = [B, P(d)]
        L.or_mtk_potential_energy.restype = d
        L.or_scale_box.argtypes = [S, P(d)]
        L.or_verlet_step_npt_mtk.argtypes = [S, d, B, N, C.c_int32, C.c_int32]
        L.or_verlet_step_npt_mtk.restype = d
        L.or_run_npt.argtypes = [S, d, C.c_int64, d, d, d, d, d, C.c_int32, C.c_int32, P(d), P(d), P(d), P(d)]
        _lib = L
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def inverse3(h_rowmajor) -> np.ndarray:
    h = np.ascontiguousarray(h_rowmajor, dtype=np.float64).reshape(9)
    out = np.zeros(9)
    lib().or_inverse3(_ptr(h, C.c_double), _ptr(out, C.c_double))
    return out.reshape(3, 3)


def lj_pair(eps, sigma, rcut, rij, shift=True):
    r = np.ascontiguousarray(rij, dtype=np.float64)
    u = np.zeros(1)
    f = np.zeros(3)
    lib().or_lj_pair(eps, sigma, rcut, int(shift), _ptr(r, C.c_double), _ptr(u, C.c_double), _ptr(f, C.c_double))
    return float(u[0]), f


class Nhc:
    """The reference's NHThermostatChain (src/ensemble/nvt.rs), chain length 3."""

    def __init__(self, t_start, t_end, tau):
        self._c = _Nhc()
        lib().or_nhc_init(C.byref(self._c), t_start, t_end, tau)

    def __getattr__(self, name):
        if name in ("xi", "eta", "g", "q"):
            return list(getattr(self._c, name))
        if name in ("t_start", "t_end", "t_target"):
            return getattr(self._c, name)
        raise AttributeError(name)

    def compute_forces(self, kinetic_energy, n_atoms):
        lib().or_nhc_compute_forces(C.byref(self._c), kinetic_energy, n_atoms)

    def propagate_half_step(self, dt):
        lib().or_nhc_propagate_half_step(C.byref(self._c), dt)

    def kinetic_energy(self):
        return lib().or_nhc_kinetic_energy(C.byref(self._c))

    def potential_energy(self, n_atoms):
        return lib().or_nhc_potential_energy(C.byref(self._c), n_atoms)

    def calculate_target_temperature(self, step, steps):
        lib().or_nhc_target(C.byref(self._c), step, steps)


def expm3(a) -> np.ndarray:
    """3x3 matrix exponential (scaling and squaring with Pade approximants, Higham 2005)."""
    m = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
    out = np.zeros(9)
    lib().or_expm3(_ptr(m, C.c_double), _ptr(out, C.c_double))
    return out.reshape(3, 3)


class Mtk:
    """The reference's MTKBarostat (src/ensemble/npt.rs)."""

    def __init__(self, p_start, tau, n_atoms, t_target):
        self._c = _Mtk()
        lib().or_mtk_init(C.byref(self._c), p_start, tau, n_atoms, t_target)

    @property
    def w(self):
        return self._c.w

    @property
    def momentum(self):
        return np.array(self._c.momentum).reshape(3, 3)

    @momentum.setter
    def momentum(self, m):
        self._c.momentum[:] = list(np.asarray(m, dtype=np.float64).reshape(9))

    @property
    def p_target(self):
        return np.array(self._c.p_target).reshape(3, 3)

    def delta_momentum(self, system, dt):
        system._refresh()
        out = np.zeros(9)
        lib().or_mtk_delta_momentum(C.byref(self._c), C.byref(system._s), dt, _ptr(out, C.c_double))
        return out.reshape(3, 3)

    def scale(self, dt, velocity_scaling):
        out = np.zeros(9)
        lib().or_mtk_scale(C.byref(self._c), dt, int(bool(velocity_scaling)), _ptr(out, C.c_double))
        return out.reshape(3, 3)

    def kinetic_energy(self):
        return lib().or_mtk_kinetic_energy(C.byref(self._c))

    def potential_energy(self, h):
        hh = np.ascontiguousarray(h, dtype=np.float64).reshape(9)
        return lib().or_mtk_potential_energy(C.byref(self._c), _ptr(hh, C.c_double))


def xsum(values) -> float:
    """The exact-sum definition shared with the GPU library: every term quantised to
    sign(t) floor(|t| 2^104), summed exactly, rounded to the nearest double (NaN for a term of
    magnitude >= 2^56 or a non-finite term)."""
    v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
    return float(lib().or_xsum_array(_ptr(v, C.c_double), len(v)))


def fcc_lattice(a, nx, ny, nz) -> np.ndarray:
    pos = np.zeros((nx * ny * nz * 4, 3))
    lib().or_fcc_lattice(a, nx, ny, nz, _ptr(pos, C.c_double))
    return pos


class System:
    """Reference-layout state: positions/velocities/forces as (N,3) float64 (x,y,z per
    atom), 1-based int32 type ids, masses per type, row-major box matrix h, and a dense
    per-type-pair LJ table (key (min, max) as the reference's get_potential_ij)."""

    def __init__(self, positions, type_ids, masses, h, table, velocities=None, pbc=(1, 1, 1), shift=True):
        self.pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3).copy()
        n = self.pos.shape[0]
        self.vel = (np.zeros((n, 3)) if velocities is None
                    else np.ascontiguousarray(velocities, dtype=np.float64).reshape(-1, 3).copy())
        self.force = np.zeros((n, 3))
        self.type_ids = np.ascontiguousarray(type_ids, dtype=np.int32).reshape(n).copy()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64).copy()
        nt = len(self.masses)
        self.eps = np.zeros(nt * nt)
        self.sigma = np.zeros(nt * nt)
        self.rcut = np.zeros(nt * nt)
        self.present = np.zeros(nt * nt, dtype=np.int32)
        for (ti, tj), (e, s, rc) in table.items():
            a, b = min(ti, tj), max(ti, tj)
            k = (a - 1) * nt + (b - 1)
            self.eps[k], self.sigma[k], self.rcut[k], self.present[k] = e, s, rc, 1
        self.h = np.ascontiguousarray(h, dtype=np.float64).reshape(3, 3).copy()
        self.hinv = inverse3(self.h)
        self._s = _System()
        s = self._s
        s.n = n
        s.n_types = nt
        s.pbc[:] = [int(p) for p in pbc]
        s.shift = int(shift)
        self._refresh()

    def _refresh(self):
        s = self._s
        s.type_ids = _ptr(self.type_ids, C.c_int32)
        s.masses = _ptr(self.masses, C.c_double)
        s.pos = _ptr(self.pos, C.c_double)
        s.vel = _ptr(self.vel, C.c_double)
        s.force = _ptr(self.force, C.c_double)
        s.h[:] = list(self.h.reshape(9))
        s.hinv[:] = list(self.hinv.reshape(9))
        s.eps = _ptr(self.eps, C.c_double)
        s.sigma = _ptr(self.sigma, C.c_double)
        s.rcut = _ptr(self.rcut, C.c_double)
        s.present = _ptr(self.present, C.c_int32)

    @property
    def n(self):
        return self.pos.shape[0]

    def compute_potential(self, manager=OFFSET, nthreads=1) -> float:
        self._refresh()
        return lib().or_compute_potential(C.byref(self._s), manager, nthreads)

    def verlet_step_nve(self, dt, manager=OFFSET, nthreads=1) -> float:
        self._refresh()
        return lib().or_verlet_step_nve(C.byref(self._s), dt, manager, nthreads)

    def run_nve(self, dt, steps, manager=OFFSET, nthreads=1):
        self._refresh()
        pe = np.zeros(steps + 1)
        ke = np.zeros(steps + 1)
        lib().or_run_nve(C.byref(self._s), dt, steps, manager, nthreads, _ptr(pe, C.c_double), _ptr(ke, C.c_double))
        return pe, ke

    def compute_potential_exact(self):
        """compute_potential with the offset manager: forces as the reference leaves them;
        returns (exact-sum energy, walk-order energy)."""
        self._refresh()
        out = np.zeros(1)
        pe = lib().or_compute_offset_exact(C.byref(self._s), _ptr(out, C.c_double))
        return float(out[0]), pe

    def run_nve_exact(self, dt, steps):
        """run_nve with the offset manager, energies as exact sums: (pe, ke, pe_walk_order)."""
        self._refresh()
        pe, ke, pw = np.zeros(steps + 1), np.zeros(steps + 1), np.zeros(steps + 1)
        lib().or_run_nve_exact(C.byref(self._s), dt, steps, _ptr(pe, C.c_double), _ptr(ke, C.c_double),
                               _ptr(pw, C.c_double))
        return pe, ke, pw

    def kinetic_energy_exact(self) -> float:
        self._refresh()
        return lib().or_exact_kinetic_energy(C.byref(self._s))

    def virial_tensor_exact(self) -> np.ndarray:
        self._refresh()
        w = np.zeros(9)
        lib().or_exact_virial_tensor(C.byref(self._s), _ptr(w, C.c_double))
        return w.reshape(3, 3)

    def verlet_step_nvt_nhc(self, dt, nhc, manager=OFFSET, nthreads=1) -> float:
        self._refresh()
        return lib().or_verlet_step_nvt_nhc(C.byref(self._s), dt, C.byref(nhc._c), manager, nthreads)

    def run_nvt(self, dt, steps, t_start, t_end, tau, manager=OFFSET, nthreads=1):
        """Simulation::run in the NVT ensemble: (pe, ke, hamiltonian) per step, entry 0 before
        the first step, and the final thermostat."""
        self._refresh()
        pe, ke, ham = np.zeros(steps + 1), np.zeros(steps + 1), np.zeros(steps + 1)
        nhc = Nhc(t_start, t_end, tau)
        lib().or_run_nvt(C.byref(self._s), dt, steps, t_start, t_end, tau, manager, nthreads,
                         _ptr(pe, C.c_double), _ptr(ke, C.c_double), _ptr(ham, C.c_double), C.byref(nhc._c))
        return pe, ke, ham, nhc

    def pressure_tensor(self) -> np.ndarray:
        self._refresh()
        out = np.zeros(9)
        lib().or_pressure_tensor(C.byref(self._s), _ptr(out, C.c_double))
        return out.reshape(3, 3)

    def _pull_box(self):
        self.h[:] = np.array(self._s.h).reshape(3, 3)
        self.hinv[:] = np.array(self._s.hinv).reshape(3, 3)

    def scale_box(self, m):
        self._refresh()
        mm = np.ascontiguousarray(m, dtype=np.float64).reshape(9)
        lib().or_scale_box(C.byref(self._s), _ptr(mm, C.c_double))
        self._pull_box()

    def verlet_step_npt_mtk(self, dt, mtk, nhc, manager=OFFSET, nthreads=1) -> float:
        self._refresh()
        pe = lib().or_verlet_step_npt_mtk(C.byref(self._s), dt, C.byref(mtk._c), C.byref(nhc._c), manager, nthreads)
        self._pull_box()
        return pe

    def run_npt(self, dt, steps, t_start, t_end, tau_t, p_start, tau_p, manager=OFFSET, nthreads=1):
        """Simulation::run in the NPT ensemble: (pe, ke, hamiltonian, boxes) per step, entry 0
        before the first step."""
        self._refresh()
        pe, ke, ham = np.zeros(steps + 1), np.zeros(steps + 1), np.zeros(steps + 1)
        boxes = np.zeros((steps + 1, 3, 3))
        lib().or_run_npt(C.byref(self._s), dt, steps, t_start, t_end, tau_t, p_start, tau_p, manager, nthreads,
                         _ptr(pe, C.c_double), _ptr(ke, C.c_double), _ptr(ham, C.c_double), _ptr(boxes, C.c_double))
        self._pull_box()
        return pe, ke, ham, boxes

    def full_list(self):
        """Reference full neighbour list at rcut: list of sorted-as-built index arrays."""
        self._refresh()
        off = np.zeros(self.n + 1, dtype=np.int64)
        total = lib().or_build_full_list(C.byref(self._s), _ptr(off, C.c_int64), None, 0)
        idx = np.zeros(max(total, 1), dtype=np.int32)
        lib().or_build_full_list(C.byref(self._s), _ptr(off, C.c_int64), _ptr(idx, C.c_int32), total)
        return off, idx[:total]

    def kinetic_energy(self) -> float:
        self._refresh()
        return lib().or_kinetic_energy(C.byref(self._s))

    def virial_tensor(self) -> np.ndarray:
        self._refresh()
        w = np.zeros(9)
        lib().or_virial_tensor(C.byref(self._s), _ptr(w, C.c_double))
        return w.reshape(3, 3)

    def pressure(self, ke) -> float:
        self._refresh()
        return lib().or_pressure(C.byref(self._s), ke)

    def temperature(self, ke) -> float:
        self._refresh()
        return lib().or_temperature(C.byref(self._s), ke)

    def min_image(self, r) -> np.ndarray:
        self._refresh()
        v = np.ascontiguousarray(r, dtype=np.float64).copy()
        lib().or_min_image(C.byref(self._s), _ptr(v, C.c_double))
        return v

    def wrap(self, r) -> np.ndarray:
        self._refresh()
        v = np.ascontiguousarray(r, dtype=np.float64).copy()
        lib().or_wrap(C.byref(self._s), _ptr(v, C.c_double))
        return v

    def max_rcut(self) -> float:
        self._refresh()
        return lib().or_max_rcut(C.byref(self._s))

    def divide_into_cells(self, rcut):
        self._refresh()
        n = np.zeros(3, dtype=np.int64)
        lib().or_divide_into_cells(C.byref(self._s), rcut, _ptr(n, C.c_int64))
        return tuple(int(x) for x in n)

    def remove_drift_and_rescale(self, temperature):
        self._refresh()
        lib().or_remove_drift_and_rescale(C.byref(self._s), temperature)

    @staticmethod
    def from_data(data, shift=True):
        """Build from a parsed data file (oracle.read_data)."""
        h = np.diag([data["xhi"] - data["xlo"], data["yhi"] - data["ylo"], data["zhi"] - data["zlo"]])
        return System(data["positions"], data["type_ids"], data["masses"], h, data["table"],
                      velocities=data["velocities"], shift=shift)


def maxwell_boltzmann(masses_per_atom, temperature, seed) -> np.ndarray:
    """This project's seeded Maxwell-Boltzmann velocities (SplitMix64 + Box-Muller draw, then the
    reference's drift removal and rescale, src/atoms/velocities.rs:35-59), computed without the GPU
    library: the CPU baseline's start state."""
    m = np.ascontiguousarray(masses_per_atom, dtype=np.float64)
    n = len(m)
    v = np.zeros((n, 3))
    lib().or_gaussian_velocities(n, _ptr(m, C.c_double), float(temperature), int(seed), _ptr(v, C.c_double))
    uniq = sorted(set(m.tolist()))
    types = np.array([uniq.index(x) + 1 for x in m.tolist()], np.int32)
    s = System(np.zeros((n, 3)), types, uniq, np.eye(3), {}, velocities=v)
    s.remove_drift_and_rescale(temperature)
    return s.vel.copy()


def num_threads_available() -> int:
    return int(lib().or_num_threads_available())
