"""Host-side readers and writers over the C ABI of include/pis_host.h: the reference's LAMMPS-style
data files (read and restart write), Rust-style float formatting, Maxwell-Boltzmann velocities,
and the System driver (input file -> run with thermo and .lammpstrj dumps)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import PisError


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def read_data(path: str) -> dict:
    L = _ffi.lib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = L.pis_data_read(path.encode(), C.byref(h), err, 512)
    if st != 0:
        raise PisError(st, err.value.decode())
    try:
        n = L.pis_data_n_atoms(h)
        nt = L.pis_data_n_types(h)
        npairs = L.pis_data_n_pairs(h)
        types = np.zeros(n, np.int32)
        masses = np.zeros(nt)
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        bounds = np.zeros(6)
        hv = C.c_int32()
        L.pis_data_get(h, types.ctypes.data_as(C.POINTER(C.c_int32)), _dp(masses), _dp(pos), _dp(vel), _dp(bounds),
                       C.byref(hv))
        pairs = (_ffi.LJPair * max(npairs, 1))()
        if npairs:
            L.pis_data_pairs(h, pairs)
        table = {(pairs[k].ti, pairs[k].tj): (pairs[k].epsilon, pairs[k].sigma, pairs[k].rcut) for k in range(npairs)}
    finally:
        L.pis_data_free(h)
    return {"n_atoms": n, "xlo": bounds[0], "xhi": bounds[1], "ylo": bounds[2], "yhi": bounds[3], "zlo": bounds[4],
            "zhi": bounds[5], "masses": masses, "type_ids": types, "positions": pos, "velocities": vel,
            "table": table, "start_velocities": not bool(hv.value)}


def write_data(path, positions, type_ids, masses, bounds, table=None, velocities=None):
    pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
    n = pos.shape[0]
    t = np.ascontiguousarray(type_ids, dtype=np.int32)
    m = np.ascontiguousarray(masses, dtype=np.float64)
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64).reshape(n, 3)
    table = table or {}
    pairs = (_ffi.LJPair * max(len(table), 1))()
    for k, ((ti, tj), (e, s, rc)) in enumerate(table.items()):
        pairs[k] = _ffi.LJPair(ti, tj, e, s, rc, 1)
    st = _ffi.lib().pis_data_write(path.encode(), n, len(m), t.ctypes.data_as(C.POINTER(C.c_int32)), _dp(m), _dp(pos),
                                   _dp(vel), _dp(b), pairs, len(table))
    if st != 0:
        raise PisError(st, "pis_data_write failed")


def format_f64(v: float) -> str:
    n = _ffi.lib().pis_format_f64(float(v), None, 0)
    buf = C.create_string_buffer(n + 1)
    _ffi.lib().pis_format_f64(float(v), buf, n + 1)
    return buf.value.decode()


def maxwell_boltzmann(masses_per_atom, temperature, seed) -> np.ndarray:
    m = np.ascontiguousarray(masses_per_atom, dtype=np.float64)
    v = np.zeros((m.shape[0], 3))
    st = _ffi.lib().pis_maxwell_boltzmann(m.shape[0], _dp(m), float(temperature), int(seed), _dp(v))
    if st != 0:
        raise PisError(st, "pis_maxwell_boltzmann failed")
    return v


class System:
    """System::new(infile).read().contextualize(); run() = Simulation::run on the GPU manager."""

    def __init__(self, infile, precision="fp64", skin=0.3):
        self._lib = _ffi.lib()
        h = C.c_void_p()
        st = self._lib.pis_system_open(infile.encode(), _ffi.PRECISION[precision], float(skin), C.byref(h))
        self._h = h
        if st != 0:
            msg = self._lib.pis_system_last_error(h).decode() if h else ""
            raise PisError(st, msg)

    @property
    def steps(self):
        return int(self._lib.pis_system_steps(self._h))

    @property
    def timestep(self):
        return float(self._lib.pis_system_timestep(self._h))

    @property
    def ensemble(self):
        return ["NVE", "NVT", "NPT"][self._lib.pis_system_ensemble(self._h)]

    def run(self, thermo_path=None):
        st = self._lib.pis_system_run(self._h, thermo_path.encode() if thermo_path else None)
        if st != 0:
            raise PisError(st, self._lib.pis_system_last_error(self._h).decode())

    def state(self, n):
        pos, vel, frc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        st = self._lib.pis_system_state(self._h, _dp(pos), _dp(vel), _dp(frc))
        if st != 0:
            raise PisError(st, self._lib.pis_system_last_error(self._h).decode())
        return pos, vel, frc

    def pairs(self) -> dict:
        """The LJ table the input built: {(ti, tj): (epsilon, sigma, rcut)}."""
        n = self._lib.pis_system_pairs(self._h, None, 0)
        buf = (_ffi.LJPair * max(n, 1))()
        self._lib.pis_system_pairs(self._h, buf, n)
        return {(buf[k].ti, buf[k].tj): (buf[k].epsilon, buf[k].sigma, buf[k].rcut) for k in range(n)}

    @property
    def dump(self):
        """(dump_step, file name) of the input's dump command."""
        step = C.c_int64()
        name = C.create_string_buffer(4096)
        st = self._lib.pis_system_dump(self._h, C.byref(step), name, 4096)
        if st != 0:
            raise PisError(st, self._lib.pis_system_last_error(self._h).decode())
        return int(step.value), name.value.decode()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pis_system_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
