"""The Rust binding of INTEGRATION.md, driven by the reference trait's default NVT step.

``PotentialManager::verlet_step_nvt_nhc`` (src/potentials/potential.rs:35-58) is a default trait
method: it scales ``atoms.velocities`` on the host, calls ``verlet_step_nve`` (the GPU manager's
override), and scales them again. A binding that uploaded ``Atoms`` only once would step stale
device velocities. ``RustBinding`` below transcribes the binding's C-ABI calls one for one: before a
step it compares the host arrays with the copy the device last returned and uploads them with
``pis_gpu_set_state`` when they differ, then ``pis_gpu_verlet_step_nve(ctx, dt, 1)`` and
``pis_gpu_get_state``. The trait method and Simulation::run's NVT loop (src/simulation.rs:41-64)
are transcribed on the host with the reference's own kinetic energy (a serial sum over the host
arrays, src/atoms/properties.rs:17-24) and checked against the oracle's NVT run.
"""
import ctypes as C
import math

import numpy as np
import pytest

from systems import liquid, melted, to_oracle

pytestmark = pytest.mark.gpu

DT, STEPS, T0, T1, TAU = 0.005, 30, 1.0 / 0.0083144621, 1.2 / 0.0083144621, 0.5


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class RustBinding:
    """LJGpuManager of INTEGRATION.md section 2, call for call."""

    def __init__(self, table, n_types, skin, flags=0, check_host_edits=True):
        from pis_gb300 import _ffi
        self.L = _ffi.lib()
        rows = (_ffi.LJPair * len(table))()
        for k, ((i, j), (e, s, rc)) in enumerate(table.items()):
            rows[k] = _ffi.LJPair(i, j, e, s, rc, 1)
        self.ctx = C.c_void_p()
        assert self.L.pis_gpu_create(rows, len(table), n_types, skin, 0, C.byref(self.ctx)) == 0
        if flags:
            assert self.L.pis_gpu_set_options(self.ctx, 2, flags) == 0
        self.mirror = None  # (positions, velocities) as the device last returned them
        self.check = check_host_edits

    def upload(self, atoms):
        t = np.ascontiguousarray(atoms.type_ids, np.int32)
        hc = np.ascontiguousarray(atoms.sim_box.h.T)
        pbc = (C.c_uint8 * 3)(1, 1, 1)
        st = self.L.pis_gpu_set_state(self.ctx, atoms.n_atoms, t.ctypes.data_as(C.POINTER(C.c_int32)),
                                      _p(atoms.masses), _p(atoms.positions), _p(atoms.velocities),
                                      _p(atoms.forces), _p(hc), pbc)
        assert st == 0

    def sync_in(self, atoms):
        if self.mirror is None or (self.check and not (np.array_equal(self.mirror[0], atoms.positions)
                                                       and np.array_equal(self.mirror[1], atoms.velocities))):
            self.upload(atoms)

    def compute_potential(self, atoms):
        self.upload(atoms)
        pe = C.c_double()
        assert self.L.pis_gpu_compute_potential(self.ctx, C.byref(pe), _p(atoms.forces)) == 0
        self.mirror = (atoms.positions.copy(), atoms.velocities.copy())
        return pe.value

    def verlet_step_nve(self, atoms, dt):
        self.sync_in(atoms)
        pe = C.c_double()
        assert self.L.pis_gpu_verlet_step_nve(self.ctx, dt, 1, C.byref(pe)) == 0
        assert self.L.pis_gpu_get_state(self.ctx, _p(atoms.positions), _p(atoms.velocities), _p(atoms.forces)) == 0
        self.mirror = (atoms.positions.copy(), atoms.velocities.copy())
        return pe.value

    def close(self):
        self.L.pis_gpu_destroy(self.ctx)


def kinetic_energy(atoms):
    """Atoms::kinetic_energy (src/atoms/properties.rs:17-24): serial sum of 0.5 m |v|^2."""
    e = 0.0
    for i in range(atoms.n_atoms):
        v = atoms.velocities[i]
        e += 0.5 * atoms.masses[atoms.type_ids[i] - 1] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return e


def trait_verlet_step_nvt_nhc(mgr, atoms, dt, chain):
    """The trait's default method (src/potentials/potential.rs:35-58), host arithmetic as written."""
    ke = kinetic_energy(atoms)
    chain.compute_forces(ke, atoms.n_atoms)
    chain.propagate_half_step(dt)
    scale = math.exp(-0.5 * dt * chain.xi[0])
    atoms.velocities[:] = atoms.velocities * scale
    pe = mgr.verlet_step_nve(atoms, dt)
    atoms.velocities[:] = atoms.velocities * scale
    ke = kinetic_energy(atoms)
    chain.compute_forces(ke, atoms.n_atoms)
    chain.propagate_half_step(dt)
    return pe


def run_nvt(mgr, atoms):
    """Simulation::run's NVT branch: initial evaluation, then per step the thermostatted step and
    the target ramp."""
    from pis_gb300.ensemble import NHThermostatChain
    chain = NHThermostatChain(T0, T1, TAU)
    pe = [mgr.compute_potential(atoms)]
    ke = [kinetic_energy(atoms)]
    for i in range(STEPS):
        pe.append(trait_verlet_step_nvt_nhc(mgr, atoms, DT, chain))
        chain.calculate_target_temperature(i, STEPS)
        ke.append(kinetic_energy(atoms))
    return np.array(pe), np.array(ke)


@pytest.fixture(scope="module")
def state(oracle_lib, cuda_lib):
    s = melted(liquid(nc=6), steps=100, dt=0.005)
    o = to_oracle(s)
    pe_ref, ke_ref, _, _ = o.run_nvt(DT, STEPS, T0, T1, TAU)
    return s, o, pe_ref, ke_ref


def _atoms(s):
    from pis_gb300.atoms import Atoms, SimulationBox
    return Atoms(s["pos"], s["types"], s["masses"], SimulationBox(s["h"]), velocities=s["vel"])


@pytest.mark.parametrize("ref_order", [False, True])
def test_binding_runs_the_default_nvt_step_like_the_oracle(state, ref_order):
    s, o, pe_ref, ke_ref = state
    atoms = _atoms(s)
    mgr = RustBinding(s["table"], 1, 0.3, flags=64 if ref_order else 0)
    pe, ke = run_nvt(mgr, atoms)
    mgr.close()
    if ref_order:
        # forces in the reference's order: the whole thermostatted trajectory is the oracle's
        assert np.array_equal(atoms.positions, o.pos) and np.array_equal(atoms.velocities, o.vel)
        assert np.array_equal(ke, ke_ref)
    else:
        assert np.abs(atoms.positions - o.pos).max() <= 1e-9
        assert np.max(np.abs(ke - ke_ref) / ke_ref) <= 1e-12
    # energies: the GPU's exact sum against the oracle's walk-order sum of the same terms
    assert np.max(np.abs(pe - pe_ref) / np.abs(pe_ref)) <= 1e-11
    # the thermostat did act: the run is not an NVE run
    assert abs(ke[-1] - ke[0]) > 1e-3 * ke[0]


def test_binding_without_the_host_edit_check_loses_the_scaling(state):
    # the binding as first written (upload once): the first scaling is never uploaded, so the
    # trajectory leaves the oracle's at once
    s, o, pe_ref, ke_ref = state
    atoms = _atoms(s)
    mgr = RustBinding(s["table"], 1, 0.3, check_host_edits=False)
    pe, ke = run_nvt(mgr, atoms)
    mgr.close()
    assert np.abs(atoms.velocities - o.vel).max() > 1e-6
