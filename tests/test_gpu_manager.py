"""``LJGpuManager`` (the would-be ``PotentialManagerKind::LJGpu`` variant) driven the way the
reference's ``Simulation::run`` drives a ``PotentialManager``: one ``compute_potential`` before
step 1, then ``verlet_step_nve`` once per step on the ``Atoms`` it mutates
(src/simulation.rs:8-39, src/potentials/potential.rs:15-33), against the oracle stepping the same
state. Host edits marked with ``Atoms.touch()`` reach the device before the next call."""
import numpy as np
import pytest

from pis_gb300.atoms import Atoms, SimulationBox
from systems import liquid, to_oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _min_image_max(a, b, L):
    d = a - b
    d -= L * np.round(d / L)
    return float(np.abs(d).max())


def test_manager_steps_like_the_reference(oracle_lib, cuda_lib):
    from pis_gb300.potentials import LJGpuManager
    s = liquid(nc=6, seed=23)
    rng = np.random.default_rng(23)
    L = s["h"][0, 0]
    s["pos"] = np.mod(s["pos"] + rng.normal(0, 0.03, s["pos"].shape), L)
    box = SimulationBox.from_lammps_data(0.0, L, 0.0, L, 0.0, L)
    atoms = Atoms(s["pos"], s["types"], s["masses"], box, velocities=s["vel"])
    mgr = LJGpuManager(s["table"], skin=0.3)
    o = to_oracle(s)

    pe = mgr.compute_potential(atoms)
    pe_ref = o.compute_potential()
    assert abs(pe - pe_ref) <= FP64_TOL * abs(pe_ref)
    assert rel_norm(atoms.forces, o.force) <= FP64_TOL

    for _ in range(10):
        pe = mgr.verlet_step_nve(atoms, 0.005)
        pe_ref = o.verlet_step_nve(0.005)
        assert abs(pe - pe_ref) <= 1e-11 * abs(pe_ref)
    assert _min_image_max(atoms.positions, o.pos, L) <= 1e-9
    assert rel_norm(atoms.velocities, o.vel) <= 1e-10
    assert rel_norm(atoms.forces, o.force) <= 1e-10
    ke = atoms.kinetic_energy()
    assert ke == pytest.approx(o.kinetic_energy(), rel=1e-10)

    # an edit on the host, marked with touch(), is uploaded before the next call
    atoms.velocities *= 0.5
    atoms.touch()
    o.vel *= 0.5
    pe = mgr.run_nve(atoms, 0.005, 20)
    pe_ref, _ = o.run_nve(0.005, 20)
    assert np.max(np.abs(pe - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-11
    assert _min_image_max(atoms.positions, o.pos, L) <= 1e-9
    assert rel_norm(atoms.velocities, o.vel) <= 1e-10
    mgr.ctx.close()
