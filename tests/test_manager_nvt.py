"""The NVT pieces of the reference-shaped Python mirror (no GPU): ``pis_gb300.ensemble.
NHThermostatChain`` against the oracle's restatement of src/ensemble/nvt.rs, bit for bit, and
``LJGpuManager.verlet_step_nvt_nhc``'s sequence of context calls against the oracle's
``verlet_step_nvt_nhc``, with a stand-in context whose calls the oracle answers."""
import numpy as np
import pytest

from pis_gb300.atoms import Atoms, SimulationBox
from pis_gb300.ensemble import NHThermostatChain
from systems import liquid, to_oracle

KB = 0.0083144621


def test_chain_matches_the_oracle_bit_for_bit(oracle_lib):
    import oracle
    rng = np.random.default_rng(2)
    for _ in range(20):
        t0, t1, tau = rng.uniform(1, 500), rng.uniform(1, 500), rng.uniform(0.05, 200)
        n, dt = int(rng.integers(1, 10 ** 6)), rng.uniform(1e-4, 0.5)
        a, b = NHThermostatChain(t0, t1, tau), oracle.Nhc(t0, t1, tau)
        assert a.q == b.q and a.target_temperature == b.t_target
        for step in range(4):
            ke = rng.uniform(0.1, 2.0) * 1.5 * n * KB * t0
            a.compute_forces(ke, n)
            b.compute_forces(ke, n)
            a.propagate_half_step(dt)
            b.propagate_half_step(dt)
            assert a.g == b.g and a.xi == b.xi
            a.calculate_target_temperature(step, 4)
            b.calculate_target_temperature(step, 4)
            assert a.target_temperature == b.t_target
        assert a.kinetic_energy() == b.kinetic_energy()
        assert a.potential_energy(n) == b.potential_energy(n)


class _OracleContext:
    """Answers the GpuContext calls the manager makes from an oracle System."""

    def __init__(self, table, n_types, skin=0.3, precision="fp64", list_kind="default"):
        self.table, self.o = table, None

    def set_state(self, positions, type_ids, masses, h, velocities=None, forces=None):
        import oracle
        self.o = oracle.System(positions, type_ids, masses, h, self.table, velocities=velocities)
        if forces is not None:
            self.o.force[:] = forces

    def compute_potential(self):
        return self.o.compute_potential(), self.o.force.copy()

    def reductions(self):
        return self.o.kinetic_energy(), self.o.virial_tensor()

    def scale_velocities(self, m):
        self.o.vel[:] = self.o.vel @ np.asarray(m).T

    def verlet_step_nve(self, dt, n_steps=1):
        return np.array([self.o.verlet_step_nve(dt) for _ in range(n_steps)])

    def get_state(self):
        return self.o.pos.copy(), self.o.vel.copy(), self.o.force.copy()


def test_manager_nvt_step_follows_the_trait_default(oracle_lib, monkeypatch):
    import oracle
    from pis_gb300 import potentials
    monkeypatch.setattr(potentials, "GpuContext", _OracleContext)
    s = liquid(nc=5, seed=12)
    L = s["h"][0, 0]
    atoms = Atoms(s["pos"], s["types"], s["masses"], SimulationBox.from_lammps_data(0, L, 0, L, 0, L),
                  velocities=s["vel"])
    mgr = potentials.LJGpuManager(s["table"])
    ref = to_oracle(s)
    t = 1.1 / KB
    chain, ref_chain = NHThermostatChain(t, t, 0.5), oracle.Nhc(t, t, 0.5)
    assert mgr.compute_potential(atoms) == ref.compute_potential()
    for i in range(8):
        pe = mgr.verlet_step_nvt_nhc(atoms, 0.005, chain)
        pe_ref = ref.verlet_step_nvt_nhc(0.005, ref_chain)
        chain.calculate_target_temperature(i, 8)
        ref_chain.calculate_target_temperature(i, 8)
        assert pe == pe_ref and chain.xi == ref_chain.xi
    assert np.array_equal(atoms.positions, ref.pos) and np.array_equal(atoms.velocities, ref.vel)
    assert np.array_equal(atoms.forces, ref.force)
