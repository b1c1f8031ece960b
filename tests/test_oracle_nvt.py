"""The oracle's restatement of the reference's NVT ensemble (no GPU): the Nose-Hoover chain of
src/ensemble/nvt.rs, PotentialManager::verlet_step_nvt_nhc (src/potentials/potential.rs:35-58)
and Simulation::run's NVT branch (src/simulation.rs:8-115)."""
import math

import numpy as np
import pytest

from systems import liquid, to_oracle

KB = 0.0083144621


class _Chain:
    """nvt.rs written out once more in Python, operation by operation, as an independent
    transcription of the same source."""

    def __init__(self, t0, t1, tau):
        self.t_start, self.t_end, self.t_target = t0, t1, t0
        q_value = KB * t0 * (tau * tau)
        self.q = [q_value / 1.0, q_value / 10.0, q_value / 100.0]
        self.xi, self.eta, self.g = [0.0] * 3, [0.0] * 3, [0.0] * 3

    def compute_forces(self, ke, n):
        self.g[0] = 2.0 * ke - float(n * 3) * KB * self.t_target
        for j in (1, 2):
            self.g[j] = self.q[j - 1] * (self.xi[j - 1] * self.xi[j - 1]) - KB * self.t_target

    def propagate_half_step(self, dt):
        self.xi[2] = 0.5 * dt * self.g[2] / self.q[2]
        for l in (1, 0):
            self.xi[l] = (0.5 * dt * self.g[l] / self.q[l]) * math.exp(-0.25 * dt * self.xi[l + 1])


def test_chain_arithmetic_bit_for_bit(oracle_lib):
    import oracle
    rng = np.random.default_rng(1)
    for _ in range(20):
        t0, t1, tau = rng.uniform(1, 500), rng.uniform(1, 500), rng.uniform(0.05, 200)
        n, dt = int(rng.integers(1, 10 ** 6)), rng.uniform(1e-4, 0.5)
        a, b = oracle.Nhc(t0, t1, tau), _Chain(t0, t1, tau)
        assert a.q == b.q and a.t_target == t0
        for _ in range(4):
            ke = rng.uniform(0.1, 2.0) * 1.5 * n * KB * t0
            a.compute_forces(ke, n)
            b.compute_forces(ke, n)
            a.propagate_half_step(dt)
            b.propagate_half_step(dt)
            assert a.g == b.g and a.xi == b.xi
        ke_b = 0.0  # accumulated in order (Python's sum() compensates since 3.12)
        for q, x in zip(b.q, b.xi):
            ke_b += 0.5 * q * (x * x)
        assert a.kinetic_energy() == ke_b
        assert a.potential_energy(n) == 0.0 and a.eta == [0.0, 0.0, 0.0]  # eta is never advanced


def test_target_temperature_ramp(oracle_lib):
    import oracle
    c = oracle.Nhc(100.0, 300.0, 1.0)
    for step, steps in ((0, 10), (3, 10), (9, 10), (7, 7)):
        c.calculate_target_temperature(step, steps)
        assert c.t_target == 100.0 + ((300.0 - 100.0) / steps) * step


def test_nvt_step_is_the_nve_step_between_two_scalings(oracle_lib):
    import oracle
    s = liquid(nc=4, seed=5)
    a, b = to_oracle(s), to_oracle(s)
    a.compute_potential()
    b.compute_potential()
    t = 1.0 / KB
    c, ref = oracle.Nhc(t, t, 0.5), _Chain(t, t, 0.5)
    for _ in range(5):
        pe = a.verlet_step_nvt_nhc(0.005, c)
        ref.compute_forces(b.kinetic_energy(), b.n)
        ref.propagate_half_step(0.005)
        scale = math.exp(-0.5 * 0.005 * ref.xi[0])
        b.vel[:] = b.vel * scale
        pe_b = b.verlet_step_nve(0.005)
        b.vel[:] = b.vel * scale
        ref.compute_forces(b.kinetic_energy(), b.n)
        ref.propagate_half_step(0.005)
        assert pe == pe_b and c.xi == ref.xi
        assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)


def test_run_nvt_outputs_and_weak_coupling_limit(oracle_lib):
    s = liquid(nc=5, seed=6)
    t = 0.9 / KB
    o = to_oracle(s)
    pe, ke, ham, c = o.run_nvt(0.005, 40, t, 2 * t, 1e6)
    # the printed Hamiltonian and the ramp after the last step (calculate_target_temperature(39, 40))
    assert ham[-1] == pe[-1] + ke[-1] + c.kinetic_energy() + c.potential_energy(o.n)
    assert c.t_target == t + ((2 * t - t) / 40) * 39
    # a very heavy thermostat (tau = 1e6) leaves the NVE trajectory all but unchanged
    r = to_oracle(s)
    pe_nve, ke_nve = r.run_nve(0.005, 40)
    assert np.abs(pe - pe_nve).max() <= 1e-9 * np.abs(pe_nve).max()
    assert np.abs(o.pos - r.pos).max() <= 1e-9
    assert pe[0] == pe_nve[0] and ke[0] == ke_nve[0]


def test_literal_chain_is_reproduced_not_corrected(oracle_lib):
    # propagate_half_step assigns xi from the current forces instead of integrating it, so a
    # light thermostat (tau = 0.1 in reduced units) over-damps the velocities; the restatement
    # keeps that behaviour rather than a textbook Nose-Hoover chain
    s = liquid(nc=5, seed=7)
    t = 1.2 / KB
    pe, ke, ham, c = to_oracle(s).run_nvt(0.005, 20, t, t, 0.1)
    temps = 2 * ke / (3 * len(s["pos"]) * KB)
    assert np.all(np.isfinite(pe)) and np.all(np.isfinite(ham))
    assert temps[1:].min() < 1e-3 * temps[0]


@pytest.mark.parametrize("manager", [0, 4])
def test_nvt_with_either_reference_manager(oracle_lib, manager):
    s = liquid(nc=5, seed=8)
    t = 0.8 / KB
    a = to_oracle(s).run_nvt(0.005, 10, t, t, 5.0, manager=0)
    b = to_oracle(s).run_nvt(0.005, 10, t, t, 5.0, manager=manager)
    assert np.allclose(a[0], b[0], rtol=1e-12, atol=0) and np.allclose(a[1], b[1], rtol=1e-12, atol=0)
