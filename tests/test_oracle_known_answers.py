"""Pins the CPU oracle (test infrastructure) before it is trusted as the checker.

The reference's own tests cover input parsing only, so its FP64 path has no golden vectors;
these known answers are derived from the reference's example inputs and from closed forms:
FCC shell counts, the perfect-lattice energy, Newton's third law, the reference's five
force managers agreeing with each other, and the reference data files read back.
"""
import math

import numpy as np
import pytest

from conftest import reference_file
from systems import argon, liquid, to_oracle


def test_lj_pair_closed_form(oracle_lib):
    import oracle
    eps, sig, rc = 0.238, 3.405, 8.5
    rij = np.array([0.3, -3.1, 1.7])
    u, f = oracle.lj_pair(eps, sig, rc, rij)
    r = np.linalg.norm(rij)
    sr6 = (sig / r) ** 6
    u_exp = 4 * eps * (sr6 * sr6 - sr6) - 4 * eps * ((sig / rc) ** 12 - (sig / rc) ** 6)
    f_exp = 24 * eps * (2 * sr6 * sr6 - sr6) / r ** 2 * rij
    assert u == pytest.approx(u_exp, rel=1e-13)
    assert np.allclose(f, f_exp, rtol=1e-13, atol=0)
    # sign convention: f is along r_j - r_i and repulsive pairs give F_i -= f (push i away)
    u2, f2 = oracle.lj_pair(eps, sig, rc, np.array([3.0, 0, 0]))
    assert f2[0] > 0


def test_inverse_and_minimum_image(oracle_lib):
    import oracle
    h = np.diag([5.0, 7.0, 11.0])
    hinv = oracle.inverse3(h)
    assert np.allclose(hinv @ h, np.eye(3), atol=1e-15)
    s = oracle.System(np.zeros((2, 3)), [1, 1], [1.0], h, {(1, 1): (1.0, 1.0, 2.5)})
    assert np.allclose(s.min_image(np.array([4.5, -6.0, 5.4])), [-0.5, 1.0, 5.4])
    assert np.allclose(s.wrap(np.array([-0.5, 7.5, 22.5])), [4.5, 0.5, 0.5])


def test_data_file_two_atoms(oracle_lib):
    import oracle
    d = oracle.read_data(reference_file("example", "data.txt"))
    assert d["n_atoms"] == 2 and d["table"] == {(1, 1): (0.238, 3.405, 8.5)}
    s = oracle.System.from_data(d)
    # min-image separation 0.5 A along x in the 5 A box (a3 sign and wrap)
    rij = s.min_image(s.pos[1] - s.pos[0])
    assert np.allclose(rij, [-0.5, 0, 0], rtol=0, atol=1e-15)
    pe = s.compute_potential(manager=oracle.ALLPAIRS)
    u, f = oracle.lj_pair(0.238, 3.405, 8.5, rij)
    assert pe == u
    assert np.array_equal(s.force[0], -f) and np.array_equal(s.force[1], f)


def test_data_file_pair_coeffs_quirk(oracle_lib):
    import oracle
    d = oracle.read_data(reference_file("example", "data_run.txt"))
    # "1 2 0.6 1.1 2.8" parses its second token as a float and overwrites (1,1)
    assert d["table"] == {(1, 1): (2.0, 0.6, 1.1), (2, 2): (0.8, 1.2, 3.0)}
    assert list(d["masses"]) == [1.0, 2.0]
    assert list(d["type_ids"]) == [1, 1, 2, 2]
    assert d["start_velocities"]


def test_argon_example_file_matches_lattice_generator(oracle_lib):
    import oracle
    from pis_gb300.lattice import fcc_lattice
    d = oracle.read_data(reference_file("example", "argon4000.txt"))
    assert d["n_atoms"] == 4000
    assert np.allclose(d["positions"], fcc_lattice(5.41, 10, 10, 10), rtol=0, atol=1e-12)
    assert np.allclose(d["positions"], oracle.fcc_lattice(5.41, 10, 10, 10), rtol=0, atol=1e-12)


def test_argon_shells_54_neighbours(oracle_lib):
    s = to_oracle(argon(a=5.41, eps=0.238, rc=8.5))
    off, idx = s.full_list()
    assert np.all(np.diff(off) == 54)


def test_argon_shells_78_at_526(oracle_lib):
    s = to_oracle(argon())
    off, _ = s.full_list()
    assert np.all(np.diff(off) == 78)


def test_perfect_lattice_energy_and_zero_force(oracle_lib):
    import oracle
    from oracle.data_file import lattice_energy_per_atom
    for mgr in (oracle.OFFSET, oracle.FULLLIST):
        s = to_oracle(argon(a=5.41, eps=0.238, rc=8.5))
        pe = s.compute_potential(manager=mgr)
        assert pe / s.n == pytest.approx(lattice_energy_per_atom(5.41, 0.238, 3.405, 8.5), rel=1e-11)
        assert np.abs(s.force).max() < 1e-12


def test_managers_agree_and_newton3(oracle_lib):
    import oracle
    rng = np.random.default_rng(0)
    base = liquid(nc=6)  # 4 cells per axis: every reference manager is exact here
    L = base["h"][0, 0]
    base["pos"] = np.mod(base["pos"] + rng.normal(0, 0.05, base["pos"].shape), L)
    ref = to_oracle(base)
    pe0 = ref.compute_potential(manager=oracle.ALLPAIRS)
    f0 = ref.force.copy()
    assert np.abs(f0.sum(axis=0)).max() < 1e-11
    for mgr in (oracle.OFFSET, oracle.VERLET27, oracle.PARALLEL, oracle.FULLLIST):
        s = to_oracle(base)
        pe = s.compute_potential(manager=mgr, nthreads=4)
        assert pe == pytest.approx(pe0, rel=1e-12)
        assert np.linalg.norm(s.force - f0) / np.linalg.norm(f0) < 1e-12


def test_reference_double_counts_below_three_cells(oracle_lib):
    # With 2 cells per axis the 14-offset stencil visits the same neighbour cell twice
    # (src/potentials/lennard_jones.rs:200-204); the oracle keeps that behaviour.
    import oracle
    base = liquid(nc=4)
    s = to_oracle(base)
    assert s.divide_into_cells(2.5) == (2, 2, 2)
    pe_all = s.compute_potential(manager=oracle.ALLPAIRS)
    pe_off = to_oracle(base).compute_potential(manager=oracle.OFFSET)
    assert abs(pe_off) > 1.5 * abs(pe_all)


def test_reference_bins_outside_atoms_into_cell_zero(oracle_lib):
    # Before the first wrap, a negative coordinate saturates to cell 0 (`f64 as usize`,
    # src/atoms/neighbour_list.rs:21-23), so the cell managers miss some pairs that the
    # all-pairs manager finds; the oracle keeps that behaviour.
    import oracle
    rng = np.random.default_rng(0)
    base = liquid(nc=6)
    base["pos"] = base["pos"] + rng.normal(0, 0.05, base["pos"].shape)
    assert (base["pos"] < 0).any()
    pe_all = to_oracle(base).compute_potential(manager=oracle.ALLPAIRS)
    pe_off = to_oracle(base).compute_potential(manager=oracle.OFFSET)
    assert abs(pe_off - pe_all) > 1e-8 * abs(pe_all)


def test_nve_energy_conservation(oracle_lib):
    s = to_oracle(liquid(nc=6))
    pe, ke = s.run_nve(0.005, 200)
    e = pe + ke
    assert np.abs(e - e[0]).max() / s.n < 5e-3


def test_velocity_generator_drift_and_temperature(oracle_lib):
    from pis_gb300.lattice import maxwell_boltzmann
    m = np.full(4000, 39.948)
    v = maxwell_boltzmann(m, 100.0, seed=7)
    assert np.abs((m[:, None] * v).sum(axis=0)).max() < 1e-10
    ke = float(np.sum(0.5 * m * np.sum(v * v, axis=1)))
    assert 2 * ke / (3 * 4000 * 0.0083144621) == pytest.approx(100.0, rel=1e-12)
    assert np.array_equal(v, maxwell_boltzmann(m, 100.0, seed=7))
    # the oracle's restatement of remove_drift + rescale leaves the generator's output fixed
    s = to_oracle(argon())
    s.vel[:] = v
    s.remove_drift_and_rescale(100.0)
    assert np.allclose(s.vel, v, rtol=1e-12, atol=1e-15)


def test_cells_follow_reference_rule(oracle_lib):
    s = to_oracle(argon())
    assert s.divide_into_cells(s.max_rcut()) == (6, 6, 6)
    assert s.divide_into_cells(s.max_rcut() + 0.3 * 3.405) == (5, 5, 5)
    s = to_oracle(liquid(nc=40))
    assert s.divide_into_cells(2.5) == (26, 26, 26)
    assert s.divide_into_cells(2.8) == (23, 23, 23)
