"""The host-side mirrors of the reference's ``Atoms`` and ``SimulationBox`` (pis_gb300/atoms.py)
against the oracle's restatement of the same functions (no GPU)."""
import numpy as np
import pytest

from pis_gb300.atoms import KB_KJPERMOLEKELVIN, Atoms, SimulationBox, inverse3
from systems import liquid, to_oracle


def test_boltzmann_constant():
    # src/constants.rs:3
    assert KB_KJPERMOLEKELVIN == 0.0083144621


@pytest.mark.parametrize("h", [np.diag([5.0, 7.0, 11.0]), np.diag([67.184, 67.184, 67.184]),
                               np.array([[4.0, 0.5, 0.25], [0.0, 3.0, -0.75], [0.0, 0.0, 6.0]])])
def test_inverse_matches_oracle_bits(oracle_lib, h):
    import oracle
    assert np.array_equal(inverse3(h), oracle.inverse3(h))


def test_box_from_lammps_data_and_volume():
    # SimulationBox::from_lammps_data (src/simulation_box.rs:44-65): columns (ax,0,0), (xy,ay,0), (xz,yz,az)
    b = SimulationBox.from_lammps_data(-1.0, 4.0, 0.0, 3.0, 2.0, 8.0, xy=0.5, xz=0.25, yz=-0.75)
    assert np.array_equal(b.h, [[5.0, 0.5, 0.25], [0.0, 3.0, -0.75], [0.0, 0.0, 6.0]])
    assert b.pbc == (True, True, True)
    assert b.volume() == 90.0
    assert np.allclose(b.h_inv @ b.h, np.eye(3), rtol=0, atol=1e-15)


def _atoms_and_oracle(oracle_lib, two_types=False):
    s = liquid(nc=4, seed=11)
    if two_types:
        s["types"] = (np.arange(len(s["pos"])) % 2 + 1).astype(np.int32)
        s["masses"] = np.array([1.0, 3.0])
        s["table"] = {(1, 1): (1.0, 1.0, 2.5), (2, 2): (1.0, 1.0, 2.5), (1, 2): (1.0, 1.0, 2.5)}
    o = to_oracle(s)
    o.compute_potential()
    box = SimulationBox.from_lammps_data(0.0, s["h"][0, 0], 0.0, s["h"][1, 1], 0.0, s["h"][2, 2])
    a = Atoms(s["pos"], s["types"], s["masses"], box, velocities=s["vel"], forces=o.force)
    return a, o


@pytest.mark.parametrize("two_types", [False, True])
def test_reductions_match_oracle(oracle_lib, two_types):
    # KE, T, virial sum_i r_i F_i^T and P (src/atoms/properties.rs:9-65); numpy sums in another
    # order, so agreement is to rounding
    a, o = _atoms_and_oracle(oracle_lib, two_types)
    ke = a.kinetic_energy()
    assert ke == pytest.approx(o.kinetic_energy(), rel=1e-13)
    assert a.temperature(ke) == pytest.approx(o.temperature(ke), rel=1e-15)
    w = a.virial_tensor()
    scale = np.abs(a.positions).max() * np.abs(a.forces).sum()
    assert np.abs(w - o.virial_tensor()).max() <= 1e-13 * scale
    assert a.pressure(ke) == pytest.approx(o.pressure(ke), rel=1e-12, abs=1e-12 * scale / a.sim_box.volume())
    # a_i = F_i / masses[type_i - 1] with 1-based types (properties.rs:9-13, 32-39)
    assert [a.mass_i(i) for i in range(4)] == [float(a.masses[t - 1]) for t in a.type_ids[:4]]
    assert np.array_equal(a.per_atom_mass(), a.masses[a.type_ids - 1])


def test_atoms_copies_inputs_and_counts_versions():
    pos = np.zeros((2, 3))
    a = Atoms(pos, [1, 1], [1.0], SimulationBox(np.eye(3) * 4.0))
    pos[0, 0] = 1.0
    assert a.positions[0, 0] == 0.0  # the container owns its arrays
    assert not a.velocities.any() and not a.forces.any()
    v0 = a.version
    assert a.touch() == v0 + 1 and a.version == v0 + 1
