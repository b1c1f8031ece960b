"""The repo's argon case end to end: 4000 Ar on a 10^3 FCC lattice (a = 5.26 A), LJ eps = 0.0104,
sigma = 3.405, rc = 2.5 sigma, skin 0.3 sigma, Maxwell-Boltzmann velocities at 100 K (seeded, zero
net momentum), velocity-Verlet NVE with dt = 0.001 for 1000 steps - the plain FP64 GPU path against
the oracle's restatement of the reference's serial manager on the same inputs."""
import numpy as np
import pytest

from systems import argon, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

SIGMA = 3.405
SKIN = 0.3 * SIGMA
STEPS = 1000


def _sets(off, idx):
    return [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


@pytest.fixture(scope="module")
def c1_runs(oracle_lib, cuda_lib):
    s = argon()
    o = to_oracle(s)
    off0, idx0 = o.full_list()
    pe_ref, ke_ref = o.run_nve(0.001, STEPS)
    g = to_gpu(s, "fp64", skin=SKIN)
    nl0 = g.neighbour_list()
    pe0, _ = g.compute_potential(want_forces=False)
    ke0, _ = g.reductions()
    pe = g.verlet_step_nve(0.001, STEPS)
    ke, w = g.reductions()
    pos, vel, frc = g.get_state()
    return dict(s=s, o=o, off0=off0, idx0=idx0, pe_ref=pe_ref, ke_ref=ke_ref, g=g, nl0=nl0, pe0=pe0, ke0=ke0,
                pe=pe, ke=ke, w=w, pos=pos, vel=vel, frc=frc)


def test_c1_neighbour_sets_at_start_and_end(c1_runs):
    r = c1_runs
    assert _sets(*r["nl0"]) == [tuple(sorted(x)) for x in _sets(r["off0"], r["idx0"])]
    assert all(len(x) == 78 for x in _sets(r["off0"], r["idx0"]))  # perfect a = 5.26 lattice at rc
    off, idx = r["o"].full_list()
    assert _sets(*r["g"].neighbour_list()) == [tuple(sorted(x)) for x in _sets(off, idx)]


def test_c1_trajectory_and_energies(c1_runs):
    r = c1_runs
    # PE is a sum of ~1.6e5 pair terms of both signs: summation order alone moves it by ~1e-12 relative
    assert abs(r["pe0"] - r["pe_ref"][0]) <= 1e-11 * abs(r["pe_ref"][0])
    assert np.max(np.abs(r["pe"] - r["pe_ref"][1:]) / np.abs(r["pe_ref"][1:])) <= 1e-11
    assert abs(r["ke"] - r["ke_ref"][-1]) <= 1e-11 * r["ke_ref"][-1]
    assert np.abs(r["pos"] - r["o"].pos).max() <= 1e-9 * SIGMA


def test_c1_forces_pe_virial_at_end_state(c1_runs):
    # forces, PE and virial of the GPU path on exactly the oracle's end state
    r = c1_runs
    o = r["o"]
    s = dict(r["s"])
    s["pos"], s["vel"] = o.pos.copy(), o.vel.copy()
    g = to_gpu(s, "fp64", skin=SKIN)
    pe, f = g.compute_potential()
    ke, w = g.reductions()
    o2 = to_oracle(s)
    pe_ref = o2.compute_potential()
    assert abs(pe - pe_ref) <= 1e-11 * abs(pe_ref)
    assert np.linalg.norm(f - o2.force) <= 1e-12 * np.linalg.norm(o2.force)
    scale = np.abs(o2.pos).max() * np.abs(o2.force).sum()
    assert np.abs(w - o2.virial_tensor()).max() <= 1e-12 * scale
    assert abs(ke - o2.kinetic_energy()) <= 1e-12 * ke


def test_c1_energy_drift_no_worse_than_reference_arithmetic(c1_runs):
    r = c1_runs
    e_ref = r["pe_ref"] + r["ke_ref"]
    ref_dev = np.abs(e_ref - e_ref[0]).max()
    gpu_e_end = r["pe"][-1] + r["ke"]
    gpu_dev = abs(gpu_e_end - (r["pe0"] + r["ke0"]))
    assert gpu_dev <= 1.5 * ref_dev + 1e-12 * abs(e_ref[0])
