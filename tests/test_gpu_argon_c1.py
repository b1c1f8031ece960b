"""The repo's argon case end to end: 4000 Ar on a 10^3 FCC lattice (a = 5.26 A), LJ eps = 0.0104,
sigma = 3.405, rc = 2.5 sigma, skin 0.3 sigma, Maxwell-Boltzmann velocities at 100 K (seeded, zero
net momentum), velocity-Verlet NVE with dt = 0.001 - the plain FP64 GPU path against the oracle's
restatement of the reference's serial manager on the same inputs.

Energies are compared as exact sums (the FP64 path's reductions and the oracle's
compute_potential_exact / run_nve_exact): the reference's own walk-order sum of the same pair terms
deviates from the exact sum by up to ~2e-12 relative here, a rounding of the reference itself.

* Default FP64 path (half list, FP64 atomics), 1000 steps against a live oracle run: neighbour sets
  identical, energy within 1e-12 of the oracle's at every step, positions within 1e-9 sigma.
* Reference-order FP64 path (PIS_OPT_REF_ORDER), 10^4 steps against the oracle's run stored in
  tests/golden/argon4000_nve1e4.npz: positions, velocities and every step's energy bit-identical,
  so its energy drift equals the reference arithmetic's exactly.
"""
import hashlib
import os

import numpy as np
import pytest

from systems import argon, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

SIGMA = 3.405
SKIN = 0.3 * SIGMA
STEPS = 1000
LONG = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "argon4000_nve1e4.npz")


def _sets(off, idx):
    return [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).digest(), np.uint8)


def _drift(e, every, dt):
    """Energy drift: slope of a linear fit of E(t), per 10^4 steps."""
    t = np.arange(len(e)) * every
    return float(np.polyfit(t, e, 1)[0] * 1e4)


@pytest.fixture(scope="module")
def c1_runs(oracle_lib, cuda_lib):
    s = argon()
    o = to_oracle(s)
    off0, idx0 = o.full_list()
    pe_ref, ke_ref, pe_walk = o.run_nve_exact(0.001, STEPS)
    g = to_gpu(s, "fp64", skin=SKIN)
    nl0 = g.neighbour_list()
    pe0, _ = g.compute_potential(want_forces=False)
    ke0, _ = g.reductions()
    pe = g.verlet_step_nve(0.001, STEPS)
    ke, w = g.reductions()
    pos, vel, frc = g.get_state()
    return dict(s=s, o=o, off0=off0, idx0=idx0, pe_ref=pe_ref, ke_ref=ke_ref, pe_walk=pe_walk, g=g, nl0=nl0,
                pe0=pe0, ke0=ke0, pe=pe, ke=ke, w=w, pos=pos, vel=vel, frc=frc)


def test_c1_neighbour_sets_at_start_and_end(c1_runs):
    r = c1_runs
    assert _sets(*r["nl0"]) == [tuple(sorted(x)) for x in _sets(r["off0"], r["idx0"])]
    assert all(len(x) == 78 for x in _sets(r["off0"], r["idx0"]))  # perfect a = 5.26 lattice at rc
    off, idx = r["o"].full_list()
    assert _sets(*r["g"].neighbour_list()) == [tuple(sorted(x)) for x in _sets(off, idx)]


def test_c1_trajectory_and_energies(c1_runs):
    r = c1_runs
    # step 0: the same pair terms, so the same exact sum
    assert r["pe0"] == r["pe_ref"][0]
    assert r["ke0"] == r["ke_ref"][0]
    # every step and the end state: the FP64 bar of 1e-12 (the trajectories differ only by the
    # order of the per-atom force sums)
    assert np.max(np.abs(r["pe"] - r["pe_ref"][1:]) / np.abs(r["pe_ref"][1:])) <= 1e-12
    assert abs(r["ke"] - r["ke_ref"][-1]) <= 1e-12 * r["ke_ref"][-1]
    assert np.abs(r["pos"] - r["o"].pos).max() <= 1e-9 * SIGMA
    # the reference's printed (walk-order) energy is within its own rounding of the exact one
    assert np.max(np.abs(r["pe_walk"] - r["pe_ref"]) / np.abs(r["pe_ref"])) <= 1e-11


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
    pe_exact, pe_walk = o2.compute_potential_exact()
    assert pe == pe_exact
    assert abs(pe - pe_walk) <= 1e-11 * abs(pe_walk)
    assert np.linalg.norm(f - o2.force) <= 1e-12 * np.linalg.norm(o2.force)
    scale = np.abs(o2.pos).max() * np.abs(o2.force).sum()
    assert np.abs(w - o2.virial_tensor_exact()).max() <= 1e-12 * scale
    assert ke == o2.kinetic_energy_exact()


@pytest.fixture(scope="module")
def c1_long(cuda_lib):
    if not os.path.exists(LONG):
        pytest.skip("argon4000_nve1e4.npz not written (tests/golden/make_c1_long.py)")
    fx = np.load(LONG)
    s = argon()
    s["vel"] = fx["vel0"].copy()
    steps, every, dt = int(fx["steps"]), int(fx["every"]), float(fx["dt"])
    g = to_gpu(s, "fp64", skin=SKIN, ref_order=True)
    pe0, _ = g.compute_potential(want_forces=False)
    ke0, _ = g.reductions()
    pe = [np.array([pe0])]
    ke = [ke0]
    for _ in range(steps // every):
        pe.append(g.verlet_step_nve(dt, every))
        ke.append(g.reductions()[0])
    pos, vel, _ = g.get_state()
    return dict(fx=fx, pe=np.concatenate(pe), ke=np.array(ke), pos=pos, vel=vel, every=every, dt=dt)


def test_c1_ref_order_1e4_steps_bit_identical(c1_long):
    r = c1_long
    fx = r["fx"]
    assert np.array_equal(r["pe"][::r["every"]], fx["pe"])
    assert np.array_equal(r["ke"], fx["ke"])
    assert np.array_equal(_sha(r["pe"]), fx["sha_pe"])
    assert np.array_equal(_sha(r["pos"]), fx["sha_pos"])
    assert np.array_equal(_sha(r["vel"]), fx["sha_vel"])
    # against the reference's printed walk-order energies
    assert np.max(np.abs(r["pe"][::r["every"]] - fx["pe_walk"]) / np.abs(fx["pe_walk"])) <= 1e-11


def test_c1_energy_drift_equals_reference_arithmetic(c1_long):
    # identical states give identical energies: the GPU's drift over 10^4 steps is the reference
    # arithmetic's, so it is no worse (no slack)
    r = c1_long
    fx = r["fx"]
    e_gpu = r["pe"][::r["every"]] + r["ke"]
    e_ref = fx["pe"] + fx["ke"]
    d_gpu, d_ref = _drift(e_gpu, r["every"], r["dt"]), _drift(e_ref, r["every"], r["dt"])
    assert abs(d_gpu) <= abs(d_ref)
    assert np.abs(e_gpu - e_gpu[0]).max() <= np.abs(e_ref - e_ref[0]).max()
