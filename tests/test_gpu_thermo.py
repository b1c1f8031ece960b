"""Thermo of every step kept on the device (pis_gpu_verlet_step_nve_thermo): the potential energy,
kinetic energy and virial trace of each step, read back once per run, against the same run stepped
one step at a time with the device reductions after each step, and against the oracle.
Simulation::output prints PE, KE, H, T and P after every step (src/simulation.rs:66-88); the
pressure needs KE and the virial trace (src/atoms/properties.rs:61-65)."""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

STEPS = 60


@pytest.fixture(scope="module")
def state(oracle_lib, cuda_lib):
    return melted(liquid(nc=6, seed=9), steps=100, dt=0.005)


@pytest.mark.parametrize("kw", [dict(precision="fp64"), dict(precision="mixed"),
                                dict(precision="mixed", unfused=True), dict(precision="fp64", ref_order=True)])
def test_thermo_rings_equal_step_by_step_reductions(state, kw):
    a = to_gpu(state, **kw)
    b = to_gpu(state, **kw)
    a.compute_potential(want_forces=False)
    b.compute_potential(want_forces=False)
    pe, ke, tr = a.verlet_step_nve_thermo(0.005, STEPS)
    pe1, ke1, tr1 = [], [], []
    for _ in range(STEPS):
        pe1.append(b.verlet_step_nve(0.005, 1)[0])
        k, w = b.reductions()
        ke1.append(k)
        tr1.append(np.trace(w))
    pe1, ke1, tr1 = map(np.array, (pe1, ke1, tr1))
    pos, _, frc = b.get_state()
    scale = np.abs(pos).max() * np.abs(frc).sum()
    pa, va, _ = a.get_state()
    pb, vb, _ = b.get_state()
    if kw.get("precision") == "fp64" and not kw.get("ref_order"):
        # the default FP64 list is a half list whose forces on j are added with atomics, so two
        # contexts differ in the last bits of the forces and hence of the trajectory
        assert np.max(np.abs(pe - pe1) / np.abs(pe1)) <= 1e-12
        assert np.max(np.abs(ke - ke1) / ke1) <= 1e-12
        assert np.abs(pa - pb).max() <= 1e-9
    else:
        assert np.array_equal(pe, pe1)
        assert np.array_equal(ke, ke1)  # the step's own sum is the reduction's
        # the two contexts' end states are the same run
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    # trace: one sum over r_i . F_i against three sums of r_i[a] F_i[a], compared to the scale of its terms
    assert np.abs(tr - tr1).max() <= 1e-12 * scale


def test_thermo_against_oracle_reference_order(state):
    # reference-order FP64: every step's PE and KE equal the oracle's exact sums; the pressure's
    # trace matches the oracle's virial at the FP64 bar
    o = to_oracle(state)
    pe_ref, ke_ref, _ = o.run_nve_exact(0.005, STEPS)
    g = to_gpu(state, "fp64", ref_order=True)
    g.compute_potential(want_forces=False)
    pe, ke, tr = g.verlet_step_nve_thermo(0.005, STEPS)
    assert np.array_equal(pe, pe_ref[1:]) and np.array_equal(ke, ke_ref[1:])
    w = o.virial_tensor_exact()
    scale = np.abs(o.pos).max() * np.abs(o.force).sum()
    assert abs(tr[-1] - np.trace(w)) <= 1e-12 * scale
