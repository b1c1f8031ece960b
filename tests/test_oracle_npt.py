"""The oracle's restatement of the reference's NPT ensemble (no GPU): the MTK barostat of
src/ensemble/npt.rs, Atoms::pressure_tensor and scale_box (src/atoms/properties.rs:45-59,
src/atoms/transformations.rs:6-15), PotentialManager::verlet_step_npt_mtk
(src/potentials/potential.rs:115-135) and Simulation::run's NPT branch. The matrix exponential
is the published scaling-and-squaring method, checked against scipy's."""
import numpy as np
import pytest

from systems import liquid, to_oracle

KB = 0.0083144621


@pytest.mark.parametrize("scale", [1e-6, 1e-2, 0.2, 0.9, 2.0, 8.0, 40.0])
def test_matrix_exponential(oracle_lib, scale):
    import oracle
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(int(scale * 1000) + 1)
    for k in range(10):
        a = rng.normal(size=(3, 3))
        a *= scale / np.abs(a).sum(axis=0).max()  # 1-norm = scale: every Pade degree and squarings
        sym = 0.5 * (a + a.T)
        sym *= scale / np.abs(sym).sum(axis=0).max()
        # symmetric (the barostat's case): against the eigen-decomposition
        w, q = np.linalg.eigh(sym)
        exact = (q * np.exp(w)) @ q.T
        assert np.abs(oracle.expm3(sym) - exact).max() <= 1e-13 * np.abs(exact).max()
        if scale <= 2.0:
            # general matrices: against scipy's expm, where both are accurate to rounding
            ref = scipy_linalg.expm(a)
            assert np.abs(oracle.expm3(a) - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    assert np.array_equal(oracle.expm3(np.zeros((3, 3))), np.eye(3))
    d = np.diag([0.1, -0.2, 0.3])
    assert np.allclose(oracle.expm3(d), np.diag(np.exp([0.1, -0.2, 0.3])), rtol=1e-15, atol=0)


def test_barostat_construction(oracle_lib):
    import oracle
    b = oracle.Mtk(0.01, 1000.0, 4000, 5.0)
    assert b.w == (3 * 4000) * KB * 5.0 * (1000.0 * 1000.0)  # npt.rs:31
    assert np.array_equal(b.p_target, 0.01 * np.eye(3)) and not b.momentum.any()
    assert b.kinetic_energy() == 0.0
    h = np.diag([2.0, 3.0, 4.0])
    assert b.potential_energy(h) == 0.01 * 9.0  # tr(P_target^T h)
    assert np.array_equal(b.scale(0.25, True), np.eye(3)) and np.array_equal(b.scale(0.25, False), np.eye(3))


def _state(seed=3):
    s = liquid(nc=5, seed=seed)
    o = to_oracle(s)
    o.compute_potential()
    return s, o


def test_pressure_tensor_and_delta_momentum(oracle_lib):
    import oracle
    s, o = _state()
    V = np.linalg.det(s["h"])
    # the kinetic tensor carries no masses (properties.rs:45-47); masses are 1 here, so give
    # the type a different mass to see it
    p = o.pressure_tensor()
    ref = (o.vel.T @ o.vel + o.pos.T @ o.force) / V
    assert np.allclose(p, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    o.masses[:] = 3.0
    assert np.array_equal(o.pressure_tensor(), p)
    b = oracle.Mtk(1.0, 2.0, o.n, 1.0 / KB)
    d = b.delta_momentum(o, 0.005)
    assert np.array_equal(d, d.T)
    assert np.allclose(d, 0.5 * ((p - np.eye(3)) + (p - np.eye(3)).T) * (V * 0.5 * 0.005), rtol=1e-12, atol=1e-15)


def test_scale_box_keeps_fractional_coordinates(oracle_lib):
    s, o = _state()
    frac = o.pos @ np.linalg.inv(s["h"]).T
    m = np.array([[1.01, 0.002, 0.0], [0.002, 0.99, -0.001], [0.0, -0.001, 1.0]])
    o.scale_box(m)
    assert np.allclose(o.h, m @ s["h"], rtol=0, atol=1e-15 * np.abs(s["h"]).max())
    assert np.allclose(o.hinv @ o.h, np.eye(3), atol=1e-14)
    assert np.allclose(o.pos @ np.linalg.inv(o.h).T, frac, rtol=0, atol=1e-13)


def test_heavy_barostat_leaves_the_nvt_run(oracle_lib):
    # W grows as tau^2: with tau = 1e7 the box and velocity scalings stay within rounding of I
    s, _ = _state(4)
    t = 0.9 / KB
    a = to_oracle(s)
    pe, ke, ham, boxes = a.run_npt(0.005, 30, t, t, 0.5, 0.0, 1e7)
    b = to_oracle(s)
    pe_t, ke_t, _, _ = b.run_nvt(0.005, 30, t, t, 0.5)
    assert np.abs(pe - pe_t).max() <= 1e-9 * np.abs(pe_t).max()
    assert np.abs(ke - ke_t).max() <= 1e-9 * np.abs(ke_t).max()
    assert np.abs(boxes[-1] - s["h"]).max() <= 1e-9 * s["h"][0, 0]


def test_light_barostat_moves_the_box_towards_the_target(oracle_lib):
    # a target pressure above the liquid's compresses it (the box keeps 3 cells per axis at rc);
    # the printed Hamiltonian adds the barostat terms. A lighter barostat or a higher target
    # (tau 0.5 at P* = 10) makes the literal scheme diverge within 60 steps.
    import oracle
    s, _ = _state(5)
    t = 0.9 / KB
    o = to_oracle(s)
    pe, ke, ham, boxes = o.run_npt(0.005, 60, t, t, 0.5, 5.0, 2.0)
    vol = np.array([np.linalg.det(b) for b in boxes])
    assert np.all(np.isfinite(pe)) and np.all(np.isfinite(ham)) and np.all(np.isfinite(boxes))
    assert vol[-1] < vol[0]
    assert np.array_equal(o.h, boxes[-1])
    # the same run step by step through the exposed pieces gives the same numbers
    p = to_oracle(s)
    p.compute_potential()
    nhc = oracle.Nhc(t, t, 0.5)
    mtk = oracle.Mtk(5.0, 2.0, p.n, t)
    for i in range(60):
        e = p.verlet_step_npt_mtk(0.005, mtk, nhc)
        nhc.calculate_target_temperature(i, 60)
        assert e == pe[i + 1]
    k = p.kinetic_energy()
    assert k == ke[-1]
    assert ham[-1] == e + k + nhc.kinetic_energy() + nhc.potential_energy(p.n) + mtk.kinetic_energy() \
        + mtk.potential_energy(p.h)


def test_managers_agree_on_a_sheared_box(oracle_lib):
    # the barostat's symmetric box scaling makes the box triclinic: the oracle's min-image
    # (s = h^-1 r, s -= round(s), r = h s) and fractional-coordinate binning must give every
    # reference manager the all-pairs answer on a mildly sheared box with 4 cells per axis
    import oracle
    s = liquid(nc=6, seed=2)
    L = s["h"][0, 0]
    h = np.array([[L, 0.3, 0.2], [0.0, L, -0.25], [0.0, 0.0, L]])
    rng = np.random.default_rng(1)
    pos = np.mod(s["pos"] / L + rng.normal(0, 0.004, s["pos"].shape), 1.0) @ h.T
    ref = oracle.System(pos, s["types"], s["masses"], h, s["table"])
    pe_ref = ref.compute_potential(manager=oracle.ALLPAIRS)
    for mgr in (oracle.OFFSET, oracle.VERLET27, oracle.FULLLIST, oracle.PARALLEL):
        o = oracle.System(pos, s["types"], s["masses"], h, s["table"])
        assert o.divide_into_cells(2.5) == (4, 4, 4)
        pe = o.compute_potential(manager=mgr, nthreads=2)
        assert abs(pe - pe_ref) <= 1e-13 * abs(pe_ref)
        assert np.linalg.norm(o.force - ref.force) <= 1e-13 * np.linalg.norm(ref.force)
