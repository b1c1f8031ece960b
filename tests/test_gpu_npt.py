"""General (triclinic) boxes on the FP64 path and the NPT (MTK) ensemble on the GPU.

The reference's barostat scales the box by the exponential of a symmetric 3x3 matrix
(src/ensemble/npt.rs:49-56, src/atoms/transformations.rs:6-15), so after one NPT step the box has
off-diagonal elements. The FP64 path bins atoms in fractional coordinates, sizes cells by the box
widths across faces, and takes minimum images and wraps with the reference's full 3x3 arithmetic
(src/simulation_box.rs:17-42). Checked against the oracle: forces, energy and a trajectory on a
sheared box (bit for bit in the reference's order), a symmetric box scaling, the pressure tensor,
and the input driver's NPT thermo against the oracle's NPT run at the printed resolution.
"""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

KB = 0.0083144621


def sheared(s, xy=0.07, xz=-0.04, yz=0.05):
    """The state in a box whose vectors are tilted: h = [[L, xy L, xz L], [0, L, yz L], [0, 0, L]]
    (columns are box vectors, as the reference's from_lammps_data builds them); positions are
    carried in fractional coordinates."""
    out = dict(s)
    L = s["h"][0, 0]
    h = np.array([[L, xy * L, xz * L], [0.0, L, yz * L], [0.0, 0.0, L]])
    out["pos"] = (s["pos"] / L) @ h.T
    out["h"] = h
    return out


@pytest.fixture(scope="module")
def state(oracle_lib, cuda_lib):
    return sheared(melted(liquid(nc=6), steps=100, dt=0.005))


@pytest.mark.parametrize("kw", [dict(list_kind="half"), dict(list_kind="full"), dict(ref_order=True)])
def test_sheared_box_forces_energy_virial(state, kw):
    o = to_oracle(state)
    pe_exact, _ = o.compute_potential_exact()
    g = to_gpu(state, "fp64", **kw)
    pe, f = g.compute_potential()
    ke, w = g.reductions()
    assert pe == pe_exact
    if kw.get("ref_order"):
        assert np.array_equal(f, o.force)
    else:
        assert np.linalg.norm(f - o.force) <= 1e-12 * np.linalg.norm(o.force)
    scale = np.abs(o.pos).max() * np.abs(o.force).sum()
    assert np.abs(w - o.virial_tensor_exact()).max() <= 1e-12 * scale
    # the same neighbour sets as the reference's full list
    off_r, idx_r = o.full_list()
    off, idx = g.neighbour_list()
    assert [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)] == \
           [tuple(sorted(idx_r[off_r[i]:off_r[i + 1]])) for i in range(len(off_r) - 1)]


def test_sheared_box_trajectory_bit_identical(state):
    o = to_oracle(state)
    pe_ref, ke_ref, _ = o.run_nve_exact(0.005, 100)
    g = to_gpu(state, "fp64", ref_order=True)
    pe0, _ = g.compute_potential(want_forces=False)
    pe = g.verlet_step_nve(0.005, 100)
    pos, vel, _ = g.get_state()
    assert pe0 == pe_ref[0] and np.array_equal(pe, pe_ref[1:])
    assert np.array_equal(pos, o.pos) and np.array_equal(vel, o.vel)


def test_sheared_slot_in_a_replica_pool(state):
    # a sheared slot beside a cubic one in an FP64 replica pool, whose rebuild kernels stride over
    # the listed chunks and cells with the triclinic instantiations: each slot's 40 steps match
    # the oracle's run (energies at the FP64 bar, positions within 1e-9 sigma)
    from pis_gb300.batch import Batch
    cubic = melted(liquid(nc=6, seed=31), steps=50, dt=0.005)
    systems = (state, cubic)
    b = Batch(4000, 3, 0, precision="fp64")
    slots = [b.admit(s["pos"], s["types"], s["masses"], s["h"], s["table"], 40, velocities=s["vel"]) for s in systems]
    b.advance(40)
    for s, slot in zip(systems, slots):
        o = to_oracle(s)
        pe_ref, _, _ = o.run_nve_exact(0.005, 40)
        hist = b.pe_history(slot, 40)
        assert np.max(np.abs(hist - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-11
        r = b.result(slot, len(s["pos"]))
        f = (r["pos"] - o.pos) @ np.linalg.inv(s["h"]).T  # fractional difference, minimum image
        f -= np.round(f)
        assert np.abs(f @ s["h"].T).max() <= 1e-9
    b.close()


def test_symmetric_box_scaling(state):
    # Atoms::scale_box with a symmetric matrix (the barostat's form): box, positions and the
    # next evaluation against the oracle
    m = np.array([[1.002, 0.0007, -0.0003], [0.0007, 0.998, 0.0011], [-0.0003, 0.0011, 1.001]])
    o = to_oracle(state)
    o.compute_potential()
    g = to_gpu(state, "fp64")
    g.compute_potential()
    o.scale_box(m)
    g.scale_box(m)
    assert np.abs(g.box() - o.h).max() <= 1e-15 * np.abs(o.h).max()
    pos, _, _ = g.get_state()
    assert np.abs(pos - o.pos).max() <= 1e-13 * np.abs(o.pos).max()
    s2 = dict(state)
    s2["pos"], s2["h"] = o.pos.copy(), o.h.copy()
    o2 = to_oracle(s2)
    pe_exact, _ = o2.compute_potential_exact()
    pe, f = g.compute_potential()
    assert abs(pe - pe_exact) <= 1e-12 * abs(pe_exact)
    assert np.linalg.norm(f - o2.force) <= 1e-11 * np.linalg.norm(o2.force)


def test_pressure_tensor(state):
    o = to_oracle(state)
    o.compute_potential()
    g = to_gpu(state, "fp64", ref_order=True)
    g.compute_potential()
    p = g.pressure_tensor()
    p_ref = o.pressure_tensor()
    assert np.abs(p - p_ref).max() <= 1e-12 * np.abs(p_ref).max()


def test_triclinic_needs_the_exact_fp64_path(state):
    from pis_gb300._ffi import PisError
    for kw in (dict(precision="mixed"), dict(precision="fp64", fp64_fast=True), dict(precision="fp64", lanes=8)):
        with pytest.raises(PisError) as e:
            to_gpu(state, **kw)
        assert e.value.name == "PIS_ERR_UNSUPPORTED"


def _parse_thermo(path):
    lines = open(path).read().split("\n")
    first = lines[0].split()
    rows = [list(map(float, l.split())) for l in lines[1:] if l.strip()]
    return float(first[1]), np.array(rows)


def test_npt_run_matches_oracle(tmp_path, oracle_lib, cuda_lib):
    # verlet_step_npt_mtk and the NPT branch of Simulation::run (src/potentials/potential.rs:112-135,
    # src/simulation.rs:41-115) through the input driver against the oracle's restatement: per-step
    # PE, KE, Hamiltonian (with the thermostat's and barostat's energies), T and P at the printed
    # resolution, while the barostat changes and tilts the box
    from pis_gb300.io import System, write_data
    s = melted(liquid(nc=6, seed=23), 100, 0.005)
    L = s["h"][0, 0]
    t0, t1, tau_t, p0, tau_p, steps, dt = 1.0 / KB, 1.1 / KB, 0.5, 1.0, 2.0, 40, 0.005
    data = tmp_path / "liquid.txt"
    write_data(str(data), s["pos"], s["types"], s["masses"], [0, L, 0, L, 0, L], s["table"], s["vel"])
    inp = tmp_path / "in.pis"
    dump = tmp_path / "traj.lammpstrj"
    inp.write_text(f"timestep {dt}\nread_data {data}\nfix f1 all npt temp {t0!r} {t1!r} {tau_t} iso {p0} {p0} {tau_p}\n"
                   f"dump d1 all atom 10 {dump}\nrun {steps}\n")
    sysm = System(str(inp), precision="fp64")
    assert sysm.ensemble == "NPT"
    thermo = tmp_path / "thermo.txt"
    sysm.run(str(thermo))
    pe0, rows = _parse_thermo(thermo)
    o = to_oracle(s)
    pe_ref, ke_ref, ham_ref, boxes = o.run_npt(dt, steps, t0, t1, tau_t, p0, tau_p)
    n = len(s["pos"])
    assert abs(pe0 - pe_ref[0]) <= 1e-12 * abs(pe_ref[0])
    assert rows.shape == (steps, 6)
    assert np.allclose(rows[:, 1], np.round(pe_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 2], np.round(ke_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 3], np.round(ham_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 4], np.round(2 * ke_ref[1:] / (3 * n * KB), 3), rtol=0, atol=1.5e-3)
    assert abs(rows[-1, 5] - round(o.pressure(ke_ref[-1]), 3)) <= 1.5e-3
    # the box did change (off-diagonal elements included) and the dump's bounds follow it
    assert abs(boxes[-1][0, 0] - L) > 1e-6 and np.abs(boxes[-1] - np.diag(np.diag(boxes[-1]))).max() > 0.0
    text = open(dump).read().split("ITEM: TIMESTEP\n")[1:]
    assert [int(t.split("\n")[0]) for t in text] == [0, 10, 20, 30, 40]
    bounds = text[-1].split("ITEM: BOX BOUNDS pp pp pp\n")[1].split("\n")[:3]
    assert abs(float(bounds[0].split()[1]) - boxes[-1][0, 0]) <= 1e-9 * L


def test_npt_refused_in_mixed_precision(tmp_path, oracle_lib, cuda_lib):
    from pis_gb300._ffi import PisError
    from pis_gb300.io import System, write_data
    s = liquid(nc=6)
    L = s["h"][0, 0]
    data = tmp_path / "liquid.txt"
    write_data(str(data), s["pos"], s["types"], s["masses"], [0, L, 0, L, 0, L], s["table"], s["vel"])
    inp = tmp_path / "in.pis"
    inp.write_text(f"timestep 0.005\nread_data {data}\nfix f1 all npt temp 100 100 0.5 iso 1 1 2\n"
                   f"dump d1 all atom 10 {tmp_path / 'd.lammpstrj'}\nrun 5\n")
    with pytest.raises(PisError) as e:
        System(str(inp), precision="mixed").run(str(tmp_path / "t.txt"))
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
