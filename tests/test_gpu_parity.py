"""Parity of the CUDA path (through the C ABI) with the CPU oracle on identical inputs.

Bars (the plain FP64 path against the reference's FP64 arithmetic):
  * per-atom neighbour sets identical;
  * forces, potential energy and virial within 1e-12 relative (normwise for vectors);
  * positions after 100 steps within 1e-9 sigma.
Mixed precision: force RMS error <= 1e-5 relative to FP64.
"""
import numpy as np
import pytest

from systems import argon, liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def displaced(sysd, frac, seed):
    rng = np.random.default_rng(seed)
    out = dict(sysd)
    a = sysd["h"][0, 0] / round((len(sysd["pos"]) / 4) ** (1 / 3))
    # wrapped into the box: the reference's cell binning is only exact for atoms inside it
    out["pos"] = np.mod(sysd["pos"] + rng.normal(0, frac * a, sysd["pos"].shape), sysd["h"][0, 0])
    return out


@pytest.fixture(scope="module")
def argon_c1(oracle_lib, cuda_lib):
    return argon()


@pytest.fixture(scope="module")
def liquid_melt(oracle_lib, cuda_lib):
    return melted(liquid(nc=6), steps=300, dt=0.005)


@pytest.mark.parametrize("list_kind", ["half", "full"])
def test_force_pe_virial_argon_fp64(argon_c1, list_kind):
    s = displaced(argon_c1, 0.03, 11)
    o = to_oracle(s)
    pe_ref = o.compute_potential()
    w_ref = o.virial_tensor()
    g = to_gpu(s, "fp64", skin=0.3 * 3.405, list_kind=list_kind)
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= FP64_TOL * abs(pe_ref)
    assert rel_norm(f, o.force) <= FP64_TOL
    ke, w = g.reductions()
    assert abs(ke - o.kinetic_energy()) <= FP64_TOL * abs(ke)
    # virial = sum_i r_i F_i^T: compare against the scale of its terms (forces cancel in the sum)
    scale = np.abs(s["pos"]).max() * np.abs(o.force).sum()
    assert np.abs(w - w_ref).max() <= FP64_TOL * scale


@pytest.mark.parametrize("lanes", [1, 8, 16])
@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("list_kind", ["half", "full"])
def test_force_pe_liquid_fp64(liquid_melt, list_kind, fast, lanes):
    o = to_oracle(liquid_melt)
    pe_ref = o.compute_potential()
    g = to_gpu(liquid_melt, "fp64", list_kind=list_kind, fp64_fast=fast, lanes=lanes)
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= FP64_TOL * abs(pe_ref)
    assert rel_norm(f, o.force) <= FP64_TOL


def _sets(off, idx):
    return [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def test_neighbour_sets_exact_argon_example_lattice(oracle_lib, cuda_lib):
    # the repo's argon4000 example: a = 5.41, rc = 8.5 -> exactly 54 neighbours (4 FCC shells)
    s = argon(a=5.41, eps=0.238, rc=8.5)
    o = to_oracle(s)
    off_r, idx_r = o.full_list()
    g = to_gpu(s, "fp64", skin=1.0)
    off, idx = g.neighbour_list()
    assert np.all(np.diff(off) == 54)
    ref_sets = [tuple(sorted(x)) for x in _sets(off_r, idx_r)]
    assert _sets(off, idx) == ref_sets


@pytest.mark.parametrize("lanes", [1, 4, 8, 32])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbour_sets_exact_liquid(liquid_melt, precision, lanes):
    o = to_oracle(liquid_melt)
    off_r, idx_r = o.full_list()
    g = to_gpu(liquid_melt, precision, lanes=lanes)
    off, idx = g.neighbour_list()
    ref_sets = [tuple(sorted(x)) for x in _sets(off_r, idx_r)]
    assert _sets(off, idx) == ref_sets


def test_trajectory_100_steps_argon(argon_c1):
    s = displaced(argon_c1, 0.03, 5)
    o = to_oracle(s)
    pe_ref, ke_ref = o.run_nve(0.001, 100)
    g = to_gpu(s, "fp64", skin=0.3 * 3.405)
    pe0, _ = g.compute_potential()
    pe = g.verlet_step_nve(0.001, 100)
    pos, vel, frc = g.get_state()
    assert abs(pe0 - pe_ref[0]) <= FP64_TOL * abs(pe_ref[0])
    assert np.max(np.abs(pe - pe_ref[1:]) / np.abs(pe_ref[1:])) <= FP64_TOL
    assert np.abs(pos - o.pos).max() <= 1e-9 * 3.405
    assert rel_norm(vel, o.vel) <= 1e-10


@pytest.mark.parametrize("fast", [False, True])
def test_trajectory_100_steps_liquid(liquid_melt, fast):
    o = to_oracle(liquid_melt)
    pe_ref, _ = o.run_nve(0.005, 100)
    g = to_gpu(liquid_melt, "fp64", fp64_fast=fast)
    g.compute_potential()
    pe = g.verlet_step_nve(0.005, 100)
    pos, vel, _ = g.get_state()
    d = pos - o.pos
    d -= liquid_melt["h"][0, 0] * np.round(d / liquid_melt["h"][0, 0])
    assert np.abs(d).max() <= 1e-9
    assert np.max(np.abs(pe - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-11
    st = g.stats()
    assert st["rebuilds"] >= 2  # the skin test fired during the run


@pytest.mark.parametrize("lanes,batch", [(1, 4), (1, 8), (1, 16), (4, 0), (8, 0), (32, 0)])
@pytest.mark.parametrize("kahan", [False, True])
def test_mixed_force_error(liquid_melt, kahan, lanes, batch):
    o = to_oracle(liquid_melt)
    pe_ref = o.compute_potential()
    g = to_gpu(liquid_melt, "mixed", mixed_kahan=kahan, lanes=lanes, batch=batch)
    pe, f = g.compute_potential()
    rms = np.sqrt(np.sum((f - o.force) ** 2) / np.sum(o.force ** 2))
    assert rms <= 1e-5, rms
    assert abs(pe - pe_ref) / abs(pe_ref) <= 1e-5


def test_mixed_trajectory_close(liquid_melt):
    o = to_oracle(liquid_melt)
    pe_ref, _ = o.run_nve(0.005, 50)
    g = to_gpu(liquid_melt, "mixed")
    g.compute_potential()
    pe = g.verlet_step_nve(0.005, 50)
    assert np.max(np.abs(pe - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-4


def test_two_type_mixture(oracle_lib, cuda_lib):
    rng = np.random.default_rng(4)
    s = liquid(nc=6, rho=0.8)
    n = len(s["pos"])
    s["types"] = rng.integers(1, 3, n).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (1.0, 1.0, 2.5), (2, 2): (0.8, 1.1, 2.75), (1, 2): (0.9, 1.05, 2.6)}
    s = displaced(s, 0.02, 2)
    o = to_oracle(s)
    pe_ref = o.compute_potential()
    for prec in ("fp64", "mixed"):
        g = to_gpu(s, prec)
        pe, f = g.compute_potential()
        tol = FP64_TOL if prec == "fp64" else 1e-5
        assert abs(pe - pe_ref) <= tol * abs(pe_ref)
        assert rel_norm(f, o.force) <= tol
        off, idx = g.neighbour_list()
        off_r, idx_r = o.full_list()
        assert _sets(off, idx) == [tuple(sorted(x)) for x in _sets(off_r, idx_r)]


def test_missing_cross_pair_is_skipped(oracle_lib, cuda_lib):
    # types 1 and 2 with no (1,2) entry: the reference prints and skips those pairs
    # (6 FCC cells -> 3 reference cells at rcut 3.0, so the reference stencil is exact)
    s = liquid(nc=6, rho=0.8)
    n = len(s["pos"])
    s["types"] = (np.arange(n) % 2 + 1).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (2.0, 0.6, 1.1), (2, 2): (0.8, 1.2, 3.0)}
    s = displaced(s, 0.02, 9)
    o = to_oracle(s)
    pe_ref = o.compute_potential()
    g = to_gpu(s, "fp64")
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= FP64_TOL * abs(pe_ref)
    assert rel_norm(f, o.force) <= FP64_TOL


def test_small_box_two_cells(oracle_lib, cuda_lib):
    # 500 atoms at rho*=0.95 (L = 8.07): only 2 cells per axis at rc + skin; the GPU path
    # de-duplicates the stencil, so compare against the all-pairs reference manager
    import oracle
    s = displaced(liquid(nc=5, rho=0.95), 0.02, 3)
    o = to_oracle(s)
    pe_ref = o.compute_potential(manager=oracle.ALLPAIRS)
    for prec in ("fp64", "mixed"):
        g = to_gpu(s, prec)
        assert g.stats()["cells"] == (2, 2, 2)
        pe, f = g.compute_potential()
        tol = FP64_TOL if prec == "fp64" else 1e-5
        assert abs(pe - pe_ref) <= tol * abs(pe_ref)
        assert rel_norm(f, o.force) <= tol


@pytest.mark.parametrize("edge_margin", [0.5, 2e-6])
def test_two_cell_box_walks(oracle_lib, cuda_lib, edge_margin):
    # two cells per axis: the 27-cell walk serves the box when its edge exceeds twice the padded
    # list radius (margin 0.5: skin 0.3), the generic walk when the edge is within 1e-5 of it
    # (skin chosen so that rcut + skin = L / 2 (1 - 2e-6)); both must give the all-pairs forces
    # (a pair listed under two images would count twice)
    import oracle
    s = displaced(liquid(nc=5, rho=0.95), 0.02, 4)
    L = s["h"][0, 0]
    skin = 0.3 if edge_margin == 0.5 else L / 2 * (1 - edge_margin) - 2.5
    o = to_oracle(s)
    pe_ref = o.compute_potential(manager=oracle.ALLPAIRS)
    for prec in ("fp64", "mixed"):
        g = to_gpu(s, prec, skin=skin, list_kind="full")
        assert g.stats()["cells"] == (2, 2, 2)
        pe, f = g.compute_potential()
        tol = FP64_TOL if prec == "fp64" else 1e-5
        assert abs(pe - pe_ref) <= tol * abs(pe_ref)
        assert rel_norm(f, o.force) <= tol
        e = g.verlet_step_nve(0.005, 20)
        assert np.all(np.isfinite(e))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_two_cell_generic_walk_in_a_replica_pool(oracle_lib, cuda_lib, prec):
    # a generic-walk box as in the test above (4 lattice cells per edge, so that its ~134 list
    # entries per atom fit a replica pool's fixed capacity) beside an ordinary liquid in one
    # replica pool, whose rebuild kernels stride over the listed chunks (the generic walk's list
    # form included): the first evaluation of each slot gives the all-pairs forces
    import oracle
    from pis_gb300.batch import Batch
    s = displaced(liquid(nc=4, rho=0.95), 0.02, 4)
    L = s["h"][0, 0]
    other = displaced(liquid(nc=6, seed=12), 0.02, 5)
    b = Batch(2000, 2, 0, precision=prec)
    slots = [b.admit(x["pos"], x["types"], x["masses"], x["h"], x["table"], 20, velocities=x["vel"], skin=sk)
             for x, sk in ((s, L / 2 * (1 - 2e-6) - 2.5), (other, 0.3))]
    tol = FP64_TOL if prec == "fp64" else 1e-5
    for x, slot in zip((s, other), slots):
        o = to_oracle(x)
        pe_ref = o.compute_potential(manager=oracle.ALLPAIRS)
        r = b.result(slot, len(x["pos"]))
        assert abs(r["pe"] - pe_ref) <= tol * abs(pe_ref)
        assert rel_norm(r["force"], o.force) <= tol
    b.advance(20)
    assert all(np.isfinite(b.result(sl, len(x["pos"]))["pe"]) for sl, x in zip(slots, (s, other)))
    b.close()


def test_errors_are_reported(oracle_lib, cuda_lib):
    from pis_gb300 import PisError
    s = liquid(nc=2)  # L = 3.36 < 2 (rc + skin)
    with pytest.raises(PisError) as e:
        to_gpu(s)
    assert e.value.name == "PIS_ERR_BOX_TOO_SMALL"
    s = liquid(nc=5)
    s["types"] = s["types"].copy()
    s["types"][3] = 2
    with pytest.raises(PisError) as e:
        to_gpu(s)
    assert e.value.name == "PIS_ERR_INVALID_ATOM_TYPE"


def test_scale_velocities(liquid_melt):
    g = to_gpu(liquid_melt)
    m = np.diag([0.5, 1.0, 2.0])
    g.scale_velocities(m)
    _, vel, _ = g.get_state()
    assert np.allclose(vel, liquid_melt["vel"] @ m.T, rtol=0, atol=1e-15)


def test_kernel_launch_counter_moves(liquid_melt):
    from pis_gb300.potentials import kernel_launches
    g = to_gpu(liquid_melt)
    before = kernel_launches()
    g.compute_potential()
    g.verlet_step_nve(0.005, 10)
    assert kernel_launches() - before >= 10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_set_state_reuses_pool_and_matches_fresh_context(liquid_melt, precision):
    # a second state of the same shape is placed in the same device pool (memory and captured
    # step graphs reused); its results must equal those of a fresh context bit for bit
    g = to_gpu(liquid_melt, precision, list_kind="full")
    g.compute_potential()
    g.verlet_step_nve(0.005, 20)
    s2 = displaced(liquid_melt, 0.01, 9)
    g.set_state(s2["pos"], s2["types"], s2["masses"], s2["h"], velocities=s2["vel"])
    pe, f = g.compute_potential()
    e = g.verlet_step_nve(0.005, 30)
    out = (np.empty((len(s2["pos"]), 3)), np.empty((len(s2["pos"]), 3)), np.empty((len(s2["pos"]), 3)))
    p, v, fo = g.get_state(out=out)
    assert p is out[0] and v is out[1] and fo is out[2]
    fresh = to_gpu(s2, precision, list_kind="full")
    pe_f, f_f = fresh.compute_potential()
    e_f = fresh.verlet_step_nve(0.005, 30)
    p_f, v_f, fo_f = fresh.get_state()
    assert pe == pe_f and np.array_equal(f, f_f) and np.array_equal(e, e_f)
    assert np.array_equal(p, p_f) and np.array_equal(v, v_f) and np.array_equal(fo, fo_f)
    assert g.stats()["steps"] == 30


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_plain_step_graphs_equal_conditional(liquid_melt, precision):
    # PIS_OPT_PLAIN_GRAPHS captures the step graphs with the rebuild kernels launched on every
    # step (exiting at once when nothing rebuilds) instead of behind a conditional node; the
    # trajectory, energies and rebuild count must be those of the default graphs bit for bit (full
    # lists: the FP64 half list scatters Newton-3 forces with atomics, whose order varies)
    from pis_gb300.potentials import kernel_launches
    a = to_gpu(liquid_melt, precision, list_kind="full")
    b = to_gpu(liquid_melt, precision, list_kind="full", plain_graphs=True)
    e_a = a.verlet_step_nve(0.005, 120)
    k0 = kernel_launches()
    e_b = b.verlet_step_nve(0.005, 120)
    assert kernel_launches() - k0 >= 120 * 4
    assert np.array_equal(e_a, e_b)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"] >= 2


@pytest.mark.parametrize("nc,stretch", [(6, (1.0, 1.1, 1.25)), (5, (1.0, 0.95, 1.2))])
def test_mixed_orthorhombic_cells(oracle_lib, cuda_lib, nc, stretch):
    # boxes whose cells differ between axes (3 x 3 x 4 cells; 2 x 2 x 3 cells, two-cell axes): the
    # mixed path's FP32 coordinates are in units of the x cell edge, so the y and z image shifts
    # are edge ratios there. Neighbour sets equal the oracle's, forces stay within the mixed bar
    # of FP64, and a 60-step run with rebuilds stays close to the FP64 run
    s = liquid(nc=nc, seed=12)
    m = np.diag(stretch)
    s["pos"] = s["pos"] @ m
    s["h"] = s["h"] @ m
    s = melted(s, steps=100, dt=0.004)
    o = to_oracle(s)
    off, idx = o.full_list()
    g = to_gpu(s, "mixed", list_kind="full")
    got = g.neighbour_list()
    sets = [tuple(sorted(idx[off[i]:off[i + 1]])) for i in range(len(off) - 1)]
    assert [tuple(got[1][got[0][i]:got[0][i + 1]]) for i in range(len(got[0]) - 1)] == sets
    f64 = to_gpu(s, "fp64")
    pe64, F64 = f64.compute_potential()
    pe, f = g.compute_potential()
    assert np.sqrt(np.sum((f - F64) ** 2) / np.sum(F64 ** 2)) <= 1e-5
    assert abs(pe - pe64) <= 1e-6 * abs(pe64)
    e = g.verlet_step_nve(0.004, 60)
    e64 = f64.verlet_step_nve(0.004, 60)
    assert np.max(np.abs(e - e64) / np.abs(e64)) <= 1e-5
    assert g.stats()["rebuilds"] >= 2


def test_large_cell_grid_segmented_scan(oracle_lib, cuda_lib):
    # 186,624 atoms on 21^3 = 9,261 cells: more than one 8,192-cell segment, so the cell scan runs
    # as one block per segment plus the carry kernel. The neighbour sets and the FP64 energy (an
    # exact sum) must equal the oracle's on the displaced lattice.
    s = liquid(nc=36, seed=31)
    rng = np.random.default_rng(31)
    L = s["h"][0, 0]
    s["pos"] = np.mod(s["pos"] + rng.normal(0, 0.05, s["pos"].shape), L)
    assert int(L // 2.8) ** 3 > 8192
    o = to_oracle(s)
    pe_exact, _ = o.compute_potential_exact()
    off, idx = o.full_list()
    g = to_gpu(s, "fp64", list_kind="full")
    pe, _ = g.compute_potential()
    assert pe == pe_exact
    go, gi = g.neighbour_list()
    assert np.array_equal(go, off)
    for i in range(len(off) - 1):
        assert np.array_equal(gi[go[i]:go[i + 1]], np.sort(idx[off[i]:off[i + 1]])), i
    m = to_gpu(s, "mixed")
    pem, _ = m.compute_potential()
    assert abs(pem - pe) <= 1e-6 * abs(pe)
