"""Mixed precision through the cluster-list kernels (PIS_OPT_CLUSTER(2 or 4)), against the oracle.

A cluster is a run of up to m spatially adjacent atoms of one cell; its list holds every atom
within the list radius of any member; one thread evaluates every (member, entry) pair
(PIS_OPT_LANES(1)) or one lane per member evaluates its own pairs (PIS_OPT_LANES(m)). The
bars are the mixed-precision ones: force RMS <= 1e-5 relative to the FP64 oracle, energies within
1e-5, neighbour sets within the cutoff identical to the reference's build_neighbour_list, and a
replica bit-identical alone and in a mix.
"""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _sets(off, idx):
    return [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def displaced(sysd, frac, seed):
    rng = np.random.default_rng(seed)
    out = dict(sysd)
    a = sysd["h"][0, 0] / round((len(sysd["pos"]) / 4) ** (1 / 3))
    out["pos"] = np.mod(sysd["pos"] + rng.normal(0, frac * a, sysd["pos"].shape), sysd["h"][0, 0])
    return out


@pytest.fixture(scope="module")
def liquid_melt(oracle_lib, cuda_lib):
    return melted(liquid(nc=6), steps=300, dt=0.005)


@pytest.mark.parametrize("lane", [False, True])
@pytest.mark.parametrize("batch", [4, 8])
@pytest.mark.parametrize("kahan", [False, True])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_force_error(liquid_melt, cluster, kahan, batch, lane):
    o = to_oracle(liquid_melt)
    pe_ref = o.compute_potential()
    g = to_gpu(liquid_melt, "mixed", mixed_kahan=kahan, batch=batch, cluster=cluster, lanes=cluster if lane else 1)
    pe, f = g.compute_potential()
    rms = np.sqrt(np.sum((f - o.force) ** 2) / np.sum(o.force ** 2))
    assert rms <= 1e-5, rms
    assert abs(pe - pe_ref) / abs(pe_ref) <= 1e-5
    st = g.stats()
    assert st["list_capacity"] > 0 and st["list_entries"] > 0


@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_neighbour_sets_exact(liquid_melt, cluster):
    o = to_oracle(liquid_melt)
    off_r, idx_r = o.full_list()
    g = to_gpu(liquid_melt, "mixed", cluster=cluster)
    off, idx = g.neighbour_list()
    assert _sets(off, idx) == [tuple(sorted(x)) for x in _sets(off_r, idx_r)]


@pytest.mark.parametrize("lane", [False, True])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_trajectory_close(liquid_melt, cluster, lane):
    o = to_oracle(liquid_melt)
    pe_ref, _ = o.run_nve(0.005, 50)
    g = to_gpu(liquid_melt, "mixed", cluster=cluster, lanes=cluster if lane else 1)
    g.compute_potential()
    pe = g.verlet_step_nve(0.005, 50)
    assert np.max(np.abs(pe - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-4
    assert g.stats()["rebuilds"] >= 2


@pytest.mark.parametrize("lane", [False, True])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_two_type_mixture(oracle_lib, cuda_lib, cluster, lane):
    rng = np.random.default_rng(4)
    s = liquid(nc=6, rho=0.8)
    n = len(s["pos"])
    s["types"] = rng.integers(1, 3, n).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (1.0, 1.0, 2.5), (2, 2): (0.8, 1.1, 2.75), (1, 2): (0.9, 1.05, 2.6)}
    s = displaced(s, 0.02, 2)
    o = to_oracle(s)
    pe_ref = o.compute_potential()
    g = to_gpu(s, "mixed", cluster=cluster, lanes=cluster if lane else 1)
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= 1e-5 * abs(pe_ref)
    assert rel_norm(f, o.force) <= 1e-5
    off, idx = g.neighbour_list()
    off_r, idx_r = o.full_list()
    assert _sets(off, idx) == [tuple(sorted(x)) for x in _sets(off_r, idx_r)]


@pytest.mark.parametrize("lane", [False, True])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_small_box_two_cells(oracle_lib, cuda_lib, cluster, lane):
    # 2 cells per axis at rc + skin: both images of the other cell are scanned
    import oracle
    s = displaced(liquid(nc=5, rho=0.95), 0.02, 3)
    o = to_oracle(s)
    pe_ref = o.compute_potential(manager=oracle.ALLPAIRS)
    g = to_gpu(s, "mixed", cluster=cluster, lanes=cluster if lane else 1)
    assert g.stats()["cells"] == (2, 2, 2)
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= 1e-5 * abs(pe_ref)
    assert rel_norm(f, o.force) <= 1e-5
    off, idx = g.neighbour_list()
    off_r, idx_r = o.full_list()
    assert _sets(off, idx) == [tuple(sorted(x)) for x in _sets(off_r, idx_r)]


@pytest.mark.parametrize("lane", [False, True])
def test_cluster_batch_alone_equals_mix(cuda_lib, lane):
    """An odd-sized replica and a liquid give bit-identical results alone and together."""
    from pis_gb300.batch import Batch
    a = liquid(nc=5, seed=21)
    a = {**a, "pos": a["pos"][:-1], "vel": a["vel"][:-1], "types": a["types"][:-1]}
    b = liquid(nc=6, rho=0.8, seed=22)

    def run(systems):
        bt = Batch(4096, 4, 0, precision="mixed", cluster=4, lanes=4 if lane else 1)
        slots = [bt.admit(x["pos"], x["types"], x["masses"], x["h"], x["table"], 80, velocities=x["vel"])
                 for x in systems]
        bt.advance(80)
        out = [bt.result(sl, len(x["pos"])) for sl, x in zip(slots, systems)]
        bt.close()
        return out

    alone = [run([a])[0], run([b])[0]]
    mix = run([a, b])
    for q in range(2):
        assert mix[q]["steps"] == 80
        assert np.array_equal(mix[q]["pos"], alone[q]["pos"]), q
        assert np.array_equal(mix[q]["vel"], alone[q]["vel"]), q
        assert mix[q]["pe"] == alone[q]["pe"] and mix[q]["ke"] == alone[q]["ke"], q


def test_cluster_option_checks(cuda_lib):
    from pis_gb300._ffi import PisError
    s = liquid(nc=6)
    with pytest.raises(PisError) as e:
        to_gpu(s, "fp64", cluster=4)
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
    with pytest.raises(PisError) as e:
        to_gpu(s, "mixed", cluster=3)
    assert e.value.name == "PIS_ERR_INVALID_ARGUMENT"
    with pytest.raises(PisError) as e:
        to_gpu(s, "mixed", cluster=4, lanes=2)
    assert e.value.name in ("PIS_ERR_UNSUPPORTED", "PIS_ERR_INVALID_ARGUMENT")


# ---- per-atom lists built per cluster (PIS_OPT_SCAN) -----------------------------------------
# The build scans candidates per cluster of m atoms but writes each atom's own list with the
# per-atom build's arithmetic and order, so every result must be bit-identical to the per-atom
# build's (FP64 half lists scatter with atomics, so there the exact neighbour sets are compared).


@pytest.mark.parametrize("scan", [2, 4])
def test_scan_build_bitwise_mixed(liquid_melt, scan):
    ref = to_gpu(liquid_melt, "mixed", scan=1)
    g = to_gpu(liquid_melt, "mixed", scan=scan)
    pe_r, f_r = ref.compute_potential()
    pe, f = g.compute_potential()
    assert pe == pe_r and np.array_equal(f, f_r)
    assert g.stats()["list_entries"] == ref.stats()["list_entries"]
    e_r = ref.verlet_step_nve(0.005, 60)
    e = g.verlet_step_nve(0.005, 60)
    assert np.array_equal(e, e_r)
    p_r, v_r, _ = ref.get_state()
    p, v, _ = g.get_state()
    assert np.array_equal(p, p_r) and np.array_equal(v, v_r)
    assert g.stats()["rebuilds"] >= 2


@pytest.mark.parametrize("scan", [2, 4])
def test_scan_build_bitwise_fp64_full(liquid_melt, scan):
    ref = to_gpu(liquid_melt, "fp64", list_kind="full", scan=1)
    g = to_gpu(liquid_melt, "fp64", list_kind="full", scan=scan)
    pe_r, f_r = ref.compute_potential()
    pe, f = g.compute_potential()
    assert pe == pe_r and np.array_equal(f, f_r)
    e_r = ref.verlet_step_nve(0.005, 30)
    e = g.verlet_step_nve(0.005, 30)
    assert np.array_equal(e, e_r)


@pytest.mark.parametrize("scan", [2, 4])
def test_scan_build_half_list_sets_and_oracle(liquid_melt, scan):
    o = to_oracle(liquid_melt)
    pe_ref = o.compute_potential()
    off_r, idx_r = o.full_list()
    g = to_gpu(liquid_melt, "fp64", scan=scan)
    pe, f = g.compute_potential()
    assert abs(pe - pe_ref) <= 1e-12 * abs(pe_ref)
    assert rel_norm(f, o.force) <= 1e-12
    off, idx = g.neighbour_list()
    assert _sets(off, idx) == [tuple(sorted(x)) for x in _sets(off_r, idx_r)]


def test_scan_build_batch_alone_equals_mix(cuda_lib):
    from pis_gb300.batch import Batch
    a = liquid(nc=5, seed=21)
    a = {**a, "pos": a["pos"][:-1], "vel": a["vel"][:-1], "types": a["types"][:-1]}
    b = liquid(nc=7, rho=0.8, seed=22)

    def run(systems, scan):
        bt = Batch(4096, 4, 0, precision="mixed", scan=scan)
        slots = [bt.admit(x["pos"], x["types"], x["masses"], x["h"], x["table"], 80, velocities=x["vel"])
                 for x in systems]
        bt.advance(80)
        out = [bt.result(sl, len(x["pos"])) for sl, x in zip(slots, systems)]
        bt.close()
        return out

    ref = run([a, b], 1)
    mix = run([a, b], 4)
    alone = run([b], 4)[0]
    for q in range(2):
        assert np.array_equal(mix[q]["pos"], ref[q]["pos"]) and np.array_equal(mix[q]["vel"], ref[q]["vel"]), q
        assert mix[q]["pe"] == ref[q]["pe"], q
    assert np.array_equal(alone["pos"], mix[1]["pos"]) and alone["pe"] == mix[1]["pe"]
