"""The fused step kernel of the mixed path (forces, kick and the next step's drift in one pass).

The fused step and the separate force / kick / drift kernels (PIS_OPT_UNFUSED) do the same
arithmetic and the same block partial sums, so trajectories, per-step energies, forces and rebuild
counts must agree bit for bit, across graph boundaries (runs that are not a multiple of the 50-step
graph), for every kernel shape the fused step serves (compensated or FP64 batch sums, 4- or 8-entry
batches, one or two atom types) and for pools whose slots stop at different steps.
"""
import numpy as np
import pytest

from systems import liquid, to_gpu

pytestmark = pytest.mark.gpu


def _hot(nc, seed, amp=0.05):
    s = liquid(nc=nc, seed=seed, t_star=1.2)
    rng = np.random.default_rng(seed)
    L = s["h"][0, 0]
    s["pos"] = np.mod(s["pos"] + rng.normal(0, amp, s["pos"].shape), L)
    return s


def _two_types(s, seed):
    rng = np.random.default_rng(seed)
    out = dict(s)
    out["types"] = rng.integers(1, 3, len(s["pos"])).astype(np.int32)
    out["masses"] = np.array([1.0, 1.5])
    out["table"] = {(1, 1): (1.0, 1.0, 2.5), (2, 2): (0.8, 1.05, 2.6), (1, 2): (0.9, 1.02, 2.55)}
    return out


@pytest.fixture(scope="module")
def hot_liquid(cuda_lib):
    return _hot(14, 5)


def _run(s, runs, **kw):
    g = to_gpu(s, "mixed", **kw)
    pe0, f0 = g.compute_potential()
    energies = [g.verlet_step_nve(0.005, k) for k in runs]
    pos, vel, frc = g.get_state()
    ke, w = g.reductions()
    st = g.stats()
    g.close()
    return pe0, f0, energies, pos, vel, frc, ke, w, st


@pytest.mark.parametrize("kahan,batch", [(True, 4), (False, 4), (True, 8), (False, 8)])
def test_fused_equals_unfused(hot_liquid, kahan, batch):
    runs = [1, 7, 50, 63]
    a = _run(hot_liquid, runs, mixed_kahan=kahan, batch=batch)
    b = _run(hot_liquid, runs, mixed_kahan=kahan, batch=batch, unfused=True)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
    for ea, eb in zip(a[2], b[2]):
        assert np.array_equal(ea, eb)
    for x, y in zip(a[3:6], b[3:6]):
        assert np.array_equal(x, y)
    assert a[6] == b[6] and np.array_equal(a[7], b[7])
    assert a[8]["rebuilds"] == b[8]["rebuilds"] >= 3
    assert a[8]["steps"] == b[8]["steps"] == sum(runs)


def test_fused_two_types_equals_unfused(cuda_lib):
    s = _two_types(_hot(8, 9), 9)
    a = _run(s, [33, 50], mixed_kahan=True, batch=4)
    b = _run(s, [33, 50], mixed_kahan=True, batch=4, unfused=True)
    for ea, eb in zip(a[2], b[2]):
        assert np.array_equal(ea, eb)
    for x, y in zip(a[3:6], b[3:6]):
        assert np.array_equal(x, y)
    assert a[8]["rebuilds"] == b[8]["rebuilds"] >= 2


def test_fused_plain_graphs_equal_conditional(hot_liquid):
    a = _run(hot_liquid, [50, 21], mixed_kahan=True, batch=4)
    b = _run(hot_liquid, [50, 21], mixed_kahan=True, batch=4, plain_graphs=True)
    for ea, eb in zip(a[2], b[2]):
        assert np.array_equal(ea, eb)
    for x, y in zip(a[3:6], b[3:6]):
        assert np.array_equal(x, y)


def test_fused_neighbour_list_after_run_matches(hot_liquid):
    # lists rebuilt inside the graphs (at odd and even steps, so from either coordinate buffer) are
    # those of the unfused path, and a force evaluation after the run agrees
    out = []
    for unfused in (False, True):
        g = to_gpu(hot_liquid, "mixed", mixed_kahan=True, batch=4, unfused=unfused)
        g.verlet_step_nve(0.005, 89)
        off, idx = g.neighbour_list()
        pe, f = g.compute_potential()
        out.append((off, idx, pe, f, g.stats()["rebuilds"]))
        g.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and np.array_equal(out[0][3], out[1][3])
    assert out[0][4] == out[1][4]


def test_fused_batch_slots_stop_at_different_steps(cuda_lib):
    from pis_gb300.batch import Batch
    systems = [_hot(10, 21), _hot(6, 22), _hot(8, 23)]
    steps = [60, 17, 41]

    def run(unfused):
        bt = Batch(40000, 4, 0, precision="mixed", batch=4, mixed_kahan=True, unfused=unfused)
        slots = [bt.admit(x["pos"], x["types"], x["masses"], x["h"], x["table"], k, velocities=x["vel"])
                 for x, k in zip(systems, steps)]
        bt.advance(60)
        out = [bt.result(sl, len(x["pos"])) for sl, x in zip(slots, systems)]
        bt.close()
        return out

    r, f = run(True), run(False)
    for q in range(3):
        assert np.array_equal(f[q]["pos"], r[q]["pos"]) and np.array_equal(f[q]["vel"], r[q]["vel"]), q
        assert f[q]["pe"] == r[q]["pe"], q


def test_unfused_option_validated(cuda_lib):
    from pis_gb300._ffi import option_flags
    assert option_flags(unfused=True) == 32
