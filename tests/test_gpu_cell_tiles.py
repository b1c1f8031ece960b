"""The mixed force kernel with neighbour-cell tiles staged in shared memory (PIS_OPT_TILE).

A 256-atom chunk whose atoms lie in one cell row copies its neighbour cells' positions into
shared memory with bulk copies and gathers from there; other chunks gather from global memory.
Either way the pair arithmetic, entry order and batching are those of the default kernel
(4-entry batches), so forces, energies and trajectories must be bit-identical to it. The
256,000-atom liquid has 23 cells per row (~460 atoms), so a large share of its chunks take the
tiled path; a 864-atom liquid (3 cells per row) exercises the fallback only.
"""
import numpy as np
import pytest

from systems import liquid, to_gpu, to_oracle

pytestmark = pytest.mark.gpu


def _perturbed(nc, seed, amp=0.06):
    s = liquid(nc=nc, seed=seed)
    rng = np.random.default_rng(seed)
    L = s["h"][0, 0]
    s["pos"] = np.mod(s["pos"] + rng.normal(0, amp, s["pos"].shape), L)
    return s


@pytest.fixture(scope="module")
def big_liquid(cuda_lib):
    return _perturbed(40, 31)


@pytest.mark.parametrize("kahan", [False, True])
def test_tiles_bitwise_equal_direct_gathers(big_liquid, kahan):
    ref = to_gpu(big_liquid, "mixed", mixed_kahan=kahan, batch=4)
    tile = to_gpu(big_liquid, "mixed", mixed_kahan=kahan, batch=4, tiles=True)
    pe_r, f_r = ref.compute_potential()
    pe_t, f_t = tile.compute_potential()
    assert pe_t == pe_r and np.array_equal(f_t, f_r)
    e_r = ref.verlet_step_nve(0.005, 60)
    e_t = tile.verlet_step_nve(0.005, 60)
    assert np.array_equal(e_t, e_r)
    p_r, v_r, _ = ref.get_state()
    p_t, v_t, _ = tile.get_state()
    assert np.array_equal(p_t, p_r) and np.array_equal(v_t, v_r)
    assert tile.stats()["rebuilds"] >= 2


def test_tiles_force_error_vs_oracle(cuda_lib, oracle_lib):
    s = _perturbed(30, 5)
    o = to_oracle(s)
    pe_ref = o.compute_potential()
    g = to_gpu(s, "mixed", batch=4, mixed_kahan=True, tiles=True)
    pe, f = g.compute_potential()
    rms = np.sqrt(np.sum((f - o.force) ** 2) / np.sum(o.force ** 2))
    assert rms <= 1e-5, rms
    assert abs(pe - pe_ref) / abs(pe_ref) <= 1e-5


def test_tiles_small_box_falls_back(cuda_lib):
    s = _perturbed(6, 7)
    ref = to_gpu(s, "mixed", batch=4)
    tile = to_gpu(s, "mixed", batch=4, tiles=True)
    assert ref.compute_potential()[0] == tile.compute_potential()[0]
    assert np.array_equal(ref.verlet_step_nve(0.005, 30), tile.verlet_step_nve(0.005, 30))


def test_tiles_batch_equals_direct(cuda_lib):
    from pis_gb300.batch import Batch
    systems = [_perturbed(24, 11), _perturbed(6, 12)]

    def run(tiles):
        bt = Batch(60000, 4, 0, precision="mixed", batch=4, tiles=tiles)
        slots = [bt.admit(x["pos"], x["types"], x["masses"], x["h"], x["table"], 40, velocities=x["vel"])
                 for x in systems]
        bt.advance(40)
        out = [bt.result(sl, len(x["pos"])) for sl, x in zip(slots, systems)]
        bt.close()
        return out

    r, t = run(False), run(True)
    for q in range(2):
        assert np.array_equal(t[q]["pos"], r[q]["pos"]) and np.array_equal(t[q]["vel"], r[q]["vel"]), q
        assert t[q]["pe"] == r[q]["pe"], q


def test_tiles_option_rejected_outside_mixed_thread_per_atom(cuda_lib):
    from pis_gb300._ffi import PisError
    s = liquid(nc=6)
    for kw in ({"precision": "fp64"}, {"precision": "mixed", "lanes": 4}, {"precision": "mixed", "tma": True},
               {"precision": "mixed", "cluster": 4}):
        prec = kw.pop("precision")
        with pytest.raises(PisError) as e:
            to_gpu(s, prec, tiles=True, **kw)
        assert e.value.name == "PIS_ERR_UNSUPPORTED"
