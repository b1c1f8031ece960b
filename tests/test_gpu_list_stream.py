"""The mixed force kernel fed by bulk copies of the neighbour list (PIS_OPT_LIST_TMA).

The variant streams each 256-atom chunk's list rows into a shared-memory ring with
cp.async.bulk and mbarriers instead of loading list words from global memory per batch. With 8
rows per stage it consumes entries in the same batches and folds them at the same points as the
direct-load kernel with PIS_OPT_BATCH(8), so forces, energies and trajectories must be
bit-identical to it; with 16 rows it is held to the mixed-precision error bar against the oracle
(force RMS <= 1e-5 relative to FP64). A batch pool whose second slot starts at an atom offset that
is not a multiple of 4 checks the row copies' alignment handling.
"""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def liquid_melt(oracle_lib, cuda_lib):
    return melted(liquid(nc=6), steps=300, dt=0.005)


@pytest.mark.parametrize("kahan", [False, True])
def test_stream_bitwise_equals_direct_loads(liquid_melt, kahan):
    ref = to_gpu(liquid_melt, "mixed", mixed_kahan=kahan, batch=8)
    tma = to_gpu(liquid_melt, "mixed", mixed_kahan=kahan, batch=8, tma=True)
    pe_r, f_r = ref.compute_potential()
    pe_t, f_t = tma.compute_potential()
    assert pe_t == pe_r
    assert np.array_equal(f_t, f_r)
    e_r = ref.verlet_step_nve(0.005, 60)
    e_t = tma.verlet_step_nve(0.005, 60)
    assert np.array_equal(e_t, e_r)
    p_r, v_r, _ = ref.get_state()
    p_t, v_t, _ = tma.get_state()
    assert np.array_equal(p_t, p_r) and np.array_equal(v_t, v_r)
    assert tma.stats()["rebuilds"] >= 2


@pytest.mark.parametrize("batch", [8, 16])
@pytest.mark.parametrize("kahan", [False, True])
def test_stream_force_error(liquid_melt, kahan, batch):
    o = to_oracle(liquid_melt)
    pe_ref = o.compute_potential()
    g = to_gpu(liquid_melt, "mixed", mixed_kahan=kahan, batch=batch, tma=True)
    pe, f = g.compute_potential()
    rms = np.sqrt(np.sum((f - o.force) ** 2) / np.sum(o.force ** 2))
    assert rms <= 1e-5, rms
    assert abs(pe - pe_ref) / abs(pe_ref) <= 1e-5


def test_stream_unaligned_slot_start(cuda_lib):
    """Slot 1 starts at atom 499 (a vacancy makes slot 0 odd-sized): its chunks begin 3 words past
    a 16-byte boundary of every list row, and slot 0's last chunk holds 243 atoms."""
    from pis_gb300.batch import Batch
    a = liquid(nc=5, seed=21)
    a = {**a, "pos": a["pos"][:-1], "vel": a["vel"][:-1], "types": a["types"][:-1]}
    b = liquid(nc=6, rho=0.8, seed=22)
    res = {}
    for tma in (False, True):
        bt = Batch(4096, 4, 0, precision="mixed", batch=8, tma=tma)
        sa = bt.admit(a["pos"], a["types"], a["masses"], a["h"], a["table"], 80, velocities=a["vel"])
        sb = bt.admit(b["pos"], b["types"], b["masses"], b["h"], b["table"], 80, velocities=b["vel"])
        bt.advance(80)
        res[tma] = (bt.result(sa, len(a["pos"])), bt.result(sb, len(b["pos"])))
        bt.close()
    for q in range(2):
        r, t = res[False][q], res[True][q]
        assert r["steps"] == t["steps"] == 80
        assert np.array_equal(t["pos"], r["pos"]) and np.array_equal(t["vel"], r["vel"]), q
        assert t["pe"] == r["pe"] and t["ke"] == r["ke"], q


def test_stream_option_rejected_outside_mixed(cuda_lib):
    from pis_gb300._ffi import PisError
    s = liquid(nc=6)
    with pytest.raises(PisError) as e:
        to_gpu(s, "fp64", tma=True)
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
    with pytest.raises(PisError):
        to_gpu(s, "mixed", tma=True, lanes=4)
