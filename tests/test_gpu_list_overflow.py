"""Neighbour-list overflow: reported when growth is off, recovered without a trace when it is on.

The reference has no list (it rebuilds its cells at every evaluation), so a list that outgrows its
capacity is this library's own failure mode. pis_gpu_set_list_capacity sets the capacity; with
automatic growth an evaluation or a run of steps that overflows is repeated from its own start
(a device copy of the state taken before it) with a larger list, so its results equal those of a
run whose list was large enough from the start - bit for bit on the reference-order FP64 path.
The overflow in the middle of a run is provoked by compressing the box (pis_gpu_scale_box), which
raises the neighbour count well above the capacity the start state needed.
"""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu

pytestmark = pytest.mark.gpu

SHRINK = np.diag([0.85, 0.85, 0.85])


@pytest.fixture(scope="module")
def state(oracle_lib, cuda_lib):
    return melted(liquid(nc=6), steps=100, dt=0.005)  # 864 atoms, ~77 list entries per atom


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overflow_is_reported_without_growth(state, precision):
    from pis_gb300._ffi import PisError
    g = to_gpu(state, precision, list_kind="full", list_capacity=32, auto_grow=False)
    with pytest.raises(PisError) as e:
        g.compute_potential()
    assert e.value.name == "PIS_ERR_LIST_OVERFLOW"
    with pytest.raises(PisError) as e:
        g.verlet_step_nve(0.005, 20)
    assert e.value.name == "PIS_ERR_LIST_OVERFLOW"


@pytest.mark.parametrize("kw", [dict(precision="fp64", ref_order=True), dict(precision="mixed"),
                                dict(precision="fp64", list_kind="half")])
def test_overflow_grows_and_matches_a_large_list(state, kw):
    # evaluation: a 32-entry list grows at once and the result is a fresh evaluation's
    big = to_gpu(state, list_capacity=256, **kw)
    small = to_gpu(state, list_capacity=32, **kw)
    pe_b, f_b = big.compute_potential()
    pe_s, f_s = small.compute_potential()
    assert small.stats()["list_capacity"] > 32
    assert pe_s == pe_b
    if kw.get("list_kind") == "half":  # atomics: summation order differs between launches
        assert np.linalg.norm(f_s - f_b) <= 1e-12 * np.linalg.norm(f_b)
    else:
        assert np.array_equal(f_s, f_b)
    # a run whose list overflows in its middle: compress the box (volume x 0.61), so the next
    # rebuild needs more entries than the grown capacity holds; the chunk is repeated from its
    # checkpoint
    for g in (big, small):
        g.verlet_step_nve(0.005, 30)
    cap_before = small.stats()["list_capacity"]
    assert cap_before <= 128
    for g in (big, small):
        g.scale_box(SHRINK)
    pe_b = big.verlet_step_nve(0.005, 50)
    pe_s = small.verlet_step_nve(0.005, 50)
    assert small.stats()["list_capacity"] > cap_before
    pos_b, vel_b, _ = big.get_state()
    pos_s, vel_s, _ = small.get_state()
    if kw.get("list_kind") == "half":
        assert np.max(np.abs(pe_s - pe_b) / np.abs(pe_b)) <= 1e-10
        assert np.abs(pos_s - pos_b).max() <= 1e-9
    else:
        assert np.array_equal(pe_s, pe_b)
        assert np.array_equal(pos_s, pos_b) and np.array_equal(vel_s, vel_b)
    assert small.stats()["steps"] == big.stats()["steps"]
