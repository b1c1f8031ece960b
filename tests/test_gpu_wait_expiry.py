"""The bounded waits of the bulk-copy (TMA) force variants run out and report, on correct kernels.

The bulk-copy list stream (PIS_OPT_LIST_TMA) and the neighbour-cell tiles (PIS_OPT_TILE) wait on
mbarriers for their copies; every wait has a poll budget. pis_gpu_set_wait_limit(ctx, 0) gives the
pipeline waits no polls at all, so each one expires at once: the block stops its pipeline, waits
with the full budget for its own copies still in flight, flags the slot, and the call returns
PIS_ERR_TIMEOUT. Nothing is broken on purpose: the copies all complete, and a context with the
default budget evaluates the same state normally afterwards.
"""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def states(oracle_lib, cuda_lib):
    small = melted(liquid(nc=8), steps=50, dt=0.005)
    # the tiles serve chunks that lie in one cell row: 26 cells per row (340,736 atoms), an FCC
    # lattice displaced at random
    big = liquid(nc=44)
    rng = np.random.default_rng(4)
    L = big["h"][0, 0]
    big["pos"] = np.mod(big["pos"] + rng.normal(0, 0.05, big["pos"].shape), L)
    return {"small": small, "big": big}


@pytest.mark.parametrize("case,kw", [("small", dict(tma=True, batch=8)), ("small", dict(tma=True, batch=16)),
                                     ("big", dict(tiles=True))])
def test_expired_wait_returns_timeout_and_the_gpu_stays_usable(states, case, kw):
    from pis_gb300._ffi import PisError
    state = states[case]
    ref = to_gpu(state, "mixed", **kw)
    pe_ref, f_ref = ref.compute_potential()
    g = to_gpu(state, "mixed", wait_limit=0, **kw)
    with pytest.raises(PisError) as e:
        g.compute_potential()
    assert e.value.name == "PIS_ERR_TIMEOUT"
    g.close()
    # the same state with the default budget afterwards: the usual result
    again = to_gpu(state, "mixed", **kw)
    pe, f = again.compute_potential()
    assert pe == pe_ref and np.array_equal(f, f_ref)
