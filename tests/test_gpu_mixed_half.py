"""The mixed path on a Newton-3 half list (PIS_LIST_HALF with PIS_PRECISION_MIXED), a measured
variant: each pair is evaluated once with the FP32 pair arithmetic of the full-list kernel, and
its force on j is added with FP64 atomics. It must meet the mixed path's bar against FP64 and
follow the full-list mixed run closely; the order of the atomic additions changes between
launches, so results agree to FP64 rounding of the force sums, not bit for bit."""
import numpy as np
import pytest

from systems import liquid, melted, to_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def liquid_melt(oracle_lib, cuda_lib):
    return melted(liquid(nc=6, seed=5), steps=200, dt=0.005)


def rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


@pytest.mark.parametrize("kahan", [False, True])
def test_half_list_forces_and_energy_against_fp64(liquid_melt, kahan):
    f64 = to_gpu(liquid_melt, "fp64")
    pe64, F64 = f64.compute_potential()
    g = to_gpu(liquid_melt, "mixed", list_kind="half", mixed_kahan=kahan)
    pe, f = g.compute_potential()
    assert rms(f, F64) <= 1e-5
    assert abs(pe - pe64) <= 1e-6 * abs(pe64)
    # half the entries of the full list
    full = to_gpu(liquid_melt, "mixed", list_kind="full")
    full.compute_potential()
    assert abs(2 * g.stats()["list_entries"] - full.stats()["list_entries"]) <= 0.01 * full.stats()["list_entries"]
    # the same state evaluated twice: equal up to the order of the atomic additions
    pe2, f2 = g.compute_potential()
    assert pe2 == pe and np.abs(f2 - f).max() <= 1e-12 * np.abs(f).max()


def test_half_list_run_follows_full_list_run(liquid_melt):
    a = to_gpu(liquid_melt, "mixed", list_kind="half")
    b = to_gpu(liquid_melt, "mixed", list_kind="full")
    a.compute_potential(want_forces=False)
    b.compute_potential(want_forces=False)
    ea = a.verlet_step_nve(0.005, 60)
    eb = b.verlet_step_nve(0.005, 60)
    assert np.max(np.abs(ea - eb) / np.abs(eb)) <= 1e-5
    assert a.stats()["rebuilds"] >= 2
    pa, _, _ = a.get_state()
    pb, _, _ = b.get_state()
    L = liquid_melt["h"][0, 0]
    d = pa - pb
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-4


def test_half_list_two_types(oracle_lib, cuda_lib):
    s = melted(liquid(nc=6, seed=6), steps=50, dt=0.005)
    n = len(s["pos"])
    s["types"] = (np.arange(n) % 2 + 1).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (1.0, 1.0, 2.5), (1, 2): (0.8, 1.1, 2.2), (2, 2): (1.2, 0.9, 2.0)}
    pe64, F64 = to_gpu(s, "fp64").compute_potential()
    pe, f = to_gpu(s, "mixed", list_kind="half").compute_potential()
    assert rms(f, F64) <= 1e-5 and abs(pe - pe64) <= 1e-6 * abs(pe64)


def test_half_list_refuses_other_mixed_variants(liquid_melt):
    from pis_gb300._ffi import PisError
    for kw in (dict(lanes=8), dict(tma=True), dict(tiles=True)):
        with pytest.raises(PisError) as e:
            to_gpu(liquid_melt, "mixed", list_kind="half", **kw)
        assert e.value.name == "PIS_ERR_UNSUPPORTED"
