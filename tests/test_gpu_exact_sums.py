"""Exact, order-independent reductions of the FP64 path and the reference-order force kernel,
against the oracle on identical inputs.

The reference adds pair energies in its cell-walk order (LJVOffsetManager::compute_potential,
src/potentials/lennard_jones.rs:186-244). On the argon case that walk-order sum is itself
1.6e-12 (relative) away from the exactly rounded sum of the same terms, so no correct program
that adds in another order can promise 1e-12 against it. The FP64 path and the oracle therefore
also form one defined exact sum (terms quantised to 2^-104, added as integers, rounded once):
the per-pair energies are the reference's bit for bit, so the GPU's energy equals the oracle's
exact energy exactly, and the walk-order energy is within its own rounding of both.

PIS_OPT_REF_ORDER goes further: each atom's force terms are subtracted in the walk's order, so
forces equal the reference's bit for bit.
"""
import numpy as np
import pytest

from systems import argon, liquid, melted, to_gpu, to_oracle

pytestmark = pytest.mark.gpu

SIGMA = 3.405


def displaced(sysd, frac, seed):
    rng = np.random.default_rng(seed)
    out = dict(sysd)
    a = sysd["h"][0, 0] / round((len(sysd["pos"]) / 4) ** (1 / 3))
    out["pos"] = np.mod(sysd["pos"] + rng.normal(0, frac * a, sysd["pos"].shape), sysd["h"][0, 0])
    return out


@pytest.fixture(scope="module")
def argon_disp(oracle_lib, cuda_lib):
    return displaced(argon(), 0.03, 11)


@pytest.fixture(scope="module")
def liquid_melt(oracle_lib, cuda_lib):
    return melted(liquid(nc=6), steps=300, dt=0.005)


@pytest.mark.parametrize("case", ["argon", "liquid"])
@pytest.mark.parametrize("variant", ["half", "full", "full_lanes8", "ref_order"])
def test_energy_equals_oracle_exact_sum(argon_disp, liquid_melt, case, variant):
    s, skin = (argon_disp, 0.3 * SIGMA) if case == "argon" else (liquid_melt, 0.3)
    o = to_oracle(s)
    pe_exact, pe_walk = o.compute_potential_exact()
    kw = dict(half=dict(list_kind="half"), full=dict(list_kind="full"),
              full_lanes8=dict(list_kind="full", lanes=8), ref_order=dict(ref_order=True))[variant]
    g = to_gpu(s, "fp64", skin=skin, **kw)
    pe, f = g.compute_potential()
    assert pe == pe_exact  # same pair terms, same defined sum
    assert abs(pe - pe_walk) <= 1e-11 * abs(pe_walk)  # the walk-order sum's own rounding
    ke, w = g.reductions()
    assert ke == o.kinetic_energy_exact()
    if variant == "ref_order":
        assert np.array_equal(f, o.force)  # the walk's forces, bit for bit
        assert np.array_equal(w, o.virial_tensor_exact())
    else:
        assert np.linalg.norm(f - o.force) <= 1e-12 * np.linalg.norm(o.force)
        scale = np.abs(s["pos"]).max() * np.abs(o.force).sum()
        assert np.abs(w - o.virial_tensor_exact()).max() <= 1e-12 * scale


def test_walk_order_sum_deviation_is_the_references_own(argon_disp):
    # the oracle's walk-order energy against the exact sum of the same terms: the size of the
    # reference's own summation error, which bounds any comparison against its printed energy
    o = to_oracle(argon_disp)
    pe_exact, pe_walk = o.compute_potential_exact()
    assert pe_exact != pe_walk
    assert abs(pe_exact - pe_walk) <= 1e-11 * abs(pe_exact)


def test_ref_order_trajectory_bit_identical_100_steps(liquid_melt):
    # 864-atom liquid (6 reference cells per axis), 100 NVE steps with list rebuilds: positions,
    # velocities and every step's energy equal the oracle's
    o = to_oracle(liquid_melt)
    pe_ref, ke_ref, _ = o.run_nve_exact(0.005, 100)
    g = to_gpu(liquid_melt, "fp64", ref_order=True)
    pe0, _ = g.compute_potential(want_forces=False)
    pe = g.verlet_step_nve(0.005, 100)
    ke, _ = g.reductions()
    pos, vel, frc = g.get_state()
    assert pe0 == pe_ref[0]
    assert np.array_equal(pe, pe_ref[1:])
    assert ke == ke_ref[-1]
    assert np.array_equal(pos, o.pos) and np.array_equal(vel, o.vel) and np.array_equal(frc, o.force)
    assert g.stats()["rebuilds"] >= 2


def test_ref_order_mixture_per_pair_cutoffs(oracle_lib, cuda_lib):
    # two types with per-pair cutoffs: the reference cells follow the largest cutoff
    s = melted(liquid(nc=6), steps=50, dt=0.005)
    n = len(s["pos"])
    s["types"] = (np.arange(n) % 2 + 1).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (1.0, 1.0, 2.5), (1, 2): (0.8, 1.1, 2.2), (2, 2): (1.2, 0.9, 2.0)}
    o = to_oracle(s)
    pe_ref, ke_ref, _ = o.run_nve_exact(0.004, 40)
    g = to_gpu(s, "fp64", ref_order=True)
    pe0, _ = g.compute_potential(want_forces=False)
    pe = g.verlet_step_nve(0.004, 40)
    pos, vel, _ = g.get_state()
    assert pe0 == pe_ref[0] and np.array_equal(pe, pe_ref[1:])
    assert np.array_equal(pos, o.pos) and np.array_equal(vel, o.vel)


def test_ref_order_refuses_small_and_half(oracle_lib, cuda_lib):
    from pis_gb300._ffi import PisError
    s = liquid(nc=4)  # 6.7 sigma: 2 cells of the cutoff per axis
    with pytest.raises(PisError) as e:
        to_gpu(s, "fp64", ref_order=True)
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
    with pytest.raises(PisError) as e:
        to_gpu(liquid(nc=6), "fp64", ref_order=True, list_kind="half")
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
    with pytest.raises(PisError) as e:
        to_gpu(liquid(nc=6), "mixed", ref_order=True)
    assert e.value.name == "PIS_ERR_UNSUPPORTED"
