"""The CUDA path (through the C ABI) against the committed golden fixtures.

The fixtures hold the CPU oracle's FP64 answers, pinned to the reference's example inputs when
they were written, so these checks need neither the oracle nor the reference at run time. Bars
as in the oracle parity tests: FP64 forces, energy and virial within 1e-12 relative (normwise
for vectors); neighbour sets identical (compared through per-atom CRC-32 and a SHA-256 of the
sorted rows); the stored NVE run reproduced to 1e-9 sigma in position and 1e-11 relative in
per-step energy; mixed precision force RMS within 1e-5 relative.
"""
import numpy as np
import pytest

from golden_data import FIXTURES, examples, load, neighbour_digest
from systems import to_gpu

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
# reduced-unit mixed-precision checks run on the liquid and the mixture
MIXED_FIXTURES = ("liquid864_melt", "mixture864")


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _sigma_max(fx):
    return float(np.max(fx["table"][:, 3]))


@pytest.mark.parametrize("name", FIXTURES)
def test_fp64_forces_energy_virial_lists(cuda_lib, name):
    fx = load(name)
    s = fx["sys"]
    g = to_gpu(s, "fp64", skin=float(fx["skin"]))
    pe, f = g.compute_potential()
    assert abs(pe - fx["pe0"]) <= FP64_TOL * abs(fx["pe0"])
    assert rel_norm(f, fx["force0"]) <= FP64_TOL
    ke, w = g.reductions()
    assert abs(ke - fx["ke0"]) <= FP64_TOL * abs(fx["ke0"])
    scale = np.abs(s["pos"]).max() * np.abs(fx["force0"]).sum()
    assert np.abs(w - fx["virial0"]).max() <= FP64_TOL * scale
    count, crc, sha = neighbour_digest(*g.neighbour_list())
    assert np.array_equal(count, fx["nl_count"])
    assert np.array_equal(crc, fx["nl_crc"]) and np.array_equal(sha, fx["nl_sha"])
    g.close()


@pytest.mark.parametrize("name", FIXTURES)
def test_fp64_trajectory(cuda_lib, name):
    fx = load(name)
    s = fx["sys"]
    steps = int(fx["steps"])
    g = to_gpu(s, "fp64", skin=float(fx["skin"]))
    g.compute_potential()
    pe = g.verlet_step_nve(float(fx["dt"]), steps)
    pos, vel, _ = g.get_state()
    g.close()
    ref = fx["pe_steps"][1:]
    assert np.max(np.abs(pe - ref) / np.abs(ref)) <= 1e-11
    L = np.diag(fx["h"])
    d = pos - fx["pos_end"]
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-9 * _sigma_max(fx)
    assert rel_norm(vel, fx["vel_end"]) <= 1e-10


@pytest.mark.parametrize("name", MIXED_FIXTURES)
def test_mixed_forces_and_energies(cuda_lib, name):
    fx = load(name)
    g = to_gpu(fx["sys"], "mixed")
    pe, f = g.compute_potential()
    rms = np.sqrt(np.sum((f - fx["force0"]) ** 2) / np.sum(fx["force0"] ** 2))
    assert rms <= 1e-5, rms
    assert abs(pe - fx["pe0"]) <= 1e-5 * abs(fx["pe0"])
    steps = min(int(fx["steps"]), 50)
    e = g.verlet_step_nve(float(fx["dt"]), steps)
    g.close()
    ref = fx["pe_steps"][1:steps + 1]
    assert np.max(np.abs(e - ref) / np.abs(ref)) <= 1e-4


def test_example_lattice_answers(cuda_lib):
    # the reference's 500-atom argon example (FCC a = 5.41, rc = 8.5), generated in its atom
    # order: 54 neighbours per atom, the recorded lattice energy, forces cancelling to roundoff
    from pis_gb300.lattice import fcc_lattice
    ex = examples()["example.txt"]
    nc = ex["cells"]
    pos = fcc_lattice(ex["lattice_a"], nc, nc, nc)
    n = len(pos)
    s = dict(pos=pos, vel=np.zeros((n, 3)), types=np.ones(n, np.int32), masses=np.array([39.948]),
             h=np.eye(3) * (ex["lattice_a"] * nc), table={(1, 1): (0.238, 3.405, 8.5)})
    g = to_gpu(s, "fp64", skin=1.0)
    off, idx = g.neighbour_list()
    assert np.all(np.diff(off) == ex["neighbours_per_atom"])
    pe, f = g.compute_potential()
    g.close()
    assert abs(pe - ex["pe"]) <= FP64_TOL * abs(ex["pe"])
    assert abs(pe / n - ex["pe_per_atom_closed_form"]) <= 1e-11 * abs(ex["pe_per_atom_closed_form"])
    assert np.abs(f).max() < 1e-12
