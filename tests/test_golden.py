"""The committed golden fixtures against the CPU oracle (no GPU).

The fixtures were written by ``tests/golden/make_golden.py`` from the oracle after it had been
checked against the reference's example inputs and closed forms. The oracle is serial FP64 with
no fused multiply-adds, so rebuilding it from source on any machine must reproduce every stored
number bit for bit; a difference means the oracle changed and no longer matches what the
fixtures (and the GPU parity tests that read them) were pinned to.
"""
import os

import numpy as np
import pytest

from conftest import REFERENCE
from golden_data import FIXTURES, examples, load, neighbour_digest
from systems import to_oracle


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(oracle_lib, name):
    fx = load(name)
    o = to_oracle(fx["sys"])
    assert o.compute_potential() == fx["pe0"]
    assert np.array_equal(o.force, fx["force0"])
    assert o.kinetic_energy() == fx["ke0"]
    assert np.array_equal(o.virial_tensor(), fx["virial0"])
    count, crc, sha = neighbour_digest(*o.full_list())
    assert np.array_equal(count, fx["nl_count"]) and np.array_equal(crc, fx["nl_crc"])
    assert np.array_equal(sha, fx["nl_sha"])
    pe, ke = o.run_nve(float(fx["dt"]), int(fx["steps"]))
    assert np.array_equal(pe, fx["pe_steps"]) and np.array_equal(ke, fx["ke_steps"])
    assert np.array_equal(o.pos, fx["pos_end"]) and np.array_equal(o.vel, fx["vel_end"])


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_states_are_physical(name):
    fx = load(name)
    n = len(fx["pos"])
    L = np.diag(fx["h"])
    assert fx["pos"].shape == (n, 3) and fx["vel"].shape == (n, 3) and fx["force0"].shape == (n, 3)
    assert np.all(fx["pos"] >= 0) and np.all(fx["pos"] < L)
    # Newton's third law on the stored forces, NVE energy conservation over the stored run
    assert np.abs(fx["force0"].sum(axis=0)).max() <= 1e-11 * np.abs(fx["force0"]).sum()
    e = fx["pe_steps"] + fx["ke_steps"]
    assert np.abs(e - e[0]).max() <= 1e-3 * np.abs(fx["pe_steps"]).max()
    assert len(fx["pe_steps"]) == int(fx["steps"]) + 1
    assert np.all(fx["nl_count"] > 0) and fx["nl_sha"].shape == (32,)


def test_two_atom_data_file_answers(oracle_lib):
    import oracle
    ex = examples()["data.txt"]
    b = ex["box"]
    h = np.diag([b[1] - b[0], b[3] - b[2], b[5] - b[4]])
    table = {(int(r[0]), int(r[1])): tuple(r[2:]) for r in ex["table"]}
    assert table == {(1, 1): (0.238, 3.405, 8.5)}
    s = oracle.System(ex["positions"], ex["type_ids"], ex["masses"], h, table)
    assert np.array_equal(s.min_image(s.pos[1] - s.pos[0]), ex["min_image_rij"])
    assert s.compute_potential(manager=oracle.ALLPAIRS) == ex["pe_allpairs"]
    assert np.array_equal(s.force, ex["forces_allpairs"])


def test_two_type_data_file_answers(oracle_lib):
    import oracle
    ex = examples()["data_run.txt"]
    b = ex["box"]
    h = np.diag([b[1] - b[0], b[3] - b[2], b[5] - b[4]])
    table = {(int(r[0]), int(r[1])): tuple(r[2:]) for r in ex["table"]}
    # the PairCoeffs quirk: "1 2 0.6 1.1 2.8" overwrites (1,1); no cross entry
    assert table == {(1, 1): (2.0, 0.6, 1.1), (2, 2): (0.8, 1.2, 3.0)}
    assert ex["masses"] == [1.0, 2.0] and ex["type_ids"] == [1, 1, 2, 2] and ex["start_velocities"]
    for mgr in (oracle.OFFSET, oracle.ALLPAIRS):
        s = oracle.System(ex["positions"], ex["type_ids"], ex["masses"], h, table)
        assert s.compute_potential(manager=mgr) == ex["pe"]
        assert np.array_equal(s.force, ex["forces"])


@pytest.mark.parametrize("name,nc", [("example.txt", 5), ("argon4000.txt", 10)])
def test_argon_lattice_example_answers(oracle_lib, name, nc):
    import oracle
    from oracle.data_file import lattice_energy_per_atom
    from pis_gb300.lattice import fcc_lattice
    ex = examples()[name]
    assert ex["n_atoms"] == 4 * nc ** 3 and ex["cells"] == nc and ex["max_dev_from_generator"] <= 1e-12
    assert ex["pe_per_atom_closed_form"] == lattice_energy_per_atom(5.41, 0.238, 3.405, 8.5)
    L = 5.41 * nc
    s = oracle.System(fcc_lattice(5.41, nc, nc, nc), np.ones(4 * nc ** 3, np.int32), [39.948], np.eye(3) * L,
                      {(1, 1): (0.238, 3.405, 8.5)})
    pe = s.compute_potential()
    assert pe == pytest.approx(ex["pe"], rel=1e-12)
    assert np.abs(s.force).max() <= max(ex["max_abs_force"], 1e-13) * 10
    off, _ = s.full_list()
    assert np.all(np.diff(off) == ex["neighbours_per_atom"])


@pytest.mark.parametrize("name", ["data.txt", "data_run.txt", "example.txt", "example2.txt", "argon4000.txt"])
def test_examples_match_reference_files(oracle_lib, name):
    # where the reference sources are mounted: its example file is the one the answers came from
    import hashlib
    import oracle
    path = os.path.join(REFERENCE, "example", name)
    if not REFERENCE or not os.path.exists(path):
        pytest.skip("reference sources not mounted")
    ex = examples()[name]
    with open(path, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == ex["sha256"]
    d = oracle.read_data(path)
    assert d["n_atoms"] == ex["n_atoms"]
    assert sorted([ti, tj, *v] for (ti, tj), v in d["table"].items()) == ex["table"]
    if "positions" in ex:
        assert np.array_equal(np.asarray(d["positions"]), ex["positions"])
