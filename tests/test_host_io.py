"""The C++ host side (include/pis_host.h) without a GPU: data-file reader parity with the oracle's
restatement of the reference reader, Rust-style float formatting, restart round trip, velocity
generator, and input-file parsing."""
import os

import numpy as np
import pytest

from conftest import reference_file


@pytest.fixture(scope="module")
def io(oracle_lib):
    from pis_gb300 import build
    build.build()
    from pis_gb300 import io as pio
    return pio


@pytest.mark.parametrize("name", ["argon4000.txt", "example.txt", "example2.txt", "data.txt", "data_run.txt"])
def test_reader_matches_oracle_reader(io, name):
    import oracle
    path = reference_file("example", name)
    a = io.read_data(path)
    b = oracle.read_data(path)
    for k in ("n_atoms", "xlo", "xhi", "ylo", "yhi", "zlo", "zhi", "start_velocities", "table"):
        assert a[k] == b[k], k
    assert np.array_equal(a["masses"], b["masses"])
    assert np.array_equal(a["type_ids"], b["type_ids"])
    assert np.array_equal(a["positions"], b["positions"])
    assert np.array_equal(a["velocities"], b["velocities"])


def test_reader_errors(io, tmp_path):
    from pis_gb300 import PisError
    p = tmp_path / "bad.txt"
    p.write_text("2 atoms\n1 atom types\n\nMasses\n1 1.0\n\nAtoms\n1 1 0 0 0\n3 1 1 1 1\n")
    with pytest.raises(PisError) as e:
        io.read_data(str(p))
    assert e.value.name == "PIS_ERR_ATOM_COUNT"
    p.write_text("1 atoms\n1 atom types\n\nAtoms\n1 1 0 x 0\n")
    with pytest.raises(PisError) as e:
        io.read_data(str(p))
    assert e.value.name == "PIS_ERR_PARSE"
    with pytest.raises(PisError) as e:
        io.read_data(str(tmp_path / "missing.txt"))
    assert e.value.name == "PIS_ERR_IO"


@pytest.mark.parametrize("v,s", [(1.0, "1"), (0.1, "0.1"), (-0.0, "-0"), (0.0, "0"), (1e21, "1000000000000000000000"),
                                 (1e-7, "0.0000001"), (2.705, "2.705"), (18.935000000000002, "18.935000000000002"),
                                 (float("nan"), "NaN"), (float("inf"), "inf"), (-1.5e-3, "-0.0015")])
def test_format_like_rust(io, v, s):
    assert io.format_f64(v) == s


def test_format_round_trips(io):
    rng = np.random.default_rng(0)
    for v in np.concatenate([rng.normal(0, 10, 200), rng.normal(0, 1e-5, 50), rng.normal(0, 1e8, 50)]):
        assert float(io.format_f64(v)) == v


def test_format_is_the_shortest_positional(io):
    # the shortest round-trip digits, nearest the value, positional: numpy's Dragon4 in unique mode
    # gives the same string over the whole range (subnormals and the largest values included)
    rng = np.random.default_rng(1)
    vals = np.concatenate([rng.normal(0, 10, 300), 10.0 ** rng.uniform(-320, 308, 300) * rng.choice([-1, 1], 300),
                           [5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, 0.1, 0.3, 1 / 3]])
    for v in vals:
        assert io.format_f64(float(v)) == np.format_float_positional(v, unique=True, trim="-")


def test_restart_round_trip(io, tmp_path):
    rng = np.random.default_rng(3)
    n = 50
    pos = rng.uniform(0, 10, (n, 3))
    vel = rng.normal(0, 1, (n, 3))
    types = rng.integers(1, 3, n).astype(np.int32)
    path = str(tmp_path / "restart.txt")
    io.write_data(path, pos, types, [1.0, 2.5], [0, 10, 0, 10, 0, 10], {(1, 1): (1.0, 1.0, 2.5)}, vel)
    d = io.read_data(path)
    assert np.array_equal(d["positions"], pos) and np.array_equal(d["velocities"], vel)
    assert np.array_equal(d["type_ids"], types) and not d["start_velocities"]
    assert d["table"] == {(1, 1): (1.0, 1.0, 2.5)}


def test_maxwell_boltzmann(io):
    m = np.full(1000, 39.948)
    v = io.maxwell_boltzmann(m, 100.0, 5)
    assert np.array_equal(v, io.maxwell_boltzmann(m, 100.0, 5))
    assert not np.array_equal(v, io.maxwell_boltzmann(m, 100.0, 6))
    assert np.abs((m[:, None] * v).sum(0)).max() < 1e-9
    ke = 0.5 * np.sum(m[:, None] * v * v)
    assert 2 * ke / (3 * 1000 * 0.0083144621) == pytest.approx(100.0, rel=1e-12)
    assert abs(np.std(v) / np.sqrt(0.0083144621 * 100 / 39.948) - 1) < 0.05


def test_input_file_parsing(io, tmp_path):
    from pis_gb300 import PisError
    d = tmp_path / "d.txt"
    d.write_text("4 atoms\n1 atom types\n0 10 xlo xhi\n0 10 ylo yhi\n0 10 zlo zhi\nMasses\n1 1.0\n"
                 "Atoms\n1 1 1 1 1\n2 1 2 2 2\n3 1 5 5 5\n4 1 6 6 6\n")
    inp = tmp_path / "in.pis"
    inp.write_text(f"timestep 0.002 # comment\nread_data {d}\nvelocity all create 50.0 7\n"
                   "pair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0\nfix f all nvt temp 1.0 2.0 0.5\n"
                   f"dump d all atom 5 {tmp_path / 'x.lammpstrj'}\nrun 30\n")
    s = io.System(str(inp))
    assert s.steps == 30 and s.timestep == 0.002 and s.ensemble == "NVT"
    s.close()
    inp.write_text("frobnicate 1 2\n")
    with pytest.raises(PisError) as e:
        io.System(str(inp))
    assert e.value.name == "PIS_ERR_PARSE"
    inp.write_text("pair_coeff 1 1 1.0 1.0\n")
    with pytest.raises(PisError) as e:
        io.System(str(inp))
    assert e.value.name == "PIS_ERR_MISSING_POTENTIAL"


_HEAD = "# t\n2 atoms\n1 atom types\n0 4 xlo xhi\n0 4 ylo yhi\n0 4 zlo zhi\n"


@pytest.mark.parametrize("text,status", [
    ("x atoms\n", "PIS_ERR_PARSE"),
    ("-2 atoms\n", "PIS_ERR_INVALID_ARGUMENT"),
    ("99999999999 atoms\n", "PIS_ERR_PARSE"),
    ("2 atoms\n1 atom types\n0 a xlo xhi\n", "PIS_ERR_PARSE"),
    (_HEAD + "Masses\n1\n", "PIS_ERR_INVALID_ARGUMENT"),
    (_HEAD + "Masses\n0 1.0\n", "PIS_ERR_INVALID_ATOM_TYPE"),
    (_HEAD + "Masses\n2 1.0\n", "PIS_ERR_INVALID_ATOM_TYPE"),
    (_HEAD + "Masses\n1 heavy\n", "PIS_ERR_PARSE"),
    (_HEAD + "PairCoeffs\n1\n", "PIS_ERR_INVALID_ARGUMENT"),
    (_HEAD + "PairCoeffs\n1 2 x 1.0\n", "PIS_ERR_PARSE"),
    (_HEAD + "PairCoeffs\n1 a 1.0 1.0\n", "PIS_ERR_PARSE"),
    (_HEAD + "PairCoeffs\n-1 1.0 1.0\n", "PIS_ERR_INVALID_ARGUMENT"),
    (_HEAD + "Atoms\n3 1 0 0 0\n", "PIS_ERR_ATOM_COUNT"),
    (_HEAD + "Atoms\n\n1 1 0 0\n", "PIS_ERR_INVALID_ARGUMENT"),
    (_HEAD + "Atoms\n1 -1 0 0 0\n", "PIS_ERR_INVALID_ARGUMENT"),
    (_HEAD + "Atoms\n1 1 0 0 0\nVelocities\n0 0 0 0\n", "PIS_ERR_ATOM_COUNT"),
    (_HEAD + "Atoms\n1 1 0 0 0\nVelocities\n1 0 0 fast\n", "PIS_ERR_PARSE"),
])
def test_reader_error_messages_match_oracle(io, tmp_path, text, status):
    # the library's reader and the oracle's restatement fail on the same line with the same
    # PisError display string (src/errors.rs; 0-based data-file line numbers)
    import oracle
    from oracle.data_file import DataFileError
    from pis_gb300 import PisError
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(PisError) as e:
        io.read_data(str(p))
    with pytest.raises(DataFileError) as o:
        oracle.read_data(str(p))
    assert e.value.name == status
    assert e.value.message == str(o.value)
