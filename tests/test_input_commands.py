"""The input-file commands of the host driver (``pis_system_open``) against the reference's own
command tests (src/tests/command_tests.rs), case for case, through an input file as
``System::read`` (src/system.rs:48-94) feeds them. No GPU: ``pis_system_open`` parses and
contextualizes on the host.

Mapping of the reference's error variants onto status codes (include/pis_gpu.h):
MissingArgument, NegativeValue and InvalidArgument -> PIS_ERR_INVALID_ARGUMENT;
FloatParseError, IntParseError and UnknownCommand -> PIS_ERR_PARSE; PotentialNotInitialized ->
PIS_ERR_MISSING_POTENTIAL; InputFileError -> PIS_ERR_IO; AtomCountMismatch -> PIS_ERR_ATOM_COUNT.
The messages follow the variants' display strings (src/errors.rs).

Two differences of form, not of behaviour: the reference's tests call each command with an
argument list directly, so they reach an empty list; through a file, a line with fewer than two
tokens is skipped before any command sees it (src/system.rs:75-77), which these tests check
instead. And the reference's context fields are not exposed one by one: the tests observe them
through what ``pis_system_open`` builds from them (steps, timestep, ensemble, the pair table,
the dump step and file, the start velocities).
"""
import numpy as np
import pytest

DATA_1TYPE = """# two atoms

2 atoms
1 atom types

0.0 6.0 xlo xhi
0.0 6.0 ylo yhi
0.0 6.0 zlo zhi

Masses

1 2.0

Atoms

1 1 0.5 0.5 0.5
2 1 1.5 2.5 3.5
"""


@pytest.fixture(scope="module")
def pio(oracle_lib):
    from pis_gb300 import build
    build.build()
    from pis_gb300 import io
    return io


def _open(pio, tmp_path, text, data=None):
    if data is not None:
        d = tmp_path / "d.txt"
        d.write_text(data)
        text = text.replace("{data}", str(d))
    p = tmp_path / "in.pis"
    p.write_text(text)
    return pio.System(str(p))


def _err(pio, tmp_path, text, data=None):
    from pis_gb300 import PisError
    with pytest.raises(PisError) as e:
        _open(pio, tmp_path, text, data)
    return e.value


# ─── Command::from_str (command_tests.rs:49-70) ───────────────────────────────

@pytest.mark.parametrize("cmd", ["timestep 0.1", "run 10", "velocity all create 1.0", "fix f all nvt",
                                 "pair_style lj/cut 2.5", "dump d all atom 5 x.lammpstrj"])
def test_known_commands_are_accepted(pio, tmp_path, cmd):
    _open(pio, tmp_path, cmd + "\n").close()


@pytest.mark.parametrize("cmd", ["unknown_command", "TIMESTEP", "TimeStep"])
def test_unknown_commands_are_rejected(pio, tmp_path, cmd):
    e = _err(pio, tmp_path, "\n\n" + cmd + " 0.1\n")
    assert e.name == "PIS_ERR_PARSE"
    assert e.message == f"Invalid command {cmd} found line: 3"


def test_bare_command_lines_are_skipped(pio, tmp_path):
    # "timestep" / "run" / "velocity" with no argument never reach the command (system.rs:75-77)
    s = _open(pio, tmp_path, "timestep\nrun\nvelocity\n# comment\n\n   \n")
    assert s.steps == 100 and s.timestep == 0.01  # SimulationContext defaults
    s.close()


# ─── timestep (command_tests.rs:73-100) ───────────────────────────────────────

def test_timestep_sets_value(pio, tmp_path):
    s = _open(pio, tmp_path, "timestep 0.001\n")
    assert s.timestep == 0.001
    s.close()


@pytest.mark.parametrize("tok", ["notanumber", "one", "0.1.2"])
def test_timestep_invalid_float(pio, tmp_path, tok):
    e = _err(pio, tmp_path, f"timestep {tok}\n")
    assert e.name == "PIS_ERR_PARSE"
    assert e.message == f"Error parsing floating number from string {tok}: invalid float literal"


@pytest.mark.parametrize("tok,value", [("1e3", 1000.0), ("+.5", 0.5), ("5.", 5.0), ("inf", float("inf"))])
def test_timestep_accepts_rust_float_forms(pio, tmp_path, tok, value):
    s = _open(pio, tmp_path, f"timestep {tok}\n")
    assert s.timestep == value
    s.close()


# ─── run (command_tests.rs:102-137) ───────────────────────────────────────────

def test_run_sets_steps(pio, tmp_path):
    s = _open(pio, tmp_path, "run 5000\n")
    assert s.steps == 5000
    s.close()


def test_run_negative_value(pio, tmp_path):
    e = _err(pio, tmp_path, "run -1\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT"
    assert e.message == "Negative value -1 not allowed on line: 1"


@pytest.mark.parametrize("tok", ["1.5", "ten", "1e3"])
def test_run_non_integer(pio, tmp_path, tok):
    e = _err(pio, tmp_path, f"run {tok}\n")
    assert e.name == "PIS_ERR_PARSE"
    assert e.message == f"Error parsing integer number from string {tok}: invalid digit found in string"


def test_run_overflow(pio, tmp_path):
    e = _err(pio, tmp_path, "run 2147483648\n")
    assert e.message.endswith("number too large to fit in target type")


# ─── velocity (command_tests.rs:140-216) ──────────────────────────────────────

@pytest.mark.parametrize("line,t,seed", [("velocity all create 300.0 12345", 300.0, 12345),
                                         ("velocity all create 300.0", 300.0, 0),
                                         ("velocity all create 300.0 42 dist gaussian", 300.0, 42),
                                         ("velocity all create 300.0 42 dist uniform", 300.0, 42),
                                         ("velocity all create 300.0 dist gaussian", 300.0, 0)])
def test_velocity_create_sets_start_velocities(pio, tmp_path, line, t, seed):
    # the temperature and seed (0 when absent) reach the start velocities; the distribution
    # keyword is parsed and, as in the reference, does not change the draw
    s = _open(pio, tmp_path, f"read_data {{data}}\n{line}\n", DATA_1TYPE)
    _, vel, frc = s.state(2)
    s.close()
    assert np.array_equal(vel, pio.maxwell_boltzmann(np.full(2, 2.0), t, seed))
    assert not frc.any()


def test_velocity_after_read_data_overrides_defaults(pio, tmp_path):
    # read_data alone starts velocities at 300 K with seed 0 (commands.rs:374-383)
    s = _open(pio, tmp_path, "read_data {data}\n", DATA_1TYPE)
    _, vel, _ = s.state(2)
    s.close()
    assert np.array_equal(vel, pio.maxwell_boltzmann(np.full(2, 2.0), 300.0, 0))


@pytest.mark.parametrize("line", ["velocity all", "velocity all create", "velocity all create 300.0 42 dist"])
def test_velocity_missing_argument(pio, tmp_path, line):
    e = _err(pio, tmp_path, "\n" + line + "\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT"
    assert e.message == "Missing argument on line 2"


@pytest.mark.parametrize("args,bad", [("all set 300.0 42", "set"), ("all scale 300.0 42", "scale"),
                                      ("all create 300.0 42 badkeyword value", "badkeyword"),
                                      ("all create 300.0 42 dist lorentzian", "lorentzian")])
def test_velocity_invalid_argument(pio, tmp_path, args, bad):
    e = _err(pio, tmp_path, f"velocity {args}\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT"
    assert e.message == f"Invalid argument: {bad} at line: 1"


def test_velocity_bad_temperature_and_negative_seed(pio, tmp_path):
    e = _err(pio, tmp_path, "velocity all create hot\n")
    assert e.name == "PIS_ERR_PARSE" and "from string hot" in e.message
    e = _err(pio, tmp_path, "velocity all create 300.0 -3\n")
    assert e.message == "Negative value -3 not allowed on line: 1"


# ─── pair_style / pair_coeff (command_tests.rs:219-255, system.rs:120-168) ─────

def test_pair_style_and_coeffs_build_the_table(pio, tmp_path):
    s = _open(pio, tmp_path, "read_data {data}\npair_style lj/cut 10.0\npair_coeff 1 1 0.238 3.405 8.5\n"
                             "pair_coeff 1 2 0.150 3.100 7.5\npair_coeff 2 2 0.1 3.0\n", DATA_1TYPE)
    assert s.pairs() == {(1, 1): (0.238, 3.405, 8.5), (1, 2): (0.15, 3.1, 7.5), (2, 2): (0.1, 3.0, 10.0)}
    s.close()


def test_pair_coeff_rows_replace_and_unreachable_rows_are_dropped(pio, tmp_path):
    # a later (i, j) row replaces the earlier one; a row written with i > j is never looked up
    s = _open(pio, tmp_path, "pair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0\npair_coeff 1 1 2.0 1.0 3.0\n"
                             "pair_coeff 2 1 0.5 0.5 1.0\n")
    assert s.pairs() == {(1, 1): (2.0, 1.0, 3.0)}
    s.close()


def test_pair_style_replaces_the_data_file_table(pio, tmp_path):
    data = DATA_1TYPE.replace("Atoms\n", "PairCoeffs\n\n1 0.238 3.405 8.5\n\nAtoms\n")
    s = _open(pio, tmp_path, "read_data {data}\n", data)
    assert s.pairs() == {(1, 1): (0.238, 3.405, 8.5)}
    s.close()
    s = _open(pio, tmp_path, "read_data {data}\npair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0\n", data)
    assert s.pairs() == {(1, 1): (1.0, 1.0, 2.5)}
    s.close()


def test_pair_coeff_without_pair_style(pio, tmp_path):
    e = _err(pio, tmp_path, "pair_coeff 1 1 0.238 3.405 8.5\n")
    assert e.name == "PIS_ERR_MISSING_POTENTIAL"
    assert e.message == "Potential manager not initialized - missing pair_style or pair_coeff commands"


@pytest.mark.parametrize("coeff,name,msg", [
    ("1", "PIS_ERR_INVALID_ARGUMENT", "Missing argument on line 3"),
    ("1 x 1.0 1.0", "PIS_ERR_PARSE", "Error parsing integer number from string x: invalid digit found in string"),
    ("1 -2 1.0 1.0", "PIS_ERR_INVALID_ARGUMENT", "Negative value -2 not allowed on line: 3"),
    ("1 1 1.0", "PIS_ERR_INVALID_ARGUMENT", "Missing argument on line 3"),
    ("1 1 eps 1.0", "PIS_ERR_PARSE", "Error parsing floating number from string eps: invalid float literal"),
])
def test_pair_coeff_errors_in_argument_order(pio, tmp_path, coeff, name, msg):
    e = _err(pio, tmp_path, f"pair_style lj/cut 2.5\n\npair_coeff {coeff}\n")
    assert e.name == name and e.message == msg


def test_pair_style_errors(pio, tmp_path):
    e = _err(pio, tmp_path, "pair_style lj/long 2.5\n")
    assert e.name == "PIS_ERR_UNKNOWN_PAIR_STYLE" and e.message == "Unknown pair style: 'lj/long'"
    e = _err(pio, tmp_path, "\npair_style lj/cut\npair_coeff 1 1 1 1\n")
    # one token after the command: the line is a command with one argument, and contextualize
    # misses the global cutoff at the pair_style line
    assert e.name == "PIS_ERR_INVALID_ARGUMENT" and e.message == "Missing argument on line 2"


# ─── dump (command_tests.rs:257-294) ──────────────────────────────────────────

def test_dump_sets_step_and_file(pio, tmp_path):
    s = _open(pio, tmp_path, "dump my_dump all atom 100 output.lammpstrj\n")
    assert s.dump == (100, "output.lammpstrj")
    s.close()
    s = _open(pio, tmp_path, "run 1\n")
    assert s.dump == (1, "dump.lammpstrj")  # DumpArgs defaults
    s.close()


@pytest.mark.parametrize("args", ["my_dump all atom 100", "my_dump all atom", "my_dump all"])
def test_dump_missing_arguments(pio, tmp_path, args):
    e = _err(pio, tmp_path, f"dump {args}\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT" and e.message == "Missing argument on line 1"


@pytest.mark.parametrize("args,bad", [("my_dump all atom every output.lammpstrj", "every"),
                                      ("my_dump all atom 1.5 output.lammpstrj", "1.5")])
def test_dump_non_integer_step(pio, tmp_path, args, bad):
    e = _err(pio, tmp_path, f"dump {args}\n")
    assert e.name == "PIS_ERR_PARSE" and e.message.startswith(f"Error parsing integer number from string {bad}: ")


# ─── fix (command_tests.rs:296-356) ───────────────────────────────────────────

@pytest.mark.parametrize("line,ensemble", [("fix myfix all nvt temp 300.0 300.0 0.1", "NVT"),
                                           ("fix myfix all npt temp 300.0 300.0 0.1 iso 1.0 1.0 1.0", "NPT"),
                                           ("fix myfix all npt iso 2.0 2.0 0.5 temp 1.0 1.0 0.1", "NPT"),
                                           ("fix myfix all npt iso 2.0 2.0 0.5", "NVE"),
                                           ("fix myfix all nve temp 300.0 300.0 0.1", "NVE")])
def test_fix_selects_the_ensemble(pio, tmp_path, line, ensemble):
    # a thermostat needs nvt/npt; the barostat alone does not select NPT (simulation.rs:118-132)
    s = _open(pio, tmp_path, line + "\n")
    assert s.ensemble == ensemble
    s.close()


@pytest.mark.parametrize("args", ["myfix all", "myfix", "myfix all nvt temp 300.0 300.0"])
def test_fix_missing_arguments(pio, tmp_path, args):
    e = _err(pio, tmp_path, f"fix {args}\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT" and e.message == "Missing argument on line 1"


@pytest.mark.parametrize("args,bad", [("myfix all nvt badkeyword 300.0 300.0 0.1", "badkeyword"),
                                      ("myfix all npt unknown 1.0 1.0 1.0", "unknown")])
def test_fix_unknown_keyword(pio, tmp_path, args, bad):
    e = _err(pio, tmp_path, f"fix {args}\n")
    assert e.name == "PIS_ERR_INVALID_ARGUMENT" and e.message == f"Invalid argument: {bad} at line: 1"


# ─── read_data (command_tests.rs:358-502) ─────────────────────────────────────

def test_read_data_populates_atoms(pio, tmp_path):
    data = DATA_1TYPE.replace("2 atoms", "3 atoms").replace("2 1 1.5 2.5 3.5\n", "2 1 1.5 2.5 3.5\n3 1 4 5 5.5\n")
    s = _open(pio, tmp_path, "read_data {data}\n", data)
    pos, _, _ = s.state(3)
    s.close()
    assert np.array_equal(pos, [[0.5, 0.5, 0.5], [1.5, 2.5, 3.5], [4.0, 5.0, 5.5]])


def test_read_data_missing_file(pio, tmp_path):
    bad = "/nonexistent/path/to/file.data"
    e = _err(pio, tmp_path, f"read_data {bad}\n")
    assert e.name == "PIS_ERR_IO"
    assert e.message.startswith(f"Failed to open input file '{bad}': ")


def test_missing_input_file(pio, tmp_path):
    from pis_gb300 import PisError
    with pytest.raises(PisError) as e:
        pio.System(str(tmp_path / "none.pis"))
    assert e.value.name == "PIS_ERR_IO" and "No such file or directory (os error 2))" in e.value.message


@pytest.mark.parametrize("bad_id", [0, 5])
def test_read_data_invalid_atom_id(pio, tmp_path, bad_id):
    data = DATA_1TYPE.replace("2 1 1.5 2.5 3.5", f"{bad_id} 1 1.5 2.5 3.5")
    e = _err(pio, tmp_path, "read_data {data}\n", data)
    assert e.name == "PIS_ERR_ATOM_COUNT"
    assert e.message == f"Atom count mismatch: expected 2, found {bad_id}"


def test_read_data_velocities_switch_off_the_draw(pio, tmp_path):
    data = DATA_1TYPE + "\nVelocities\n\n1 0.1 0.2 0.3\n2 0.4 0.5 0.6\n"
    for cmd in ("read_data {data}\n", "velocity all create 50.0 9\nread_data {data}\n"):
        s = _open(pio, tmp_path, cmd, data)
        _, vel, _ = s.state(2)
        s.close()
        assert np.array_equal(vel, [[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]])


def test_reference_example_input(pio, monkeypatch):
    # the reference's own run script (example/input.pis, run from the reference's root as its
    # test_command.sh does): every command it uses parses, and contextualize builds its state
    import os
    from conftest import REFERENCE
    if not REFERENCE or not os.path.exists(os.path.join(REFERENCE, "example", "input.pis")):
        pytest.skip("reference sources not mounted")
    monkeypatch.chdir(REFERENCE)
    s = pio.System("example/input.pis")
    assert s.timestep == 0.25 and s.steps == 3000 and s.ensemble == "NPT"
    assert s.dump == (10, "dump.lammpstrj")
    assert s.pairs() == {(1, 1): (0.238, 3.405, 8.5)}  # the data file's PairCoeffs
    _, vel, _ = s.state(4000)
    s.close()
    assert np.array_equal(vel, pio.maxwell_boltzmann(np.full(4000, 39.948), 5.0, 12345))


def test_pair_style_supplies_the_table_a_data_file_lacks(pio, tmp_path):
    # example/example2.txt has no PairCoeffs: the input's pair_style / pair_coeff build the table,
    # the global cutoff filling the missing per-pair one
    import os
    from conftest import REFERENCE
    from golden_data import examples
    from pis_gb300.lattice import fcc_lattice
    data = os.path.join(REFERENCE, "example", "example2.txt")
    if not REFERENCE or not os.path.exists(data):
        pytest.skip("reference sources not mounted")
    ex = examples()["example2.txt"]
    s = _open(pio, tmp_path, f"read_data {data}\npair_style lj/cut 8.5\npair_coeff 1 1 0.238 3.405\n")
    assert s.pairs() == {(1, 1): (0.238, 3.405, 8.5)}
    pos, _, _ = s.state(ex["n_atoms"])
    s.close()
    assert np.abs(pos - fcc_lattice(ex["lattice_a"], 5, 5, 5)).max() <= ex["max_dev_from_generator"]
    s = _open(pio, tmp_path, f"read_data {data}\n")
    assert s.pairs() == {}
    s.close()
