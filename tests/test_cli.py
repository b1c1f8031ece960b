"""The ``pis_gpu_run -i`` command line on its error paths (no GPU: every case fails before a
device is touched), against the reference's ``main`` (src/main.rs:50-62): the error's display
string on stderr after ``Error: `` and exit status 1."""
import os
import subprocess

import pytest


@pytest.fixture(scope="module")
def cli(oracle_lib):
    from pis_gb300 import build
    build.build()
    return os.path.join(build.OUT_DIR, "pis_gpu_run")


def _run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=60)


def test_usage_without_input(cli):
    r = _run(cli)
    assert r.returncode == 2 and "usage:" in r.stderr


def test_missing_input_file(cli, tmp_path):
    path = str(tmp_path / "absent.pis")
    r = _run(cli, "-i", path)
    assert r.returncode == 1
    assert r.stderr == f"Error: Failed to open input file '{path}': No such file or directory (os error 2))\n"


@pytest.mark.parametrize("text,msg", [
    ("timestep 0.01\nrun -5\n", "Negative value -5 not allowed on line: 2"),
    ("# comment\nfrobnicate 1\n", "Invalid command frobnicate found line: 2"),
    ("pair_coeff 1 1 1.0 1.0\n", "Potential manager not initialized - missing pair_style or pair_coeff commands"),
    ("run 10\n", "Potential manager not initialized - missing pair_style or pair_coeff commands"),
    ("pair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0\nrun 10\n", "No atoms defined in input file"),
])
def test_input_errors_are_reported_like_the_reference(cli, tmp_path, text, msg):
    p = tmp_path / "in.pis"
    p.write_text(text)
    r = _run(cli, "--infile", str(p))
    assert r.returncode == 1
    assert r.stderr == f"Error: {msg}\n"
