"""The host driver (System::read -> contextualize -> run) and the pis_gpu_run CLI on the GPU:
thermo lines and dumps against the oracle's NVE run on the same input."""
import os
import subprocess

import numpy as np
import pytest

from systems import liquid, melted, to_oracle

pytestmark = pytest.mark.gpu

KB = 0.0083144621


def _write_inputs(tmp_path, s, steps=20, dt=0.005, extra=""):
    from pis_gb300.io import write_data
    L = s["h"][0, 0]
    data = tmp_path / "liquid.txt"
    write_data(str(data), s["pos"], s["types"], s["masses"], [0, L, 0, L, 0, L], s["table"], s["vel"])
    inp = tmp_path / "in.pis"
    dump = tmp_path / "traj.lammpstrj"
    inp.write_text(f"timestep {dt}\nread_data {data}\n{extra}dump d1 all atom 10 {dump}\nrun {steps}\n")
    return inp, dump


def _parse_thermo(path):
    lines = open(path).read().split("\n")
    first = lines[0].split()
    rows = [list(map(float, l.split())) for l in lines[1:] if l.strip()]
    return float(first[1]), np.array(rows)


def test_system_run_matches_oracle(tmp_path, oracle_lib, cuda_lib):
    from pis_gb300.io import System
    s = melted(liquid(nc=6, seed=17), 100, 0.005)
    inp, dump = _write_inputs(tmp_path, s)
    sysm = System(str(inp), precision="fp64")
    thermo = tmp_path / "thermo.txt"
    sysm.run(str(thermo))
    pe0, rows = _parse_thermo(thermo)
    o = to_oracle(s)
    pe_ref, ke_ref = o.run_nve(0.005, 20)
    assert abs(pe0 - pe_ref[0]) <= 1e-12 * abs(pe_ref[0])
    assert rows.shape == (20, 6) and list(rows[:, 0]) == list(range(1, 21))
    # thermo prints {:.3}: compare at that resolution
    assert np.allclose(rows[:, 1], np.round(pe_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 2], np.round(ke_ref[1:], 3), rtol=0, atol=1.5e-3)
    n = len(s["pos"])
    assert np.allclose(rows[:, 4], np.round(2 * ke_ref[1:] / (3 * n * KB), 3), rtol=0, atol=1.5e-3)
    # pressure on the final state: (2 KE + tr sum r F^T) / (3 V)
    p_ref = o.pressure(ke_ref[-1])
    assert abs(rows[-1, 5] - round(p_ref, 3)) <= 1.5e-3
    # the dump holds steps 0, 10 and 20; step 20 positions equal the oracle's
    text = open(dump).read().split("ITEM: TIMESTEP\n")[1:]
    assert [int(t.split("\n")[0]) for t in text] == [0, 10, 20]
    last = text[-1].split("ITEM: ATOMS id type x y z\n")[1].strip().split("\n")
    pos = np.array([[float(x) for x in l.split()[2:]] for l in last])
    d = pos - o.pos
    d -= s["h"][0, 0] * np.round(d / s["h"][0, 0])
    assert np.abs(d).max() <= 1e-9


def test_cli_matches_library_run(tmp_path, oracle_lib, cuda_lib):
    from pis_gb300 import build
    from pis_gb300.io import System
    s = melted(liquid(nc=6, seed=18), 50, 0.005)
    inp, _ = _write_inputs(tmp_path, s, steps=10)
    t_lib = tmp_path / "lib.txt"
    System(str(inp), precision="fp64").run(str(t_lib))
    t_cli = tmp_path / "cli.txt"
    cli = os.path.join(build.OUT_DIR, "pis_gpu_run")
    r = subprocess.run([cli, "-i", str(inp), "--thermo", str(t_cli)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert open(t_cli).read() == open(t_lib).read()


def _check_nvt_thermo(rows, pe0, s, o, pe_ref, ke_ref, ham_ref, steps):
    n = len(s["pos"])
    assert abs(pe0 - pe_ref[0]) <= 1e-12 * abs(pe_ref[0])
    assert rows.shape == (steps, 6) and list(rows[:, 0]) == list(range(1, steps + 1))
    # thermo prints {:.3}: compare at that resolution
    assert np.allclose(rows[:, 1], np.round(pe_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 2], np.round(ke_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 3], np.round(ham_ref[1:], 3), rtol=0, atol=1.5e-3)
    assert np.allclose(rows[:, 4], np.round(2 * ke_ref[1:] / (3 * n * KB), 3), rtol=0, atol=1.5e-3)
    assert abs(rows[-1, 5] - round(o.pressure(ke_ref[-1]), 3)) <= 1.5e-3


def test_nvt_run_matches_oracle(tmp_path, oracle_lib, cuda_lib):
    # verlet_step_nvt_nhc and the NVT branch of Simulation::run (src/potentials/potential.rs:35-58,
    # src/simulation.rs:41-115) against the oracle's restatement: per-step PE, KE, Hamiltonian,
    # T and the final P, with the thermostat ramping its target from T* = 1.0 to 1.2 (tau* = 0.5)
    from pis_gb300.io import System
    s = melted(liquid(nc=6, seed=21), 100, 0.005)
    t0, t1, tau, steps = 1.0 / KB, 1.2 / KB, 0.5, 30
    inp, _ = _write_inputs(tmp_path, s, steps=steps, extra=f"fix f1 all nvt temp {t0!r} {t1!r} {tau}\n")
    sysm = System(str(inp), precision="fp64")
    assert sysm.ensemble == "NVT"
    thermo = tmp_path / "thermo.txt"
    sysm.run(str(thermo))
    pe0, rows = _parse_thermo(thermo)
    o = to_oracle(s)
    pe_ref, ke_ref, ham_ref, _ = o.run_nvt(0.005, steps, t0, t1, tau)
    _check_nvt_thermo(rows, pe0, s, o, pe_ref, ke_ref, ham_ref, steps)


def test_nvt_runs_and_thermostats(tmp_path, oracle_lib, cuda_lib):
    from pis_gb300.io import System
    s = liquid(nc=6, seed=19)
    # reference units: T* = KB * T, so T = 1.2 / KB targets T* = 1.2
    t_target = 1.2 / KB
    inp, _ = _write_inputs(tmp_path, s, steps=200, extra=f"fix f1 all nvt temp {t_target} {t_target} 0.1\n")
    sysm = System(str(inp), precision="mixed")
    assert sysm.ensemble == "NVT"
    thermo = tmp_path / "thermo.txt"
    sysm.run(str(thermo))
    _, rows = _parse_thermo(thermo)
    assert rows.shape[0] == 200 and np.all(np.isfinite(rows))
