"""Host-side logic of bench.py (no GPU): the synthetic replica mix and served job stream, the
drift fit, the clock-record summary, the traffic lookup, the peak fallback and the bounded
CPU-baseline sample."""
import json
import math

import numpy as np
import pytest

import bench


def test_replica_mix_matches_its_specification():
    # 512 replicas: N log-uniform in [500, 32000] -> k = round(cbrt(N / 4)) in [5, 20],
    # rho* in U[0.70, 0.95], T* in U[0.5, 1.5], one seed per replica
    jobs = bench.batch_jobs()
    assert len(jobs) == 512
    k = np.array([j.k for j in jobs])
    assert k.min() >= 5 and k.max() <= 20 and len(set(k)) >= 14
    assert all(0.70 <= j.rho <= 0.95 and 0.5 <= j.t_star <= 1.5 for j in jobs)
    assert len({j.seed for j in jobs}) == 512
    atoms = int(np.sum(4 * k ** 3))
    assert 3.3e6 < atoms < 4.5e6  # ~3.9M atoms, mean N ~ 7,600
    again = bench.batch_jobs()
    assert [(j.k, j.rho, j.t_star, j.seed) for j in jobs] == [(j.k, j.rho, j.t_star, j.seed) for j in again]


def test_served_stream_matches_its_specification():
    reqs = bench.serve_requests(2000, rate=200.0, step_scale=1.0)
    t = np.array([r[0] for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert 1 / 200 * 0.9 < np.mean(np.diff(t)) < 1 / 200 * 1.1  # Poisson arrivals at 200 jobs/s
    k = np.array([r[1].k for r in reqs])
    steps = np.array([r[1].steps for r in reqs])
    assert k.min() >= 6 and k.max() <= 40
    assert steps.min() >= 100 and steps.max() <= 5000 and abs(steps.mean() - 2550) < 150
    n = 4 * k.astype(np.int64) ** 3
    # log-uniform N: the median sits near the geometric mean of [1000, 256000]
    assert 0.6 < np.median(n) / math.sqrt(1000 * 256000) < 1.6
    scaled = bench.serve_requests(50, rate=200.0, step_scale=0.2)
    assert all(20 <= r[1].steps <= 1000 for r in scaled)


def test_drift_fit_recovers_a_linear_trend():
    chunk, n = 500, 1000
    t = np.arange(21) * chunk
    e = -5000.0 + 2.5e-4 * t + 1e-9 * np.sin(t)
    d = bench.drift_stats(e, n, chunk)
    assert d["drift_per_atom_per_1e4_steps"] == pytest.approx(2.5e-4 * 1e4 / n, rel=1e-6)
    assert d["max_abs_dev_per_atom"] == pytest.approx(2.5e-4 * 10000 / n, rel=1e-6)


def test_clock_summary():
    cs = bench.ClockSampler(0)
    cs.lines = ["0, 1965, 2070, 900.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
                "0, 1980, 2070, 910.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
                "0, 2010, 2070, 880.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
                "garbage"]
    s = cs.summary()
    assert s["sm_mhz"] == 1980 and s["sm_max_mhz"] == 2070 and s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 3
    cs.lines = ["0, 1500, 2070, 700, 0x8, Active, Not Active, Active, Not Active"]
    assert bench.ClockSampler.summary(cs)["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    cs.lines = []
    assert cs.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}


def test_traffic_lookup_scales_by_atoms():
    per_launch = bench.read_traffic("step_mixed", 256000)
    assert per_launch is not None and per_launch > 0
    assert bench.read_traffic("step_mixed", 2048000) == pytest.approx(8 * per_launch)
    assert bench.read_traffic("no_such_kernel", 1000) is None


def test_peaks_fall_back_without_measurements(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (bench.HBM_FALLBACK_GBS, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 7000.5}))
    assert bench.peaks() == (7000.5, "measured")


def test_cpu_sample_is_bounded(oracle_lib):
    import oracle
    pos, vel, L = bench.make_state(5, 3)
    v, steps, el = bench.cpu_sample(pos, vel, L, 2, oracle.PARALLEL, min_seconds=0.05, max_steps=500)
    assert v > 0 and steps >= 1 and (el >= 0.05 or steps == 500)
    v1, steps1, _ = bench.cpu_sample(pos, vel, L, 1, oracle.OFFSET, min_seconds=0.0, max_steps=3)
    assert steps1 == 1 and v1 > 0  # at least one whole step, even with no time bound


def test_reference_arm_state_equals_gpu_arm_state(oracle_lib):
    # the reference arm rebuilds the start state without the GPU library: lattice and velocities
    # equal the GPU arm's bit for bit
    import oracle
    from pis_gb300.lattice import lj_liquid
    pos, vel, L = lj_liquid(5, bench.RHO, bench.TSTAR, 1)
    a = (4.0 / bench.RHO) ** (1.0 / 3.0)
    assert np.array_equal(oracle.fcc_lattice(a, 5, 5, 5), pos)
    assert np.array_equal(oracle.maxwell_boltzmann(np.ones(len(pos)), bench.TSTAR / oracle.KB, 1), vel)
    assert L == a * 5


def test_reference_arm_does_not_load_the_gpu_library(oracle_lib, tmp_path):
    # a small reference-arm run in a fresh process: one JSON line, and libpis_gpu.so never mapped
    import subprocess
    import sys
    code = ("import argparse, bench\n"
            "a = argparse.Namespace(cells=6, equil=2, steps=1, warmup=1, gpus=1)\n"
            "bench.run_reference(a, 0, 1)\n"
            "print('mapped' if 'libpis_gpu' in open('/proc/self/maps').read() else 'unmapped')\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["config"]["atoms"] == 864 and rec["cpu_baseline"]["kind"] == "port"
    assert lines[-1] == "unmapped"


def test_roofline_bytes_follow_the_per_atom_step_count():
    # compulsory bytes of one atom-step: 4 per list entry + 100 (position 24, velocity 48, force 24,
    # type 4) -> about 410 B at 77.6 entries; flops 23 per entry + 3 per in-cutoff pair -> ~1,950
    assert bench.ALG_BYTES_PER_ATOM + 4 * 77.6 == pytest.approx(410.4)
    assert 77.6 * bench.FLOPS_PER_CANDIDATE + 55.3 * bench.FLOPS_PER_PAIR_ENERGY == pytest.approx(1950.7, abs=1)
    f = bench.pipe_fraction(2e12, 100.0, 40.0)
    assert f["achieved"] == pytest.approx(20.0) and f["frac"] == pytest.approx(0.5)
    assert bench.pipe_fraction(1.0, 0.0, 40.0) is None
