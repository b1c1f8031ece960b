"""Batched replicas and the served-job loop (pis_batch_*, pis_serve_run) through the C ABI.

Each slot's arithmetic is independent of every other slot's, so a job must give bit-identical
results alone and in any mix (mixed precision: the full-list path has no atomics). FP64 replicas
are checked against the oracle, and a replica with injected NaN velocities must fail alone.
"""
import numpy as np
import pytest

from systems import liquid, to_oracle

pytestmark = pytest.mark.gpu

JOBS = [(5, 0.95, 0.5, 11), (6, 0.80, 1.2, 12), (7, 0.70, 0.9, 13), (5, 0.85, 1.5, 14), (8, 0.8442, 0.72, 15)]


def _batch(precision="mixed", atoms=20000, slots=8):
    from pis_gb300.batch import Batch
    return Batch(atoms, slots, 0, precision=precision)


def _run_alone(k, rho, t, seed, steps):
    from pis_gb300.batch import lj_job
    b = _batch()
    s = b.admit_lj(lj_job(k, rho, t, steps, seed))
    b.advance(steps)
    r = b.result(s, 4 * k ** 3)
    b.close()
    return r


def test_alone_equals_mix_bitwise(cuda_lib):
    from pis_gb300.batch import lj_job
    steps = 120
    alone = [_run_alone(k, rho, t, seed, steps) for (k, rho, t, seed) in JOBS]
    b = _batch()
    slots = {}
    # staggered admission: three jobs first, the rest join while those are running
    for q in (0, 1, 2):
        k, rho, t, seed = JOBS[q]
        slots[q] = b.admit_lj(lj_job(k, rho, t, steps, seed))
    b.advance(37)
    for q in (3, 4):
        k, rho, t, seed = JOBS[q]
        slots[q] = b.admit_lj(lj_job(k, rho, t, steps, seed))
    b.advance(steps)  # the early jobs stop at their own step count
    assert sorted(b.poll()) == sorted(slots.values())
    for q, (k, rho, t, seed) in enumerate(JOBS):
        r = b.result(slots[q], 4 * k ** 3)
        assert r["steps"] == steps
        assert np.array_equal(r["pos"], alone[q]["pos"]), q
        assert np.array_equal(r["vel"], alone[q]["vel"]), q
        assert r["pe"] == alone[q]["pe"] and r["ke"] == alone[q]["ke"], q
    b.close()


def test_batch_matches_single_context(cuda_lib):
    from pis_gb300.batch import Batch
    from pis_gb300.potentials import GpuContext
    s = liquid(nc=6, seed=8)
    b = Batch(4000, 2, 0, precision="mixed")
    slot = b.admit(s["pos"], s["types"], s["masses"], s["h"], s["table"], 60, velocities=s["vel"])
    b.advance(60)
    r = b.result(slot, len(s["pos"]))
    g = GpuContext(s["table"], 1, precision="mixed")
    g.set_state(s["pos"], s["types"], s["masses"], s["h"], velocities=s["vel"])
    g.compute_potential(False)
    g.verlet_step_nve(0.005, 60)
    pos, vel, _ = g.get_state()
    assert np.array_equal(pos, r["pos"]) and np.array_equal(vel, r["vel"])


def test_fp64_replicas_match_oracle(oracle_lib, cuda_lib):
    from pis_gb300.batch import Batch
    systems = [liquid(nc=6, rho=0.8442, seed=21), liquid(nc=7, rho=0.8, seed=22)]
    b = Batch(6000, 4, 0, precision="fp64")
    slots = [b.admit(s["pos"], s["types"], s["masses"], s["h"], s["table"], 40, velocities=s["vel"]) for s in systems]
    b.advance(40)
    for s, slot in zip(systems, slots):
        o = to_oracle(s)
        pe_ref, _ = o.run_nve(0.005, 40)
        r = b.result(slot, len(s["pos"]))
        d = r["pos"] - o.pos
        d -= s["h"][0, 0] * np.round(d / s["h"][0, 0])
        assert np.abs(d).max() <= 1e-9
        hist = b.pe_history(slot, 40)
        assert np.max(np.abs(hist - pe_ref[1:]) / np.abs(pe_ref[1:])) <= 1e-11


def test_served_stream_results_match_alone(cuda_lib):
    from pis_gb300.batch import lj_job
    reqs = [(0.00, lj_job(5, 0.9, 0.8, 80, 31)), (0.00, lj_job(6, 0.8, 1.0, 150, 32)),
            (0.02, lj_job(5, 0.75, 1.3, 60, 33)), (0.05, lj_job(7, 0.85, 0.6, 100, 34)),
            (0.05, lj_job(6, 0.95, 1.1, 40, 35)), (0.08, lj_job(5, 0.8442, 0.72, 120, 36))]
    b = _batch(atoms=4500, slots=3)  # too small for all at once: later requests wait for releases
    res, wall = b.serve(reqs, graph_steps=25)
    assert wall > 0
    # the per-graph accounting adds up to every job's atoms x steps
    st = b.serve_stats()
    assert st["atom_steps"] == sum(4 * job.k ** 3 * job.steps for _, job in reqs)
    assert st["graphs"] >= max(job.steps for _, job in reqs) // 25
    assert 0 <= st["saturated_graphs"] <= st["graphs"] and 0 < st["device_s"]
    for (t, job), r in zip(reqs, res):
        assert r["status"] == 0
        assert r["steps"] == job.steps
        assert r["admitted_s"] >= t - 1e-9 and r["finished_s"] >= r["admitted_s"]
        alone = _run_alone(job.k, job.rho, job.t_star, job.seed, job.steps)
        assert r["pe"] == alone["pe"] and r["ke"] == alone["ke"]
    b.close()


def test_serve_graphs_longer_than_the_partial_ring(cuda_lib):
    # 150 steps per serving iteration run as fused graphs of at most 64 steps (the rows of the
    # per-step partial ring whose sums end each graph): results equal the jobs run alone
    from pis_gb300.batch import lj_job
    reqs = [(0.0, lj_job(5, 0.85, 0.9, 170, 41)), (0.0, lj_job(6, 0.8, 1.1, 130, 42)),
            (0.0, lj_job(5, 0.9, 0.7, 64, 43))]
    b = _batch(atoms=3000, slots=3)
    res, _ = b.serve(reqs, graph_steps=150)
    st = b.serve_stats()
    b.close()
    assert st["atom_steps"] == sum(4 * job.k ** 3 * job.steps for _, job in reqs)
    for (_, job), r in zip(reqs, res):
        assert r["status"] == 0 and r["steps"] == job.steps
        alone = _run_alone(job.k, job.rho, job.t_star, job.seed, job.steps)
        assert r["pe"] == alone["pe"] and r["ke"] == alone["ke"]


def test_serve_accounting_at_saturation(cuda_lib):
    # six jobs at once on two slots: the first graphs run while requests wait for a slot
    from pis_gb300.batch import lj_job
    reqs = [(0.0, lj_job(5, 0.8, 1.0, 60 + 10 * q, 70 + q)) for q in range(6)]
    b = _batch(atoms=2000, slots=2)
    res, _ = b.serve(reqs, graph_steps=20)
    st = b.serve_stats()
    b.close()
    assert all(r["status"] == 0 for r in res)
    assert st["atom_steps"] == sum(500 * job.steps for _, job in reqs)
    assert 0 < st["saturated_graphs"] < st["graphs"]
    assert 0 < st["saturated_atom_steps"] < st["atom_steps"] and 0 < st["saturated_device_s"] < st["device_s"]


def test_admission_refuses_what_does_not_fit(cuda_lib):
    from pis_gb300 import PisError
    from pis_gb300.batch import lj_job
    b = _batch(atoms=1000, slots=2)
    big = lj_job(8, 0.8, 1.0, 10, 1)  # 2048 atoms
    assert not b.fits_lj(big)
    with pytest.raises(PisError) as e:
        b.admit_lj(big)
    assert e.value.name == "PIS_ERR_NO_MEMORY"
    small = lj_job(5, 0.8, 1.0, 10, 1)
    assert b.fits_lj(small)
    b.admit_lj(small)
    b.close()


def test_nan_replica_fails_alone(cuda_lib):
    from pis_gb300 import PisError
    from pis_gb300.batch import Batch
    good = liquid(nc=6, seed=41)
    bad = liquid(nc=6, seed=42)
    bad["vel"] = bad["vel"].copy()
    bad["vel"][17] = np.nan
    b = Batch(4000, 2, 0, precision="mixed")
    sg = b.admit(good["pos"], good["types"], good["masses"], good["h"], good["table"], 50, velocities=good["vel"])
    sb = b.admit(bad["pos"], bad["types"], bad["masses"], bad["h"], bad["table"], 50, velocities=bad["vel"])
    b.advance(50)
    with pytest.raises(PisError) as e:
        b.result(sb, len(bad["pos"]))
    assert e.value.name == "PIS_ERR_NAN_DETECTED"
    r = b.result(sg, len(good["pos"]))
    ref = Batch(2000, 1, 0, precision="mixed")
    s2 = ref.admit(good["pos"], good["types"], good["masses"], good["h"], good["table"], 50, velocities=good["vel"])
    ref.advance(50)
    r2 = ref.result(s2, len(good["pos"]))
    assert np.array_equal(r["pos"], r2["pos"])


@pytest.mark.parametrize("precision,opts", [("fp64", {}), ("mixed", {}),
                                            ("mixed", dict(lanes=1, batch=4, mixed_kahan=True))])
def test_slot_forces_equal_a_single_context(cuda_lib, precision, opts):
    # the forces a slot returns after a run are the evaluation of its state: the same state in a
    # single context gives the same forces, in every slot of a pool (after 50 steps from the
    # lattice start, whose forces vanish by symmetry)
    from pis_gb300.batch import Batch, lj_job
    from pis_gb300.potentials import GpuContext
    table = {(1, 1): (1.0, 1.0, 2.5)}
    jobs = [lj_job(5, 0.88, 0.95, 50, 61), lj_job(9, 0.71, 1.5, 50, 62), lj_job(7, 0.94, 0.5, 50, 63)]
    b = Batch(8000, 4, 0, precision=precision, **opts)
    slots = [b.admit_lj(j) for j in jobs]
    b.advance(50)
    for j, sl in zip(jobs, slots):
        n = 4 * j.k ** 3
        r = b.result(sl, n)
        L = np.cbrt(4.0 / j.rho) * j.k
        g = GpuContext(table, 1, precision=precision, **opts)
        g.set_state(r["pos"], np.ones(n, np.int32), [1.0], np.eye(3) * L, velocities=r["vel"])
        pe, f = g.compute_potential()
        g.close()
        assert np.all(np.isfinite(r["force"]))
        # FP64: the same pair terms (the half list's atomics add them in another order). Mixed:
        # the pool's FP32 cell-relative coordinates are the build's plus the FP32 displacement
        # since, a fresh context's are rounded from the FP64 positions, so the two are two mixed
        # evaluations of one state, each within the mixed path's error of the FP64 forces
        tol = 1e-12 if precision == "fp64" else 1e-5
        assert np.linalg.norm(r["force"] - f) <= tol * np.linalg.norm(f), (j.k, precision)
        assert abs(r["pe"] - pe) <= tol * abs(pe)
        if precision == "mixed":
            g64 = GpuContext(table, 1, precision="fp64")
            g64.set_state(r["pos"], np.ones(n, np.int32), [1.0], np.eye(3) * L, velocities=r["vel"])
            _, f64 = g64.compute_potential()
            g64.close()
            assert np.sqrt(np.sum((r["force"] - f64) ** 2) / np.sum(f64 ** 2)) <= 1e-5
    b.close()
