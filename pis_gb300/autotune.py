"""Autotuner for the kernel shape knobs of the MD step.

The measured knobs are the ones the C ABI exposes as variants: lanes per atom in the list build
and force kernels (PIS_OPT_LANES), list entries per gather batch in the mixed force kernel
(PIS_OPT_BATCH), FP64 batch sums versus compensated FP32 sums (PIS_OPT_MIXED_KAHAN), the list
streamed into shared memory by bulk copies (PIS_OPT_LIST_TMA), cluster lists (PIS_OPT_CLUSTER)
and the cluster-scanned per-atom list build (PIS_OPT_SCAN). For a
given workload the tuner times a short run of every candidate on the real system (CUDA events on
the engine's stream) and keeps the fastest. Results are cached in a JSON file keyed by GPU name,
precision and size class (atoms per system rounded to a power of two), so a workload is tuned
once per machine.
"""
from __future__ import annotations

import json
import os

import numpy as np

from .build import OUT_DIR

CACHE = os.path.join(OUT_DIR, "autotune.json")

MIXED_CANDIDATES = [
    {"lanes": 1, "batch": 4, "mixed_kahan": False},
    {"lanes": 1, "batch": 8, "mixed_kahan": False},
    {"lanes": 1, "batch": 4, "mixed_kahan": True},
    {"lanes": 1, "batch": 8, "mixed_kahan": True},
    {"lanes": 1, "batch": 4, "mixed_kahan": True, "scan": 4},
    {"lanes": 1, "batch": 8, "mixed_kahan": True, "tma": True},
    {"lanes": 1, "batch": 4, "mixed_kahan": True, "cluster": 4},
]
FP64_CANDIDATES = [
    {"lanes": 1, "fp64_fast": False},
    {"lanes": 4, "fp64_fast": False},
    {"lanes": 1, "fp64_fast": True},
    {"lanes": 4, "fp64_fast": True},
]


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def size_class(n_atoms: int) -> int:
    return 1 << max(0, int(np.ceil(np.log2(max(1, n_atoms)))))


def _load() -> dict:
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(d, fh, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _key(precision: str, n_atoms: int) -> str:
    return f"{_gpu_name()}|{precision}|{size_class(n_atoms)}"


def tune_system(table, n_types, positions, type_ids, masses, h, velocities, precision="mixed", skin=0.3, dt=0.005,
                steps=60, use_cache=True) -> dict:
    """Fastest variant options for one system (a GpuContext workload)."""
    from .potentials import GpuContext
    key = _key(precision, len(positions))
    cache = _load()
    if use_cache and key in cache:
        return dict(cache[key]["options"])
    cands = MIXED_CANDIDATES if precision == "mixed" else FP64_CANDIDATES
    if precision == "fp64":
        steps = max(6, steps // 6)
    timings = []
    for opt in cands:
        g = GpuContext(table, n_types, skin=skin, precision=precision, **opt)
        g.set_state(positions, type_ids, masses, h, velocities=velocities)
        g.compute_potential(want_forces=False)
        g.run_timed(dt, 5)
        ms, _ = g.run_timed(dt, steps)
        g.close()
        timings.append((ms / steps, opt))
    best = min(timings, key=lambda t: t[0])
    cache[key] = {"options": best[1], "ms_per_step": best[0],
                  "all": [{"options": o, "ms_per_step": t} for t, o in timings]}
    _store(cache)
    return dict(best[1])


def tune_batch(jobs, precision="mixed", steps=40, use_cache=True) -> dict:
    """Fastest variant options for a batch of LJ jobs (pis_batch pool)."""
    from .batch import Batch, lj_pool_cells
    atoms = sum(4 * j.k ** 3 for j in jobs)
    key = _key(precision, atoms) + f"|batch{len(jobs)}"
    cache = _load()
    if use_cache and key in cache:
        return dict(cache[key]["options"])
    cells = sum(lj_pool_cells(j.k, j.rho) for j in jobs)
    cands = MIXED_CANDIDATES if precision == "mixed" else FP64_CANDIDATES
    if precision == "fp64":
        steps = max(6, steps // 6)
    timings = []
    for opt in cands:
        b = Batch(atoms + 1024, len(jobs), cells + 1024, precision=precision, **opt)
        for j in jobs:
            b.admit_lj(j)
        b.run_timed(5)
        ms = b.run_timed(steps)
        b.close()
        timings.append((ms / steps, opt))
    best = min(timings, key=lambda t: t[0])
    cache[key] = {"options": best[1], "ms_per_step": best[0],
                  "all": [{"options": o, "ms_per_step": t} for t, o in timings]}
    _store(cache)
    return dict(best[1])
