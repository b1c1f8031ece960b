"""Benchmark of the PIS LJ MD step on GB300.

Workload (one "step" = one velocity-Verlet NVE step of the hot path: integrate, skin test and
conditional neighbour-list rebuild, LJ forces/energy, integrate, reductions): the reduced-unit
LJ liquid with N = 2,048,000 atoms (80^3 FCC cells, rho* = 0.8442, T* = 0.72, rc = 2.5,
skin = 0.3, dt* = 0.005), melted from the lattice with seeded Maxwell-Boltzmann velocities.
Synthetic data: the reference ships no benchmark inputs; this is its own lattice generator's
layout with this project's seeded velocities.

`value` is the mixed-precision path's whole-job atom-steps/s (device-timed, state resident in
HBM); `fp64` reports the plain FP64 GPU path on the same state; `e2e` repeats the mixed
measurement through the C ABI with host buffers (upload, force, K steps with per-step energy
read-back, download). `--impl reference` times the CPU restatement of the reference's
multithreaded manager (LJVParallelManager) on the same workload with all host cores.

Multi-GPU: replicas only (each rank advances its own independent system; no collective on the
data path); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TABLE = {(1, 1): (1.0, 1.0, 2.5)}
RHO, TSTAR, DT, SKIN = 0.8442, 0.72, 0.005, 0.3
HBM_FALLBACK_GBS = 6800.0
# Work per atom-step of the LJ pair loop: 23 flops per list entry (displacement, minimum image,
# r^2, reciprocal, powers, force factor, force components, cutoff test) plus 3 for the energy of an
# in-cutoff pair; compulsory bytes 4 per list entry plus 100 per atom (own position 24, velocity
# read and write 48, force write 24, type 4).
FLOPS_PER_CANDIDATE = 23
FLOPS_PER_PAIR_ENERGY = 3
ALG_BYTES_PER_ATOM = 100


def probe_peaks():
    """FP32 and FP64 pipe peaks (TFLOP/s) of this GPU, probed in this run by the library's
    measurement hook (independent fused multiply-add chains on every SM)."""
    import ctypes as C
    from pis_gb300 import _ffi
    a, b = C.c_double(), C.c_double()
    if _ffi.lib().pis_gpu_probe_peaks(C.byref(a), C.byref(b)) != 0:
        return None, None
    return a.value, b.value


def pipe_fraction(flops, kernel_ms, peak_tflops):
    if not peak_tflops or not kernel_ms:
        return None
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    return {"achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s", "frac": achieved / peak_tflops,
            "peak_source": "probed in this run"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cells", type=int, default=80, help="FCC cells per edge (80 -> 2,048,000 atoms)")
    p.add_argument("--equil", type=int, default=300, help="unreported mixed-precision melt steps")
    p.add_argument("--fp64-steps", type=int, default=200)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-batch", action="store_true", help="skip the 512-replica batched measurement")
    p.add_argument("--batch-steps", type=int, default=2000)
    p.add_argument("--no-serve", action="store_true", help="skip the served-stream measurement")
    p.add_argument("--serve-jobs", type=int, default=128)
    p.add_argument("--serve-fp64-jobs", type=int, default=12)
    p.add_argument("--no-drift", action="store_true", help="skip the 10^4-step energy-drift runs")
    p.add_argument("--no-driver", action="store_true", help="skip the input-file driver measurement")
    p.add_argument("--drift-steps", type=int, default=10000)
    p.add_argument("--mixed-options", default=None,
                   help='kernel variant of the mixed path as JSON (GpuContext keywords, e.g. '
                        '\'{"batch": 8, "tma": true}\'); default: the autotuner\'s choice')
    return p.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("PIS_BENCH_GLOO") is None else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_state(cells, seed):
    from pis_gb300.lattice import lj_liquid
    pos, vel, L = lj_liquid(cells, RHO, TSTAR, seed)
    return pos, vel, L


def cpu_sample(pos, vel, L, threads, manager, min_seconds=10.0, max_steps=50):
    """The oracle's restatement of a reference force manager stepping the state on host cores:
    whole NVE steps until at least ``min_seconds`` have passed (or ``max_steps``), after the
    initial force evaluation. Returns (atom-steps/s, steps, seconds)."""
    import oracle
    n = len(pos)
    s = oracle.System(pos, np.ones(n, np.int32), [1.0], np.eye(3) * L, TABLE, velocities=vel)
    s.compute_potential(manager=manager, nthreads=threads)
    steps, t0 = 0, time.perf_counter()
    while True:
        s.verlet_step_nve(DT, manager=manager, nthreads=threads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or steps >= max_steps:
            return n * steps / el, steps, el


def run_reference(args, rank, world):
    """The reference arm: the oracle's restatement of the reference's multithreaded manager
    (LJVParallelManager, src/potentials/lennard_jones.rs:253-336, OpenMP on all host cores) on the
    same workload. The start state is built without the GPU library (the oracle's copies of the
    lattice order and of this project's velocity generator) and melted on the CPU for the same
    number of unreported steps as the GPU arm's melt (in FP64 here, in mixed precision there: the
    same liquid statistically, not bit for bit). To keep the melt to seconds, a periodic block of
    base^3 FCC cells (base the largest divisor of the cell count up to 20) is melted and tiled to
    the full box: a periodic liquid tiled periodically is a liquid of the same density, temperature
    and neighbour statistics."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = oracle.num_threads_available()
    a = (4.0 / RHO) ** (1.0 / 3.0)
    base = max([d for d in range(8, 21) if args.cells % d == 0], default=args.cells)
    pos0 = oracle.fcc_lattice(a, base, base, base)
    n0 = len(pos0)
    L0 = a * base
    vel0 = oracle.maxwell_boltzmann(np.ones(n0), TSTAR / oracle.KB, 1)
    s0 = oracle.System(pos0, np.ones(n0, np.int32), [1.0], np.eye(3) * L0, TABLE, velocities=vel0)
    s0.compute_potential(manager=oracle.PARALLEL, nthreads=threads)
    t_melt = time.perf_counter()
    for _ in range(args.equil):
        s0.verlet_step_nve(DT, manager=oracle.PARALLEL, nthreads=threads)
    t_melt = time.perf_counter() - t_melt
    rep = args.cells // base
    shifts = np.array([(x, y, z) for x in range(rep) for y in range(rep) for z in range(rep)], dtype=np.float64) * L0
    pos = (s0.pos[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    vel = np.tile(s0.vel, (rep ** 3, 1))
    n = len(pos)
    L = L0 * rep
    s = oracle.System(pos, np.ones(n, np.int32), [1.0], np.eye(3) * L, TABLE, velocities=vel)
    s.compute_potential(manager=oracle.PARALLEL, nthreads=threads)
    # bounded sample: each step of the 2M-atom system costs ~0.5 s on 16 cores
    k = max(1, min(args.steps, 5))
    w = max(0, min(args.warmup, 3))
    for _ in range(w):
        s.verlet_step_nve(DT, manager=oracle.PARALLEL, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(k):
        s.verlet_step_nve(DT, manager=oracle.PARALLEL, nthreads=threads)
    el = time.perf_counter() - t0
    v = n * k / el
    line = {
        "impl": "reference", "metric": "atom-steps/s", "value": v, "unit": "atom-steps/s", "n_gpus": world,
        "steps": k, "warmup": w, "ms_per_step": el / k * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, n),
        "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{k} NVE steps of the {n}-atom liquid ({base}^3-cell block melted on the CPU "
                                   f"for {args.equil} steps in {t_melt:.1f} s and tiled {rep}^3, untimed), after {w} "
                                   "warm-up step(s); LJVParallelManager restated with OpenMP (oracle/pis_oracle.cpp)"},
        "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, n):
    return {"workload": f"LJ liquid N={n} (FCC {args.cells}^3 melted), rho*={RHO}, T*={TSTAR}, rc=2.5, "
                        f"skin={SKIN}, dt*={DT}, NVE",
            "atoms": n, "rho": RHO, "t_star": TSTAR, "rcut": 2.5, "skin": SKIN, "dt": DT,
            "equilibration_steps": args.equil, "l2": "inputs larger than L2 (state + list ~2 GB resident)",
            "parallelism": f"replicas{args.gpus}" if args.gpus > 1 else "single"}


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    from pis_gb300 import build as B
    B.build()
    from pis_gb300.potentials import GpuContext, kernel_launches

    pos, vel, L = make_state(args.cells, 1 + rank)
    n = len(pos)
    types = np.ones(n, np.int32)
    h = np.eye(3) * L
    hbm_peak, peak_src = peaks()

    # ---- mixed precision (the headline form) -------------------------------------------------
    mix = GpuContext(TABLE, 1, skin=SKIN, precision="mixed")
    mix.set_state(pos, types, [1.0], h, velocities=vel)
    mix.compute_potential(want_forces=False)
    mix.run_timed(DT, max(args.equil, 1))          # melt (unreported)
    melt_pos, melt_vel, _ = mix.get_state()
    mix.close()
    # kernel shape from the project's autotuner (cached per GPU / precision / size class)
    from pis_gb300.autotune import tune_system
    if args.mixed_options:
        tuned = json.loads(args.mixed_options)
    else:
        tuned = tune_system(TABLE, 1, melt_pos, types, [1.0], h, melt_vel, precision="mixed", skin=SKIN, dt=DT)
    mix = GpuContext(TABLE, 1, skin=SKIN, precision="mixed", **tuned)
    mix.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
    mix.compute_potential(want_forces=False)
    mix.run_timed(DT, max(args.warmup, 3))         # warm-up
    barrier(world)
    st0 = mix.stats()
    launches0 = kernel_launches()
    with ClockSampler(local) as clk:
        ms, _ = mix.run_timed(DT, args.steps)
    launches = kernel_launches() - launches0
    ms = max_over_ranks(ms, world)
    st = mix.stats()
    rebuilds_per_step = (st["rebuilds"] - st0["rebuilds"]) / args.steps
    value = world * n * args.steps / (ms * 1e-3)
    # stage breakdown (events captured in the graphs), separate pass of the same length
    ms_s, stages = mix.run_timed(DT, args.steps, stages=True)
    stages_per = stages / args.steps
    list_per_atom = st["list_entries"] / n
    fused = bool(st.get("fused_step"))
    step_kernel = "k_step_mixed" if fused else "k_force_mixed"
    # Algorithmic bytes of one atom-step (the compulsory HBM traffic of a full-list step with FP64
    # state): list indices 4 nn + own position 24 + velocity read/write 48 + force write 24 + type 4
    # (= 4 nn + 100, about 404 B at nn = 76); neighbour-position gathers count as cache-resident.
    force_bytes = n * ALG_BYTES_PER_ATOM + st["list_entries"] * 4
    # what this implementation's layout moves per atom-step (double4 padding, the acceleration
    # stream, build snapshot, FP32 coordinates), for comparison with the measured DRAM traffic
    if fused:
        impl_bytes = n * (4 + 16 + 32 + 64 + 64 + 64 + 32 + 16 + 16) + st["list_entries"] * 4
    else:
        impl_bytes = n * (4 + 16 + 32) + st["list_entries"] * 4
    force_ms = stages_per[2]
    achieved = force_bytes / (force_ms * 1e-3) / 1e9
    pairs_per_step = 27.6 * n  # in-cutoff unordered pairs per step at rho* = 0.8442
    traffic = read_traffic("step_mixed" if fused else "force_mixed", n)
    # FP32 work of the pair loop: 23 flops per list entry plus 3 per in-cutoff (full-list) pair
    fp32_flops = n * (list_per_atom * FLOPS_PER_CANDIDATE + 2 * 27.6 * FLOPS_PER_PAIR_ENERGY)
    fp32_peak, fp64_peak = probe_peaks()

    # ---- plain FP64 on the same state --------------------------------------------------------
    f64 = GpuContext(TABLE, 1, skin=SKIN, precision="fp64")
    f64.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
    pe64, F64 = f64.compute_potential()
    f64.run_timed(DT, 3)
    k64 = max(3, min(args.fp64_steps, args.steps))
    ms64, _ = f64.run_timed(DT, k64)
    ms64 = max_over_ranks(ms64, world)
    v64 = world * n * k64 / (ms64 * 1e-3)
    k64s = min(k64, 20)
    _, st64 = f64.run_timed(DT, k64s, stages=True)
    force64_ms = st64[2] / k64s
    list64 = f64.stats()["list_entries"] / n  # half list
    fp64_flops = n * (list64 * FLOPS_PER_CANDIDATE + 27.6 * FLOPS_PER_PAIR_ENERGY)
    # mixed precision on a Newton-3 half list (forces on j by FP64 atomics; a measured variant)
    mh = GpuContext(TABLE, 1, skin=SKIN, precision="mixed", list_kind="half", mixed_kahan=True)
    mh.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
    mh.compute_potential(want_forces=False)
    mh.run_timed(DT, 3)
    msh, _ = mh.run_timed(DT, k64)
    _, sth = mh.run_timed(DT, k64s, stages=True)
    mixed_half = {"value": world * n * k64 / (max_over_ranks(msh, world) * 1e-3), "unit": "atom-steps/s",
                  "steps": k64, "ms_per_step": msh / k64, "force_ms_per_step": float(sth[2]) / k64s,
                  "list_entries_per_atom": mh.stats()["list_entries"] / n}
    mh.close()
    f64f = GpuContext(TABLE, 1, skin=SKIN, precision="fp64", fp64_fast=True)
    f64f.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
    f64f.compute_potential(want_forces=False)
    f64f.run_timed(DT, 3)
    ms64f, _ = f64f.run_timed(DT, k64)
    v64f = world * n * k64 / (max_over_ranks(ms64f, world) * 1e-3)
    f64f.close()
    # error of the timed kernel variant, and of the default options (FP64 sums of 32-entry FP32
    # batches instead of compensated sums)
    errs = {}
    for name, kw in (("timed", tuned), ("default_options", {})):
        mixf = GpuContext(TABLE, 1, skin=SKIN, precision="mixed", **kw)
        mixf.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
        pem, Fm = mixf.compute_potential()
        errs[name] = (float(np.sqrt(np.sum((Fm - F64) ** 2) / np.sum(F64 ** 2))), abs(pem - pe64) / abs(pe64))
        if name == "timed":
            # atoms whose force differs by more than 1e-2 eps/sigma: a pair within ~1e-7 of the cutoff
            # decided differently by the FP32 test (the LJ force jumps by 0.039 eps/sigma at rc = 2.5)
            dF = np.linalg.norm(Fm - F64, axis=1)
            edge = dF > 1e-2
            cut_edge = {"atoms_over_1e-2": int(edge.sum()),
                        "force_rms_rel_other_atoms": float(np.sqrt(np.sum((Fm - F64)[~edge] ** 2) / np.sum(F64 ** 2)))}
        mixf.close()
    force_rms, pe_rel = errs["timed"]
    f64.close()

    # ---- end to end through the C ABI with host buffers -------------------------------------
    # inputs and outputs in pinned host memory; the timed region holds the upload, the initial
    # force evaluation, K steps with every step's energy read back, and the download
    k_e2e = args.steps

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    e2e_pos = pinned((n, 3), torch.float64)
    e2e_vel = pinned((n, 3), torch.float64)
    e2e_types = pinned((n,), torch.int32)
    e2e_pos[:] = melt_pos
    e2e_vel[:] = melt_vel
    e2e_types[:] = types
    e2e_out = (pinned((n, 3), torch.float64), pinned((n, 3), torch.float64), pinned((n, 3), torch.float64))
    # one untimed pass of the same calls first (W steps): the step graphs of this entry point are
    # captured there, as the timed steps of `value` follow their own warm-up
    mix.set_state(e2e_pos, e2e_types, [1.0], h, velocities=e2e_vel)
    mix.compute_potential(want_forces=False)
    mix.verlet_step_nve(DT, max(args.warmup, 3))
    mix.get_state(out=e2e_out)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    mix.set_state(e2e_pos, e2e_types, [1.0], h, velocities=e2e_vel)
    mix.compute_potential(want_forces=False)
    pe_steps = mix.verlet_step_nve(DT, k_e2e)
    out_pos, out_vel, out_f = mix.get_state(out=e2e_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = world * n * k_e2e / e2e_s
    h2d = e2e_pos.nbytes + e2e_vel.nbytes + e2e_types.nbytes
    d2h = sum(a.nbytes for a in e2e_out) + pe_steps.nbytes
    mix.close()

    drift = None if args.no_drift else run_drift(args, melt_pos, melt_vel, types, h, tuned)
    batched = None if args.no_batch else run_batched(args, rank, world)
    mix_errors = None if (args.no_batch or args.no_drift) else run_batch_errors(args, tuned)
    served = None if (args.no_serve or rank != 0) else run_served(args, tuned)
    driver = None if (args.no_driver or rank != 0) else run_driver(args, tuned)

    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        threads = oracle.num_threads_available()
        v_cpu, k_cpu, el = cpu_sample(melt_pos, melt_vel, L, threads, oracle.PARALLEL)
        v_ser, k_ser, el_ser = cpu_sample(melt_pos, melt_vel, L, 1, oracle.OFFSET)
        cpu = {"value": v_cpu, "unit": "atom-steps/s", "cores": threads, "kind": "port",
               "sample": f"{k_cpu} NVE steps of the same {n}-atom liquid ({el:.1f} s), LJVParallelManager "
                         "restated with OpenMP (oracle/pis_oracle.cpp)",
               "serial": {"value": v_ser, "unit": "atom-steps/s", "cores": 1, "kind": "port",
                          "sample": f"{k_ser} NVE step(s) of the same liquid ({el_ser:.1f} s), LJVOffsetManager "
                                    "(the CLI's manager) restated serially (oracle/pis_oracle.cpp)"}}

    if rank == 0:
        roofline = {"bound": "hbm", "kernel": step_kernel, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "peak_source": peak_src, "traffic": traffic,
                    "algorithmic_bytes_per_launch": force_bytes,
                    "implementation_bytes_per_launch": impl_bytes,
                    "traffic_over_algorithmic": (traffic / force_bytes) if traffic else None,
                    "fp32_pipe": pipe_fraction(fp32_flops, force_ms, fp32_peak),
                    "fp64_pipe_plain_fp64_force": pipe_fraction(fp64_flops, force64_ms, fp64_peak)}
        batched_summary = None
        if batched:
            batched_summary = {k: batched[k] for k in ("replicas", "atoms", "mixed", "fp64", "mixed_over_fp64")}
            if mix_errors:
                batched_summary["errors"] = mix_errors["summary"]
        line = {
            "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32-pair/f64-accumulate",
            "data": "synthetic", "config": workload_config(args, n),
            "precision": "mixed",
            # details first; the figures the summary keys below restate come last on the line
            "served": served,
            "driver": driver,
            "drift": drift,
            "batched_detail": batched,
            "batched_errors_vs_fp64": mix_errors,
            "stages_ms_per_step": {"integrate1": stages_per[0], "rebuild": stages_per[1], "force": stages_per[2],
                                   "integrate2": stages_per[3], "reduce": stages_per[4]},
            "fp64_stages_ms_per_step": [float(x) / k64s for x in st64],
            "tuned_options": tuned,
            "rebuilds_per_step": rebuilds_per_step,
            "list_entries_per_atom": list_per_atom,
            "pairs_per_s": world * pairs_per_step * args.steps / (ms * 1e-3),
            "fp64_fast": {"value": v64f, "unit": "atom-steps/s", "steps": k64, "dtype": "f64",
                          "note": "FMA / Newton-reciprocal variant, same cutoff decisions"},
            "mixed_half_list": mixed_half,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d / k_e2e,
                    "d2h_bytes_per_step": d2h / k_e2e, "seconds": e2e_s,
                    "path": "set_state + compute_potential + verlet_step_nve(K) + get_state, pinned host buffers, "
                            "after one untimed pass of the same calls"},
            "roofline": roofline,
            "error_vs_fp64": {"force_rms_rel": force_rms, "pe_rel": pe_rel, "cutoff_edge": cut_edge,
                              "default_options": {"force_rms_rel": errs["default_options"][0],
                                                  "pe_rel": errs["default_options"][1]}},
            "batched": batched_summary,
            "fp64": {"value": v64, "unit": "atom-steps/s", "steps": k64, "ms_per_step": ms64 / k64,
                     "dtype": "f64", "list": "half"},
            "mixed_over_fp64": value / v64,
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batch_jobs(seed=2024, count=512):
    """512 replicas: N log-uniform in [500, 32000] rounded to 4 k^3 FCC, rho* in U[0.70, 0.95],
    T* in U[0.5, 1.5], per-replica seeds."""
    import math
    from pis_gb300.batch import lj_job
    rng = np.random.default_rng(seed)
    jobs = []
    for r in range(count):
        N = math.exp(rng.uniform(math.log(500), math.log(32000)))
        k = int(min(20, max(5, round((N / 4) ** (1 / 3)))))
        jobs.append(lj_job(k, rng.uniform(0.70, 0.95), rng.uniform(0.5, 1.5), 10 ** 9, 1000 + r))
    return jobs


def run_batched(args, rank, world):
    """All 512 replicas advanced together (one launch per kernel per step, 50-step graphs)."""
    from pis_gb300.batch import Batch, lj_pool_cells
    jobs = batch_jobs(seed=2024 + rank)
    atoms = sum(4 * j.k ** 3 for j in jobs)
    cells = sum(lj_pool_cells(j.k, j.rho) for j in jobs)
    out = {"replicas": len(jobs), "atoms": atoms, "steps": args.batch_steps}
    from pis_gb300.autotune import tune_batch
    tuned = tune_batch(jobs, precision="mixed")
    out["tuned_options"] = tuned
    for prec, kw in (("mixed", tuned), ("fp64", {}), ("fp64_fast", {"fp64_fast": True})):
        precision = "mixed" if prec == "mixed" else "fp64"
        k = args.batch_steps if prec == "mixed" else max(3, args.batch_steps // 10)
        b = Batch(atoms + 1024, len(jobs), cells + 1024, precision=precision, **kw)
        for j in jobs:
            b.admit_lj(j)
        b.run_timed(100)  # warm-up and melt
        barrier(world)
        ms = max_over_ranks(b.run_timed(k), world)
        out[prec] = world * atoms * k / (ms * 1e-3)
        b.close()
    out["mixed_over_fp64"] = out["mixed"] / out["fp64"]
    return out


def representative(jobs, count=6):
    """Indices of the smallest and largest systems, the median one, and the hottest, coldest and
    densest of the rest."""
    order = sorted(range(len(jobs)), key=lambda r: jobs[r].k)
    pick = [order[0], order[-1], order[len(order) // 2]]
    for key in (lambda r: jobs[r].t_star, lambda r: -jobs[r].t_star, lambda r: jobs[r].rho):
        for r in sorted(range(len(jobs)), key=key, reverse=True):
            if r not in pick:
                pick.append(r)
                break
    return pick[:count]


def job_errors(jobs, pick, steps, tuned, chunk=500, melt=300):
    """Error of the mixed path against FP64 on the jobs `pick`: each job's lattice start is melted
    for `melt` steps in an FP64 pool (a perfect lattice has forces of ~1e-14, so errors relative to
    them mean nothing); the melted state is admitted to an FP64 pool and to a mixed pool; force RMS
    and energy error of their first evaluations, then `steps` NVE steps in each with the total
    energy every `chunk` steps and its drift per atom per 10^4 steps."""
    from pis_gb300.batch import Batch, lj_pool_cells
    sel = [jobs[r] for r in pick]
    atoms = sum(4 * j.k ** 3 for j in sel)
    cells = sum(lj_pool_cells(j.k, j.rho) for j in sel)
    b = Batch(atoms + 1024, len(sel), cells + 1024, precision="fp64")
    slots = [b.admit_lj(type(j)(j.k, j.rho, j.t_star, j.rcut, j.skin, j.dt, melt, j.seed)) for j in sel]
    b.advance(melt)
    melted = [b.result(sl, 4 * j.k ** 3) for sl, j in zip(slots, sel)]
    b.close()
    res = {}
    for prec in ("fp64", "mixed"):
        kw = tuned if prec == "mixed" else {}
        b = Batch(atoms + 1024, len(sel), cells + 1024, precision=prec, **kw)
        slots = []
        for j, m in zip(sel, melted):
            n = 4 * j.k ** 3
            L = np.cbrt(4.0 / j.rho) * j.k
            slots.append(b.admit(m["pos"], np.ones(n, np.int32), [1.0], np.eye(3) * L, {(1, 1): (1.0, 1.0, j.rcut)},
                                 steps, velocities=m["vel"], skin=j.skin, dt=j.dt))
        first = [b.result(sl, 4 * j.k ** 3) for sl, j in zip(slots, sel)]
        series = [[f["pe"] + f["ke"]] for f in first]
        for _ in range(steps // chunk):
            b.advance(chunk)
            for q, sl in enumerate(slots):
                r = b.result(sl, state=False)
                series[q].append(r["pe"] + r["ke"])
        res[prec] = (first, series)
        b.close()
    reps = []
    for q, (r, j) in enumerate(zip(pick, sel)):
        n = 4 * j.k ** 3
        f64, fm = res["fp64"][0][q], res["mixed"][0][q]
        s64 = drift_stats(np.array(res["fp64"][1][q]), n, chunk)
        sm = drift_stats(np.array(res["mixed"][1][q]), n, chunk)
        reps.append({"job": r, "atoms": n, "rho": j.rho, "t_star": j.t_star,
                     "force_rms_rel": float(np.sqrt(np.sum((fm["force"] - f64["force"]) ** 2) / np.sum(f64["force"] ** 2))),
                     "pe_rel": abs(fm["pe"] - f64["pe"]) / abs(f64["pe"]),
                     "drift_fp64": s64["drift_per_atom_per_1e4_steps"], "drift_mixed": sm["drift_per_atom_per_1e4_steps"],
                     "drift_fit_stderr_fp64": s64["fit_stderr_per_atom_per_1e4_steps"],
                     "drift_fit_stderr_mixed": sm["fit_stderr_per_atom_per_1e4_steps"]})
    summary = {"jobs": len(reps), "steps": steps, "melt_steps": melt,
               "max_force_rms_rel": max(x["force_rms_rel"] for x in reps),
               "max_pe_rel": max(x["pe_rel"] for x in reps),
               "max_abs_drift_mixed": max(abs(x["drift_mixed"]) for x in reps),
               "max_abs_drift_fp64": max(abs(x["drift_fp64"]) for x in reps)}
    return {"per_job": reps, "summary": summary}


def run_batch_errors(args, tuned, count=6):
    """Mixed against FP64 on representative replicas of the 512-replica mix, 10^4 NVE steps."""
    jobs = batch_jobs(seed=2024)
    return job_errors(jobs, representative(jobs, count), args.drift_steps, tuned)


def energy_series(ctx, steps, chunk):
    """Total energy every `chunk` steps (PE from the step, KE from the device reductions)."""
    pe0, _ = ctx.compute_potential(want_forces=False)
    ke0, _ = ctx.reductions()
    e = [pe0 + ke0]
    for _ in range(steps // chunk):
        pe = ctx.verlet_step_nve(DT, chunk)
        ke, _ = ctx.reductions()
        e.append(pe[-1] + ke)
    return np.array(e)


def drift_stats(e, n, chunk):
    """Slope of a linear fit of E(t) per atom per 10^4 steps, with the fit's standard error (the
    residuals are the energy's own fluctuation, which per atom grows as N shrinks; being
    correlated in time they make this a lower bound on the slope's uncertainty)."""
    t = np.arange(len(e)) * chunk
    slope, icpt = np.polyfit(t, e, 1)
    res = e - (slope * t + icpt)
    se = np.sqrt(np.sum(res ** 2) / max(len(e) - 2, 1) / np.sum((t - t.mean()) ** 2)) if len(e) > 2 else 0.0
    return {"drift_per_atom_per_1e4_steps": float(slope * 1e4 / n), "fit_stderr_per_atom_per_1e4_steps": float(se * 1e4 / n),
            "max_abs_dev_per_atom": float(np.abs(e - e[0]).max() / n)}


def run_drift(args, melt_pos, melt_vel, types, h, tuned):
    """NVE energy drift over 10^4 steps: the mixed path on the 2.048M-atom liquid, and the plain
    FP64 path (the reference's arithmetic) and the mixed path from three melted states of the
    256,000-atom liquid (FP64 at 2M atoms would take minutes). Both paths drift by ~1e-5 eps/atom
    per 10^4 steps at dt* = 0.005: the floor is the shifted-energy cutoff's force jump, not the
    precision, and it varies by about +-50 % between starting states."""
    from pis_gb300.potentials import GpuContext
    from pis_gb300.lattice import lj_liquid
    out = {"steps": args.drift_steps}
    n = len(melt_pos)
    g = GpuContext(TABLE, 1, skin=SKIN, precision="mixed", **tuned)
    g.set_state(melt_pos, types, [1.0], h, velocities=melt_vel)
    # equilibrate to 2000 steps from the lattice before the NVE record (a liquid still relaxing
    # from the melt drifts more), as the 256k states below
    extra = max(0, 2000 - args.equil)
    if extra:
        g.compute_potential(want_forces=False)
        g.run_timed(DT, extra)
    out["mixed_2m"] = drift_stats(energy_series(g, args.drift_steps, 500), n, 500)
    out["mixed_2m"]["equilibration_steps"] = args.equil + extra
    g.close()
    # FP64 (the reference's arithmetic) against mixed from the same states: the drift varies by
    # about +-50 % between starting states, so three states and their means
    per = {"fp64_256k": [], "mixed_256k": []}
    for seed in (4, 5, 6):
        pos, vel, L = lj_liquid(40, RHO, TSTAR, seed)
        ns = len(pos)
        g = GpuContext(TABLE, 1, skin=SKIN, precision="mixed")
        g.set_state(pos, np.ones(ns, np.int32), [1.0], np.eye(3) * L, velocities=vel)
        g.compute_potential(want_forces=False)
        g.run_timed(DT, 2000)  # melt
        p4, v4, _ = g.get_state()
        g.close()
        for name, kw in (("fp64_256k", {"precision": "fp64"}), ("mixed_256k", {"precision": "mixed", **tuned})):
            g = GpuContext(TABLE, 1, skin=SKIN, **kw)
            g.set_state(p4, np.ones(ns, np.int32), [1.0], np.eye(3) * L, velocities=v4)
            per[name].append(drift_stats(energy_series(g, args.drift_steps, 500), ns, 500))
            g.close()
    for name, runs in per.items():
        vals = [r["drift_per_atom_per_1e4_steps"] for r in runs]
        out[name] = {"drift_per_atom_per_1e4_steps": float(np.mean(vals)), "per_state": vals,
                     "max_abs_dev_per_atom": max(r["max_abs_dev_per_atom"] for r in runs), "states": len(vals)}
    return out


def serve_requests(count, seed=77, rate=200.0, step_scale=1.0):
    """Poisson arrivals (rate jobs/s) of LJ jobs: N log-uniform in [1000, 256000] rounded to 4 k^3,
    rho* in U[0.70, 0.95], T* in U[0.5, 1.5], steps U[100, 5000] (times step_scale)."""
    import math
    from pis_gb300.batch import lj_job
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for q in range(count):
        t += rng.exponential(1.0 / rate)
        N = math.exp(rng.uniform(math.log(1000), math.log(256000)))
        k = int(min(40, max(6, round((N / 4) ** (1 / 3)))))
        steps = int(round(rng.uniform(100, 5000) * step_scale))
        reqs.append((t, lj_job(k, rng.uniform(0.70, 0.95), rng.uniform(0.5, 1.5), steps, 5000 + q)))
    return reqs


def serve_stats(reqs, res, wall):
    work = sum(4 * j.k ** 3 * j.steps for _, j in reqs)
    lat = np.array([r["finished_s"] - r["arrival_s"] for r in res])
    wait = np.array([r["admitted_s"] - r["arrival_s"] for r in res])
    return {"jobs": len(reqs), "atom_steps": work, "atom_steps_per_s": work / wall, "wall_s": wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "p50_queue_wait_s": float(np.percentile(wait, 50)), "p99_queue_wait_s": float(np.percentile(wait, 99)),
            "all_ok": all(r["status"] == 0 for r in res)}


def run_served(args, tuned):
    """The served stream as stated: Poisson arrivals at 200 jobs/s, steps U[100, 5000], a fixed job
    count; continuous batching on one mixed-precision pool (50-step graphs). The plain FP64 path
    serves the first jobs of the same stream one at a time (a subset: one at a time it would take
    minutes). An arrival-rate sweep runs a lighter stream (steps x 0.2) below and above saturation.
    Mixed-precision error against FP64 on representative jobs of the stream, 10^4 steps each."""
    from pis_gb300.batch import Batch, lj_pool_cells
    reqs = serve_requests(args.serve_jobs)
    work = sum(4 * j.k ** 3 * j.steps for _, j in reqs)
    out = {"jobs": len(reqs), "arrival_rate_per_s": 200.0, "step_scale": 1.0, "atom_steps": work,
           "offered_atom_steps_per_s": work / max(reqs[-1][0], 1e-9), "graph_steps": 50}
    max_atoms = 4 * 40 ** 3 * 8
    max_cells = max(lj_pool_cells(j.k, j.rho) for _, j in reqs) * 16
    # continuous batching on a 4.1M-atom pool (128 slots), and on a 2.0M-atom pool (64 slots);
    # "saturated": the rate of the graphs queued while a request waited for pool space
    for name, atoms, slots in (("mixed_batched", 2 * max_atoms, 128), ("mixed_batched_2m_pool", max_atoms, 64)):
        b = Batch(atoms, slots, max_cells * slots // 64, precision="mixed")
        res, wall = b.serve(reqs, graph_steps=50)
        out[name] = serve_stats(reqs, res, wall)
        out[name].update(pool_atoms=atoms, slots=slots, graphs=b.serve_stats())
        b.close()
    out["mixed_batched"]["saturated_atom_steps_per_s"] = out["mixed_batched"]["graphs"]["saturated_atom_steps_per_device_s"]
    sub = reqs[:args.serve_fp64_jobs]
    b = Batch(max_atoms, 1, max_cells, precision="fp64")
    res, wall = b.serve(sub, graph_steps=50)
    b.close()
    out["fp64_one_at_a_time"] = serve_stats(sub, res, wall)
    out["fp64_one_at_a_time"]["subset"] = f"the first {len(sub)} jobs of the stream"
    # arrival-rate sweep of the continuous-batching path
    sweep = []
    for rate in (100.0, 200.0, 400.0, 800.0):
        rq = serve_requests(128, seed=78, rate=rate, step_scale=0.2)
        w = sum(4 * j.k ** 3 * j.steps for _, j in rq)
        cells = max(lj_pool_cells(j.k, j.rho) for _, j in rq) * 16
        b = Batch(max_atoms, 64, cells, precision="mixed")
        res, wall = b.serve(rq, graph_steps=50)
        b.close()
        st = serve_stats(rq, res, wall)
        st.update(rate_per_s=rate, step_scale=0.2, offered_atom_steps_per_s=w / max(rq[-1][0], 1e-9))
        sweep.append(st)
    out["mixed_rate_sweep"] = sweep
    if not args.no_drift:
        jobs = [j for _, j in reqs]
        out["errors_vs_fp64"] = job_errors(jobs, representative(jobs, 4), args.drift_steps, tuned)
    return out


def run_driver(args, tuned, steps=10000, dump_every=2500):
    """The input-file driver (System::run on the GPU manager: a thermo line i PE KE H T P every step,
    a LAMMPS dump every dump_every steps) against pis_gpu_verlet_step_nve with every step's energy
    read back, both on the same melted 256,000-atom liquid, mixed precision, wall clock."""
    import tempfile
    from pis_gb300.io import System, write_data
    from pis_gb300.lattice import lj_liquid
    from pis_gb300.potentials import GpuContext
    pos, vel, L = lj_liquid(40, RHO, TSTAR, 7)
    n = len(pos)
    types = np.ones(n, np.int32)
    g = GpuContext(TABLE, 1, skin=SKIN, precision="mixed")
    g.set_state(pos, types, [1.0], np.eye(3) * L, velocities=vel)
    g.compute_potential(want_forces=False)
    g.run_timed(DT, 500)
    p, v, _ = g.get_state()
    g.close()
    out = {"atoms": n, "steps": steps, "thermo_every": 1, "dump_every": dump_every}
    with tempfile.TemporaryDirectory() as d:
        data = os.path.join(d, "liquid.txt")
        write_data(data, p, types, [1.0], [0, L, 0, L, 0, L], TABLE, v)
        inp = os.path.join(d, "in.pis")
        with open(inp, "w") as fh:
            fh.write(f"timestep {DT}\nread_data {data}\ndump d1 all atom {dump_every} {os.path.join(d, 'traj')}\n"
                     f"run {steps}\n")
        sysm = System(inp, precision="mixed", skin=SKIN)
        t0 = time.perf_counter()
        sysm.run(os.path.join(d, "thermo.txt"))
        wall = time.perf_counter() - t0
        with open(os.path.join(d, "thermo.txt")) as fh:
            lines = sum(1 for _ in fh)
        sysm.close()
    out["driver"] = {"atom_steps_per_s": n * steps / wall, "wall_s": wall, "thermo_lines": lines}
    g = GpuContext(TABLE, 1, skin=SKIN, precision="mixed")
    g.set_state(p, types, [1.0], np.eye(3) * L, velocities=v)
    g.compute_potential(want_forces=False)
    g.verlet_step_nve(DT, 50)
    t0 = time.perf_counter()
    g.compute_potential(want_forces=False)
    g.verlet_step_nve(DT, steps)
    wall = time.perf_counter() - t0
    g.close()
    out["verlet_step_nve"] = {"atom_steps_per_s": n * steps / wall, "wall_s": wall}
    out["driver_over_verlet_step_nve"] = out["driver"]["atom_steps_per_s"] / out["verlet_step_nve"]["atom_steps_per_s"]
    return out


def read_traffic(kernel, n):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, scaled to n atoms."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as fh:
            for line in fh:
                f = line.split()
                if len(f) >= 3 and f[0] == kernel:
                    return float(f[1]) * n / float(f[2])
    except OSError:
        pass
    return None


if __name__ == "__main__":
    main()
