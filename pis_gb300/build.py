"""Build the CUDA library ``pis_gb300/_build/libpis_gpu.so`` for sm_103a (in-tree).

Translation units compile in parallel with nvcc, then link into one shared library whose
C ABI is declared in ``include/pis_gpu.h``. Host code is compiled with
``-ffp-contract=off`` so host-side FP64 constants (box inverse, pair constants) round exactly
as the reference's Rust code does on every architecture.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpis_gpu.so")

CU_SOURCES = ["engine.cu", "pis_gpu.cu", "pis_batch.cu", "noalloc.cu", "probe.cu"]
CXX_SOURCES = ["host_io.cpp", "host_system.cpp"]
CLI_SOURCE = "pis_gpu_run.cpp"
CLI = os.path.join(OUT_DIR, "pis_gpu_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC, "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pis_gb300")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES + CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            jobs.append([nvcc, *ARCH, *flags, "-c", path, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    cli_src = os.path.join(CSRC, CLI_SOURCE)
    if force or _stale(CLI, [cli_src, LIB] + hdrs):
        run([nvcc, *ARCH, *flags, "-o", CLI, cli_src, "-L", OUT_DIR, "-lpis_gpu", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
