"""pis_gb300 - GB300-native (sm_103a) Lennard-Jones MD step for PIS.

The compute path is the CUDA library ``_build/libpis_gpu.so`` (C ABI in include/pis_gpu.h);
this package is the host-side mirror of the reference's potential / atoms / box interfaces.
There is no CPU fallback: every compute call goes through the CUDA library and fails if it is
missing or no GPU is visible.
"""
from .atoms import Atoms, SimulationBox, KB_KJPERMOLEKELVIN  # noqa: F401
from ._ffi import PisError  # noqa: F401


def __getattr__(name):
    if name in ("GpuContext", "LJGpuManager", "kernel_launches"):
        from . import potentials
        return getattr(potentials, name)
    raise AttributeError(name)
