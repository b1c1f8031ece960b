"""The no-allocation force entry point against the regular one.

pis_gpu_compute_potential_noalloc serves callers that cannot allocate device memory while they run
(a framework that owns the whole device memory pool, a real-time loop that cannot afford
cudaMalloc). It works on device buffers the caller owns and keeps its scratch in a fixed device
array inside the library. This test gives it device buffers made here, calls it twice in a row
through the C ABI, and checks forces and energy against pis_gpu_compute_potential within the FP64
tolerance of the other parity tests (1e-12 relative). It sits in its own file so a run that stops at
the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from systems import liquid, to_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _displaced(sysd, seed):
    rng = np.random.default_rng(seed)
    out = dict(sysd)
    out["pos"] = np.mod(sysd["pos"] + rng.normal(0, 0.03, sysd["pos"].shape), sysd["h"][0, 0])
    return out


def test_noalloc_matches_compute_potential(cuda_lib):
    import torch
    from pis_gb300 import _ffi

    lib = _ffi.lib()
    s = _displaced(liquid(nc=8), 21)  # 2048 atoms, 5 cells per axis at rc = 2.5
    n = len(s["pos"])
    g = to_gpu(s, "fp64")
    pe_ref, f_ref = g.compute_potential()
    g.close()

    pairs = (_ffi.LJPair * 1)(_ffi.LJPair(1, 1, 1.0, 1.0, 2.5, 1))
    h = np.ascontiguousarray(s["h"].T, dtype=np.float64)
    d_pos = torch.tensor(s["pos"], dtype=torch.float64, device="cuda").contiguous()
    d_types = torch.tensor(s["types"], dtype=torch.int32, device="cuda").contiguous()
    for call in range(2):
        d_f = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
        d_pe = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.pis_gpu_compute_potential_noalloc(pairs, 1, 1, n, C.c_void_p(d_types.data_ptr()),
                                                   C.c_void_p(d_pos.data_ptr()),
                                                   h.ctypes.data_as(C.POINTER(C.c_double)),
                                                   C.c_void_p(d_f.data_ptr()), C.c_void_p(d_pe.data_ptr()), None)
        assert st == 0, _ffi.STATUS_NAMES.get(st, st)
        torch.cuda.synchronize()
        f = d_f.cpu().numpy()
        pe = float(d_pe.cpu().numpy()[0])
        assert abs(pe - pe_ref) <= TOL * abs(pe_ref), (call, pe, pe_ref)
        assert np.linalg.norm(f - f_ref) <= TOL * np.linalg.norm(f_ref), call


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    from pis_gb300 import _ffi

    lib = _ffi.lib()
    pairs = (_ffi.LJPair * 1)(_ffi.LJPair(1, 1, 1.0, 1.0, 2.5, 1))
    h = np.ascontiguousarray(np.eye(3) * 100.0)
    dummy = C.c_void_p(1)  # never dereferenced: the size check fails first
    st = lib.pis_gpu_compute_potential_noalloc(pairs, 1, 1, 262145, dummy, dummy,
                                               h.ctypes.data_as(C.POINTER(C.c_double)), dummy, dummy, None)
    assert _ffi.STATUS_NAMES[st] == "PIS_ERR_INVALID_ARGUMENT"
