"""The no-allocation force entry point against the regular one and the oracle.

pis_gpu_compute_potential_noalloc serves callers that cannot allocate device memory while they run
(a framework that owns the whole device memory pool, a real-time loop that cannot afford
cudaMalloc). It works on device buffers the caller owns and keeps its scratch in a fixed device
array inside the library. This test gives it device buffers made here, calls it twice in a row
through the C ABI, and checks forces and energy against pis_gpu_compute_potential within the FP64
tolerance of the other parity tests (1e-12 relative). It sits in its own file so a run that stops at
the first failure has already run every other test. It also checks the call against the oracle
directly, on a two-type mixture with per-pair cutoffs in a box of exactly 3 cells per axis, that
device free memory does not change across a call, that out-of-range type ids give a NaN energy,
and the size limits.
"""
import ctypes as C

import numpy as np
import pytest

from systems import liquid, melted, to_gpu, to_oracle

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


def _call(lib, table, n_types, d_types, d_pos, h, d_f, d_pe):
    from pis_gb300 import _ffi
    pairs = (_ffi.LJPair * len(table))()
    for k, ((i, j), (e, sg, rc)) in enumerate(table.items()):
        pairs[k] = _ffi.LJPair(i, j, e, sg, rc, 1)
    hc = np.ascontiguousarray(np.asarray(h, dtype=np.float64).T)
    return lib.pis_gpu_compute_potential_noalloc(pairs, len(table), n_types, d_pos.shape[0],
                                                 C.c_void_p(d_types.data_ptr()), C.c_void_p(d_pos.data_ptr()),
                                                 hc.ctypes.data_as(C.POINTER(C.c_double)),
                                                 C.c_void_p(d_f.data_ptr()), C.c_void_p(d_pe.data_ptr()), None)


@pytest.fixture(scope="module")
def mixture(oracle_lib, cuda_lib):
    s = melted(liquid(nc=5), steps=40, dt=0.005)  # 500 atoms, 8.4 sigma: 3 cells per axis at rc = 2.5
    n = len(s["pos"])
    s["types"] = (np.arange(n) % 2 + 1).astype(np.int32)
    s["masses"] = np.array([1.0, 2.0])
    s["table"] = {(1, 1): (1.0, 1.0, 2.5), (1, 2): (0.8, 1.1, 2.2), (2, 2): (1.2, 0.9, 2.0)}
    return s


def test_noalloc_mixture_three_cells_against_oracle_and_regular_path(mixture):
    import torch
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    s = mixture
    n = len(s["pos"])
    o = to_oracle(s)
    pe_exact, _ = o.compute_potential_exact()
    g = to_gpu(s, "fp64")
    pe_reg, f_reg = g.compute_potential()
    g.close()
    d_pos = torch.tensor(s["pos"], dtype=torch.float64, device="cuda").contiguous()
    d_types = torch.tensor(s["types"], dtype=torch.int32, device="cuda").contiguous()
    for call in range(2):
        d_f = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
        d_pe = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(lib, s["table"], 2, d_types, d_pos, s["h"], d_f, d_pe) == 0
        torch.cuda.synchronize()
        f, pe = d_f.cpu().numpy(), float(d_pe.cpu().numpy()[0])
        assert pe == pe_exact and pe == pe_reg  # the same exact sum of the same pair terms
        assert np.linalg.norm(f - o.force) <= TOL * np.linalg.norm(o.force), call
        assert np.linalg.norm(f - f_reg) <= TOL * np.linalg.norm(f_reg), call


def test_noalloc_allocates_nothing(mixture):
    # device-wide free memory is the same before and after a call (after the first, which may
    # load the module's code)
    import torch
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    s = mixture
    n = len(s["pos"])
    d_pos = torch.tensor(s["pos"], dtype=torch.float64, device="cuda").contiguous()
    d_types = torch.tensor(s["types"], dtype=torch.int32, device="cuda").contiguous()
    d_f = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    d_pe = torch.zeros((1,), dtype=torch.float64, device="cuda")
    assert _call(lib, s["table"], 2, d_types, d_pos, s["h"], d_f, d_pe) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, s["table"], 2, d_types, d_pos, s["h"], d_f, d_pe) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_out_of_range_type_gives_nan_then_recovers(mixture):
    import torch
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    s = mixture
    n = len(s["pos"])
    d_pos = torch.tensor(s["pos"], dtype=torch.float64, device="cuda").contiguous()
    d_f = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    d_pe = torch.zeros((1,), dtype=torch.float64, device="cuda")
    bad = s["types"].copy()
    bad[7] = 3  # beyond n_types = 2
    bad[11] = 0
    d_bad = torch.tensor(bad, dtype=torch.int32, device="cuda").contiguous()
    assert _call(lib, s["table"], 2, d_bad, d_pos, s["h"], d_f, d_pe) == 0
    torch.cuda.synchronize()
    assert np.isnan(float(d_pe.cpu().numpy()[0]))
    f = d_f.cpu().numpy()
    assert np.all(f[7] == 0.0) and np.all(f[11] == 0.0) and np.all(np.isfinite(f))
    d_types = torch.tensor(s["types"], dtype=torch.int32, device="cuda").contiguous()
    assert _call(lib, s["table"], 2, d_types, d_pos, s["h"], d_f, d_pe) == 0
    torch.cuda.synchronize()
    pe_exact, _ = to_oracle(s).compute_potential_exact()
    assert float(d_pe.cpu().numpy()[0]) == pe_exact


def test_noalloc_rejects_more_cells_than_its_scratch(cuda_lib):
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    pairs = (_ffi.LJPair * 1)(_ffi.LJPair(1, 1, 1.0, 1.0, 2.5, 1))
    h = np.ascontiguousarray(np.eye(3) * 105.0)  # 42^3 = 74,088 cells at rc = 2.5
    dummy = C.c_void_p(1)  # never dereferenced: the size check fails first
    st = lib.pis_gpu_compute_potential_noalloc(pairs, 1, 1, 1000, dummy, dummy,
                                               h.ctypes.data_as(C.POINTER(C.c_double)), dummy, dummy, None)
    assert _ffi.STATUS_NAMES[st] == "PIS_ERR_INVALID_ARGUMENT"
