"""The C-ABI library builds, loads and exports every symbol its headers declare (no GPU needed:
nothing here calls into the device)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = []
    for name in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        syms += re.findall(r"\b(pis_[a-z0-9_]+)\s*\(", text)
    return sorted(set(syms))


@pytest.fixture(scope="module")
def built_lib():
    from pis_gb300 import build
    return ctypes.CDLL(build.build())


def test_every_declared_symbol_is_exported(built_lib):
    syms = declared_symbols()
    assert "pis_gpu_create" in syms and "pis_gpu_verlet_step_nve" in syms
    missing = [s for s in syms if not hasattr(built_lib, s)]
    assert not missing, missing


def test_ffi_signatures_cover_header():
    from pis_gb300 import _ffi
    bound = {name for name, _, _ in _ffi.SIGNATURES}
    gpu_syms = [s for s in declared_symbols() if s.startswith("pis_gpu_")]
    assert set(gpu_syms) <= bound


def test_version_string(built_lib):
    built_lib.pis_gpu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in built_lib.pis_gpu_version()


def test_create_validates_without_gpu():
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    h = ctypes.c_void_p()
    pair = (_ffi.LJPair * 1)(_ffi.LJPair(1, 3, 1.0, 1.0, 2.5, 1))
    assert lib.pis_gpu_create(pair, 1, 2, 0.3, 0, ctypes.byref(h)) == 1  # type 3 > n_types
    pair = (_ffi.LJPair * 1)(_ffi.LJPair(1, 1, 1.0, 1.0, 2.5, 1))
    assert lib.pis_gpu_create(pair, 1, 1, 0.3, 7, ctypes.byref(h)) == 1  # unknown precision
    assert lib.pis_gpu_create(pair, 1, 1, 0.3, 0, ctypes.byref(h)) == 0
    lib.pis_gpu_destroy(h)


def test_product_never_imports_oracle():
    for dirpath, _, files in os.walk(os.path.join(ROOT, "pis_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "from oracle" not in text, f
                assert "liboracle" not in text, f


def _ctx(lib, precision):
    from pis_gb300 import _ffi
    h = ctypes.c_void_p()
    pair = (_ffi.LJPair * 1)(_ffi.LJPair(1, 1, 1.0, 1.0, 2.5, 1))
    assert lib.pis_gpu_create(pair, 1, 1, 0.3, precision, ctypes.byref(h)) == 0
    return h


@pytest.mark.parametrize("precision,flags,status", [
    (1, 0, 0),                                      # defaults
    (1, 4 | (8 << 16), 0),                          # bulk-copy list stream, 8 rows per stage
    (1, (4 << 24) | (4 << 8), 0),                   # clusters of 4, a lane per member
    (1, (2 << 24) | (2 << 8), 0),                   # clusters of 2, a lane per member
    (1, 4 << 28, 0),                                # two-stage build
    (0, 4 << 28, 0),                                # two-stage build, FP64 path
    (0, 4, 26),                                     # bulk-copy stream needs the mixed path
    (1, 4 | (4 << 8), 26),                          # ... and one thread per atom
    (0, 4 << 24, 26),                               # cluster lists need the mixed path
    (1, (4 << 24) | (2 << 8), 1),                   # 2 lanes only with clusters of 2
    (1, 3 << 24, 1),                                # clusters of 3
    (1, 3 << 28, 1),                                # build clusters of 3
    (1, 5 << 16, 1),                                # batch of 5
    (1, 1 << 7, 1),                                 # unknown flag bit
])
def test_set_options_validates_without_gpu(precision, flags, status):
    from pis_gb300 import _ffi
    lib = _ffi.lib()
    h = _ctx(lib, precision)
    assert lib.pis_gpu_set_options(h, 0, flags) == status
    lib.pis_gpu_destroy(h)


def test_option_flags_match_header():
    from pis_gb300 import _ffi
    text = open(os.path.join(ROOT, "include", "pis_gpu.h")).read()
    assert "#define PIS_OPT_LIST_TMA 4" in text and "PIS_OPT_CLUSTER(m) ((m) << 24)" in text
    assert "PIS_OPT_SCAN(m) ((m) << 28)" in text and "PIS_ERR_TIMEOUT = 27" in text
    assert _ffi.option_flags(tma=True, batch=8) == 4 | (8 << 16)
    assert _ffi.option_flags(cluster=4, lanes=4, scan=0) == (4 << 24) | (4 << 8)
    assert _ffi.option_flags(scan=4, mixed_kahan=True) == (4 << 28) | 2
    assert _ffi.STATUS_NAMES[27] == "PIS_ERR_TIMEOUT"
    for name, value in (("PIS_OPT_TILE", 8), ("PIS_OPT_PLAIN_GRAPHS", 16), ("PIS_OPT_UNFUSED", 32),
                        ("PIS_OPT_REF_ORDER", 64)):
        assert f"#define {name} {value}" in text
    assert _ffi.option_flags(tiles=True) == 8
    assert _ffi.option_flags(ref_order=True) == 64
    assert _ffi.option_flags(plain_graphs=True, unfused=True) == 16 | 32


def test_stats_struct_matches_header():
    # the ctypes mirror of pis_gpu_stats lists the header's fields in order
    import ctypes
    from pis_gb300 import _ffi
    text = open(os.path.join(ROOT, "include", "pis_gpu.h")).read()
    body = text[text.index("typedef struct {\n    int64_t n_atoms;"):text.index("} pis_gpu_stats;")]
    names = [f[0] for f in _ffi.Stats._fields_]
    for n in names:
        assert n in body, n
    assert names[-2:] == ["fused_step", "reserved_"]
    assert ctypes.sizeof(_ffi.Stats) == 8 * 4 + 4 * 4 + 8 * 11 + 8


def test_serve_stats_struct_matches_header():
    import ctypes
    from pis_gb300 import _ffi
    text = open(os.path.join(ROOT, "include", "pis_gpu.h")).read()
    body = text[text.rindex("typedef struct {", 0, text.index("} pis_serve_stats;")):text.index("} pis_serve_stats;")]
    fields = re.findall(r"(int64_t|double)\s+([^;]+);", body)
    names = [n.strip() for _, group in fields for n in group.split(",")]
    assert names == [f[0] for f in _ffi.ServeStats._fields_]
    assert ctypes.sizeof(_ffi.ServeStats) == 6 * 8
