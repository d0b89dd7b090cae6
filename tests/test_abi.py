"""The C ABI: libwlgpu.so builds for sm_103a, loads without a GPU, exports every
function include/wlgpu.h declares, and the header compiles as plain C.
CPU only (no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "wlgpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wl_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from wavelets_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from wavelets_gb300 import lib as L
    assert set(declared_functions()) <= set(L.EXPORTS)


def test_header_is_plain_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "wlgpu.h"\nint main(void){wl_params p; wl_params_default(&p);'
                   'return p.bin_count == 256 ? 0 : 1;}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-c", str(src), "-I",
                        os.path.dirname(HEADER), "-o", str(tmp_path / "t.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_defaults_match_reference(lib):
    """wl_params_default = the reference's defaults (wavelet.h:48-53)."""
    from wavelets_gb300 import lib as L
    p = L.WlParams()
    lib.wl_params_default(ctypes.byref(p))
    assert list(p.steps) == [-1, -1, -1]
    assert p.wavelet == 2 and p.bin_count == 256 and p.quant_alg == 2
    assert abs(p.threshold_fraction - 0.5) < 1e-7 and p.compress_zeros == 1


def test_init_without_gpu_fails_cleanly(lib):
    """No GPU in this container: wl_init reports an error instead of exiting."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    lib.wl_init.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    assert lib.wl_init(0, ctypes.byref(h)) != 0


def test_serve_create_without_gpu_fails_cleanly(lib):
    """No GPU: the server reports an error instead of starting lanes."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    from wavelets_gb300 import lib as L
    cfg = L.WlServeConfig()
    lib.wl_serve_config_default.argtypes = [ctypes.POINTER(L.WlServeConfig)]
    lib.wl_serve_config_default(ctypes.byref(cfg))
    assert cfg.lanes == 2 and cfg.memory_budget == 16 << 30 and cfg.max_batch == 1024
    h = ctypes.c_void_p()
    lib.wl_serve_create.argtypes = [ctypes.c_int, ctypes.POINTER(L.WlServeConfig),
                                    ctypes.POINTER(ctypes.c_void_p)]
    assert lib.wl_serve_create(0, ctypes.byref(cfg), ctypes.byref(h)) != 0
    assert not h.value


def test_tile_table_round_trip(lib):
    """The tile table needs no GPU: lines imported come back exported, bad
    lines are refused, reset empties it."""
    from wavelets_gb300 import lib as L
    L.tune_reset()
    assert L.tune_table() == ""
    L.tune_load("0 0 6 64 8 10.5 9.25 11 0 8 7.5\n3 3 9 32 4\n\n")
    rows = L.tune_rows(L.tune_table())
    assert rows[(0, 0, 6)] == ((64, 8), (10.5, 9.25, 11.0, 0.0, 8.0, 7.5))
    assert rows[(3, 3, 9)][0] == (32, 4)
    for bad in ("0 0 6 48 4\n", "0 0 6 32 6\n", "6 0 6 32 4\n", "0 8 6 32 4\n",
                "0 0 10 32 4\n", "0 0 6 32\n"):
        with pytest.raises(L.WlError):
            L.tune_load(bad)
    L.tune_reset()
    assert L.tune_table() == ""
