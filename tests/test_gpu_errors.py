"""-err error metrics on the GPU (wl_error_metrics, wl_error_metrics_file,
the command line's -err) against the oracle's restatement of the reference's
computeErrorRates (test_compress_common.cc:587-694; ErrorAccumulator,
test_compress_common.h:90-160), which itself reproduces the reference's
printed -err lines (tests/test_oracle.py).

Both sides measure the same compressed stream.  The sums over the original
alone are equal up to summation order; the error sums differ only where the
GPU's lifting inverse transform and the reference's filter bank round a
restored value to a different integer (a last-bit difference on a .5 or
integer boundary), so they are held to ERR_RTOL and the PSNR to
PSNR_TOL_DB."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle
from wavelets_gb300 import cubefile, lib, params as P, synth

pytestmark = pytest.mark.gpu

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
ERR = MANIFEST.get("err", [])
ERR_RTOL = 0.02       # relative difference of the error sums and getters
PSNR_TOL_DB = 0.05
SUM_RTOL = 1e-12      # sums over the original values (summation order only)


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _close(got, want):
    assert got["count"] == want["count"]
    if want["count"] == 0:
        assert got["mse"] == 0 and got["psnr"] == 0 and got["relative_error"] == 0
        return
    for k in ("sum_value", "sum_value_squared"):
        assert abs(got[k] - want[k]) <= SUM_RTOL * max(1.0, abs(want[k])), k
    for k in ("sum_diff", "sum_diff_squared", "l1", "l2", "mse", "average_error",
              "relative_error"):
        assert abs(got[k] - want[k]) <= ERR_RTOL * max(abs(want[k]), 1e-3), (k, got[k], want[k])
    assert abs(got["psnr"] - want["psnr"]) <= PSNR_TOL_DB, (got["psnr"], want["psnr"])


def _flags(p):
    prm, _, _ = P.parse_flags(MANIFEST["params"][p])
    return prm


@pytest.mark.parametrize("e", ERR, ids=[f"{e['input']}.{e['params']}" for e in ERR])
def test_error_metrics_file_against_oracle(ctx, e, tmp_path):
    inp = os.path.join(GOLDEN, e["input"])
    out = str(tmp_path / "o.cube")
    prm = _flags(e["params"])
    prm.exact_transform = True  # the reference's compressed file, byte for byte
    ctx.compress_file(inp, out, prm)
    got = ctx.error_metrics_file(inp, out)
    want = oracle.error_metrics(inp, out)
    _close(got, want)


@pytest.mark.parametrize("name", ["plain2d", "volume"])
def test_error_metrics_bench_cubelets_against_oracle(ctx, name, tmp_path):
    """The single-cubelet benchmark workloads (default lifting transform),
    the original passed as an array and the peak given explicitly."""
    import bench
    (a, p), = bench.WORKLOADS[name][0](20261205, 1)
    if name == "volume":
        a = a[:96, :128, :160]  # keeps the oracle's restore quick
    comp = ctx.compress(a, p)
    peak = 255.0 if a.dtype == np.uint8 else 1.0
    got = ctx.error_metrics(comp, a, peak)
    inp, cub = str(tmp_path / "in.cube"), str(tmp_path / "c.cube")
    cubefile.write_file(inp, [cubefile.from_array(a, maximum_value=int(peak))])
    with open(cub, "wb") as f:
        f.write(lib.encode_cube(comp))
    want = oracle.error_metrics(inp, cub)
    _close(got, want)


def test_error_metrics_u16_and_device_original(ctx):
    """16-bit data (compared like the reference's INT32 carriage) from a
    device pointer equals the same from host memory."""
    a = synth.scaled_blob_cubelet(np.random.default_rng(41), (24, 40, 56), np.uint16)
    comp = ctx.compress(a, P.Params(steps=(3, 3, 3), threshold_fraction=0.9,
                                    quant_alg=P.UNIFORM, bin_count=1024))
    host = ctx.error_metrics(comp, a, 65535.0)
    dev = lib.DeviceBuffer(a.nbytes)
    dev.upload(a)
    st = lib.WlErrorStats()
    r = comp.to_struct()
    import ctypes
    L = lib.load()
    assert L.wl_error_metrics(ctx.h, ctypes.byref(r), ctypes.c_void_p(dev.ptr), lib.WL_U16, 1,
                              ctypes.c_float(65535.0), ctypes.byref(st)) == lib.WL_OK
    dev.free()
    assert st.as_dict() == host
    assert host["count"] == a.size and host["psnr"] > 30


def test_error_metrics_without_peak_computes_nothing(ctx):
    a = synth.volume_f32(5, (8, 8, 8), 4)
    comp = ctx.compress(a, P.Params(steps=(2, 2, 2)))
    m = ctx.error_metrics(comp, a, 0.0)
    assert m["count"] == 0 and m["mse"] == 0 and m["psnr"] == 0


def test_cli_err_line(ctx, tmp_path):
    """The command line's -err prints the reference's line, with the numbers
    of the golden fixture (same stream, exact transform order)."""
    from wavelets_gb300 import build
    e = next(x for x in ERR if x["input"] == "uint8_1x64x64.in.cube")
    cli = os.path.join(os.path.dirname(lib.LIB_PATH), "wl_compress")
    r = subprocess.run([cli, "-q", "-err", "-exact", *MANIFEST["params"][e["params"]],
                        os.path.join(GOLDEN, e["input"]), str(tmp_path / "o.cube")],
                       capture_output=True, text=True, check=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("Mean squared error:")]
    assert len(line) == 1
    want = open(os.path.join(GOLDEN, e["err"])).read().split("\n")[0]
    g = [float(x.split(":")[1]) for x in line[0].split(",")]
    w = [float(x.split(":")[1]) for x in want.split(",")]
    assert abs(g[0] - w[0]) <= ERR_RTOL * w[0] + 1e-3
    assert abs(g[2] - w[2]) <= PSNR_TOL_DB
