"""The -opt parameter sweep (optimizeParameters -> plotAll) on the GPU
against the table the reference itself printed for the same input (fixtures
from tests/golden/make_golden.py).  With the transform in the reference's
float order the coefficients, thresholds, bins and Huffman tables are the
reference's, so every point's size is identical; the PSNR differs only by
the float rounding of the inverse transform."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from wavelets_gb300 import cubefile, lib, params as P

pytestmark = pytest.mark.gpu

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
OPT = MANIFEST["opt"]
PSNR_TOL_DB = 0.05


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _table(case):
    with open(os.path.join(GOLDEN, case["table"])) as f:
        lines = f.read().splitlines()
    assert lines[0] == "Threshold\tBins\tsize\tpSNR"
    return [ln.split("\t") for ln in lines[1:]]


@pytest.mark.parametrize("case", OPT["cases"], ids=lambda c: f"{c['case']}.{c['params']}")
def test_opt_sweep_matches_reference(ctx, case):
    p, _, _ = P.parse_flags(OPT["params"][case["params"]])
    p.exact_transform = True
    a = cubefile.read_file(os.path.join(GOLDEN, case["input"]))[0].array()
    got = ctx.optimize(a, p)
    want = _table(case)
    assert len(got) == len(want) == 1600
    worst = 0.0
    for (f, b, size, psnr), row in zip(got, want):
        assert f"{f:.3f}" == row[0] and b == int(row[1])
        assert size == int(row[2]), (row, size)
        worst = max(worst, abs(psnr - float(row[3])))
    assert worst <= PSNR_TOL_DB, worst


def test_opt_cli_prints_the_reference_table(ctx, tmp_path):
    case = OPT["cases"][0]
    exe = os.path.join(os.path.dirname(lib.LIB_PATH), "wl_compress")
    out = subprocess.run([exe, "-q", "-exact", *OPT["params"][case["params"]],
                          os.path.join(GOLDEN, case["input"]), str(tmp_path / "none.cube")],
                         capture_output=True, text=True, check=True).stdout.splitlines()
    want = _table(case)
    assert out[0] == "Threshold\tBins\tsize\tpSNR"
    assert len(out) == 1 + len(want)
    for got, row in zip(out[1:], want):
        g = got.split("\t")
        assert g[:3] == row[:3]
    assert not (tmp_path / "none.cube").exists()  # like the reference: no output


def test_opt_lifting_mode_close_to_reference(ctx):
    """Default (lifting) transform: sizes within 2% of the reference's."""
    case = OPT["cases"][0]
    p, _, _ = P.parse_flags(OPT["params"][case["params"]])
    a = cubefile.read_file(os.path.join(GOLDEN, case["input"]))[0].array()
    got = ctx.optimize(a, p)
    for (f, b, size, psnr), row in zip(got, _table(case)):
        assert abs(size - int(row[2])) <= 0.02 * int(row[2]) + 8
        assert abs(psnr - float(row[3])) <= 0.5
