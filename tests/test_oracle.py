"""The oracle (oracle/port) against the reference's own outputs.

The fixtures in tests/golden were produced by the reference compiled from its
own sources (tests/golden/make_golden.py); here the CPU restatement must
reproduce them bit for bit.  CPU only.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle
from wavelets_gb300 import cubefile
from conftest import GOLDEN

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))


def _case_ids():
    return [f"{c['case']}.{c['params']}" for c in MANIFEST["cases"]]


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_case_ids())
def test_oracle_cli_matches_reference_bytes(case, tmp_path):
    args = MANIFEST["params"][case["params"]]
    out = tmp_path / "o.cube"
    dec = tmp_path / "d.cube"
    inp = os.path.join(GOLDEN, case["input"])
    assert oracle.main(args + [inp, str(out)]) == 0
    assert out.read_bytes() == open(os.path.join(GOLDEN, case["output"]), "rb").read()
    assert oracle.main(["-d", str(out), str(dec)]) == 0
    assert dec.read_bytes() == open(os.path.join(GOLDEN, case["decompressed"]), "rb").read()


def test_oracle_kat_cdf97_one_step():
    kat = MANIFEST["kat_cdf97_1step"]
    v = np.array(kat["input"], np.float32).reshape(1, 1, 16)
    out = oracle.forward(v, (1, 0, 0))
    want = np.array([float.fromhex(h) for h in kat["output_hex"]], np.float32)
    assert np.array_equal(out, want)
    # the values printed in the reference's comment (6 significant digits)
    assert np.allclose(out, kat["published"], rtol=2e-5, atol=2e-6)
    back = oracle.inverse(out, (1, 1, 16), (1, 0, 0))
    assert np.allclose(back.ravel(), kat["input"], atol=1e-5)


@pytest.mark.parametrize("case", [c for c in MANIFEST["cases"] if c["params"] in ("p1", "p2", "p3")],
                         ids=lambda c: f"{c['case']}.{c['params']}")
def test_oracle_stages_match_reference(case):
    """Coefficients and the compressed stream from the stage functions."""
    inp = cubefile.read_file(os.path.join(GOLDEN, case["input"]))[0]
    ref = cubefile.read_file(os.path.join(GOLDEN, case["output"]))[0]
    p = ref.params
    a = inp.array().astype(np.float32)
    Z, Y, X = a.shape
    sx, sy, sz = p.steps
    pad = lambda n, s: ((n - 1) // (1 << s) + 1) * (1 << s)
    Xp, Yp, Zp = pad(X, sx), pad(Y, sy), pad(Z, sz)
    v = np.pad(a, ((0, Zp - Z), (0, Yp - Y), (0, Xp - X)), mode="edge")
    coeffs = oracle.forward(v, (sx, sy, sz), p.wavelet)
    golden = np.fromfile(os.path.join(GOLDEN, case["coeffs"]), np.float32)
    assert np.array_equal(coeffs, golden)
    qalg = {cubefile.PB_UNIFORM: oracle.UNIFORM, cubefile.PB_LOG: oracle.LOG,
            cubefile.PB_LLOYD: oracle.LLOYD}[p.quant_alg]
    enc = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, qalg,
                        p.huffman_dup_key is not None)
    assert np.float32(enc["threshold"]) == np.float32(p.threshold_value)
    assert np.array_equal(enc["words"], ref.words())
    assert list(enc["decode"]) == list(p.huffman_decode_table)
    dec = oracle.huffman_decode(enc["words"], enc["decode"], enc["dup_key"],
                                enc["dup_value"], coeffs.size)
    assert np.array_equal(dec, enc["bins"])


def test_padded_length_and_ceil_log2_asserts():
    """test_haar_cpu.cc:135-169 expectations, via the oracle's step clamp."""
    from wavelets_gb300 import params
    for x, want in [(1, 0), (2, 1), (3, 2), (4, 2), (5, 3), (8, 3), (9, 4),
                    (511, 9), (512, 9), (513, 10)]:
        assert params.ceil_log2(x) == want
    for n, s, want in [(4, 1, 4), (5, 1, 6), (5, 2, 8), (6, 1, 6), (6, 2, 8)]:
        assert params.padded_length(n, s) == want


def test_reference_cli_flags_rejected_like_reference(tmp_path):
    inp = os.path.join(GOLDEN, MANIFEST["cases"][0]["input"])
    assert oracle.main(["-thresh", "1.5", inp, str(tmp_path / "x.cube")]) != 0
    assert oracle.main(["-qalg", "count", inp, str(tmp_path / "x.cube")]) != 0


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_case_ids())
def test_float64_lifting_agrees_with_reference_coefficients(case):
    """The float64 lifting yardstick reproduces the reference's own float32
    coefficients to float32 rounding (pins the yardstick before it measures
    the GPU transform)."""
    from oracle import lifting64
    from wavelets_gb300 import params as P
    p, _, _ = P.parse_flags(MANIFEST["params"][case["params"]])
    a = cubefile.read_file(os.path.join(GOLDEN, case["input"]))[0].array()
    got, st = lifting64.forward(a, p.steps, p.wavelet, p.transform_2d)
    assert [int(s) for s in case["stats"]["steps"]] == list(st)
    ref = np.fromfile(os.path.join(GOLDEN, case["coeffs"]), np.float32).astype(np.float64)
    assert got.shape == ref.shape
    scale = float(np.abs(got).max())
    if scale == 0:
        assert np.abs(ref).max() == 0
        return
    assert float(np.abs(got - ref).max()) / scale <= 2e-6


ERR = MANIFEST.get("err", [])


@pytest.mark.parametrize("e", ERR, ids=[f"{e['input']}.{e['params']}" for e in ERR])
def test_oracle_err_line_matches_reference(e, tmp_path):
    """-err: the error line the reference printed (computeErrorRates,
    test_compress_common.cc:587-694, printed at test_compress_cpu.cc:155-156),
    reproduced character for character by the oracle's command line."""
    args = MANIFEST["params"][e["params"]]
    r = subprocess.run([oracle.cli_path(), "-q", "-err", *args,
                        os.path.join(GOLDEN, e["input"]), str(tmp_path / "o.cube")],
                       capture_output=True, text=True, check=True)
    got = [ln for ln in r.stdout.splitlines() if ln.startswith("Mean squared")]
    want = open(os.path.join(GOLDEN, e["err"])).read().split("\n")[0]
    assert got == [want]
    # the library-level numbers print to the same line
    m = oracle.error_metrics(os.path.join(GOLDEN, e["input"]), str(tmp_path / "o.cube"))
    assert "Mean squared error: %.3f, relative error: %g, peak SNR: %.3f" % (
        np.float32(m["mse"]), np.float32(m["relative_error"]), np.float32(m["psnr"])) == want
