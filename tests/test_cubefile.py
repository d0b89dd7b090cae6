"""Host-side parity of the Python `.cube` codec and the reference flag parser
(no GPU), pinned to files the reference itself wrote (tests/golden, made by
tests/golden/make_golden.py from the reference's own command line).

* cubefile: every golden file -- the reference's inputs, compressed outputs
  and decompressed outputs -- decodes and re-encodes to the same bytes
  (CubeletStreamWriter / CubeletStreamReader, cubelet_file.cc:259-327,
  :330-540; wavelet_compress.proto).
* params.parse_flags: the flags each golden was made with
  (test_compress_common.cc:35-192) parse to the parameters the reference
  recorded in its compressed output: clamped steps (setWaveletSteps,
  test_compress_common.cc:362-374), wavelet, threshold fraction (as a
  float32), bin count, quantizer, the zero-run key (present unless -noz) and
  the 2-D flag.
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from wavelets_gb300 import cubefile as cf, params as P

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.cube")))

WAVE_WIRE = {P.HAAR: cf.PB_HAAR, P.CDF97: cf.PB_CDF97}
QALG_WIRE = {P.UNIFORM: cf.PB_UNIFORM, P.LOG: cf.PB_LOG, P.LLOYD: cf.PB_LLOYD}


def test_goldens_present():
    assert len(FILES) >= 70


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_reference_file_round_trips_byte_exact(path):
    raw = open(path, "rb").read()
    cubelets = cf.decode_file(raw)
    assert cubelets
    assert cf.encode_file(cubelets, footer=raw.endswith(b"cube")) == raw


def _first_case_per_params():
    seen, out = set(), []
    for c in MANIFEST["cases"]:
        if c["params"] not in seen:
            seen.add(c["params"])
            out.append(c)
    return out


CASES = _first_case_per_params()


@pytest.mark.parametrize("case", CASES, ids=[c["params"] + "-" + c["case"] for c in CASES])
def test_flags_parse_to_the_parameters_the_reference_recorded(case):
    p, decompress, rest = P.parse_flags(MANIFEST["params"][case["params"]])
    assert not decompress and not rest
    cub = cf.read_file(os.path.join(GOLDEN, case["output"]))[0]
    q = cub.params
    assert cub.compression == cf.COMP_WAVELET
    assert tuple(q.steps) == tuple(P.clamp_steps(p.steps, q.original_size))
    assert q.wavelet == WAVE_WIRE[p.wavelet]
    assert q.threshold_fraction == float(np.float32(p.threshold_fraction))
    assert q.bin_count == p.bin_count
    assert q.quant_alg == QALG_WIRE[p.quant_alg]
    assert (q.huffman_dup_key is not None) == p.compress_zeros
    if p.compress_zeros:
        assert q.huffman_dup_key == p.bin_count
    assert bool(q.transform_2d) == p.transform_2d


def test_parse_flags_step_forms_and_errors():
    assert P.parse_flags(["-steps", "3"])[0].steps == (3, 3, 3)
    assert P.parse_flags(["-steps", "3,2"])[0].steps == (3, 2, 0)
    assert P.parse_flags(["-steps", "1,2,3"])[0].steps == (1, 2, 3)
    p, d, rest = P.parse_flags(["-d", "in.cube", "out.cube"])
    assert d and rest == ["in.cube", "out.cube"]
    with pytest.raises(ValueError):
        P.parse_flags(["-steps", "1,2,3,4"])
    with pytest.raises(ValueError):
        P.parse_flags(["-thresh", "1.5"])
