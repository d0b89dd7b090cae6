"""Failure paths of the C ABI: malformed input is rejected on the host with a
status code before anything is launched, and the context stays usable
afterwards.  The reference has no counterpart beyond printing and exit(1)
(cucheck.h:9-21, parseOptions); here every case returns WL_EFORMAT,
WL_EINVAL or WL_ENOMEM and wl_last_error says why.  No case faults the GPU:
each is refused by the host-side checks (file codec, check_result,
check_params, the workspace cap)."""
import ctypes
import dataclasses
import os

import numpy as np
import pytest

from conftest import GOLDEN
from wavelets_gb300 import cubefile, lib, params as P, synth

pytestmark = pytest.mark.gpu

COMP = os.path.join(GOLDEN, "uint8_1x64x64.p1.cube")   # a reference-compressed file
INP = os.path.join(GOLDEN, "uint8_1x64x64.in.cube")


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _status(fn, *a):
    try:
        fn(*a)
    except lib.WlError as e:
        return e.status
    return lib.WL_OK


def _still_works(ctx):
    a = synth.volume_f32(3, (8, 8, 8), 4)
    back = ctx.decompress(ctx.compress(a, P.Params(steps=(2, 2, 2))))
    assert back.shape == a.shape


def test_truncated_compressed_file(ctx, tmp_path):
    data = open(COMP, "rb").read()
    for cut in (len(data) - 5, 70, 40, 10):
        p = tmp_path / f"t{cut}.cube"
        p.write_bytes(data[:cut])
        assert _status(ctx.decompress_file, str(p), str(tmp_path / "d.cube")) == lib.WL_EFORMAT
    _still_works(ctx)


def test_truncated_input_file(ctx, tmp_path):
    data = open(INP, "rb").read()
    p = tmp_path / "t.cube"
    p.write_bytes(data[:len(data) - 100])
    assert _status(ctx.compress_file, str(p), str(tmp_path / "o.cube"),
                   P.Params()) == lib.WL_EFORMAT
    _still_works(ctx)


def test_corrupt_header(ctx, tmp_path):
    data = bytearray(open(COMP, "rb").read())
    data[0:4] = b"XXXX"
    p = tmp_path / "h.cube"
    p.write_bytes(bytes(data))
    assert _status(ctx.decompress_file, str(p), str(tmp_path / "d.cube")) == lib.WL_EFORMAT
    assert _status(ctx.compress_file, str(p), str(tmp_path / "o.cube"),
                   P.Params()) == lib.WL_EFORMAT


def test_compressed_size_not_whole_words(ctx, tmp_path):
    """The stream's byte count (4 x words, writeQuantData) must be whole
    32-bit words."""
    c = cubefile.read_file(COMP)[0]
    bad = dataclasses.replace(c, data=c.data + b"\0\0")
    p = tmp_path / "w.cube"
    cubefile.write_file(str(p), [bad], footer=False)
    assert _status(ctx.decompress_file, str(p), str(tmp_path / "d.cube")) == lib.WL_EFORMAT
    _still_works(ctx)


def _result(ctx):
    a = synth.scaled_blob_cubelet(np.random.default_rng(2), (12, 20, 28), np.uint8)
    return ctx.compress(a, P.Params(steps=(2, 2, 2), threshold_fraction=0.8))


def test_decode_table_child_out_of_range(ctx):
    c = _result(ctx)
    dec = np.array(c.decode, np.int32)
    node = next(i for i in range(0, dec.size, 2) if dec[i] != 0)  # an inner node
    dec[node] = 10 ** 6
    bad = dataclasses.replace(c, decode=dec)
    assert _status(ctx.decompress, bad) == lib.WL_EFORMAT
    dec2 = np.array(c.decode, np.int32)
    dec2[node + 1] = -3
    assert _status(ctx.decompress, dataclasses.replace(c, decode=dec2)) == lib.WL_EFORMAT
    _still_works(ctx)


def test_stream_too_short_for_its_cubelet(ctx):
    c = _result(ctx)
    bad = dataclasses.replace(c, words=np.array(c.words[: max(1, c.words.size // 4)]))
    assert _status(ctx.decompress, bad) == lib.WL_EFORMAT
    _still_works(ctx)


def test_bin_count_out_of_range(ctx):
    a = synth.volume_f32(4, (8, 8, 8), 4)
    for bins in (1, 4097, -5):
        assert _status(ctx.compress, a, P.Params(bin_count=bins)) == lib.WL_EINVAL
    assert _status(ctx.compress, a, P.Params(quant_alg=P.LLOYD, bin_count=2)) == lib.WL_EINVAL
    assert _status(ctx.compress, a, P.Params(threshold_fraction=1.5)) == lib.WL_EINVAL
    c = _result(ctx)
    assert _status(ctx.decompress, dataclasses.replace(c, bin_count=1)) == lib.WL_EFORMAT
    assert _status(ctx.decompress, dataclasses.replace(c, bin_count=5000)) == lib.WL_EFORMAT
    _still_works(ctx)


def test_inconsistent_sizes(ctx):
    c = _result(ctx)
    assert _status(ctx.decompress, dataclasses.replace(c, original_size=(999, 1, 1))) == \
        lib.WL_EFORMAT
    assert _status(ctx.decompress, dataclasses.replace(c, steps=(31, 0, 0))) == lib.WL_EFORMAT


def test_workspace_limit_gives_enomem_and_recovers():
    """A context capped below what a call needs fails with WL_ENOMEM before
    freeing or launching anything; raising the cap makes the same call work."""
    c = lib.Context(0)
    try:
        a = synth.volume_f32(6, (64, 64, 64), 8)
        c.set_memory_limit(1 << 20)
        assert _status(c.compress, a, P.Params(steps=(3, 3, 3))) == lib.WL_ENOMEM
        assert "limit" in c.lib.wl_last_error(c.h).decode()
        assert c.memory_held() <= 1 << 20
        c.set_memory_limit(0)
        comp = c.compress(a, P.Params(steps=(3, 3, 3)))
        held = c.memory_held()
        c.set_memory_limit(held)  # at the cap: the same geometry still fits
        assert np.array_equal(c.compress(a, P.Params(steps=(3, 3, 3))).words, comp.words)
        big = synth.volume_f32(7, (128, 128, 128), 8)
        assert _status(c.compress, big, P.Params(steps=(3, 3, 3))) == lib.WL_ENOMEM
        assert np.array_equal(c.compress(a, P.Params(steps=(3, 3, 3))).words, comp.words)
    finally:
        c.close()


def test_error_metrics_size_mismatch(ctx, tmp_path):
    other = os.path.join(GOLDEN, "uint8_2x33x17.in.cube")
    assert _status(ctx.error_metrics_file, other, COMP) == lib.WL_EINVAL
    assert _status(ctx.error_metrics_file, COMP, COMP) == lib.WL_EFORMAT
