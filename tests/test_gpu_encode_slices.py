"""The bit packer's slices: every slice count gives the same packed bits.

The Huffman tokens of each 4096-element chunk are packed by F lanes (1 to 32)
that each take a contiguous share of the chunk's tokens; the count is chosen
from the batch size, so large batches pack with one lane per chunk and small
ones with up to 32.  The stream must not depend on it (the reference writes
one stream per cubelet, BitStreamWriter bit_stream.h:60-162): each count is
forced on the same batches and the results are compared word for word with
the default, which the oracle tests pin to the reference.
"""
import numpy as np
import pytest

from wavelets_gb300 import lib, params as P, synth

pytestmark = pytest.mark.gpu

SLICES = (1, 2, 4, 8, 16, 32)


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _batch(seed):
    """Shapes, types and quantizers that give sparse and dense chunks, short
    and long codes, with and without zero runs."""
    rng = np.random.default_rng(seed)
    items = []
    for i in range(14):
        shape = tuple(int(rng.choice([5, 16, 33, 48, 64, 96])) for _ in range(3))
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        alg = [P.LLOYD, P.LOG, P.UNIFORM][i % 3]
        p = P.Params(wavelet=P.HAAR if i % 2 else P.CDF97, quant_alg=alg,
                     bin_count=[256, 4096, 1024, 255, 64, 2048, 16][i % 7],
                     threshold_fraction=[0.9, 0.5, 0.0, 0.99][i % 4],
                     compress_zeros=i % 5 != 3)
        items.append((synth.scaled_blob_cubelet(rng, shape, dt), p))
    # chunks of white noise: nearly every element is a value token
    noise = rng.integers(0, 65536, (40, 64, 80)).astype(np.uint16)
    items.append((noise, P.Params(quant_alg=P.LOG, bin_count=4096, threshold_fraction=0.05)))
    return items


def _same(a, b):
    assert a.longest_code == b.longest_code
    assert np.array_equal(a.words, b.words)
    assert np.array_equal(a.decode, b.decode)


@pytest.mark.parametrize("seed", [11, 12])
def test_every_slice_count_packs_the_same_bits(ctx, seed):
    items = _batch(seed)
    want = ctx.compress_batch(items)
    try:
        for f in SLICES:
            ctx.set_encode_slices(f)
            got = ctx.compress_batch(items)
            for w, g in zip(want, got):
                _same(w, g)
    finally:
        ctx.set_encode_slices(0)


def test_single_cubelet_every_slice_count(ctx):
    rng = np.random.default_rng(3)
    a = synth.scaled_blob_cubelet(rng, (96, 128, 64), np.uint8)
    p = P.Params(wavelet=P.CDF97, quant_alg=P.LLOYD, bin_count=256, threshold_fraction=0.9)
    want = ctx.compress(a, p)
    try:
        for f in SLICES:
            ctx.set_encode_slices(f)
            _same(want, ctx.compress(a, p))
    finally:
        ctx.set_encode_slices(0)


def test_slice_count_rejects_bad_values(ctx):
    for bad in (-1, 3, 64):
        with pytest.raises(lib.WlError):
            ctx.set_encode_slices(bad)
