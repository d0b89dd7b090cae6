"""A volume split into overlapping cubelets is compressed in place (each
cubelet read from the volume through its row and slice pitches): the
streams equal those of the cubelets copied out, whether the volume is in
device, page-locked or pageable memory."""
import numpy as np
import pytest

from wavelets_gb300 import lib, params as P, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _same(a, b):
    return (np.array_equal(a.words, b.words) and np.array_equal(a.decode, b.decode)
            and a.threshold_value == b.threshold_value)


def test_split_in_place_equals_copies(ctx):
    vol = synth.phantom_u16(3, size=96, ellipsoids=12)[:70, :90, :]  # (Z, Y, X) = 70, 90, 96
    vol = np.ascontiguousarray(vol)
    p = P.Params(steps=(3, 3, 3), wavelet=P.CDF97, threshold_fraction=0.97,
                 quant_alg=P.LOG, bin_count=512)
    grid, got = ctx.compress_split(vol, cube=(32, 32, 32), overlap=4, params=p)
    copies = [np.ascontiguousarray(vol[oz:oz + sz, oy:oy + sy, ox:ox + sx])
              for (ox, oy, oz), (sx, sy, sz) in grid]
    ref = ctx.compress_batch([(c, p) for c in copies])
    assert len(grid) == 4 * 4 * 3  # x: 96, y: 90, z: 70 in steps of 28
    assert all(_same(a, b) for a, b in zip(got, ref))

    dev = lib.DeviceBuffer(vol.nbytes)
    dev.upload(vol)
    _, on_dev = ctx.compress_split(vol, cube=(32, 32, 32), overlap=4, params=p, ptr=dev.ptr,
                                   on_device=True)
    assert all(_same(a, b) for a, b in zip(on_dev, ref))
    pin = lib.PinnedBuffer(vol.nbytes)
    pin.array(vol.dtype, vol.shape)[...] = vol
    _, pinned = ctx.compress_split(vol, cube=(32, 32, 32), overlap=4, params=p, ptr=pin.ptr)
    assert all(_same(a, b) for a, b in zip(pinned, ref))

    # round trip: every cubelet restores its own part of the volume
    back = np.zeros(vol.shape, np.float64)
    for ((ox, oy, oz), (sx, sy, sz)), c in zip(grid, got):
        back[oz:oz + sz, oy:oy + sy, ox:ox + sx] = ctx.decompress(c)
    mse = float(np.mean((back - vol) ** 2))
    assert 10 * np.log10(65535.0 ** 2 / mse) > 40.0
