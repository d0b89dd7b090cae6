"""The seeded synthetic workloads (no GPU): shapes, element types, mixes and
value ranges of the benchmark configurations they stand in for -- the
2048x2048 u8 image (64 blobs + gradient + N(0,3), clipped 0..255), the 256^3
f32 volume (200 Gaussians, amplitude in [-1, 1], + N(0,0.01)), the 512 mixed
cubelets (axes from {16..256}, 50% u8 / 30% u16 / 20% f32, Haar or CDF 9/7
half each, contents scaled to the element type's range), the serving pool
(axes log-uniform 16..512, at most 256 MiB, u8/u16/f32 in thirds) and the
ellipsoid phantom (densities 0..4095 + N(0,20)) -- and that each is the same
for the same seed."""
import collections

import numpy as np

from wavelets_gb300 import synth


def test_plain_2d():
    img = synth.plain_2d()
    assert img.shape == (1, 2048, 2048) and img.dtype == np.uint8
    assert img.min() == 0 and img.max() == 255  # clipped at both ends
    assert img.std() > 20
    assert np.array_equal(img, synth.plain_2d())


def test_volume_f32():
    v = synth.volume_f32()
    assert v.shape == (256, 256, 256) and v.dtype == np.float32
    assert np.isfinite(v).all()
    # sums of 200 blobs of amplitude in [-1, 1]: both signs, a few units at most
    assert v.min() < -0.5 and v.max() > 0.5
    assert np.abs(v).max() < 10


def test_mixed_batch():
    items = synth.mixed_batch(count=512)
    assert len(items) == 512
    dtypes = collections.Counter(a.dtype.name for a, _ in items)
    # 512 draws of a 50/30/20 mix (bounds about three standard deviations)
    assert 0.43 <= dtypes["uint8"] / 512 <= 0.57
    assert 0.23 <= dtypes["uint16"] / 512 <= 0.37
    assert 0.14 <= dtypes["float32"] / 512 <= 0.26
    waves = collections.Counter(w for _, w in items)
    assert set(waves) == {1, 2} and 0.42 <= waves[1] / 512 <= 0.58
    for a, _ in items:
        assert a.ndim == 3 and all(n in synth.AXIS_CHOICES for n in a.shape)
        if a.dtype == np.uint8:
            assert a.min() == 0 and a.max() == 255
        elif a.dtype == np.uint16:
            assert a.min() == 0 and a.max() == 65535
    again = synth.mixed_batch(count=4)
    assert all(np.array_equal(a, b) and w == v
               for (a, w), (b, v) in zip(again, items[:4]))


def test_serving_pool():
    pool = synth.serving_pool(count=24)
    assert len(pool) == 24
    for i, a in enumerate(pool):
        assert a.dtype == (np.uint8, np.uint16, np.float32)[i % 3]
        assert a.nbytes <= 256 << 20
        assert all(16 <= n <= 512 for n in a.shape)


def test_phantom_u16():
    ph = synth.phantom_u16(size=96)
    assert ph.shape == (96, 96, 96) and ph.dtype == np.uint16
    # densities 0..4095 plus N(0, 20): a few sigma above 4095 at most
    assert ph.max() <= 4095 + 200
    assert len(np.unique(ph[48])) > 50
    assert np.array_equal(ph, synth.phantom_u16(size=96))
