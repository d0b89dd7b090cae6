"""Seeded synthetic cubelets for the benchmark and tests.

The reference's sample images are partly missing from its checkout and no
public dataset is named for this path, so seeded synthetic volumes with the
shapes, sizes and value distributions of the benchmark workloads stand in:

* ``plain_2d``    2048x2048x1 uint8: 64 Gaussian blobs (sigma 8-256 px,
  amplitude 20-120) + a linear gradient + N(0,3) noise, clipped to 0..255.
* ``volume_f32``  256^3 float32: 200 axis-aligned anisotropic 3-D Gaussians
  (sigma 2-64 voxels per axis, amplitude in [-1,1]) + N(0,0.01) noise.
* ``mixed_batch`` 512 cubelets, axis lengths from {16,32,48,64,96,128,256},
  dtypes 50% uint8 / 30% uint16 / 20% float32, blob contents scaled to the
  dtype range.
* ``phantom_u16`` an ellipsoid phantom (40 ellipsoids with piecewise-constant
  densities 0..4095 + N(0,20)) for the large-volume split workload.

Blobs are evaluated only inside +-4 sigma of their centre (the tail beyond is
below 3.4e-4 of the amplitude), which keeps generation fast.
"""
from __future__ import annotations

import numpy as np

AXIS_CHOICES = (16, 32, 48, 64, 96, 128, 256)


def _gauss1d(n, centre, sigma):
    lo = max(0, int(np.floor(centre - 4 * sigma)))
    hi = min(n, int(np.ceil(centre + 4 * sigma)) + 1)
    x = np.arange(lo, hi, dtype=np.float32)
    return lo, hi, np.exp(-0.5 * ((x - centre) / sigma) ** 2).astype(np.float32)


def add_blobs(vol: np.ndarray, rng: np.random.Generator, count: int,
              sigma_range, amp_range) -> None:
    """Add ``count`` separable Gaussian blobs to ``vol`` (any of 1-3 dims) in
    place; each axis gets its own sigma (anisotropic, axis-aligned)."""
    shape = vol.shape
    for _ in range(count):
        amp = np.float32(rng.uniform(*amp_range))
        slices, factors = [], []
        for n in shape:
            c = rng.uniform(0, n)
            s = rng.uniform(*sigma_range)
            lo, hi, g = _gauss1d(n, c, s)
            slices.append(slice(lo, hi))
            factors.append(g)
        if any(f.size == 0 for f in factors):
            continue
        blob = factors[0]
        for f in factors[1:]:
            blob = np.multiply.outer(blob, f)
        vol[tuple(slices)] += amp * blob


def plain_2d(seed: int = 20261203, size: int = 2048) -> np.ndarray:
    """(1, size, size) uint8 image of blobs + gradient + noise."""
    rng = np.random.default_rng(seed)
    img = np.zeros((size, size), np.float32)
    add_blobs(img, rng, 64, (8.0, 256.0), (20.0, 120.0))
    gy, gx = rng.uniform(-40, 40, size=2)
    ramp = (np.arange(size, dtype=np.float32) / size)
    img += np.float32(gy) * ramp[:, None] + np.float32(gx) * ramp[None, :]
    img += rng.normal(0.0, 3.0, img.shape).astype(np.float32)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)[None]


def volume_f32(seed: int = 20261204, size=(256, 256, 256), blobs: int = 200) -> np.ndarray:
    """(depth, height, width) float32 volume of blobs + N(0, 0.01) noise."""
    rng = np.random.default_rng(seed)
    vol = np.zeros(size, np.float32)
    add_blobs(vol, rng, blobs, (2.0, 64.0), (-1.0, 1.0))
    vol += rng.normal(0.0, 0.01, vol.shape).astype(np.float32)
    return vol


def scaled_blob_cubelet(rng: np.random.Generator, shape, dtype) -> np.ndarray:
    """Blob contents scaled to the dtype's range (used by the mixed batch)."""
    vol = np.zeros(shape, np.float32)
    smax = max(2.0, min(shape) / 2.0)
    add_blobs(vol, rng, 12, (2.0, smax), (-1.0, 1.0))
    vol += rng.normal(0.0, 0.01, shape).astype(np.float32)
    if dtype == np.float32:
        return vol
    lo, hi = float(vol.min()), float(vol.max())
    span = hi - lo if hi > lo else 1.0
    top = 255.0 if dtype == np.uint8 else 65535.0
    return np.clip(np.rint((vol - lo) / span * top), 0, top).astype(dtype)


def mixed_batch(seed: int = 20261205, count: int = 512):
    """List of (depth, height, width) arrays of mixed shapes and dtypes, plus
    the wavelet choice for each (1 = Haar, 2 = CDF9/7, half each)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        shape = tuple(int(rng.choice(AXIS_CHOICES)) for _ in range(3))
        u = rng.uniform()
        dtype = np.uint8 if u < 0.5 else (np.uint16 if u < 0.8 else np.float32)
        wavelet = 1 if rng.uniform() < 0.5 else 2
        out.append((scaled_blob_cubelet(rng, shape, dtype), wavelet))
    return out


def phantom_u16(seed: int = 20261206, size: int = 1024, ellipsoids: int = 40) -> np.ndarray:
    """size^3 uint16 ellipsoid phantom: each ellipsoid sets its voxels to a
    density drawn from 0..4095 (later ones overwrite earlier ones), + N(0,20)."""
    rng = np.random.default_rng(seed)
    vol = np.zeros((size, size, size), np.float32)
    for _ in range(ellipsoids):
        c = rng.uniform(0.15, 0.85, 3) * size
        r = rng.uniform(0.03, 0.3, 3) * size
        dens = np.float32(rng.uniform(0, 4095))
        lo = np.maximum(0, np.floor(c - r)).astype(int)
        hi = np.minimum(size, np.ceil(c + r) + 1).astype(int)
        z = ((np.arange(lo[0], hi[0], dtype=np.float32) - c[0]) / r[0]) ** 2
        y = ((np.arange(lo[1], hi[1], dtype=np.float32) - c[1]) / r[1]) ** 2
        x = ((np.arange(lo[2], hi[2], dtype=np.float32) - c[2]) / r[2]) ** 2
        inside = (z[:, None, None] + y[None, :, None] + x[None, None, :]) <= 1.0
        sub = vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[inside] = dens
    for z0 in range(0, size, 64):
        sl = vol[z0:z0 + 64]
        sl += rng.normal(0.0, 20.0, sl.shape).astype(np.float32)
    return np.clip(np.rint(vol), 0, 65535).astype(np.uint16)


def small_cases(seed: int = 7):
    """Small and odd shapes for parity tests: (name, array) pairs."""
    rng = np.random.default_rng(seed)
    cases = []
    for shape, dt in [((1, 64, 64), np.uint8), ((8, 16, 32), np.float32),
                      ((5, 7, 9), np.uint8), ((3, 2, 5), np.float32),
                      ((16, 16, 16), np.uint16), ((1, 1, 37), np.float32),
                      ((2, 33, 17), np.uint8), ((12, 20, 24), np.float32)]:
        a = scaled_blob_cubelet(rng, shape, dt)
        cases.append((f"{dt.__name__}_{'x'.join(map(str, shape))}", a))
    return cases


def serving_pool(seed: int = 20261207, count: int = 64, cap_bytes: int = 256 << 20,
                 base_size: int = 128):
    """Request payloads for the serving workload: every axis log-uniform in
    16..512, dtypes uint8 / uint16 / float32 in equal parts, input at most
    cap_bytes (redrawn otherwise).  Contents are mirrored crops of one blob
    volume, scaled to the dtype range (cheap to make at any size)."""
    rng = np.random.default_rng(seed)
    base = np.zeros((base_size,) * 3, np.float32)
    add_blobs(base, rng, 40, (2.0, base_size / 2.0), (-1.0, 1.0))
    base += rng.normal(0.0, 0.01, base.shape).astype(np.float32)
    lo, hi = float(base.min()), float(base.max())
    span = hi - lo if hi > lo else 1.0
    dtypes = (np.uint8, np.uint16, np.float32)
    out = []
    for i in range(count):
        dt = dtypes[i % 3]
        while True:
            shape = tuple(int(np.exp(rng.uniform(np.log(16), np.log(512)))) for _ in range(3))
            if int(np.prod(shape)) * np.dtype(dt).itemsize <= cap_bytes:
                break
        idx = []
        for n in shape:  # mirrored walk through the base volume from a random start
            k = (rng.integers(0, base_size) + np.arange(n)) % (2 * base_size)
            idx.append(np.where(k < base_size, k, 2 * base_size - 1 - k))
        v = base[np.ix_(*idx)]
        if dt == np.float32:
            out.append(np.ascontiguousarray(v))
        else:
            top = 255.0 if dt == np.uint8 else 65535.0
            out.append(np.clip(np.rint((v - lo) / span * top), 0, top).astype(dt))
    return out
