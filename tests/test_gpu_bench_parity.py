"""Parity at the benchmark workloads: the cubelets bench.py compresses,
checked one by one against the oracle (never against the GPU itself).

* Mixed batch (512 cubelets, axes 16..256, u8/u16/f32, Haar | CDF 9/7,
  Lloyd 256 trained 20 iterations, keep 10%): the whole batch is compressed
  from device memory in one call, exactly as the bench's timed step does;
  then a sample of 40+ cubelets that covers every axis length on every axis,
  every element type with both wavelets, and the largest cubelets of each
  type, is checked:
    - transform within 1e-5 (max error relative to the largest coefficient)
      of the reference's float32 transform (dwt_cpu.cc:943-992);
    - threshold, largest |c|, zero bin bit-exact (thresh_cpu.cc:80-109);
    - bins given the GPU's codebook (QuantCodebook::quant, quant.h:515-526)
      and the Huffman stream and decode table bit-exact
      (huffman.h:278-296, huffman.cc:177-211);
    - codebook quality: distortion of the reference's coefficients under the
      GPU codebook (20 Lloyd iterations on the |c| histogram) against the
      reference's own codebook (lloyds.cpp:30-141 to convergence), and the
      PSNR of the restored cubelet against the reference's whole path.
* Split volume (1024^3 u16 phantom, 128^3 cubelets with 8-voxel overlap,
  CDF 9/7 4,4,4, keep 3%, log 512): all 729 cubelets compressed in place from
  the device-resident volume; 8 cubelets, among them 64-voxel edge cubelets,
  checked the same way (log bins bit-exact through the oracle's quantizer).
* The single-cubelet workloads at full size (2048^2 u8 11,11,0; 256^3 f32
  3,3,3): transform within 1e-5 of the reference's float32 transform.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

import bench
from oracle import jobs, oracle
from wavelets_gb300 import lib, params as P, synth

pytestmark = pytest.mark.gpu

TRANSFORM_RTOL = 1e-5          # max|gpu - ref| / max|ref|
LLOYD_DISTORTION_RATIO = 1.10  # GPU codebook distortion <= 1.10 x the reference's
PSNR_SLACK_DB = 0.25           # restored PSNR >= the reference path's - 0.25 dB
REPORT = []                    # (workload, cubelet, figures) printed at the end


@pytest.fixture(scope="module")
def pool():
    # spawned workers: the oracle never runs in a process that inherited CUDA
    p = mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1))
    yield p
    p.terminate()
    p.join()


@pytest.fixture(scope="module")
def ctx(pool):
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()
    if REPORT:
        print("\nbenchmark-workload parity figures:")
        for row in REPORT:
            print("  ", row)


def _rel_err(got, ref):
    scale = float(np.abs(ref).max())
    if scale == 0:
        return float(np.abs(got).max())
    return float(np.abs(got.astype(np.float64) - ref).max()) / scale


def _steps(a, p):
    return P.clamp_steps(p.steps, lib._size_of(a))


def c3_sample(items, fill=40):
    """Cubelets covering every (axis, length) pair, every (type, wavelet)
    pair, the largest cubelet of each type up to 8 M voxels, then the
    smallest others up to `fill`."""
    need = {("ax", k, L) for k in range(3) for L in synth.AXIS_CHOICES}
    need |= {("tw", dt, w) for dt in ("uint8", "uint16", "float32") for w in (P.HAAR, P.CDF97)}

    def keys(i):
        a, p = items[i]
        ks = {("ax", k, L) for k, L in enumerate(lib._size_of(a))}
        ks.add(("tw", str(a.dtype), p.wavelet))
        return ks
    order = sorted(range(len(items)), key=lambda i: items[i][0].size)
    chosen = []
    while need:
        gain, best = max((len(keys(i) & need), -k) for k, i in enumerate(order)
                         if i not in chosen)
        i = order[-best]
        chosen.append(i)
        need -= keys(i)
    for dt in ("uint8", "uint16", "float32"):
        big = [i for i in order if str(items[i][0].dtype) == dt and items[i][0].size <= 8 << 20]
        if big and big[-1] not in chosen:
            chosen.append(big[-1])
    for i in order:
        if len(chosen) >= fill:
            break
        if i not in chosen:
            chosen.append(i)
    return sorted(chosen)


@pytest.fixture(scope="module")
def c3(ctx, pool):
    items = bench.mixed_workload(20261205, 512)
    offs, off = [], 0
    for a, _ in items:
        offs.append(off)
        off += (a.nbytes + 255) // 256 * 256
    dev = lib.DeviceBuffer(off)
    for (a, _), o in zip(items, offs):
        dev.upload(a, o)
    out = ctx.compress_batch([(dev.ptr + o, lib.NP_TO_WL[a.dtype], lib._size_of(a), p)
                              for (a, p), o in zip(items, offs)], on_device=True)
    dev.free()
    sample = c3_sample(items)
    refs = pool.map(jobs.forward, [(items[i][0], _steps(*items[i]), items[i][1].wavelet)
                                   for i in sample])
    return items, out, sample, dict(zip(sample, refs))


def test_c3_sample_covers_the_workload(c3):
    items, _, sample, _ = c3
    seen = {(k, L) for i in sample for k, L in enumerate(lib._size_of(items[i][0]))}
    assert seen == {(k, L) for k in range(3) for L in synth.AXIS_CHOICES}
    kinds = {(str(items[i][0].dtype), items[i][1].wavelet) for i in sample}
    assert len(kinds) == 6
    assert len(sample) >= 40


def test_c3_transform_matches_reference(ctx, c3):
    items, _, sample, refs = c3
    worst = 0.0
    for i in sample:
        a, p = items[i]
        coeffs, _ = ctx.forward_transform(a, p)
        err = _rel_err(coeffs, refs[i])
        worst = max(worst, err)
        assert err <= TRANSFORM_RTOL, (i, a.shape, str(a.dtype), p.wavelet, err)
    REPORT.append(("mixed", "transform max rel err over sample", f"{worst:.2e}"))


def test_c3_integer_stages_bit_exact(ctx, c3):
    """Each cubelet's result from the 512-cubelet batch against the oracle
    fed that cubelet's GPU coefficients."""
    items, out, sample, _ = c3
    for i in sample:
        a, p = items[i]
        comp = out[i]
        coeffs, stored = ctx.forward_transform(a, p)
        assert tuple(stored) == tuple(comp.size)
        thr = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, oracle.UNIFORM)
        assert np.float32(comp.threshold_value) == np.float32(thr["threshold"]), i
        assert np.float32(comp.max_value) == np.float32(thr["max_abs"]), i
        assert np.float32(comp.min_coef) == np.float32(thr["min"]), i
        assert np.float32(comp.max_coef) == np.float32(thr["max"]), i
        # zero bin of the mirrored codebook (setBinsFromCodebook,
        # test_compress_common.cc:784-846): (bins - 1) / 2 ... as the reference
        ref_lloyd = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, oracle.LLOYD)
        assert comp.zero_bin == ref_lloyd["zero_bin"], i
        assert len(comp.boundaries) == len(ref_lloyd["boundaries"])
        assert len(comp.values) == len(ref_lloyd["values"])
        bins = oracle.quantize(coeffs, oracle.LLOYD, p.bin_count, comp.threshold_value,
                               comp.max_value, comp.boundaries)
        enc = oracle.huffman_encode(bins, p.bin_count, comp.zero_bin)
        assert comp.dup_key == enc["dup_key"] and comp.dup_value == enc["dup_value"], i
        assert list(comp.decode) == list(enc["decode"]), i
        assert comp.longest_code == enc["longest"], i
        assert np.array_equal(comp.words, enc["words"]), i


def test_c3_codebook_and_psnr_against_reference_path(ctx, c3, pool):
    """The Lloyd codebook is trained differently (20 iterations on the |c|
    histogram), so it is held to a distortion ratio, and the restored
    cubelet to the reference path's PSNR."""
    items, out, sample, refs = c3
    sub = sample[::2]
    jobs_ = [(items[i][0], _steps(*items[i]), items[i][1].wavelet,
              items[i][1].threshold_fraction, items[i][1].bin_count, oracle.LLOYD) for i in sub]
    ref_paths = pool.map(jobs.reference_path, jobs_)
    ratios, deltas = [], []
    for i, (restored, bnd, vals, thr) in zip(sub, ref_paths):
        a, p = items[i]
        comp = out[i]
        coeffs = refs[i]  # the reference's own coefficients
        assert np.float32(thr) == np.float32(comp.threshold_value) or \
            abs(thr - comp.threshold_value) <= 1e-5 * float(np.abs(coeffs).max())

        def mse(b, v):
            q = oracle.quantize(coeffs, oracle.LLOYD, p.bin_count, 0, 0, b)
            return float(np.mean((v.astype(np.float64)[q] - coeffs) ** 2))
        m_gpu, m_ref = mse(comp.boundaries, comp.values), mse(bnd, vals)
        ratio = m_gpu / m_ref if m_ref > 0 else 1.0
        ratios.append(ratio)
        x = a.astype(np.float64)
        peak = 255.0 if a.dtype == np.uint8 else (65535.0 if a.dtype == np.uint16
                                                  else float(x.max() - x.min()))
        back = ctx.decompress(comp).astype(np.float64)

        def psnr(y):
            m = float(np.mean((y - x) ** 2))
            return 10 * np.log10(peak * peak / m) if m > 0 else 999.0
        p_gpu, p_ref = psnr(back), psnr(restored.astype(np.float64))
        deltas.append(p_gpu - p_ref)
        assert ratio <= LLOYD_DISTORTION_RATIO, (i, ratio)
        assert p_gpu >= p_ref - PSNR_SLACK_DB, (i, p_gpu, p_ref)
    REPORT.append(("mixed", f"Lloyd distortion ratio GPU/reference over {len(sub)} cubelets",
                   f"mean {np.mean(ratios):.4f} max {np.max(ratios):.4f}"))
    REPORT.append(("mixed", "restored PSNR GPU - reference path (dB)",
                   f"mean {np.mean(deltas):+.3f} min {np.min(deltas):+.3f} "
                   f"max {np.max(deltas):+.3f}"))


# ------------------------------------------------------------ split volume
@pytest.fixture(scope="module")
def c5(ctx, pool):
    items = bench.split_workload(20261205, 0)
    vol, grid = bench.split_workload.volume, bench.split_workload.grid
    Z, Y, X = vol.shape
    dev = lib.DeviceBuffer(vol.nbytes)
    dev.upload(vol)
    es = vol.dtype.itemsize
    out = ctx.compress_batch(
        [(dev.ptr + (ox + X * (oy + Y * oz)) * es, lib.NP_TO_WL[vol.dtype], size, p, (X, X * Y))
         for ((ox, oy, oz), size), (_, p) in zip(grid, items)], on_device=True)
    dev.free()
    n = round(len(grid) ** (1 / 3))
    pick = [(0, 0, 0), (n - 1, n - 1, n - 1), (n - 1, 0, 0), (0, n - 1, 0), (0, 0, n - 1),
            (4, 4, 4), (n - 1, n - 1, 0), (3, 5, 7)]
    sample = [gx + n * (gy + n * gz) for gx, gy, gz in pick]
    subs = {i: np.ascontiguousarray(items[i][0]) for i in sample}
    refs = pool.map(jobs.forward, [(subs[i], _steps(*items[i]), items[i][1].wavelet)
                                   for i in sample])
    return items, grid, out, sample, subs, dict(zip(sample, refs))


def test_c5_sample_has_edge_cubelets(c5):
    _, grid, _, sample, _, _ = c5
    assert len(grid) == 729
    sizes = [grid[i][1] for i in sample]
    assert (64, 64, 64) in sizes and (64, 128, 128) in sizes and (128, 128, 128) in sizes


def test_c5_transform_and_integer_stages(ctx, c5):
    items, grid, out, sample, subs, refs = c5
    worst = 0.0
    for i in sample:
        a, p = subs[i], items[i][1]
        coeffs, stored = ctx.forward_transform(a, p)
        err = _rel_err(coeffs, refs[i])
        worst = max(worst, err)
        assert err <= TRANSFORM_RTOL, (i, grid[i], err)
        comp = out[i]
        assert tuple(stored) == tuple(comp.size)
        enc = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, oracle.LOG)
        assert np.float32(comp.threshold_value) == np.float32(enc["threshold"]), i
        assert np.float32(comp.max_value) == np.float32(enc["max_abs"]), i
        assert comp.zero_bin == enc["zero_bin"], i
        assert (comp.dup_key, comp.dup_value) == (enc["dup_key"], enc["dup_value"]), i
        assert list(comp.decode) == list(enc["decode"]), i
        assert comp.longest_code == enc["longest"], i
        assert np.array_equal(comp.words, enc["words"]), i
    REPORT.append(("split1024", "transform max rel err over 8 cubelets", f"{worst:.2e}"))


# ------------------------------------------------------------ full-size single cubelets
@pytest.mark.parametrize("name", ["plain2d", "volume"])
def test_full_size_transform_matches_reference(ctx, pool, name):
    (a, p), = bench.WORKLOADS[name][0](20261205, 1)
    coeffs, _ = ctx.forward_transform(a, p)
    ref = pool.apply(jobs.forward, ((a, _steps(a, p), p.wavelet),))
    err = _rel_err(coeffs, ref)
    REPORT.append((name, "transform max rel err", f"{err:.2e}"))
    assert err <= TRANSFORM_RTOL, err
