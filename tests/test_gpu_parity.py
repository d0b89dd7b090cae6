"""GPU parity: libwlgpu (through its C ABI) against the reference's outputs
and the oracle.

* exact mode (reference float order): the .cube files the GPU writes are
  byte-identical to the reference's own output files in tests/golden;
* lifting mode: coefficients within 1e-5 of the reference's (relative to the
  largest coefficient), and threshold / bins / histogram / Huffman stream
  bit-exact against the oracle fed the GPU's coefficients;
* decompression within tolerance of the oracle's; batch == single.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle
from wavelets_gb300 import cubefile, lib, params as P, synth

pytestmark = pytest.mark.gpu

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
TRANSFORM_RTOL = 1e-5  # max|gpu - ref| / max|ref| for the lifting transform
QALG = {cubefile.PB_UNIFORM: oracle.UNIFORM, cubefile.PB_LOG: oracle.LOG,
        cubefile.PB_LLOYD: oracle.LLOYD}


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _params(case, exact=False):
    p, _, _ = P.parse_flags(MANIFEST["params"][case["params"]])
    p.exact_transform = exact
    return p


def _ids(cases):
    return [f"{c['case']}.{c['params']}" for c in cases]


def _input(case):
    c = cubefile.read_file(os.path.join(GOLDEN, case["input"]))[0]
    a = c.array()
    return a


NON_LLOYD = [c for c in MANIFEST["cases"] if "lloyd" not in MANIFEST["params"][c["params"]]]
LLOYD = [c for c in MANIFEST["cases"] if "lloyd" in MANIFEST["params"][c["params"]]]


@pytest.mark.parametrize("case", NON_LLOYD, ids=_ids(NON_LLOYD))
def test_exact_mode_file_identical_to_reference(ctx, case, tmp_path):
    out = str(tmp_path / "o.cube")
    ctx.compress_file(os.path.join(GOLDEN, case["input"]), out, _params(case, exact=True))
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, case["output"]), "rb").read()


@pytest.mark.parametrize("case", LLOYD, ids=_ids(LLOYD))
def test_exact_mode_lloyd_matches_reference_except_codebook(ctx, case, tmp_path):
    """The codebook is trained on the |coefficient| histogram (20 Lloyd
    iterations), not on every sorted value as the reference does, so only
    the codebook-independent fields must match; the codebook must be close."""
    out = str(tmp_path / "o.cube")
    ctx.compress_file(os.path.join(GOLDEN, case["input"]), out, _params(case, exact=True))
    got = cubefile.read_file(out)[0]
    want = cubefile.read_file(os.path.join(GOLDEN, case["output"]))[0]
    assert (got.width, got.height, got.depth) == (want.width, want.height, want.depth)
    g, w = got.params, want.params
    assert (g.steps, g.wavelet, g.bin_count, g.quant_alg, g.original_size,
            g.original_data_type) == (w.steps, w.wavelet, w.bin_count, w.quant_alg,
                                      w.original_size, w.original_data_type)
    assert np.float32(g.threshold_value) == np.float32(w.threshold_value)
    assert len(g.bin_values) == len(w.bin_values)
    assert len(g.bin_boundaries) == len(w.bin_boundaries)
    # distortion of the reference's coefficients under each codebook
    coeffs = np.fromfile(os.path.join(GOLDEN, case["coeffs"]), np.float32)

    def mse(par):
        bins = oracle.quantize(coeffs, oracle.LLOYD, par.bin_count, 0, 0,
                               np.array(par.bin_boundaries, np.float32))
        return float(np.mean((np.array(par.bin_values, np.float64)[bins] - coeffs) ** 2))
    m_gpu, m_ref = mse(g), mse(w)
    LLOYD_DISTORTION_RATIO = 1.5
    assert m_gpu <= LLOYD_DISTORTION_RATIO * m_ref + 1e-12 * float(np.abs(coeffs).max()) ** 2, \
        (m_gpu, m_ref)


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_ids(MANIFEST["cases"]))
def test_decompress_reference_files(ctx, case, tmp_path):
    """Decompress the reference's compressed file; compare with the
    reference's own decompression (lifting synthesis vs the reference filter
    bank: float tolerance, +-1 for integer outputs that round or truncate)."""
    out = str(tmp_path / "d.cube")
    ctx.decompress_file(os.path.join(GOLDEN, case["output"]), out)
    got = cubefile.read_file(out)[0]
    want = cubefile.read_file(os.path.join(GOLDEN, case["decompressed"]))[0]
    assert (got.width, got.height, got.depth, got.data_type) == \
        (want.width, want.height, want.depth, want.data_type)
    g = got.array().astype(np.float64)
    w = want.array().astype(np.float64)
    if want.data_type == cubefile.FLOAT32:
        scale = max(1.0, float(np.abs(w).max()))
        assert np.abs(g - w).max() <= 1e-4 * scale
    else:
        # the last step rounds or truncates a float, so a 1e-6 difference in
        # the float reconstruction flips values sitting on a .5 (or integer)
        # boundary by one
        diff = np.abs(g - w)
        assert diff.max() <= 1
        assert (diff > 0).mean() < 0.05


CDF = [c for c in MANIFEST["cases"] if "haar" not in MANIFEST["params"][c["params"]]]


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_ids(MANIFEST["cases"]))
def test_transform_matches_reference(ctx, case):
    p = _params(case)
    coeffs, stored = ctx.forward_transform(_input(case), p)
    ref = np.fromfile(os.path.join(GOLDEN, case["coeffs"]), np.float32)
    assert coeffs.shape == ref.shape
    scale = float(np.abs(ref).max())
    if scale == 0:
        assert np.abs(coeffs).max() == 0
        return
    err = float(np.abs(coeffs.astype(np.float64) - ref).max()) / scale
    assert err <= TRANSFORM_RTOL, err
    if p.wavelet == P.HAAR or p.exact_transform:
        assert np.array_equal(coeffs, ref)


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_ids(MANIFEST["cases"]))
def test_exact_transform_bit_identical(ctx, case):
    coeffs, _ = ctx.forward_transform(_input(case), _params(case, exact=True))
    ref = np.fromfile(os.path.join(GOLDEN, case["coeffs"]), np.float32)
    assert np.array_equal(coeffs, ref)


def _check_integer_stages(ctx, arr, p):
    """GPU result vs the oracle fed the GPU's own coefficients."""
    comp = ctx.compress(arr, p)
    coeffs, stored = ctx.forward_transform(arr, p)
    assert tuple(stored) == tuple(comp.size)
    if p.quant_alg == P.LLOYD:
        # codebook: trained differently (histogram Lloyd); bins exact given it
        bins = oracle.quantize(coeffs, oracle.LLOYD, p.bin_count, comp.threshold_value,
                               comp.max_value, comp.boundaries)
        zb = comp.zero_bin if p.compress_zeros else -1
        enc = oracle.huffman_encode(bins, p.bin_count, zb)
        ref_thr = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, oracle.UNIFORM,
                                p.compress_zeros)["threshold"]
        assert np.float32(comp.threshold_value) == np.float32(ref_thr)
    else:
        enc = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, p.quant_alg,
                            p.compress_zeros)
        assert np.float32(comp.threshold_value) == np.float32(enc["threshold"])
        assert np.float32(comp.max_value) == np.float32(enc["max_abs"])
        assert comp.zero_bin == (enc["zero_bin"] if p.compress_zeros else comp.zero_bin)
    assert comp.dup_key == enc["dup_key"]
    assert comp.dup_value == enc["dup_value"]
    assert list(comp.decode) == list(enc["decode"])
    assert comp.longest_code == enc["longest"]
    assert np.array_equal(comp.words, enc["words"])
    return comp, coeffs


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_ids(MANIFEST["cases"]))
def test_integer_stages_bit_exact(ctx, case):
    _check_integer_stages(ctx, _input(case), _params(case))


EDGE = [
    ("zeros", np.zeros((4, 4, 4), np.float32), P.Params()),
    ("const", np.full((1, 8, 8), 7, np.uint8), P.Params(quant_alg=P.UNIFORM)),
    ("tiny", np.arange(2, dtype=np.float32).reshape(1, 1, 2), P.Params()),
    ("one", np.ones((1, 1, 1), np.float32), P.Params()),
    ("bins2", synth.volume_f32(3, (8, 8, 8), 4), P.Params(bin_count=2, quant_alg=P.UNIFORM)),
    ("bins3log", synth.volume_f32(4, (8, 8, 8), 4), P.Params(bin_count=3)),
    ("bins4096", synth.volume_f32(5, (16, 16, 16), 8), P.Params(bin_count=4096, quant_alg=P.UNIFORM,
                                                                 threshold_fraction=0.2)),
    ("noz", synth.volume_f32(6, (9, 10, 11), 8), P.Params(compress_zeros=False)),
    ("thresh0", synth.volume_f32(7, (8, 8, 8), 8), P.Params(threshold_fraction=0.0)),
    ("thresh1", synth.volume_f32(8, (8, 8, 8), 8), P.Params(threshold_fraction=1.0)),
    ("steps0", synth.volume_f32(9, (5, 6, 7), 4), P.Params(steps=(0, 0, 0))),
    ("steps_mixed", synth.volume_f32(10, (12, 20, 24), 8), P.Params(steps=(1, 0, 2))),
    ("haar_u16", synth.scaled_blob_cubelet(np.random.default_rng(3), (16, 16, 16), np.uint16),
     P.Params(wavelet=P.HAAR, quant_alg=P.UNIFORM, bin_count=1024)),
    ("lloyd_even", synth.volume_f32(11, (16, 24, 32), 10), P.Params(quant_alg=P.LLOYD, bin_count=256,
                                                                     threshold_fraction=0.9)),
    ("lloyd_odd", synth.volume_f32(12, (16, 16, 16), 10), P.Params(quant_alg=P.LLOYD, bin_count=255,
                                                                    threshold_fraction=0.8)),
    ("long_runs", np.pad(np.ones((2, 2, 2), np.float32), ((0, 30), (0, 30), (0, 62))),
     P.Params(threshold_fraction=0.99)),
    # nearly equal code lengths: speculative decoding does not resynchronise
    ("flat_codes", np.random.default_rng(9).uniform(-1, 1, (32, 32, 64)).astype(np.float32),
     P.Params(steps=(0, 0, 0), threshold_fraction=0.0, quant_alg=P.UNIFORM, bin_count=256)),
]


@pytest.mark.parametrize("name,arr,p", EDGE, ids=[e[0] for e in EDGE])
def test_edge_cases(ctx, name, arr, p):
    comp, coeffs = _check_integer_stages(ctx, arr, p)
    # the reference's table walk decodes the GPU stream to bins of the right count
    bins = oracle.huffman_decode(comp.words, comp.decode, comp.dup_key, comp.dup_value,
                                 coeffs.size)
    assert bins.size == coeffs.size
    # GPU decompression (GPU Huffman decode) == oracle dequantize + inverse
    got = ctx.decompress(comp, np.float32)
    qalg = {P.UNIFORM: oracle.UNIFORM, P.LOG: oracle.LOG, P.LLOYD: oracle.LLOYD}[p.quant_alg]
    deq = oracle.dequantize(bins, qalg, p.bin_count, comp.threshold_value, comp.max_value,
                            comp.values if p.quant_alg == P.LLOYD else None)
    if comp.steps == (0, 0, 0):
        Xp, Yp, Zp = comp.size
    else:
        Zp, Xp, Yp = comp.size
    ref = oracle.inverse(deq, (Zp, Yp, Xp), comp.steps, p.wavelet)
    a3 = arr if arr.ndim == 3 else arr.reshape((1,) * (3 - arr.ndim) + arr.shape)
    ref = ref[:a3.shape[0], :a3.shape[1], :a3.shape[2]]
    assert got.shape == ref.shape
    # a 3-bin log quantizer has a zero scale on one side; the reference's own
    # dequantizer then yields NaN/inf there, and so does this one
    fin = np.isfinite(ref)
    assert np.array_equal(fin, np.isfinite(got))
    if fin.any():
        scale = max(1e-30, float(np.abs(ref[fin]).max()))
        assert float(np.abs(got[fin].astype(np.float64) - ref[fin]).max()) <= 1e-4 * scale


def test_batch_equals_single(ctx):
    rng = np.random.default_rng(5)
    items = []
    for i in range(12):
        shape = tuple(int(rng.choice([4, 8, 12, 16, 32])) for _ in range(3))
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        p = P.Params(wavelet=P.HAAR if i % 2 else P.CDF97,
                     quant_alg=[P.UNIFORM, P.LOG, P.LLOYD][i % 3],
                     bin_count=[256, 1024, 255][i % 3], threshold_fraction=0.9)
        items.append((synth.scaled_blob_cubelet(rng, shape, dt), p))
    batch = ctx.compress_batch(items)
    for (a, p), b in zip(items, batch):
        s = ctx.compress(a, p)
        assert np.array_equal(s.words, b.words)
        assert np.array_equal(s.decode, b.decode)
        assert s.threshold_value == b.threshold_value
        assert np.array_equal(s.boundaries, b.boundaries)


def test_pinned_inputs_read_in_place(ctx):
    """Page-locked host inputs are read by the first pass without a staging
    copy; pageable, pinned and device inputs give identical streams."""
    from wavelets_gb300 import lib as L
    rng = np.random.default_rng(9)
    items = []
    for i in range(10):
        shape = tuple(int(rng.choice([5, 8, 16, 33, 48])) for _ in range(3))
        dt = [np.uint8, np.uint16, np.float32, np.int32][i % 4]
        p = P.Params(wavelet=P.HAAR if i % 2 else P.CDF97,
                     quant_alg=[P.UNIFORM, P.LOG, P.LLOYD][i % 3], threshold_fraction=0.8)
        items.append((synth.scaled_blob_cubelet(rng, shape, dt), p))
    offs, off = [], 0
    for a, _ in items:
        offs.append(off)
        off += (a.nbytes + 255) & ~255
    pin = L.PinnedBuffer(off)
    dev = L.DeviceBuffer(off)
    host = pin.array(np.uint8, (off,))
    for (a, _), o in zip(items, offs):
        host[o:o + a.nbytes] = a.view(np.uint8).ravel()
    dev.upload(host)
    pinned = ctx.compress_batch([(pin.ptr + o, L.NP_TO_WL[a.dtype], L._size_of(a), p)
                                 for (a, p), o in zip(items, offs)], raw=True)
    ondev = ctx.compress_batch([(dev.ptr + o, L.NP_TO_WL[a.dtype], L._size_of(a), p)
                                for (a, p), o in zip(items, offs)], on_device=True)
    pageable = ctx.compress_batch(items)
    for x, y, z in zip(pinned, ondev, pageable):
        assert np.array_equal(x.words, y.words) and np.array_equal(x.words, z.words)
        assert x.threshold_value == y.threshold_value == z.threshold_value
    pin.free()


def test_roundtrip_against_oracle(ctx):
    """GPU decompression vs the oracle's dequantize + inverse transform of
    the same stream."""
    arr = synth.volume_f32(13, (32, 48, 64), 30)
    p = P.Params(steps=(3, 3, 3), threshold_fraction=0.95, quant_alg=P.UNIFORM, bin_count=1024)
    comp = ctx.compress(arr, p)
    got = ctx.decompress(comp)
    n = int(np.prod(comp.size))
    bins = oracle.huffman_decode(comp.words, comp.decode, comp.dup_key, comp.dup_value, n)
    deq = oracle.dequantize(bins, oracle.UNIFORM, p.bin_count, comp.threshold_value,
                            comp.max_value)
    Zp, Xp, Yp = comp.size
    ref = oracle.inverse(deq, (Zp, Yp, Xp), comp.steps, p.wavelet)
    ref = ref[:arr.shape[0], :arr.shape[1], :arr.shape[2]]
    assert got.shape == arr.shape
    scale = float(np.abs(ref).max())
    assert float(np.abs(got.astype(np.float64) - ref).max()) <= 1e-4 * scale


def test_round_trip_psnr_full_volume_f32(ctx):
    """256^3 float32 volume, CDF9/7 3,3,3, keep 5%, uniform 1024 bins:
    decompressed PSNR (peak = max - min of the original) and the Huffman
    stream identical to the oracle's coding of the GPU coefficients."""
    arr = synth.volume_f32()
    p = P.Params(steps=(3, 3, 3), threshold_fraction=0.95, quant_alg=P.UNIFORM, bin_count=1024)
    comp, coeffs = _check_integer_stages(ctx, arr, p)
    back = ctx.decompress(comp)
    peak = float(arr.max() - arr.min())
    mse = float(np.mean((back.astype(np.float64) - arr) ** 2))
    psnr = 10 * np.log10(peak * peak / mse)
    assert psnr > 30, psnr


def test_plain_2d_u8_full_size(ctx):
    """2048x2048 uint8, CDF9/7 11,11,0, keep 10%, log 256 bins."""
    arr = synth.plain_2d()
    p = P.Params(steps=(11, 11, 0), threshold_fraction=0.9, quant_alg=P.LOG, bin_count=256)
    comp, coeffs = _check_integer_stages(ctx, arr, p)
    back = ctx.decompress(comp)
    mse = float(np.mean((back.astype(np.float64) - arr) ** 2))
    psnr = 10 * np.log10(255.0 ** 2 / mse)
    assert psnr > 25, psnr


FP64_RTOL = 2e-6  # max|gpu - fp64 lifting| / max|fp64| (the reference itself: <= 4.6e-7)


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=_ids(MANIFEST["cases"]))
def test_transform_error_against_float64_lifting(ctx, case):
    """The GPU transform (default lifting mode) against the float64 lifting
    yardstick: within FP64_RTOL of the largest coefficient."""
    from oracle import lifting64
    p = _params(case)
    coeffs, _ = ctx.forward_transform(_input(case), p)
    ref, _ = lifting64.forward(_input(case), p.steps, p.wavelet, p.transform_2d)
    scale = float(np.abs(ref).max())
    if scale == 0:
        assert np.abs(coeffs).max() == 0
        return
    assert float(np.abs(coeffs - ref).max()) / scale <= FP64_RTOL


@pytest.mark.parametrize("shape,steps,wavelet", [((256, 256, 256), (3, 3, 3), P.CDF97),
                                                 ((1, 2048, 2048), (11, 11, 0), P.CDF97),
                                                 ((96, 128, 48), (-1, -1, -1), P.HAAR)])
def test_full_size_transform_error_against_float64_lifting(ctx, shape, steps, wavelet):
    """Full-size volumes of the benchmark workloads: error stated and bounded."""
    from oracle import lifting64
    if shape[0] == 1:
        a = synth.plain_2d()
    elif shape == (256, 256, 256):
        a = synth.volume_f32()
    else:
        a = synth.scaled_blob_cubelet(np.random.default_rng(3), shape, np.uint16)
    p = P.Params(steps=steps, wavelet=wavelet)
    coeffs, _ = ctx.forward_transform(a, p)
    ref, _ = lifting64.forward(a, steps, wavelet)
    err = float(np.abs(coeffs - ref).max()) / float(np.abs(ref).max())
    print(f"transform error vs float64 lifting, {shape} {steps}: {err:.3e}")
    assert err <= FP64_RTOL



@pytest.mark.parametrize("z,zsteps", [(16, 4), (16, 1), (32, 2), (48, 4), (48, 1), (48, 3),
                                      (64, 6), (96, 5), (96, 2), (128, 3), (192, 6),
                                      (192, 1), (256, 8), (256, 4)])
@pytest.mark.parametrize("wavelet", [P.CDF97, P.HAAR])
def test_row_register_z_lengths_against_float64_lifting(ctx, z, zsteps, wavelet):
    """z rows of every length the row-register pass takes (8 or 6 elements
    per lane, every level count), 240 rows so that the last block is ragged."""
    from oracle import lifting64
    a = synth.scaled_blob_cubelet(np.random.default_rng(z * 31 + zsteps), (z, 12, 20),
                                  np.float32)
    steps = (2, 2, zsteps)
    p = P.Params(steps=steps, wavelet=wavelet)
    coeffs, _ = ctx.forward_transform(a, p)
    ref, _ = lifting64.forward(a, steps, wavelet)
    err = float(np.abs(coeffs - ref).max()) / float(np.abs(ref).max())
    assert err <= FP64_RTOL


@pytest.mark.parametrize("z,zsteps", [(16, 4), (16, 1), (32, 2), (48, 4), (48, 1), (48, 3),
                                      (64, 6), (96, 5), (96, 2), (128, 3), (192, 6),
                                      (192, 1), (256, 8), (256, 4)])
@pytest.mark.parametrize("wavelet", [P.CDF97, P.HAAR])
def test_row_register_inverse_z_lengths_round_trip(ctx, z, zsteps, wavelet):
    """The inverse transform (its z rows in registers for these lengths)
    restores the forward transform's input; 240 rows, the last block ragged."""
    a = synth.scaled_blob_cubelet(np.random.default_rng(z * 17 + zsteps), (z, 12, 20),
                                  np.float32)
    steps = (2, 2, zsteps)
    p = P.Params(steps=steps, wavelet=wavelet)
    coeffs, stored = ctx.forward_transform(a, p)
    back = ctx.inverse_transform(coeffs, stored, steps, wavelet, (20, 12, z))
    err = float(np.abs(back - a).max()) / float(np.abs(a).max())
    assert err <= 2e-6


@pytest.mark.parametrize("two_d_steps", [(-1, -1, -1), (3, 2, 0), (0, 2, 3), (4, 4, 1)])
def test_2d_mode_batched_equals_single_and_round_trips(ctx, two_d_steps, tmp_path):
    """-2d on the column-tile kernel (lifting): a batch of mixed sizes equals
    each cubelet alone, the stored size is the padded (x, y, z), and the
    restored volume is as close to the input as the reference path's own
    round trip (oracle port, same flags)."""
    rng = np.random.default_rng(31)
    items = []
    for i, shape in enumerate([(3, 64, 64), (5, 40, 24), (2, 17, 33), (4, 128, 96)]):
        a = synth.scaled_blob_cubelet(rng, shape, [np.uint8, np.uint16, np.float32, np.uint8][i])
        items.append((a, P.Params(steps=two_d_steps, transform_2d=True, threshold_fraction=0.5,
                                  quant_alg=P.UNIFORM, bin_count=1024)))
    batch = ctx.compress_batch(items)
    flags = ["-2d", "-steps", ",".join(str(s) for s in two_d_steps), "-thresh", "0.5",
             "-qalg", "uniform", "-qcount", "1024"]
    for k, ((a, p), c) in enumerate(zip(items, batch)):
        single = ctx.compress(a, p)
        assert np.array_equal(single.words, c.words)
        assert c.transform_2d
        st = P.clamp_steps(p.steps, lib._size_of(a))
        assert tuple(c.size) == tuple(P.padded_length(n, s) for n, s in zip(lib._size_of(a), st))
        back = ctx.decompress(c).astype(np.float64)
        x = a.astype(np.float64)
        # the reference path's round trip (16-bit data travels as INT32)
        inp, outp, decp = (str(tmp_path / f"{k}.{e}.cube") for e in ("in", "o", "d"))
        src = a.astype(np.int32) if a.dtype == np.uint16 else a
        cubefile.write_file(inp, [cubefile.from_array(src)])
        assert oracle.main(flags + [inp, outp]) == 0
        assert oracle.main(["-d", outp, decp]) == 0
        ref = cubefile.read_file(decp)[0].array().astype(np.float64)
        rms_gpu = float(np.sqrt(np.mean((back - x) ** 2)))
        rms_ref = float(np.sqrt(np.mean((ref - x) ** 2)))
        span = float(x.max() - x.min()) or 1.0
        assert rms_gpu <= 1.02 * rms_ref + 1e-3 * span, (k, rms_gpu, rms_ref)


def test_decompress_batch_equals_single(ctx):
    """wl_decompress_batch over mixed cubelets (sizes, element types, both
    wavelets, 3-D and -2d, all three quantizers, a single-symbol stream, the
    reference's own files) restores each exactly as wl_decompress_cubelet."""
    rng = np.random.default_rng(51)
    items = []
    for i, shape in enumerate([(8, 32, 16), (2, 64, 64), (16, 16, 16), (3, 5, 7), (32, 48, 40),
                               (1, 9, 130), (4, 40, 24)]):
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        a = synth.scaled_blob_cubelet(rng, shape, dt)
        items.append((a, P.Params(steps=(2, 2, 2) if i % 2 else (-1, -1, -1),
                                  wavelet=P.HAAR if i % 3 == 0 else P.CDF97,
                                  quant_alg=[P.LOG, P.UNIFORM, P.LLOYD][i % 3],
                                  transform_2d=(i == 6), threshold_fraction=0.8)))
    items.append((np.full((4, 8, 8), 7, np.uint8), P.Params(steps=(2, 2, 2))))  # one symbol
    items.append((synth.scaled_blob_cubelet(rng, (12, 20, 16), np.uint16),  # no zero runs
                  P.Params(steps=(2, 2, 2), compress_zeros=False, threshold_fraction=0.7)))
    comp = ctx.compress_batch(items)
    for name in ("uint8_1x64x64.p1.cube", "float32_12x20x24.p2.cube", "uint8_5x7x9.p8.cube"):
        c = cubefile.read_file(os.path.join(GOLDEN, name))[0]
        tmp = lib.Compressed(
            (c.width, c.height, c.depth), tuple(c.params.original_size),
            {cubefile.UINT8: lib.NP_TO_WL[np.dtype(np.uint8)],
             cubefile.INT32: lib.NP_TO_WL[np.dtype(np.int32)],
             cubefile.FLOAT32: lib.NP_TO_WL[np.dtype(np.float32)]}[c.params.original_data_type],
            tuple(c.params.steps), c.params.wavelet,
            {cubefile.PB_LOG: P.LOG, cubefile.PB_UNIFORM: P.UNIFORM,
             cubefile.PB_LLOYD: P.LLOYD}[c.params.quant_alg],
            c.params.bin_count, c.params.threshold_fraction, c.params.threshold_value,
            c.params.quant_max_value or 0.0, 0.0, 0.0, 0,
            c.params.huffman_dup_key if c.params.huffman_dup_key is not None else -1,
            c.params.huffman_dup_value if c.params.huffman_dup_value is not None else -1, 0,
            c.words().copy(), np.array(c.params.huffman_decode_table, np.int32),
            np.array(c.params.bin_boundaries or [], np.float32),
            np.array(c.params.bin_values or [], np.float32), bool(c.params.transform_2d))
        comp.append(tmp)
    single = [ctx.decompress(c) for c in comp]
    batch = ctx.decompress_batch(comp)
    for i, (x, y) in enumerate(zip(batch, single)):
        assert x.dtype == y.dtype and np.array_equal(x, y), i
    # the same into device memory
    offs, total = [], 0
    for y in single:
        offs.append(total)
        total += (y.nbytes + 255) // 256 * 256
    buf = lib.DeviceBuffer(total)
    try:
        ctx.decompress_batch(comp, device_outs=[buf.ptr + o for o in offs])
        for i, (o, y) in enumerate(zip(offs, single)):
            assert np.array_equal(buf.download(y.shape, y.dtype, o), y), i
    finally:
        buf.free()


@pytest.mark.parametrize("L,s", [(13, 4), (30, 5), (45, 4), (60, 6), (90, 5), (120, 7),
                                 (180, 6), (250, 8), (250, 2)])
@pytest.mark.parametrize("axis", ["x", "y"])
@pytest.mark.parametrize("dtype", [np.float32, np.uint8, np.uint16])
def test_row_register_inverse_xy_lengths_round_trip(ctx, L, s, axis, dtype):
    """Inverse y and x passes (and the forward y pass) on every row length the
    row-register tile kernels take (padded 16..256, 48, 96, 192), the inverse
    x pass cropping to the original length and converting to the output type:
    forward against the float64 lifting yardstick, and the restored volume
    equals the input (floats within 2e-6, integers within 1)."""
    shape = (9, 7, L) if axis == "x" else (9, L, 7)
    steps = (s, 1, 1) if axis == "x" else (1, s, 1)
    a = synth.scaled_blob_cubelet(np.random.default_rng(L * 7 + s), shape, dtype)
    p = P.Params(steps=steps)
    coeffs, stored = ctx.forward_transform(a, p)
    # the forward y pass on these lengths runs through the tile kernel too
    from oracle import lifting64
    ref64, _ = lifting64.forward(a, steps, p.wavelet)
    assert float(np.abs(coeffs - ref64).max()) / float(np.abs(ref64).max()) <= FP64_RTOL
    cs = P.clamp_steps(steps, lib._size_of(a))
    back = ctx.inverse_transform(coeffs, stored, cs, p.wavelet, lib._size_of(a), dtype)
    if dtype == np.float32:
        err = float(np.abs(back - a).max()) / float(np.abs(a).max())
        assert err <= 2e-6
    else:
        assert int(np.abs(back.astype(np.int64) - a).max()) <= 1
    # and through the compressed stream: the GPU restore against the oracle's
    comp = ctx.compress(a, P.Params(steps=steps, threshold_fraction=0.5, quant_alg=P.UNIFORM,
                                    bin_count=1024))
    got = ctx.decompress(comp, np.float32)
    n = int(np.prod(comp.size))
    bins = oracle.huffman_decode(comp.words, comp.decode, comp.dup_key, comp.dup_value, n)
    deq = oracle.dequantize(bins, oracle.UNIFORM, 1024, comp.threshold_value, comp.max_value)
    Zp, Xp, Yp = comp.size
    ref = oracle.inverse(deq, (Zp, Yp, Xp), comp.steps, p.wavelet)[:shape[0], :shape[1], :shape[2]]
    assert float(np.abs(got - ref).max()) <= 1e-4 * float(np.abs(ref).max())
