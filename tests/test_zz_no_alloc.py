"""wl_select_threshold_noalloc: threshold selection with no device
allocation, for callers that may not call cudaMalloc (stream capture, fixed
memory budgets, real-time loops).  Its scratch is a static device array, so
this test also checks that a second call right after the first (different
data) starts from clean scratch.  Compared against wl_compress_cubelet on
the same coefficients and against the oracle (thresh_cpu, thresh_cpu.cc:80-109,
fed those coefficients); the values are order statistics and extremes, so
they must match exactly.  The cases include element counts that are not a
multiple of the 4096-element chunk (a ragged last chunk, and a single partial
chunk) and the fraction 1.0.  Named test_zz_* so pytest collects it last."""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from wavelets_gb300 import lib, params as P, synth

pytestmark = pytest.mark.gpu


def test_noalloc_threshold_matches_compress():
    from wavelets_gb300 import build
    build.build()
    L = lib.load()
    ctx = lib.Context(0)
    cases = [
        (synth.volume_f32(21, (32, 48, 64), 20),
         P.Params(steps=(3, 3, 3), threshold_fraction=0.95, quant_alg=P.UNIFORM, bin_count=1024)),
        (synth.plain_2d(22, 512), P.Params(steps=(9, 9, 0), threshold_fraction=0.9)),
        # 2 x 33 x 17 (padded 2 x 40 x 24 = 1920 < one chunk)
        (synth.scaled_blob_cubelet(np.random.default_rng(23), (2, 33, 17), np.uint8),
         P.Params(steps=(3, 3, 1), threshold_fraction=0.7)),
        # 37 x 41 x 43, no steps: 65231 elements, the last chunk ragged
        (synth.scaled_blob_cubelet(np.random.default_rng(24), (37, 41, 43), np.float32),
         P.Params(steps=(0, 0, 0), threshold_fraction=0.5)),
        (synth.volume_f32(25, (24, 40, 48), 10),
         P.Params(steps=(3, 3, 3), threshold_fraction=1.0)),
    ]
    dout = lib.DeviceBuffer(64)
    try:
        for arr, p in cases:  # two calls in a row on different data
            comp = ctx.compress(arr, p)
            coeffs, _ = ctx.forward_transform(arr, p)
            dbuf = lib.DeviceBuffer(coeffs.nbytes)
            dbuf.upload(coeffs)
            st = L.wl_select_threshold_noalloc(ctypes.c_void_p(dbuf.ptr), coeffs.size,
                                               ctypes.c_float(p.threshold_fraction), None,
                                               ctypes.c_void_p(dout.ptr))
            assert st == lib.WL_OK
            ctx.sync()
            got = np.zeros(5, np.float32)
            assert L.wl_copy_to_host(ctypes.c_void_p(got.ctypes.data),
                                     ctypes.c_void_p(dout.ptr), 20) == lib.WL_OK
            assert got[0] == np.float32(comp.threshold_value)
            assert got[1] == np.float32(comp.min_coef)
            assert got[2] == np.float32(comp.max_coef)
            assert got[3] == np.float32(comp.max_value)
            ref = oracle.encode(coeffs, p.threshold_fraction, p.bin_count, oracle.UNIFORM)
            assert got[0] == np.float32(ref["threshold"])
            assert (got[1], got[2], got[3]) == (np.float32(ref["min"]), np.float32(ref["max"]),
                                                np.float32(ref["max_abs"]))
            # second largest |c|
            assert got[4] == np.sort(np.abs(coeffs))[-2]
            dbuf.free()
    finally:
        dout.free()
        ctx.close()


def test_noalloc_rejects_oversize():
    L = lib.load()
    st = L.wl_select_threshold_noalloc(ctypes.c_void_p(1), (64 << 20) + 1, ctypes.c_float(0.5),
                                       None, ctypes.c_void_p(1))
    assert st == lib.WL_EINVAL


def test_noalloc_inside_stream_capture():
    """The use the entry point exists for: after one call outside capture
    (which looks up the scratch address), a call captured into a CUDA graph
    on a non-blocking stream, replayed on two different inputs in the same
    buffer, gives what direct calls give."""
    torch = pytest.importorskip("torch")
    from wavelets_gb300 import build
    build.build()
    L = lib.load()
    rng = np.random.default_rng(31)
    n = 3 * 4096 + 777  # a ragged last chunk
    data = [rng.standard_normal(n).astype(np.float32) * s for s in (1.0, 40.0)]
    frac = ctypes.c_float(0.9)
    dbuf = lib.DeviceBuffer(n * 4)
    dout = lib.DeviceBuffer(64)

    def read():
        got = np.zeros(5, np.float32)
        assert L.wl_copy_to_host(ctypes.c_void_p(got.ctypes.data),
                                 ctypes.c_void_p(dout.ptr), 20) == lib.WL_OK
        return got

    try:
        want = []
        for d in data:  # direct calls (the first also looks up the scratch)
            dbuf.upload(d)
            assert L.wl_select_threshold_noalloc(ctypes.c_void_p(dbuf.ptr), n, frac, None,
                                                 ctypes.c_void_p(dout.ptr)) == lib.WL_OK
            torch.cuda.synchronize()
            want.append(read())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            s = torch.cuda.current_stream().cuda_stream
            st = L.wl_select_threshold_noalloc(ctypes.c_void_p(dbuf.ptr), n, frac,
                                               ctypes.c_void_p(s), ctypes.c_void_p(dout.ptr))
        assert st == lib.WL_OK
        for d, w in zip(data, want):
            dbuf.upload(d)
            torch.cuda.synchronize()
            g.replay()
            torch.cuda.synchronize()
            assert np.array_equal(read(), w)
        del g
    finally:
        dbuf.free()
        dout.free()
