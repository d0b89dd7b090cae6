"""Oracle work items for a process pool (spawned workers: the GPU tests start
their pool with the ``spawn`` method, so a worker never inherits a CUDA
context).  TEST INFRASTRUCTURE, like the rest of ``oracle/``: the checker,
never the product.

Each job takes plain numpy arrays and parameters and returns numpy arrays or
numbers, so it pickles across processes.
"""
import os
import tempfile

import numpy as np

from . import oracle


def padded_repeat(a, steps):
    """readData + padData with REPEAT (test_compress_common.cc:269-357,
    :386-423): the cubelet as float32, every axis padded to a multiple of
    2^steps by repeating its last value.  a is (Z, Y, X); steps (x, y, z)."""
    v = np.asarray(a).astype(np.float32)
    Z, Y, X = v.shape
    sx, sy, sz = steps
    pad = lambda n, s: ((n - 1) // (1 << s) + 1) * (1 << s)
    return np.pad(v, ((0, pad(Z, sz) - Z), (0, pad(Y, sy) - Y), (0, pad(X, sx) - X)),
                  mode="edge")


def forward(job):
    """(array (Z,Y,X), clamped steps (x,y,z), wavelet) -> the reference's
    float32 coefficients in the stored Z-X-Y order (cdf97_3d / haar_3d,
    dwt_cpu.cc:943-992, :624-648)."""
    a, steps, wavelet = job
    return oracle.forward(padded_repeat(a, steps), steps, wavelet)


def reference_path(job):
    """The reference's own compress + decompress of one cubelet (oracle port
    of compressFile / decompressFile, test_compress_cpu.cc:68-241), with its
    own quantizer training (Lloyd: lloyds.cpp:30-141 on every sorted |c|).

    job = (array (Z,Y,X), clamped steps, wavelet, fraction, bins, quant_alg).
    Returns (restored array in the reference's output type, codebook
    boundaries, codebook values, threshold)."""
    from wavelets_gb300 import cubefile
    a, steps, wavelet, frac, bins, qalg = job
    with tempfile.TemporaryDirectory() as d:
        comp, back = os.path.join(d, "c.cube"), os.path.join(d, "d.cube")
        oracle.compress_volume(a, steps, wavelet, frac, bins, qalg, True, comp)
        rc = oracle.main(["-q", "-d", comp, back])
        if rc != 0:
            raise RuntimeError("oracle decompress failed")
        c = cubefile.read_file(comp)[0].params
        restored = cubefile.read_file(back)[0].array()
    return (restored, np.array(c.bin_boundaries, np.float32),
            np.array(c.bin_values, np.float32), float(c.threshold_value))
