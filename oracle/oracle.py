"""ctypes wrapper around the test oracle (oracle/port, a CPU restatement of
the reference path).  TEST INFRASTRUCTURE: imported only by tests/, the smoke
check and bench.py's CPU-baseline leg, as the checker -- never by the product.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

HAAR, CDF97 = 1, 2
UNIFORM, LOG, LLOYD = 1, 2, 3
UINT8, INT32, FLOAT32 = 1, 2, 3


class Result(ctypes.Structure):
    _fields_ = [("threshold", ctypes.c_float), ("min_value", ctypes.c_float),
                ("max_value", ctypes.c_float), ("max_abs", ctypes.c_float),
                ("nonzero_count", ctypes.c_int), ("zero_bin", ctypes.c_int),
                ("bin_count", ctypes.c_int), ("quant_alg", ctypes.c_int),
                ("n_boundaries", ctypes.c_int), ("n_values", ctypes.c_int),
                ("n_words", ctypes.c_int), ("n_decode", ctypes.c_int),
                ("longest_code", ctypes.c_int), ("dup_key", ctypes.c_int),
                ("dup_value", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path, _ = build_oracle.build_port()
        _lib = ctypes.CDLL(path)
    return _lib


def cli_path():
    return build_oracle.build_port()[1]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def forward(vol_xyz: np.ndarray, steps, wavelet=CDF97) -> np.ndarray:
    """vol_xyz: padded (Z, Y, X) float32 array.  Returns the flat rotated
    coefficients."""
    v = np.ascontiguousarray(vol_xyz, np.float32)
    Z, Y, X = v.shape
    out = np.empty(v.size, np.float32)
    lib().orc_forward(_ptr(v), X, Y, Z, *map(int, steps), int(wavelet), _ptr(out))
    return out


def inverse(coeffs: np.ndarray, shape_zyx, steps, wavelet=CDF97) -> np.ndarray:
    c = np.ascontiguousarray(coeffs, np.float32)
    Z, Y, X = shape_zyx
    out = np.empty(c.size, np.float32)
    lib().orc_inverse(_ptr(c), X, Y, Z, *map(int, steps), int(wavelet), _ptr(out))
    return out.reshape(Z, Y, X)


def encode(coeffs: np.ndarray, frac: float, bin_count: int, quant_alg: int,
           compress_zeros: bool = True):
    """Threshold + quantize + Huffman on given coefficients.  Returns a dict."""
    c = np.ascontiguousarray(coeffs, np.float32).ravel()
    n = c.size
    res = Result()
    bins = np.empty(n, np.int32)
    cap = n * 2 + 1024
    words = np.empty(cap, np.uint32)
    dec = np.empty(8 * (bin_count + 2), np.int32)
    hist = np.empty(bin_count + 1, np.int64)
    bnd = np.zeros(bin_count + 1, np.float32)
    vals = np.zeros(bin_count + 1, np.float32)
    rc = lib().orc_encode(_ptr(c), n, ctypes.c_float(frac), bin_count, quant_alg,
                          int(compress_zeros), ctypes.byref(res), _ptr(bins),
                          _ptr(words), cap, _ptr(dec), dec.size, _ptr(hist),
                          _ptr(bnd), _ptr(vals))
    if rc != 0:
        raise RuntimeError("oracle encode buffer too small")
    return {"threshold": res.threshold, "min": res.min_value, "max": res.max_value,
            "max_abs": res.max_abs, "nonzero": res.nonzero_count,
            "zero_bin": res.zero_bin, "bins": bins, "hist": hist,
            "words": words[:res.n_words].copy(), "decode": dec[:res.n_decode].copy(),
            "longest": res.longest_code, "dup_key": res.dup_key,
            "dup_value": res.dup_value,
            "boundaries": bnd[:res.n_boundaries].copy(),
            "values": vals[:res.n_values].copy()}


def huffman_encode(bins, bin_count, zero_bin):
    """Reference Huffman coding of given bins (zero_bin < 0: no zero runs)."""
    b = np.ascontiguousarray(bins, np.int32).ravel()
    res = Result()
    cap = b.size * 2 + 1024
    words = np.empty(cap, np.uint32)
    dec = np.empty(8 * (bin_count + 2), np.int32)
    hist = np.empty(bin_count + 1, np.int64)
    rc = lib().orc_huffman_encode(_ptr(b), b.size, bin_count, zero_bin, ctypes.byref(res),
                                  _ptr(words), cap, _ptr(dec), dec.size, _ptr(hist))
    if rc != 0:
        raise RuntimeError("oracle huffman buffer too small")
    return {"words": words[:res.n_words].copy(), "decode": dec[:res.n_decode].copy(),
            "hist": hist, "longest": res.longest_code, "dup_key": res.dup_key,
            "dup_value": res.dup_value}


def quantize(coeffs, quant_alg, bin_count, threshold, max_abs, boundaries=None):
    c = np.ascontiguousarray(coeffs, np.float32).ravel()
    out = np.empty(c.size, np.int32)
    b = None if boundaries is None else np.ascontiguousarray(boundaries, np.float32)
    lib().orc_quantize(_ptr(c), c.size, quant_alg, bin_count, ctypes.c_float(threshold),
                       ctypes.c_float(max_abs), _ptr(b), None, _ptr(out))
    return out


def dequantize(bins, quant_alg, bin_count, threshold, max_abs, values=None):
    b = np.ascontiguousarray(bins, np.int32).ravel()
    out = np.empty(b.size, np.float32)
    v = None if values is None else np.ascontiguousarray(values, np.float32)
    lib().orc_dequantize(_ptr(b), b.size, quant_alg, bin_count, ctypes.c_float(threshold),
                         ctypes.c_float(max_abs), _ptr(v), _ptr(out))
    return out


def huffman_decode(words, table, dup_key, dup_value, n):
    w = np.ascontiguousarray(words, np.uint32)
    t = np.ascontiguousarray(table, np.int32)
    out = np.zeros(n, np.int32)
    got = lib().orc_huffman_decode(_ptr(w), w.size, _ptr(t), t.size, dup_key,
                                   dup_value, _ptr(out), n)
    return out[:got]


def compress_volume(arr_zyx, steps, wavelet, frac, bin_count, quant_alg,
                    compress_zeros=True, out_path=None):
    """Full CPU compress of one raw volume (pad, transform, encode, write)."""
    a = np.ascontiguousarray(arr_zyx)
    if a.dtype == np.uint8:
        dt = UINT8
    elif a.dtype in (np.uint16, np.int32):
        a = a.astype(np.int32)
        dt = INT32
    else:
        a = a.astype(np.float32)
        dt = FLOAT32
    Z, Y, X = a.shape
    res = Result()
    p = out_path.encode() if out_path else None
    rc = lib().orc_compress_volume(_ptr(a), dt, X, Y, Z, *map(int, steps), int(wavelet),
                                   ctypes.c_float(frac), bin_count, quant_alg,
                                   int(compress_zeros), p, ctypes.byref(res))
    if rc != 0:
        raise RuntimeError("oracle compress failed")
    return res


def error_metrics(orig_path, comp_path):
    """-err metrics of the first compressed cubelet of comp_path against the
    first uncompressed cubelet of orig_path (computeErrorRates,
    test_compress_common.cc:587-694).  Returns a dict of the accumulator's
    sums, count and getters."""
    sums = (ctypes.c_double * 4)()
    count = ctypes.c_longlong()
    g = (ctypes.c_float * 6)()
    rc = lib().orc_error_metrics(orig_path.encode(), comp_path.encode(), sums,
                                 ctypes.byref(count), g)
    if rc != 0:
        raise RuntimeError("oracle error metrics failed")
    return {"sum_value": sums[0], "sum_value_squared": sums[1], "sum_diff": sums[2],
            "sum_diff_squared": sums[3], "count": count.value, "average_error": g[0],
            "l1": g[1], "l2": g[2], "mse": g[3], "psnr": g[4], "relative_error": g[5]}


def main(args):
    """Run the oracle's command line (the reference's flags)."""
    argv = ["oracle_cli"] + list(args)
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    return lib().orc_main(len(argv), arr)
