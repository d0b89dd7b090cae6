"""Python binding of libwlgpu's C ABI (include/wlgpu.h) through ctypes.

Arrays follow the reference's cube layout: a numpy array of shape
(depth, height, width) holds a cubelet whose x (width) index is fastest,
i.e. size = (X, Y, Z) = (shape[2], shape[1], shape[0]).

The compute path is the CUDA library only: if ``libwlgpu.so`` is missing or
no GPU is visible, these calls raise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import List, Optional, Sequence

import numpy as np

from . import params as P

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libwlgpu.so")

WL_OK, WL_EINVAL, WL_ENOMEM, WL_ETIMEOUT, WL_EFORMAT, WL_ECUDA, WL_EIO = range(7)
WL_U8, WL_I32, WL_F32, WL_U16 = 1, 2, 3, 4
STATUS_NAMES = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ETIMEOUT", 4: "EFORMAT",
                5: "ECUDA", 6: "EIO"}

NP_TO_WL = {np.dtype(np.uint8): WL_U8, np.dtype(np.int32): WL_I32,
            np.dtype(np.float32): WL_F32, np.dtype(np.uint16): WL_U16}
WL_TO_NP = {v: k for k, v in NP_TO_WL.items()}


class WlParams(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int * 3), ("wavelet", ctypes.c_int),
                ("threshold_fraction", ctypes.c_float), ("bin_count", ctypes.c_int),
                ("quant_alg", ctypes.c_int), ("compress_zeros", ctypes.c_int),
                ("lloyd_iters", ctypes.c_int), ("exact_transform", ctypes.c_int),
                ("transform_2d", ctypes.c_int)]


class WlResult(ctypes.Structure):
    _fields_ = [("size", ctypes.c_int * 3), ("original_size", ctypes.c_int * 3),
                ("original_dtype", ctypes.c_int), ("steps", ctypes.c_int * 3),
                ("wavelet", ctypes.c_int), ("quant_alg", ctypes.c_int),
                ("bin_count", ctypes.c_int), ("threshold_fraction", ctypes.c_float),
                ("threshold_value", ctypes.c_float), ("max_value", ctypes.c_float),
                ("min_coef", ctypes.c_float), ("max_coef", ctypes.c_float),
                ("zero_bin", ctypes.c_int), ("dup_key", ctypes.c_int),
                ("dup_value", ctypes.c_int), ("longest_code", ctypes.c_int),
                ("n_words", ctypes.c_int), ("words", ctypes.POINTER(ctypes.c_uint32)),
                ("n_decode", ctypes.c_int), ("decode", ctypes.POINTER(ctypes.c_int32)),
                ("n_boundaries", ctypes.c_int), ("n_values", ctypes.c_int),
                ("boundaries", ctypes.POINTER(ctypes.c_float)),
                ("values", ctypes.POINTER(ctypes.c_float)),
                ("owner", ctypes.c_void_p), ("transform_2d", ctypes.c_int)]


class WlCubelet(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int),
                ("size", ctypes.c_int * 3), ("params", WlParams),
                ("row_pitch", ctypes.c_longlong), ("slice_pitch", ctypes.c_longlong)]


REQ_COMPRESS, REQ_DECOMPRESS = 1, 2


class WlServeConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("memory_budget", ctypes.c_size_t),
                ("max_batch", ctypes.c_int), ("stage_host_inputs", ctypes.c_int),
                ("max_batch_bytes", ctypes.c_size_t), ("express_lanes", ctypes.c_int),
                ("small_request_bytes", ctypes.c_size_t), ("express_priority", ctypes.c_int)]


class WlRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("cubelet", WlCubelet),
                ("compressed", ctypes.POINTER(WlResult)), ("out_dtype", ctypes.c_int),
                ("out", ctypes.c_void_p), ("out_on_device", ctypes.c_int)]


class WlContainerStats(ctypes.Structure):
    _fields_ = [("cubelets", ctypes.c_int), ("copied", ctypes.c_int),
                ("bytes_in", ctypes.c_ulonglong), ("bytes_out", ctypes.c_ulonglong),
                ("seconds", ctypes.c_double), ("read_seconds", ctypes.c_double),
                ("compute_seconds", ctypes.c_double), ("write_seconds", ctypes.c_double)]


class WlOptPoint(ctypes.Structure):
    _fields_ = [("threshold_fraction", ctypes.c_float), ("bin_count", ctypes.c_int),
                ("size_bytes", ctypes.c_int), ("psnr", ctypes.c_float)]


class WlErrorStats(ctypes.Structure):
    _fields_ = [("count", ctypes.c_longlong), ("average_error", ctypes.c_float),
                ("l1", ctypes.c_float), ("l2", ctypes.c_float), ("mse", ctypes.c_float),
                ("psnr", ctypes.c_float), ("relative_error", ctypes.c_float),
                ("sum_value", ctypes.c_double), ("sum_value_squared", ctypes.c_double),
                ("sum_diff", ctypes.c_double), ("sum_diff_squared", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class WlRequestInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("queue_ms", ctypes.c_double),
                ("service_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("batch_size", ctypes.c_int), ("lane", ctypes.c_int)]


EXPORTS = {
    "wl_params_default": (None, [ctypes.POINTER(WlParams)]),
    "wl_result_free": (None, [ctypes.POINTER(WlResult)]),
    "wl_init": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "wl_destroy": (None, [ctypes.c_void_p]),
    "wl_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "wl_compress_cubelet": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                           ctypes.POINTER(WlParams), ctypes.POINTER(WlResult)]),
    "wl_compress_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlCubelet), ctypes.c_int,
                                         ctypes.c_int, ctypes.POINTER(WlResult)]),
    "wl_decompress_cubelet": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlResult),
                                             ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "wl_compress_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                        ctypes.POINTER(WlParams)]),
    "wl_decompress_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]),
    "wl_encode_cube": (ctypes.c_int, [ctypes.POINTER(WlResult), ctypes.c_int,
                                      ctypes.POINTER(ctypes.POINTER(ctypes.c_uint8)),
                                      ctypes.POINTER(ctypes.c_size_t)]),
    "wl_free": (None, [ctypes.c_void_p]),
    "wl_last_timings": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "wl_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "wl_forward_transform": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(WlParams),
                                            ctypes.c_void_p, ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_int)]),
    "wl_inverse_transform": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.c_int, ctypes.c_void_p]),
    "wl_device_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "wl_device_free": (None, [ctypes.c_void_p]),
    "wl_copy_to_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "wl_copy_to_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "wl_last_launch_count": (ctypes.c_int, [ctypes.c_void_p]),
    "wl_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "wl_kernel_timings": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "wl_select_threshold_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong,
                                                   ctypes.c_float, ctypes.c_void_p,
                                                   ctypes.c_void_p]),
    "wl_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "wl_host_free": (None, [ctypes.c_void_p]),
    "wl_serve_config_default": (None, [ctypes.POINTER(WlServeConfig)]),
    "wl_serve_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(WlServeConfig),
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "wl_serve_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlRequest),
                                       ctypes.POINTER(ctypes.c_ulonglong)]),
    "wl_serve_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int,
                                     ctypes.POINTER(WlResult), ctypes.POINTER(WlRequestInfo)]),
    "wl_serve_submit_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlRequest),
                                             ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong)]),
    "wl_serve_wait_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong),
                                           ctypes.c_int, ctypes.POINTER(WlResult),
                                           ctypes.POINTER(ctypes.c_int)]),
    "wl_set_host_input_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "wl_serve_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "wl_serve_destroy": (None, [ctypes.c_void_p]),
    "wl_results_free": (None, [ctypes.POINTER(WlResult), ctypes.c_int]),
    "wl_decompress_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlResult), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "wl_compress_container": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                             ctypes.POINTER(WlParams), ctypes.c_size_t,
                                             ctypes.POINTER(WlContainerStats)]),
    "wl_decompress_container": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p,
                                               ctypes.c_char_p, ctypes.c_size_t,
                                               ctypes.POINTER(WlContainerStats)]),
    "wl_optimize": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                   ctypes.c_int, ctypes.POINTER(WlParams),
                                   ctypes.POINTER(WlOptPoint), ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int)]),
    "wl_optimize_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p,
                                        ctypes.POINTER(WlParams), ctypes.POINTER(WlOptPoint),
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "wl_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "wl_tune_export": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_size_t)]),
    "wl_tune_import": (ctypes.c_int, [ctypes.c_char_p]),
    "wl_tune_reset": (None, []),
    "wl_set_graph_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "wl_set_encode_slices": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "wl_graph_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "wl_graph_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "wl_error_metrics": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WlResult),
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float, ctypes.POINTER(WlErrorStats)]),
    "wl_set_memory_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t]),
    "wl_set_stream_priority": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "wl_memory_held": (ctypes.c_size_t, [ctypes.c_void_p]),
    "wl_error_metrics_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                             ctypes.POINTER(WlErrorStats)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libwlgpu.so (built by wavelets_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libwlgpu.so not built ({path}); run wavelets_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class WlError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def make_params(p: Optional[P.Params] = None) -> WlParams:
    p = p or P.Params()
    w = WlParams()
    w.steps[:] = [int(s) for s in p.steps]
    w.wavelet = int(p.wavelet)
    w.threshold_fraction = float(p.threshold_fraction)
    w.bin_count = int(p.bin_count)
    w.quant_alg = int(p.quant_alg)
    w.compress_zeros = 1 if p.compress_zeros else 0
    w.lloyd_iters = int(p.lloyd_iters)
    w.exact_transform = 1 if p.exact_transform else 0
    w.transform_2d = 1 if getattr(p, "transform_2d", False) else 0
    return w


@dataclasses.dataclass
class Compressed:
    """A compressed cubelet (copy of a wl_result)."""
    size: tuple              # stored (rotated) width, height, depth
    original_size: tuple     # X, Y, Z
    original_dtype: int
    steps: tuple
    wavelet: int
    quant_alg: int
    bin_count: int
    threshold_fraction: float
    threshold_value: float
    max_value: float
    min_coef: float
    max_coef: float
    zero_bin: int
    dup_key: int
    dup_value: int
    longest_code: int
    words: np.ndarray
    decode: np.ndarray
    boundaries: np.ndarray
    values: np.ndarray
    transform_2d: bool = False  # 2-D mode: size is the padded (x, y, z), not rotated

    @classmethod
    def from_struct(cls, r: WlResult) -> "Compressed":
        def arr(ptr, n, dt):
            if n <= 0 or not ptr:
                return np.zeros(0, dt)
            a = np.empty(n, dt)
            ctypes.memmove(a.ctypes.data, ctypes.cast(ptr, ctypes.c_void_p).value, a.nbytes)
            return a
        return cls(tuple(r.size), tuple(r.original_size), r.original_dtype, tuple(r.steps),
                   r.wavelet, r.quant_alg, r.bin_count, r.threshold_fraction,
                   r.threshold_value, r.max_value, r.min_coef, r.max_coef, r.zero_bin,
                   r.dup_key, r.dup_value, r.longest_code,
                   arr(r.words, r.n_words, np.uint32), arr(r.decode, r.n_decode, np.int32),
                   arr(r.boundaries, r.n_boundaries, np.float32),
                   arr(r.values, r.n_values, np.float32), bool(r.transform_2d))

    def to_struct(self):
        """A WlResult pointing into this object's arrays (keep self alive)."""
        r = WlResult()
        r.size[:] = self.size
        r.original_size[:] = self.original_size
        r.original_dtype = self.original_dtype
        r.steps[:] = self.steps
        r.wavelet, r.quant_alg, r.bin_count = self.wavelet, self.quant_alg, self.bin_count
        r.threshold_fraction = self.threshold_fraction
        r.threshold_value = self.threshold_value
        r.max_value = self.max_value
        r.min_coef, r.max_coef = self.min_coef, self.max_coef
        r.zero_bin, r.dup_key, r.dup_value = self.zero_bin, self.dup_key, self.dup_value
        r.longest_code = self.longest_code
        r.transform_2d = 1 if self.transform_2d else 0
        self._keep = [np.ascontiguousarray(self.words, np.uint32),
                      np.ascontiguousarray(self.decode, np.int32),
                      np.ascontiguousarray(self.boundaries, np.float32),
                      np.ascontiguousarray(self.values, np.float32)]
        w, d, b, v = self._keep
        r.n_words = w.size
        r.words = w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        r.n_decode = d.size
        r.decode = d.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        r.n_boundaries = b.size
        r.boundaries = b.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        r.n_values = v.size
        r.values = v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        return r

    @property
    def compressed_bytes(self) -> int:
        return int(self.words.size) * 4


def _size_of(arr: np.ndarray):
    a = arr if arr.ndim == 3 else arr.reshape((1,) * (3 - arr.ndim) + arr.shape)
    Z, Y, X = a.shape
    return (X, Y, Z)


class _ResultsOwner:
    """Releases the library results whose arrays numpy views point into."""

    def __init__(self, lib, outs, n):
        self.lib, self.outs, self.n = lib, outs, n

    def __del__(self):
        try:
            self.lib.wl_results_free(self.outs, self.n)
        except Exception:
            pass


class PreparedBatch:
    """A batch description (the wl_cubelet array) built once and compressed
    any number of times: inputs that stay at the same addresses -- pinned
    staging buffers, device arrays -- are described once, so a call costs
    only the library's own work."""

    def __init__(self, cubs, n, on_device, keep):
        self.cubs, self.n, self.on_device, self._keep = cubs, n, on_device, keep


class ResultBatch:
    """The results of one compression call, left in the library's structs
    until asked for: results() makes the Compressed objects (zero-copy),
    release() frees them without looking."""

    def __init__(self, lib, outs, n):
        self.lib, self.outs, self.n = lib, outs, n
        self._live = True

    def __len__(self):
        return self.n

    def compressed_bytes(self) -> int:
        rec = np.frombuffer(self.outs, _result_dtype_cached(), count=self.n)
        return int(rec["n_words"].astype(np.int64).sum()) * 4

    def results(self) -> List["Compressed"]:
        assert self._live, "results already taken or released"
        self._live = False
        return adopt_results(self.lib, self.outs, self.n)

    def release(self):
        if self._live:
            self._live = False
            self.lib.wl_results_free(self.outs, self.n)

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def _result_dtype():
    """numpy mirror of WlResult for vectorised field access."""
    names, formats, offsets = [], [], []
    for name, ct in WlResult._fields_:
        f = getattr(WlResult, name)
        if name in ("words", "decode", "boundaries", "values", "owner"):
            fmt = np.uint64
        elif isinstance(ct, type) and issubclass(ct, ctypes.Array):
            fmt = (np.int32, (ct._length_,))
        elif ct is ctypes.c_float:
            fmt = np.float32
        else:
            fmt = np.int32
        names.append(name)
        formats.append(fmt)
        offsets.append(f.offset)
    return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                     "itemsize": ctypes.sizeof(WlResult)})


_RESULT_DT = None


def _result_dtype_cached():
    global _RESULT_DT
    if _RESULT_DT is None:
        _RESULT_DT = _result_dtype()
    return _RESULT_DT


def adopt_results(lib, outs, n) -> List["Compressed"]:
    """Compressed objects over the results' arrays without copying them.  The
    library keeps a batch's arrays in one block; the numpy views hold a
    reference that releases the results when the last view goes away."""
    global _RESULT_DT
    if _RESULT_DT is None:
        _RESULT_DT = _result_dtype()
    rec = np.frombuffer(outs, _RESULT_DT, count=n)
    ptrs = np.stack([rec["words"], rec["decode"], rec["boundaries"], rec["values"]], 1)
    cnts = np.stack([rec["n_words"], rec["n_decode"], rec["n_boundaries"], rec["n_values"]],
                    1).astype(np.int64)
    used = (cnts > 0) & (ptrs != 0)
    if n == 0 or not used.any() or not (rec["owner"] != 0).all():
        res = [Compressed.from_struct(outs[i]) for i in range(n)]
        lib.wl_results_free(outs, n)
        return res
    # one numpy view per storage block (a pipelined batch has several); all
    # views share the owner that releases the batch's results
    owner = _ResultsOwner(lib, outs, n)
    slab = rec["owner"]
    ends_abs = ptrs + 4 * cnts.astype(np.uint64)
    bases, lo_of = {}, {}
    for sid in np.unique(slab).tolist():
        sel = used & (slab == sid)[:, None]
        if not sel.any():
            continue
        lo = int(ptrs[sel].min())
        buf = (ctypes.c_char * (int(ends_abs[sel].max()) - lo)).from_address(lo)
        buf._owner = owner
        bases[sid], lo_of[sid] = np.frombuffer(buf, np.uint8), lo
    slab_l = slab.tolist()
    lo_row = np.array([lo_of.get(x, 0) for x in slab_l], np.uint64)[:, None]
    rel = np.where(used, ptrs - lo_row, 0).astype(np.int64).tolist()
    ends = (np.where(used, ptrs - lo_row, 0).astype(np.int64)
            + 4 * np.where(used, cnts, 0)).tolist()
    empty_base = np.zeros(0, np.uint8)
    f = {k: rec[k].tolist() for k in _RESULT_DT.names if k not in ("words", "decode",
                                                                    "boundaries", "values", "owner")}
    e32, ef = np.zeros(0, np.float32), np.zeros(0, np.float32)
    res = []
    for i in range(n):
        o, z = rel[i], ends[i]
        base = bases.get(slab_l[i], empty_base)
        res.append(Compressed(
            tuple(f["size"][i]), tuple(f["original_size"][i]), f["original_dtype"][i],
            tuple(f["steps"][i]), f["wavelet"][i], f["quant_alg"][i], f["bin_count"][i],
            f["threshold_fraction"][i], f["threshold_value"][i], f["max_value"][i],
            f["min_coef"][i], f["max_coef"][i], f["zero_bin"][i], f["dup_key"][i],
            f["dup_value"][i], f["longest_code"][i],
            base[o[0]:z[0]].view(np.uint32), base[o[1]:z[1]].view(np.int32),
            base[o[2]:z[2]].view(np.float32) if z[2] > o[2] else e32,
            base[o[3]:z[3]].view(np.float32) if z[3] > o[3] else ef,
            bool(f["transform_2d"][i])))
    return res


class Context:
    """A libwlgpu context (one CUDA stream + device workspace) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        st = self.lib.wl_init(device, ctypes.byref(h))
        if st != WL_OK:
            raise WlError(st, f"wl_init(device={device}) failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.wl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != WL_OK:
            raise WlError(st, self.lib.wl_last_error(self.h).decode())

    def compress(self, arr, params: Optional[P.Params] = None, ptr: Optional[int] = None,
                 dtype: Optional[int] = None, size=None) -> Compressed:
        """Compress one cubelet given as a numpy array, or as a raw pointer
        (host or device: set ``ptr`` plus ``dtype``/``size`` and pass
        ``arr=None``; device pointers use compress_device)."""
        return self._compress(arr, params, ptr, dtype, size, on_device=False)

    def compress_device(self, ptr: int, dtype: int, size, params=None) -> Compressed:
        return self._compress(None, params, ptr, dtype, size, on_device=True)

    def _compress(self, arr, params, ptr, dtype, size, on_device):
        if arr is not None:
            a = np.ascontiguousarray(arr)
            dtype = NP_TO_WL[a.dtype]
            size = _size_of(a)
            ptr = a.ctypes.data
        sz = (ctypes.c_int * 3)(*size)
        res = WlResult()
        st = self.lib.wl_compress_cubelet(self.h, ctypes.c_void_p(ptr), dtype, sz,
                                          1 if on_device else 0, ctypes.byref(make_params(params)),
                                          ctypes.byref(res))
        self._check(st)
        return adopt_results(self.lib, (WlResult * 1)(res), 1)[0]

    def prepare_batch(self, items: Sequence, params=None, on_device: bool = False,
                      raw: bool = False) -> PreparedBatch:
        """Describe a batch once (see compress_batch for items)."""
        n = len(items)
        cubs = (WlCubelet * n)()
        keep = []
        for i, it in enumerate(items):
            if raw or on_device:
                ptr, dt, size, prm = it[:4]
                if len(it) > 4:  # (row pitch, slice pitch) of a sub-volume
                    cubs[i].row_pitch, cubs[i].slice_pitch = it[4]
            else:
                if isinstance(it, tuple):
                    a, prm = it
                else:
                    a, prm = it, params
                a = np.ascontiguousarray(a)
                keep.append(a)
                ptr, dt, size = a.ctypes.data, NP_TO_WL[a.dtype], _size_of(a)
            cubs[i].data = ptr
            cubs[i].dtype = dt
            cubs[i].size[:] = size
            cubs[i].params = make_params(prm if prm is not None else params)
        return PreparedBatch(cubs, n, on_device, keep)

    def compress_prepared(self, pb: PreparedBatch, lazy: bool = False):
        """Compress a prepared batch; lazy returns a ResultBatch."""
        outs = (WlResult * pb.n)()
        st = self.lib.wl_compress_batch(self.h, pb.cubs, pb.n, 1 if pb.on_device else 0, outs)
        self._check(st)
        rb = ResultBatch(self.lib, outs, pb.n)
        return rb if lazy else rb.results()

    def compress_batch(self, items: Sequence, params=None, on_device: bool = False,
                       raw: bool = False) -> List[Compressed]:
        """items: list of numpy arrays, or (array, Params) pairs, or, with
        on_device/raw, (ptr, dtype, size, Params) tuples."""
        return self.compress_prepared(self.prepare_batch(items, params, on_device, raw))

    def compress_split(self, volume, cube=(128, 128, 128), overlap=8, params=None,
                       ptr=None, on_device=False):
        """Split a (Z, Y, X) volume into overlapping cubelets (the reference's
        `cube split`) and compress them in one batch, reading each cubelet in
        place from the volume (numpy array, or `ptr` to device / page-locked
        memory holding it).  Returns (grid, results) in the reference's
        cubelet order; grid holds (offset, size) in x, y, z order."""
        from wavelets_gb300.split import split_grid
        a = volume
        Z, Y, X = a.shape
        es = a.dtype.itemsize
        if ptr is None and not a.flags.c_contiguous:
            raise ValueError("volume must be C-contiguous")
        base = ptr if ptr is not None else a.ctypes.data
        grid = split_grid((X, Y, Z), cube, overlap)
        items = []
        for (ox, oy, oz), size in grid:
            off = (ox + X * (oy + Y * oz)) * es
            items.append((base + off, NP_TO_WL[a.dtype], size, params, (X, X * Y)))
        return grid, self.compress_batch(items, on_device=on_device, raw=not on_device)

    def decompress(self, c: Compressed, dtype=None) -> np.ndarray:
        """Restore a cubelet; dtype defaults to the original."""
        wl_dt = NP_TO_WL[np.dtype(dtype)] if dtype is not None else c.original_dtype
        X, Y, Z = c.original_size
        out = np.empty((Z, Y, X), WL_TO_NP[wl_dt])
        r = c.to_struct()
        st = self.lib.wl_decompress_cubelet(self.h, ctypes.byref(r), wl_dt,
                                            ctypes.c_void_p(out.ctypes.data), 0)
        self._check(st)
        return out

    def prepare_decompress(self, cs: Sequence[Compressed], dtypes=None, device_outs=None):
        """The wl_decompress_batch arguments for these results (reusable:
        run_decompress(prep) restores them again without rebuilding them)."""
        n = len(cs)
        rs = (WlResult * n)()
        keep = []
        outs, ptrs = [], (ctypes.c_void_p * n)()
        dts = (ctypes.c_int * n)()
        for i, c in enumerate(cs):
            r = c.to_struct()
            keep.append(c)
            ctypes.memmove(ctypes.byref(rs, i * ctypes.sizeof(WlResult)), ctypes.byref(r),
                           ctypes.sizeof(WlResult))
            wl_dt = (NP_TO_WL[np.dtype(dtypes[i])] if dtypes is not None and dtypes[i] is not None
                     else c.original_dtype)
            if device_outs is not None:
                ptrs[i] = device_outs[i]
            else:
                X, Y, Z = c.original_size
                o = np.empty((Z, Y, X), WL_TO_NP[wl_dt])
                outs.append(o)
                ptrs[i] = o.ctypes.data
            dts[i] = wl_dt
        return {"n": n, "rs": rs, "dts": dts, "ptrs": ptrs, "outs": outs, "keep": keep,
                "on_device": device_outs is not None}

    def run_decompress(self, prep):
        """One wl_decompress_batch call with prepared arguments."""
        self._check(self.lib.wl_decompress_batch(self.h, prep["rs"], prep["n"], prep["dts"],
                                                 prep["ptrs"], 1 if prep["on_device"] else 0))
        return None if prep["on_device"] else prep["outs"]

    def decompress_batch(self, cs: Sequence[Compressed], dtypes=None, device_outs=None):
        """Restore many cubelets in one batched call (dtypes default to each
        one's original).  With device_outs (one device address per cubelet,
        original_size elements of its type each) the cubelets are restored
        into device memory and nothing is returned; else into new arrays."""
        return self.run_decompress(self.prepare_decompress(cs, dtypes, device_outs))

    def forward_transform(self, arr, params: Optional[P.Params] = None):
        """Coefficients of the forward transform in the stored (rotated) order
        and the stored size (width, height, depth)."""
        a = np.ascontiguousarray(arr)
        size = _size_of(a)
        prm = params or P.Params()
        steps = P.clamp_steps(prm.steps, size)
        n = 1
        for s, L in zip(steps, size):
            n *= P.padded_length(L, s)
        out = np.empty(n, np.float32)
        stored = (ctypes.c_int * 3)()
        st = self.lib.wl_forward_transform(self.h, ctypes.c_void_p(a.ctypes.data),
                                           NP_TO_WL[a.dtype], (ctypes.c_int * 3)(*size),
                                           ctypes.byref(make_params(prm)),
                                           ctypes.c_void_p(out.ctypes.data), n, stored)
        self._check(st)
        return out, tuple(stored)

    def inverse_transform(self, coeffs, stored_size, steps, wavelet, original_size,
                          dtype=np.float32):
        c = np.ascontiguousarray(coeffs, np.float32)
        X, Y, Z = original_size
        out = np.empty((Z, Y, X), dtype)
        st = self.lib.wl_inverse_transform(self.h, ctypes.c_void_p(c.ctypes.data),
                                           (ctypes.c_int * 3)(*stored_size),
                                           (ctypes.c_int * 3)(*steps), int(wavelet),
                                           (ctypes.c_int * 3)(*original_size),
                                           NP_TO_WL[np.dtype(dtype)],
                                           ctypes.c_void_p(out.ctypes.data))
        self._check(st)
        return out

    def error_metrics(self, c: Compressed, original: np.ndarray, max_possible: float = 0.0):
        """The reference's -err metrics of a compressed cubelet against its
        original array (wl_error_metrics)."""
        a = np.ascontiguousarray(original)
        st = WlErrorStats()
        r = c.to_struct()
        self._check(self.lib.wl_error_metrics(self.h, ctypes.byref(r),
                                              ctypes.c_void_p(a.ctypes.data),
                                              NP_TO_WL[a.dtype], 0, ctypes.c_float(max_possible),
                                              ctypes.byref(st)))
        return st.as_dict()

    def error_metrics_file(self, original_path: str, compressed_path: str):
        st = WlErrorStats()
        self._check(self.lib.wl_error_metrics_file(self.h, original_path.encode(),
                                                   compressed_path.encode(), ctypes.byref(st)))
        return st.as_dict()

    def compress_file(self, inp: str, out: str, params: Optional[P.Params] = None):
        self._check(self.lib.wl_compress_file(self.h, inp.encode(), out.encode(),
                                              ctypes.byref(make_params(params))))

    def decompress_file(self, inp: str, out: str):
        self._check(self.lib.wl_decompress_file(self.h, inp.encode(), out.encode()))

    def timings(self):
        """Device time (ms) of the last compress: transform, select,
        quantize+count, Huffman build, encode, total."""
        t = (ctypes.c_float * 6)()
        self._check(self.lib.wl_last_timings(self.h, t))
        return list(t)

    def launch_count(self) -> int:
        return int(self.lib.wl_last_launch_count(self.h))

    def set_profiling(self, on: bool):
        self._check(self.lib.wl_set_profiling(self.h, 1 if on else 0))

    KERNEL_GROUPS = ("dwt_x", "dwt_y", "dwt_z", "select", "quant_setup", "quantize",
                     "runs", "huffman_build", "encode")

    def kernel_timings(self):
        t = (ctypes.c_float * 9)()
        self._check(self.lib.wl_kernel_timings(self.h, t))
        return dict(zip(self.KERNEL_GROUPS, list(t)))

    def sync(self):
        self._check(self.lib.wl_sync(self.h))

    def autotune(self, max_len: int = 0, reps: int = 0) -> str:
        """Time every tile height of every column-transform size class on
        this context's device and keep the fastest (process-wide); returns
        the table as text (see tune_table)."""
        self._check(self.lib.wl_autotune(self.h, int(max_len), int(reps)))
        return tune_table()

    def optimize(self, arr: np.ndarray, params: Optional[P.Params] = None):
        """The reference's -opt sweep on an 8-bit cubelet: a list of
        (threshold fraction, bin count, size in bytes, PSNR)."""
        a = np.ascontiguousarray(arr, np.uint8)
        sz = (ctypes.c_int * 3)(*_size_of(a))
        n = ctypes.c_int()
        prm = make_params(params)
        self._check(self.lib.wl_optimize(self.h, ctypes.c_void_p(a.ctypes.data), sz, 0,
                                         ctypes.byref(prm), None, 0, ctypes.byref(n)))
        pts = (WlOptPoint * n.value)()
        self._check(self.lib.wl_optimize(self.h, ctypes.c_void_p(a.ctypes.data), sz, 0,
                                         ctypes.byref(prm), pts, n.value, ctypes.byref(n)))
        return [(p.threshold_fraction, p.bin_count, p.size_bytes, p.psnr) for p in pts]

    def compress_container(self, in_path: str, out_path: str, params=None,
                           batch_bytes: int = 0) -> dict:
        """Compress every cubelet of a .cube file into a new .cube file
        (reading, GPU work and writing overlapped); returns the stage times."""
        st = WlContainerStats()
        self._check(self.lib.wl_compress_container(self.h, in_path.encode(), out_path.encode(),
                                                   ctypes.byref(make_params(params)),
                                                   int(batch_bytes), ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in WlContainerStats._fields_}

    def decompress_container(self, in_path: str, out_path: str, batch_bytes: int = 0) -> dict:
        """Restore every compressed cubelet of a .cube file into a new one."""
        st = WlContainerStats()
        self._check(self.lib.wl_decompress_container(self.h, in_path.encode(), out_path.encode(),
                                                     int(batch_bytes), ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in WlContainerStats._fields_}

    def set_host_input_mode(self, mode: int):
        """0: read page-locked host inputs in place; 1: copy them with the
        copy engine first."""
        self._check(self.lib.wl_set_host_input_mode(self.h, int(mode)))

    def set_memory_limit(self, nbytes: int):
        """Cap the context's device workspace (0: no cap); see wl_set_memory_limit."""
        self._check(self.lib.wl_set_memory_limit(self.h, nbytes))

    def memory_held(self) -> int:
        return self.lib.wl_memory_held(self.h)

    def set_encode_slices(self, slices: int):
        """Bit-packer lanes per 4096-element chunk (1, 2, 4, 8, 16, 32);
        0 = chosen from the batch size.  The output does not depend on it."""
        self._check(self.lib.wl_set_encode_slices(self.h, int(slices)))

    def set_graph_mode(self, mode: int):
        """1: capture a batch geometry seen twice in a row as a CUDA graph
        and replay it; 0: always launch directly."""
        self._check(self.lib.wl_set_graph_mode(self.h, int(mode)))

    def graph_stats(self):
        t = (ctypes.c_longlong * 4)()
        self._check(self.lib.wl_graph_stats(self.h, t))
        out = dict(zip(("direct", "captures", "replays", "failed"), [int(x) for x in t]))
        err = self.lib.wl_graph_error(self.h)
        if err:
            out["error"] = err.decode()
        return out


TUNE_PASSES = ("fwd_x", "fwd_y", "fwd_z", "inv_z", "inv_y", "inv_x")


def tune_table() -> str:
    """The process-wide tile table: one line per tuned size class,
    "pass type class rows warps" and the microseconds of the six candidate
    shapes (TILE_SHAPES)."""
    lib = load()
    n = ctypes.c_size_t()
    st = lib.wl_tune_export(None, 0, ctypes.byref(n))
    if st:
        raise WlError(st, "tune export")
    buf = ctypes.create_string_buffer(n.value + 1)
    st = lib.wl_tune_export(buf, n.value + 1, ctypes.byref(n))
    if st:
        raise WlError(st, "tune export")
    return buf.value.decode()


def tune_load(text: str):
    """Install tile-table lines (as tune_table returns them)."""
    st = load().wl_tune_import(text.encode())
    if st:
        raise WlError(st, "malformed tile table")


def tune_reset():
    load().wl_tune_reset()


TILE_SHAPES = ((32, 4), (64, 4), (128, 4), (32, 8), (64, 8), (128, 8))


def tune_rows(text: str):
    """Parse a tile table: {(pass, type, class): ((rows, warps), times)} with
    the microseconds of the TILE_SHAPES candidates (0 = not measured)."""
    out = {}
    for ln in text.splitlines():
        f = ln.split()
        if len(f) >= 5:
            out[(int(f[0]), int(f[1]), int(f[2]))] = (
                (int(f[3]), int(f[4])), tuple(float(x) for x in f[5:11]))
    return out


def encode_cube(c: Compressed, footer: bool = False) -> bytes:
    """The .cube file bytes the reference would write for this cubelet."""
    lib = load()
    r = c.to_struct()
    buf = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_size_t()
    st = lib.wl_encode_cube(ctypes.byref(r), 1 if footer else 0, ctypes.byref(buf), ctypes.byref(n))
    if st != WL_OK:
        raise WlError(st, "wl_encode_cube failed")
    data = ctypes.string_at(buf, n.value)
    lib.wl_free(buf)
    return data


class DeviceBuffer:
    """Device memory from wl_device_alloc."""

    def __init__(self, nbytes: int):
        self.lib = load()
        self.nbytes = nbytes
        self.ptr = self.lib.wl_device_alloc(nbytes)
        if not self.ptr:
            raise MemoryError("wl_device_alloc failed")

    def upload(self, arr: np.ndarray, offset: int = 0):
        a = np.ascontiguousarray(arr)
        assert offset + a.nbytes <= self.nbytes
        st = self.lib.wl_copy_to_device(ctypes.c_void_p(self.ptr + offset),
                                        ctypes.c_void_p(a.ctypes.data), a.nbytes)
        if st != WL_OK:
            raise WlError(st, "upload failed")

    def download(self, shape, dtype, offset: int = 0) -> np.ndarray:
        """A host copy of the bytes at offset as an array of shape and dtype."""
        out = np.empty(shape, dtype)
        assert offset + out.nbytes <= self.nbytes
        st = self.lib.wl_copy_to_host(ctypes.c_void_p(out.ctypes.data),
                                      ctypes.c_void_p(self.ptr + offset), out.nbytes)
        if st != WL_OK:
            raise WlError(st, "download failed")
        return out

    def free(self):
        if self.ptr:
            self.lib.wl_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host memory from wl_host_alloc, viewable as numpy."""

    def __init__(self, nbytes: int):
        self.lib = load()
        self.nbytes = nbytes
        self.ptr = self.lib.wl_host_alloc(nbytes)
        if not self.ptr:
            raise MemoryError("wl_host_alloc failed")

    def array(self, dtype, shape):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        assert n <= self.nbytes
        buf = (ctypes.c_uint8 * n).from_address(self.ptr)
        return np.frombuffer(buf, dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.lib.wl_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """The serving loop of libwlgpu: compress and decompress requests admitted
    as they arrive, batched continuously onto `lanes` concurrent lanes, gated
    by a device working-memory budget.  Inputs and outputs are kept alive here
    until their request has been waited for."""

    def __init__(self, lanes: int = 2, memory_budget: int = 16 << 30, max_batch: int = 1024,
                 device: int = 0, stage_host_inputs: bool = True, max_batch_bytes: int = 0,
                 express_lanes: int = 0, small_request_bytes: int = 4 << 20,
                 express_priority: bool = False):
        self.lib = load()
        cfg = WlServeConfig()
        self.lib.wl_serve_config_default(ctypes.byref(cfg))
        cfg.lanes, cfg.memory_budget, cfg.max_batch = lanes, memory_budget, max_batch
        cfg.stage_host_inputs = 1 if stage_host_inputs else 0
        cfg.max_batch_bytes = max_batch_bytes
        cfg.express_lanes = express_lanes
        cfg.small_request_bytes = small_request_bytes
        cfg.express_priority = 1 if express_priority else 0
        h = ctypes.c_void_p()
        st = self.lib.wl_serve_create(device, ctypes.byref(cfg), ctypes.byref(h))
        if st != WL_OK:
            raise WlError(st, f"wl_serve_create(device={device}) failed")
        self.h = h
        self._keep = {}

    def _submit(self, req, keep):
        t = ctypes.c_ulonglong()
        st = self.lib.wl_serve_submit(self.h, ctypes.byref(req), ctypes.byref(t))
        if st != WL_OK:
            raise WlError(st, self.lib.wl_serve_last_error(self.h).decode())
        self._keep[t.value] = (req, keep)
        return t.value

    def submit_compress(self, arr=None, params=None, ptr=None, dtype=None, size=None) -> int:
        """Compress a numpy array (host) or a raw (ptr, wl dtype, size) input."""
        req = WlRequest()
        req.kind = REQ_COMPRESS
        keep = None
        if arr is not None:
            keep = np.ascontiguousarray(arr)
            ptr, dtype, size = keep.ctypes.data, NP_TO_WL[keep.dtype], _size_of(keep)
        req.cubelet.data = ptr
        req.cubelet.dtype = dtype
        req.cubelet.size[:] = size
        req.cubelet.params = make_params(params)
        return self._submit(req, keep)

    def submit_batch(self, pb: "PreparedBatch") -> np.ndarray:
        """Queue every cubelet of a prepared batch back to back (a free lane
        takes them together); returns their tickets."""
        reqs = getattr(pb, "_reqs", None)
        if reqs is None:
            reqs = (WlRequest * pb.n)()
            for i in range(pb.n):
                reqs[i].kind = REQ_COMPRESS
                reqs[i].cubelet = pb.cubs[i]
            pb._reqs = reqs
        t = (ctypes.c_ulonglong * pb.n)()
        st = self.lib.wl_serve_submit_batch(self.h, reqs, pb.n, t)
        if st != WL_OK:
            raise WlError(st, self.lib.wl_serve_last_error(self.h).decode())
        return t

    def wait_batch(self, tickets) -> "ResultBatch":
        """Wait for the tickets of submit_batch; the results as a ResultBatch."""
        n = len(tickets)
        outs = (WlResult * n)()
        sts = (ctypes.c_int * n)()
        st = self.lib.wl_serve_wait_batch(self.h, tickets, n, outs, sts)
        rb = ResultBatch(self.lib, outs, n)
        if st != WL_OK:
            rb.release()
            raise WlError(st, self.lib.wl_serve_last_error(self.h).decode())
        return rb

    def submit_decompress(self, c: "Compressed", out: np.ndarray) -> int:
        """Restore `c` into the host array `out` (original size, any dtype)."""
        req = WlRequest()
        req.kind = REQ_DECOMPRESS
        r = c.to_struct()
        req.compressed = ctypes.pointer(r)
        req.out_dtype = NP_TO_WL[out.dtype]
        req.out = out.ctypes.data
        req.out_on_device = 0
        return self._submit(req, (c, r, out))

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(Compressed or None, info dict); None while a poll finds it pending."""
        res = (WlResult * 1)()
        info = WlRequestInfo()
        st = self.lib.wl_serve_wait(self.h, ticket, timeout_ms, res, ctypes.byref(info))
        if st == WL_ETIMEOUT:
            return None, None
        req, _ = self._keep.pop(ticket)
        if st != WL_OK:
            raise WlError(st, self.lib.wl_serve_last_error(self.h).decode())
        d = {k: getattr(info, k) for k, _ in WlRequestInfo._fields_}
        if req.kind == REQ_COMPRESS:
            return adopt_results(self.lib, res, 1)[0], d
        return None, d

    def close(self):
        if getattr(self, "h", None):
            self.lib.wl_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
