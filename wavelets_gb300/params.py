"""Compression parameters with the reference's names, defaults and flag
semantics.

Defaults follow wavelet.h:48-53 (steps -1 = as many as the axis allows,
threshold fraction 0.5, 256 bins, CDF9/7, log quantizer).  ``parse_flags``
accepts the reference command line (test_compress_common.cc:73-192):
``-steps a`` sets all three axes, ``-steps a,b`` sets z to 0; ``-thresh`` is
the fraction of coefficients REMOVED (so "keep the top 10%" is 0.9).
"""
from __future__ import annotations

import dataclasses

HAAR, CDF97 = 1, 2
UNIFORM, LOG, LLOYD = 1, 2, 3
WAVELET_NAMES = {"haar": HAAR, "cdf97": CDF97}
QUANT_NAMES = {"uniform": UNIFORM, "log": LOG, "lloyd": LLOYD}


def ceil_log2(x: int) -> int:
    """ceilLog2 (dwt_cpu.cc:75-78)."""
    return 0 if x == 0 else (x - 1).bit_length()


def padded_length(length: int, steps: int) -> int:
    """dwt_padded_length with powerOfTwo=false (dwt_cpu.cc:212-219)."""
    mod = 1 << steps
    return mod * ((length - 1) // mod + 1)


def clamp_steps(steps, size):
    """setWaveletSteps (test_compress_common.cc:362-374): negative or too many
    steps become ceil(log2(axis length))."""
    out = []
    for s, n in zip(steps, size):
        m = ceil_log2(n)
        out.append(m if (s < 0 or s > m) else s)
    return tuple(out)


@dataclasses.dataclass
class Params:
    steps: tuple = (-1, -1, -1)      # x, y, z
    wavelet: int = CDF97
    threshold_fraction: float = 0.5
    bin_count: int = 256
    quant_alg: int = LOG
    compress_zeros: bool = True
    lloyd_iters: int = 20            # Lloyd-on-histogram iterations
    exact_transform: bool = False    # reference float order instead of lifting
    transform_2d: bool = False       # -2d: a 2-D transform of every z layer


def parse_flags(args):
    """Parse the reference's flags; returns (Params, decompress, rest)."""
    p = Params()
    decompress = False
    i = 0
    args = list(args)
    while i < len(args) and args[i].startswith("-") and args[i] != "-":
        a = args[i]
        if a == "-d":
            decompress = True
        elif a == "-noz":
            p.compress_zeros = False
        elif a == "-2d":
            p.transform_2d = True
        elif a in ("-q", "-v", "-err", "-pb", "-enc", "-opt"):
            pass
        elif a == "-exact":
            p.exact_transform = True
        elif a in ("-steps", "-thresh", "-qcount", "-wave", "-qalg", "-bq", "-aq",
                   "-lloyd-iters") and i + 1 < len(args):
            v = args[i + 1]
            i += 1
            if a == "-steps":
                parts = [int(x) for x in v.split(",")]
                if len(parts) == 1:
                    p.steps = (parts[0],) * 3
                elif len(parts) == 2:
                    p.steps = (parts[0], parts[1], 0)
                elif len(parts) == 3:
                    p.steps = tuple(parts)
                else:
                    raise ValueError(f"Invalid # of wavelet transform steps: {v!r}")
            elif a == "-thresh":
                t = float(v)
                if not 0 <= t <= 1:
                    raise ValueError(f"Invalid threshold proportion: {v!r}")
                p.threshold_fraction = t
            elif a == "-qcount":
                b = int(v)
                if b < 1:
                    raise ValueError(f"Invalid # quantize bins: {v!r}")
                p.bin_count = b
            elif a == "-wave":
                if v not in WAVELET_NAMES:
                    raise ValueError(f"Invalid wavelet: {v!r}")
                p.wavelet = WAVELET_NAMES[v]
            elif a == "-qalg":
                if v not in QUANT_NAMES:
                    raise ValueError(f"Invalid quantize algorithm: {v!r}")
                p.quant_alg = QUANT_NAMES[v]
            elif a == "-lloyd-iters":
                p.lloyd_iters = int(v)
        else:
            raise ValueError(f"Unrecognized option: {a!r}")
        i += 1
    return p, decompress, args[i:]
