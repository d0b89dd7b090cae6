"""Float64 lifting transform: the precision yardstick for the GPU transform.
TEST INFRASTRUCTURE: used only by tests/ as a checker.

It computes the same 3-D multi-level transform as the reference's CPU path
(cdf97_3d / haar_3d, dwt_cpu.cc:943-992 and :624-648): REPEAT padding of each
axis to a multiple of 2^steps (padData, test_compress_common.cc:386-423), all
x levels, then all y levels, then all z levels; each level leaves the low
band in the first half and the high band in the second half of the current
span (dwt_cpu.cc:703-728); the result is stored in the reference's rotated
Z-X-Y order, element (x, y, z) at z + Zp*(x + Xp*y).

CDF 9/7 is evaluated as the four lifting steps (alpha, beta, gamma, delta)
with low * K and high * (-1/K), which equals the reference's sqrt(2)-
normalised 9/7 filter bank (dwt_cpu.cc:15-43) in exact arithmetic; whole-
sample mirroring at the row ends (MirroredArray, dwt_cpu.h:153-184) becomes
s[h] = s[h-1] and d[-1] = d[0].  Haar is (a + b, a - b) / sqrt(2)
(dwt_cpu.cc:159-162).  Every operation is in float64.
"""
import numpy as np

ALPHA = -1.586134342059924
BETA = -0.052980118572961
GAMMA = 0.882911075530934
DELTA = 0.443506852043971
K = 1.149604398860241


def ceil_log2(n: int) -> int:
    return 0 if n <= 1 else int(n - 1).bit_length()


def padded_length(n: int, steps: int) -> int:
    m = 1 << steps
    return m * ((n - 1) // m + 1)


def _cdf97_level(x: np.ndarray) -> np.ndarray:
    """One analysis level along the last axis (even length)."""
    e, o = x[..., 0::2].copy(), x[..., 1::2].copy()

    def nxt(v):
        return np.concatenate([v[..., 1:], v[..., -1:]], -1)

    def prv(v):
        return np.concatenate([v[..., :1], v[..., :-1]], -1)

    o += ALPHA * (e + nxt(e))
    e += BETA * (prv(o) + o)
    o += GAMMA * (e + nxt(e))
    e += DELTA * (prv(o) + o)
    return np.concatenate([e * K, o * (-1.0 / K)], -1)


def _haar_level(x: np.ndarray) -> np.ndarray:
    e, o = x[..., 0::2], x[..., 1::2]
    r = np.sqrt(0.5)
    return np.concatenate([(e + o) * r, (e - o) * r], -1)


def _axis(x: np.ndarray, steps: int, wavelet: int) -> np.ndarray:
    level = _haar_level if wavelet == 1 else _cdf97_level
    n = x.shape[-1]
    for _ in range(steps):
        x[..., :n] = level(x[..., :n])
        n //= 2
    return x


def forward(vol_zyx: np.ndarray, steps, wavelet: int = 2, transform_2d: bool = False):
    """vol_zyx: (Z, Y, X) array of any dtype.  steps: (sx, sy, sz), negative
    for the maximum.  Returns (flat float64 coefficients in the stored order --
    Z-X-Y, or x fastest in 2-D mode -- and the clamped steps).

    2-D mode (-2d, test_compress_common.cc:519-541; cdf97_2d / haar_2d
    dwt_cpu.cc:811-864, :495-547): every z layer gets its x levels, then its
    y levels, with no axis rotation; a step count below 1 means the maximum
    for the padded length, and layers whose padded size does not suit the
    step counts are left as they are."""
    Z, Y, X = vol_zyx.shape
    st = []
    for s, n in zip(steps, (X, Y, Z)):
        m = ceil_log2(n)
        st.append(m if s < 0 or s > m else s)
    Xp, Yp, Zp = (padded_length(n, s) for n, s in zip((X, Y, Z), st))
    v = np.pad(vol_zyx.astype(np.float64), ((0, Zp - Z), (0, Yp - Y), (0, Xp - X)), mode="edge")
    if transform_2d:
        if st == [0, 0, 0]:
            return v.ravel(), tuple(st)
        sx = st[0] if 1 <= st[0] <= ceil_log2(Xp) else ceil_log2(Xp)
        sy = st[1] if 1 <= st[1] <= ceil_log2(Yp) else ceil_log2(Yp)
        if Xp % (1 << sx) or Yp % (1 << sy):
            return v.ravel(), tuple(st)
        v = _axis(v, sx, wavelet)                                        # x
        v = np.moveaxis(_axis(np.moveaxis(v, 1, 2).copy(), sy, wavelet), 2, 1)   # y
        return v.ravel(), tuple(st)
    v = _axis(v, st[0], wavelet)                                    # x: last axis
    v = np.moveaxis(_axis(np.moveaxis(v, 1, 2).copy(), st[1], wavelet), 2, 1)   # y
    v = np.moveaxis(_axis(np.moveaxis(v, 0, 2).copy(), st[2], wavelet), 2, 0)   # z
    if st == [0, 0, 0]:
        return v.ravel(), tuple(st)          # no rotation when every step count is 0
    return np.transpose(v, (1, 2, 0)).ravel(), tuple(st)            # [y][x][z]
