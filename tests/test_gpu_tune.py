"""Tile autotuner and CUDA graph replay.

Every tile shape of the column-tile transform does the same arithmetic on
every element, so forcing any shape for every size class gives bit-identical
streams; the autotuner fills the table with measured choices; a batch whose
geometry repeats is captured once and replayed, with results identical to
direct launches (for log batches too, whose host table step splits the work
into two graphs), and a grown buffer forces a fresh capture."""
import numpy as np
import pytest

from wavelets_gb300 import lib, params as P, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    lib.tune_reset()
    c.close()


def _mix(seed, count, quant=None):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(count):
        shape = tuple(int(rng.choice([7, 16, 24, 48, 64, 96, 128, 256])) for _ in range(3))
        while np.prod(shape) > (1 << 21):
            shape = tuple(max(7, s // 2) for s in shape)
        dt = [np.uint8, np.uint16, np.float32, np.int32][i % 4]
        q = quant if quant is not None else [P.LOG, P.UNIFORM, P.LLOYD][i % 3]
        p = P.Params(steps=(3, 3, 3) if i % 4 else (-1, -1, -1),
                     wavelet=P.HAAR if i % 5 == 0 else P.CDF97,
                     quant_alg=q, bin_count=[256, 1024, 255][i % 3], threshold_fraction=0.9)
        items.append((synth.scaled_blob_cubelet(rng, shape, dt), p))
    return items


def _same(a, b):
    return (np.array_equal(a.words, b.words) and np.array_equal(a.decode, b.decode)
            and a.threshold_value == b.threshold_value
            and np.array_equal(a.boundaries, b.boundaries))


def _forced(rows, warps):
    """Table lines forcing one tile shape for every class where it fits
    (512-element rows cannot take 128-row tiles)."""
    lines = []
    for k in range(6):
        for t in range(8):
            for c in range(10):
                r = rows if not (rows == 128 and c == 9) else 64
                lines.append(f"{k} {t} {c} {r} {warps}")
    return "\n".join(lines) + "\n"


def test_tile_shapes_give_identical_results(ctx):
    items = _mix(21, 24)
    ctx.set_graph_mode(0)
    got = {}
    for shape in lib.TILE_SHAPES:
        lib.tune_load(_forced(*shape))
        comp = ctx.compress_batch(items)
        dec = [ctx.decompress(c, dtype=a.dtype) for c, (a, _) in zip(comp[:8], items[:8])]
        got[shape] = (comp, dec)
    lib.tune_reset()
    ref_c, ref_d = got[(32, 4)]
    for shape in lib.TILE_SHAPES[1:]:
        c, d = got[shape]
        for i, (x, y) in enumerate(zip(c, ref_c)):
            assert _same(x, y), (shape, i)
        for i, (x, y) in enumerate(zip(d, ref_d)):
            assert np.array_equal(x, y), (shape, i)
    ctx.set_graph_mode(1)


def test_autotune_fills_table(ctx):
    text = ctx.autotune(max_len=128, reps=3)
    rows = lib.tune_rows(text)
    # classes 1..7 of six forward-x types, four inverse-x types, four float passes
    assert len(rows) == 7 * (6 + 4 + 4)
    for (k, t, c), (shape, us) in rows.items():
        assert shape in lib.TILE_SHAPES
        measured = [u for u in us if u > 0]
        assert len(measured) == 6  # every shape fits rows of up to 128 elements
        assert min(measured) == us[lib.TILE_SHAPES.index(shape)]
    # results do not depend on the table
    items = _mix(22, 12)
    tuned = ctx.compress_batch(items)
    lib.tune_reset()
    default = ctx.compress_batch(items)
    for x, y in zip(tuned, default):
        assert _same(x, y)


@pytest.mark.parametrize("quant", [P.LLOYD, P.LOG, None])
def test_graph_replay_matches_direct(ctx, quant):
    items = _mix(23, 16, quant)
    rng = np.random.default_rng(5)
    other = [(synth.scaled_blob_cubelet(rng, a.shape, a.dtype), p) for a, p in items]
    ctx.set_graph_mode(0)
    ref = ctx.compress_batch(items)
    ref2 = ctx.compress_batch(other)
    ctx.set_graph_mode(1)
    s0 = ctx.graph_stats()
    runs = [ctx.compress_batch(items) for _ in range(4)]
    s1 = ctx.graph_stats()
    assert "error" not in s1, s1
    segs = 2 if any(p.quant_alg == P.LOG for _, p in items) else 1
    assert s1["captures"] - s0["captures"] == segs
    assert s1["replays"] - s0["replays"] == 2 * segs
    for r in runs:
        for x, y in zip(r, ref):
            assert _same(x, y)
    # other data of the same geometry replays the same graph
    got2 = ctx.compress_batch(other)
    assert ctx.graph_stats()["replays"] - s1["replays"] == segs
    for x, y in zip(got2, ref2):
        assert _same(x, y)


def test_graph_recaptured_after_buffers_grow(ctx):
    small = _mix(24, 4, P.LLOYD)
    big = _mix(25, 40, P.LLOYD)
    ctx.set_graph_mode(0)
    ref = ctx.compress_batch(small)
    ctx.set_graph_mode(1)
    for _ in range(3):
        ctx.compress_batch(small)
    ctx.compress_batch(big)   # grows the context's buffers
    s0 = ctx.graph_stats()
    for _ in range(3):
        got = ctx.compress_batch(small)
    s1 = ctx.graph_stats()
    assert s1["captures"] - s0["captures"] == 1
    for x, y in zip(got, ref):
        assert _same(x, y)
