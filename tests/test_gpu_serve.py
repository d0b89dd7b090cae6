"""The serving loop: requests admitted as they arrive and batched onto
concurrent lanes give, request by request, exactly what the same request
gives alone (bit-identical streams and restored volumes), whatever batch,
lane and neighbours it ran with."""
import threading

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
    c.close()


def _mix(seed, count):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(count):
        shape = tuple(int(rng.choice([7, 16, 24, 32, 48, 64])) for _ in range(3))
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        p = P.Params(steps=(3, 3, 3) if i % 4 else (-1, -1, -1),
                     wavelet=P.HAAR if i % 5 == 0 else P.CDF97,
                     quant_alg=[P.LOG, P.UNIFORM, P.LLOYD][i % 3],
                     bin_count=[256, 1024, 255][i % 3], threshold_fraction=0.9)
        items.append((synth.scaled_blob_cubelet(rng, shape, dt), p))
    return items


def _same(a, b):
    return (np.array_equal(a.words, b.words) and np.array_equal(a.decode, b.decode)
            and a.threshold_value == b.threshold_value
            and np.array_equal(a.boundaries, b.boundaries))


@pytest.mark.parametrize("cfg", [dict(lanes=3, memory_budget=1 << 30, max_batch=16),
                                 dict(lanes=3, memory_budget=1 << 30, max_batch=64,
                                      express_lanes=1, small_request_bytes=64 << 10,
                                      max_batch_bytes=256 << 10)],
                         ids=["fifo", "express+bytecap"])
def test_served_results_equal_standalone(ctx, cfg):
    """With or without an express lane for small requests and a byte cap per
    batch (requests then complete out of submission order), every result is
    the standalone one."""
    items = _mix(11, 48)
    ref = [ctx.compress(a, p) for a, p in items]
    dec_src = ref[:12]
    ref_dec = [ctx.decompress(c) for c in dec_src]

    srv = lib.Server(**cfg)
    tickets = [None] * (len(items) + len(dec_src))
    outs = [np.empty_like(r) for r in ref_dec]

    def submit(lo, hi):
        for k in range(lo, hi):
            if k < len(items):
                a, p = items[k]
                tickets[k] = srv.submit_compress(a, p)
            else:
                j = k - len(items)
                tickets[k] = srv.submit_decompress(dec_src[j], outs[j])

    n = len(tickets)
    threads = [threading.Thread(target=submit, args=(i * n // 4, (i + 1) * n // 4)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got, infos = [], []
    for t in tickets:
        c, info = srv.wait(t)
        got.append(c)
        infos.append(info)
    srv.close()
    for k in range(len(items)):
        assert _same(got[k], ref[k]), k
    for j in range(len(dec_src)):
        assert np.array_equal(outs[j], ref_dec[j]), j
    assert all(i["status"] == 0 for i in infos)
    assert all(i["total_ms"] >= i["service_ms"] >= 0 for i in infos)
    # requests that waited together shared a batch
    assert max(i["batch_size"] for i in infos) > 1
    assert len({i["lane"] for i in infos}) > 1


def test_memory_budget_serialises_admission(ctx):
    """With a budget below one request's working set every request runs
    alone (admission waits for the device to drain) and results still match."""
    items = _mix(12, 10)
    ref = [ctx.compress(a, p) for a, p in items]
    srv = lib.Server(lanes=2, memory_budget=1 << 16, max_batch=64)
    tickets = [srv.submit_compress(a, p) for a, p in items]
    res = [srv.wait(t) for t in tickets]
    srv.close()
    for (c, info), r in zip(res, ref):
        assert _same(c, r)
        assert info["batch_size"] == 1


def test_poll_and_device_inputs(ctx):
    items = _mix(13, 6)
    ref = [ctx.compress(a, p) for a, p in items]
    offs, off = [], 0
    for a, _ in items:
        offs.append(off)
        off += (a.nbytes + 255) & ~255
    dev = lib.DeviceBuffer(off)
    for (a, _), o in zip(items, offs):
        dev.upload(a, o)
    srv = lib.Server(lanes=2)
    tickets = [srv.submit_compress(ptr=dev.ptr + o, dtype=lib.NP_TO_WL[a.dtype],
                                   size=lib._size_of(a), params=p)
               for (a, p), o in zip(items, offs)]
    done = {}
    for _ in range(20000):
        for t in tickets:
            if t not in done:
                c, info = srv.wait(t, timeout_ms=0)
                if c is not None:
                    done[t] = c
        if len(done) == len(tickets):
            break
    for t in tickets:
        if t not in done:
            done[t] = srv.wait(t)[0]
    srv.close()
    for t, r in zip(tickets, ref):
        assert _same(done[t], r)


@pytest.mark.parametrize("stage", [True, False])
def test_batch_submission_matches_standalone(ctx, stage):
    """A prepared batch submitted whole (twice, overlapping on two lanes) gives
    each cubelet's standalone result, with page-locked inputs copied by the
    copy engine or read in place."""
    items = _mix(14, 24)
    ref = [ctx.compress(a, p) for a, p in items]
    off, offs = 0, []
    for a, _ in items:
        offs.append(off)
        off += (a.nbytes + 255) & ~255
    pin = lib.PinnedBuffer(off)
    flat = pin.array(np.uint8, (off,))
    for (a, _), o in zip(items, offs):
        flat[o:o + a.nbytes] = a.view(np.uint8).ravel()
    pb = ctx.prepare_batch([(pin.ptr + o, lib.NP_TO_WL[a.dtype], lib._size_of(a), p)
                            for (a, p), o in zip(items, offs)], raw=True)
    srv = lib.Server(lanes=2, max_batch=len(items), stage_host_inputs=stage)
    t1 = srv.submit_batch(pb)
    t2 = srv.submit_batch(pb)
    r1 = srv.wait_batch(t1).results()
    r2 = srv.wait_batch(t2).results()
    srv.close()
    for a, b, r in zip(r1, r2, ref):
        assert _same(a, r) and _same(b, r)


def test_staged_host_inputs_match(ctx):
    items = _mix(15, 12)
    ref = [ctx.compress(a, p) for a, p in items]
    off, offs = 0, []
    for a, _ in items:
        offs.append(off)
        off += (a.nbytes + 255) & ~255
    pin = lib.PinnedBuffer(off)
    flat = pin.array(np.uint8, (off,))
    for (a, _), o in zip(items, offs):
        flat[o:o + a.nbytes] = a.view(np.uint8).ravel()
    raw = [(pin.ptr + o, lib.NP_TO_WL[a.dtype], lib._size_of(a), p)
           for (a, p), o in zip(items, offs)]
    ctx.set_host_input_mode(1)
    got = ctx.compress_batch(raw, raw=True)
    ctx.set_host_input_mode(0)
    for g, r in zip(got, ref):
        assert _same(g, r)


def test_express_lane_does_not_hold_large_requests(ctx):
    """Requests too large for the express lane, submitted one at a time and
    waited for, are served by the other lane (each submission wakes every
    lane)."""
    items = _mix(14, 4)
    ref = [ctx.compress(a, p) for a, p in items]
    srv = lib.Server(lanes=2, express_lanes=1, small_request_bytes=1 << 10)
    try:
        for (a, p), r in zip(items, ref):
            assert a.nbytes > 1 << 10
            c, info = srv.wait(srv.submit_compress(a, p), timeout_ms=30000)
            assert c is not None and _same(c, r)
            assert info["lane"] == 1
    finally:
        srv.close()
