"""Whole .cube containers through the overlapped read / GPU / write pipeline:
every cubelet compressed exactly as alone, in order, with its offset, an
already-compressed cubelet copied unchanged, the index footer pointing at
every cubelet's data, small staging buffers (many batches, buffer reuse),
and the restore pipeline giving each cubelet's own decompression.  The
first cubelet of the compressed container is also restored by the oracle
(the reference's decompressFile takes a file's first compressed cubelet)."""
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle
from wavelets_gb300 import cubefile, lib, params as P, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from wavelets_gb300 import build
    build.build()
    c = lib.Context(0)
    yield c
    c.close()


def _inputs():
    rng = np.random.default_rng(41)
    arrays, cubelets = [], []
    shapes = [(8, 32, 16), (2, 64, 64), (16, 16, 16), (3, 5, 7), (32, 48, 40), (1, 9, 130)]
    for i, shape in enumerate(shapes):
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        a = synth.scaled_blob_cubelet(rng, shape, dt)
        arrays.append(a)
        cubelets.append(cubefile.from_array(a, offset=(10 * i, 20 * i, 30 * i)))
    return arrays, cubelets


def _index_offsets(buf):
    assert buf[-4:] == b"cube"
    (n,) = struct.unpack_from("<i", buf, len(buf) - 8)
    index = buf[len(buf) - 8 - n:len(buf) - 8]
    offs = []
    for field, wire, v in cubefile._fields(index):
        assert field == 5
        offs.append(cubefile.Cubelet.decode_meta(v).data_file_offset)
    return offs


def test_container_round_trip(ctx, tmp_path):
    arrays, cubelets = _inputs()
    pre = cubefile.read_file(os.path.join(GOLDEN, "uint8_1x64x64.p1.cube"))[0]
    cubelets.insert(3, pre)  # already compressed: copied unchanged
    inp, comp, back = (str(tmp_path / n) for n in ("in.cube", "c.cube", "d.cube"))
    cubefile.write_file(inp, cubelets)
    p = P.Params(steps=(2, 2, 2), threshold_fraction=0.8, quant_alg=P.LOG, bin_count=256)
    st = ctx.compress_container(inp, comp, p, batch_bytes=64 << 10)
    assert st["cubelets"] == len(cubelets) and st["copied"] == 1
    buf = open(comp, "rb").read()
    out = cubefile.decode_file(buf)
    assert len(out) == len(cubelets)
    # the index footer points at every cubelet's data
    offs, pos = [], 64
    for c in out:
        (n,) = struct.unpack_from("<I", buf, pos)
        pos += 4 + n
        offs.append(pos)
        pos += len(c.data)
    assert _index_offsets(buf) == offs
    k = 0
    for i, c in enumerate(out):
        if i == 3:
            assert c.data == pre.data and c.params.encode() == pre.params.encode()
            continue
        a = arrays[k]
        want = ctx.compress(a.astype(np.int32) if a.dtype == np.uint16 else a, p)
        assert np.array_equal(c.words(), want.words)
        assert np.array_equal(np.array(c.params.huffman_decode_table), want.decode)
        assert c.offset == (10 * k, 20 * k, 30 * k)
        assert c.compression == cubefile.COMP_WAVELET
        k += 1
    # restore the container
    st2 = ctx.decompress_container(comp, back, batch_bytes=32 << 10)
    assert st2["cubelets"] == len(cubelets) and st2["copied"] == 0
    rest = cubefile.read_file(back)
    k = 0
    for i, c in enumerate(rest):
        if i == 3:
            assert (c.width, c.height, c.depth) == tuple(pre.params.original_size)
            continue
        a = arrays[k]
        src = a.astype(np.int32) if a.dtype == np.uint16 else a
        want = ctx.decompress(ctx.compress(src, p))
        assert np.array_equal(c.array(), want)
        assert c.offset == (10 * k, 20 * k, 30 * k)
        k += 1
    # the reference's decompressFile restores the container's first cubelet
    assert oracle.main(["-d", comp, str(tmp_path / "o.cube")]) == 0
    ref = cubefile.read_file(str(tmp_path / "o.cube"))[0].array().astype(np.float64)
    assert np.abs(ref - rest[0].array().astype(np.float64)).max() <= 1


def test_container_rejects_a_non_cube_file(ctx, tmp_path):
    bad = tmp_path / "bad.cube"
    bad.write_bytes(b"not a cube file" * 10)
    with pytest.raises(lib.WlError):
        ctx.compress_container(str(bad), str(tmp_path / "x.cube"), P.Params())
