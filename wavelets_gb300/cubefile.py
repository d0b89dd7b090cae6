"""Reader and writer for the reference's ``.cube`` container, in Python.

File layout (reference cubelet_file.h:17-45): a 64-byte header whose first
line is ``"SCU cubelets 1.0\\n"``, then for each cubelet a little-endian u32
length, an encoded ``CubeletBuffer`` message and the cubelet's raw bytes; an
optional footer (``0xFFFFFFFF``, an encoded ``CubeletIndexBuffer``, its u32
length and the 4 bytes ``cube``) closes a complete file
(cubelet_file.cc:303-327).  The messages follow wavelet_compress.proto:7-174
in proto2 wire format: fields in field-number order, optional fields only when
set, repeated scalars packed.  The writer sets exactly the fields the
reference's ``Cube::copyToCubeletBuffer`` sets (wavelet.cc:283-343), so files
written here are byte-identical to the reference's.

This module is the Python-side convenience used by tests, the benchmark and
Python callers; the C++ library has its own codec (csrc/cubelet_io.cpp).
"""
from __future__ import annotations

import dataclasses
import struct
from typing import List, Optional

import numpy as np

HEADER_LINE = b"SCU cubelets 1.0\n"
HEADER_SIZE = 64

# CubeletBuffer.DataType (wavelet_compress.proto:95-99)
UINT8, INT32, FLOAT32 = 1, 2, 3
# CubeletBuffer.CompressionAlgorithm (wavelet_compress.proto:113-127)
COMP_NONE, COMP_ZLIB, COMP_WAVELET = 0, 1, 2
# CompressionParametersBuffer enums on the wire (wavelet_compress.proto:23-49)
PB_HAAR, PB_CDF97, PB_CDF53 = 1, 2, 3
PB_LOG, PB_UNIFORM, PB_LLOYD = 1, 2, 3

DTYPE_NUMPY = {UINT8: np.uint8, INT32: np.int32, FLOAT32: np.float32}


# ---------------------------------------------------------------- wire format
def _varint(v: int) -> bytes:
    if v < 0:
        v &= (1 << 64) - 1
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def _tag(field: int, wire: int) -> bytes:
    return _varint((field << 3) | wire)


def _f32(x: float) -> bytes:
    return struct.pack("<f", x)


def _len_delim(field: int, body: bytes) -> bytes:
    return _tag(field, 2) + _varint(len(body)) + body


def _read_varint(buf: bytes, pos: int):
    v = 0
    shift = 0
    while True:
        if pos >= len(buf) or shift > 63:
            raise ValueError("truncated varint")
        b = buf[pos]
        pos += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, pos
        shift += 7


def _as_int32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v & 0x80000000 else v


def _fields(buf: bytes):
    """Yield (field, wire, value) for every field of an encoded message.
    value is an int for varint/fixed fields and bytes for length-delimited."""
    pos = 0
    while pos < len(buf):
        tag, pos = _read_varint(buf, pos)
        field, wire = tag >> 3, tag & 7
        if wire == 0:
            v, pos = _read_varint(buf, pos)
        elif wire == 1:
            if pos + 8 > len(buf):
                raise ValueError("truncated fixed64")
            v = struct.unpack_from("<Q", buf, pos)[0]
            pos += 8
        elif wire == 2:
            n, pos = _read_varint(buf, pos)
            if pos + n > len(buf):
                raise ValueError("truncated length-delimited field")
            v = bytes(buf[pos:pos + n])
            pos += n
        elif wire == 5:
            if pos + 4 > len(buf):
                raise ValueError("truncated fixed32")
            v = struct.unpack_from("<I", buf, pos)[0]
            pos += 4
        else:
            raise ValueError(f"unsupported wire type {wire}")
        yield field, wire, v


def _u32_to_f32(u: int) -> float:
    return struct.unpack("<f", struct.pack("<I", u))[0]


# ------------------------------------------------------------------ messages
@dataclasses.dataclass
class CompressionParams:
    """CompressionParametersBuffer (wavelet_compress.proto:7-77).  Enum fields
    hold the *wire* values (PB_*)."""
    steps: tuple = (0, 0, 0)
    wavelet: int = PB_CDF97
    threshold_fraction: Optional[float] = None
    threshold_value: Optional[float] = None
    bin_count: int = 256
    quant_alg: Optional[int] = None
    quant_max_value: Optional[float] = None
    bin_boundaries: List[float] = dataclasses.field(default_factory=list)
    bin_values: List[float] = dataclasses.field(default_factory=list)
    huffman_decode_table: List[int] = dataclasses.field(default_factory=list)
    original_size: Optional[tuple] = None
    original_data_type: Optional[int] = None
    transform_2d: Optional[bool] = None
    huffman_dup_key: Optional[int] = None
    huffman_dup_value: Optional[int] = None

    def encode(self) -> bytes:
        o = bytearray()
        for f, v in zip((1, 2, 3), self.steps):
            o += _tag(f, 0) + _varint(int(v))
        o += _tag(4, 0) + _varint(self.wavelet)
        if self.threshold_fraction is not None:
            o += _tag(6, 5) + _f32(self.threshold_fraction)
        if self.threshold_value is not None:
            o += _tag(7, 5) + _f32(self.threshold_value)
        o += _tag(8, 0) + _varint(self.bin_count)
        if self.quant_alg is not None:
            o += _tag(9, 0) + _varint(self.quant_alg)
        if self.quant_max_value is not None:
            o += _tag(10, 5) + _f32(self.quant_max_value)
        if self.bin_boundaries:
            o += _len_delim(11, np.asarray(self.bin_boundaries, "<f4").tobytes())
        if self.bin_values:
            o += _len_delim(12, np.asarray(self.bin_values, "<f4").tobytes())
        if self.huffman_decode_table:
            o += _len_delim(13, b"".join(_varint(int(x)) for x in self.huffman_decode_table))
        if self.original_size is not None:
            for f, v in zip((14, 15, 16), self.original_size):
                o += _tag(f, 0) + _varint(int(v))
        if self.original_data_type is not None:
            o += _tag(17, 0) + _varint(self.original_data_type)
        if self.transform_2d is not None:
            o += _tag(18, 0) + _varint(1 if self.transform_2d else 0)
        if self.huffman_dup_key is not None:
            o += _tag(19, 0) + _varint(self.huffman_dup_key)
        if self.huffman_dup_value is not None:
            o += _tag(20, 0) + _varint(self.huffman_dup_value)
        return bytes(o)

    @classmethod
    def decode(cls, buf: bytes) -> "CompressionParams":
        p = cls()
        steps = [0, 0, 0]
        orig = [None, None, None]
        seen = set()
        for field, wire, v in _fields(buf):
            seen.add(field)
            if field in (1, 2, 3):
                steps[field - 1] = _as_int32(v)
            elif field == 4:
                p.wavelet = v
            elif field == 6:
                p.threshold_fraction = _u32_to_f32(v)
            elif field == 7:
                p.threshold_value = _u32_to_f32(v)
            elif field == 8:
                p.bin_count = _as_int32(v)
            elif field == 9:
                p.quant_alg = v
            elif field == 10:
                p.quant_max_value = _u32_to_f32(v)
            elif field in (11, 12):
                vals = list(np.frombuffer(v, "<f4").astype(float)) if wire == 2 else [_u32_to_f32(v)]
                (p.bin_boundaries if field == 11 else p.bin_values).extend(vals)
            elif field == 13:
                if wire == 2:
                    pos = 0
                    while pos < len(v):
                        x, pos = _read_varint(v, pos)
                        p.huffman_decode_table.append(_as_int32(x))
                else:
                    p.huffman_decode_table.append(_as_int32(v))
            elif field in (14, 15, 16):
                orig[field - 14] = v
            elif field == 17:
                p.original_data_type = v
            elif field == 18:
                p.transform_2d = bool(v)
            elif field == 19:
                p.huffman_dup_key = _as_int32(v)
            elif field == 20:
                p.huffman_dup_value = _as_int32(v)
        for req in (1, 2, 3, 4, 8):
            if req not in seen:
                raise ValueError(f"CompressionParametersBuffer: required field {req} missing")
        p.steps = tuple(steps)
        if any(o is not None for o in orig):
            p.original_size = tuple(0 if o is None else o for o in orig)
        return p


@dataclasses.dataclass
class Cubelet:
    """One cubelet: CubeletBuffer metadata (wavelet_compress.proto:83-158) and
    its raw bytes (uncompressed voxels, or Huffman words when compressed)."""
    width: int
    height: int
    depth: int
    data_type: int
    data: bytes = b""
    offset: tuple = (0, 0, 0)
    maximum_value: int = 0
    compression: int = COMP_NONE
    params: Optional[CompressionParams] = None
    data_file_offset: int = 0

    @property
    def byte_count(self) -> int:
        return len(self.data)

    def array(self) -> np.ndarray:
        """Voxels of an uncompressed cubelet as a (depth, height, width) array."""
        if self.compression != COMP_NONE:
            raise ValueError("cubelet is compressed")
        return np.frombuffer(self.data, DTYPE_NUMPY[self.data_type]).reshape(
            self.depth, self.height, self.width)

    def words(self) -> np.ndarray:
        return np.frombuffer(self.data, "<u4")

    def encode_meta(self) -> bytes:
        o = bytearray()
        o += _tag(1, 0) + _varint(self.width)
        o += _tag(2, 0) + _varint(self.height)
        o += _tag(3, 0) + _varint(self.depth)
        for f, v in zip((4, 5, 6), self.offset):
            o += _tag(f, 0) + _varint(int(v))
        o += _tag(7, 0) + _varint(self.data_type)
        o += _tag(8, 0) + _varint(self.byte_count)
        o += _tag(9, 0) + _varint(self.compression)
        if self.data_file_offset > 0:
            o += _tag(13, 0) + _varint(self.data_file_offset)
        if self.compression == COMP_WAVELET:
            o += _len_delim(14, (self.params or CompressionParams()).encode())
        if self.maximum_value > 0:
            o += _tag(15, 0) + _varint(self.maximum_value)
        return bytes(o)

    @classmethod
    def decode_meta(cls, buf: bytes) -> "Cubelet":
        c = cls(0, 0, 0, 0)
        byte_count = 0
        seen = set()
        for field, wire, v in _fields(buf):
            seen.add(field)
            if field == 1:
                c.width = v
            elif field == 2:
                c.height = v
            elif field == 3:
                c.depth = v
            elif field in (4, 5, 6):
                off = list(c.offset)
                off[field - 4] = v
                c.offset = tuple(off)
            elif field == 7:
                c.data_type = v
            elif field == 8:
                byte_count = v
            elif field == 9:
                c.compression = v
            elif field == 13:
                c.data_file_offset = v
            elif field == 14:
                c.params = CompressionParams.decode(v)
            elif field == 15:
                c.maximum_value = _as_int32(v)
        for req in (1, 2, 3, 7, 8):
            if req not in seen:
                raise ValueError(f"CubeletBuffer: required field {req} missing")
        c._byte_count = byte_count
        return c


def from_array(arr: np.ndarray, maximum_value: int = 0, offset=(0, 0, 0)) -> Cubelet:
    """An uncompressed cubelet from a (depth, height, width) array (a 2-D array
    is one layer).  uint16 data is carried as INT32 with ``maximum_value`` set,
    as the reference's own 16-bit importer does (shortImagesToCubelets.cc:24-49)."""
    a = np.asarray(arr)
    if a.ndim == 2:
        a = a[None]
    if a.dtype == np.uint8:
        dt = UINT8
    elif a.dtype == np.uint16:
        dt = INT32
        a = a.astype(np.int32)
        if maximum_value <= 0:
            maximum_value = 65535
    elif a.dtype == np.int32:
        dt = INT32
    elif a.dtype == np.float32:
        dt = FLOAT32
    else:
        raise ValueError(f"unsupported dtype {a.dtype}")
    d, h, w = a.shape
    return Cubelet(w, h, d, dt, np.ascontiguousarray(a).tobytes(), offset=offset,
                   maximum_value=maximum_value)


# ---------------------------------------------------------------- file level
def header_bytes() -> bytes:
    line = HEADER_LINE + b"\0" * (24 - len(HEADER_LINE))
    return line + b"\0" * 40


def encode_file(cubelets: List[Cubelet], footer: bool = True) -> bytes:
    out = bytearray(header_bytes())
    index_entries = []
    for c in cubelets:
        meta = c.encode_meta()
        out += struct.pack("<I", len(meta)) + meta
        data_off = len(out)
        out += c.data
        # the index copy carries the data offset (cubelet_file.cc:281)
        idx = dataclasses.replace(c, data_file_offset=data_off)
        index_entries.append(idx.encode_meta())
    if footer:
        index = b"".join(_len_delim(5, m) for m in index_entries)
        out += struct.pack("<i", -1) + index + struct.pack("<i", len(index)) + b"cube"
    return bytes(out)


def write_file(path: str, cubelets: List[Cubelet], footer: bool = True) -> None:
    with open(path, "wb") as f:
        f.write(encode_file(cubelets, footer))


def decode_file(buf: bytes) -> List[Cubelet]:
    if len(buf) < HEADER_SIZE or buf[:len(HEADER_LINE)] != HEADER_LINE:
        raise ValueError("not a cubelet file")
    pos = HEADER_SIZE
    cubelets = []
    while pos + 4 <= len(buf):
        (n,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        if n == 0xFFFFFFFF:
            break
        if pos + n > len(buf):
            raise ValueError("truncated cubelet metadata")
        c = Cubelet.decode_meta(buf[pos:pos + n])
        pos += n
        bc = c._byte_count
        if pos + bc > len(buf):
            raise ValueError("truncated cubelet data")
        c.data = bytes(buf[pos:pos + bc])
        c.data_file_offset = 0
        pos += bc
        cubelets.append(c)
    return cubelets


def read_file(path: str) -> List[Cubelet]:
    with open(path, "rb") as f:
        return decode_file(f.read())
