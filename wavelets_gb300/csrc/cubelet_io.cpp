// .cube container codec (reference cubelet_file.h:17-45, cubelet_file.cc).
//
// A 64-byte header ("SCU cubelets 1.0\n" + zeros), then per cubelet a
// little-endian u32 length, a CubeletBuffer message and the raw bytes; an
// optional footer 0xFFFFFFFF, CubeletIndexBuffer, its u32 length, "cube".
// Messages use the proto2 wire format of wavelet_compress.proto; fields are
// written in field-number order and exactly the optional fields the
// reference's Cube::copyToCubeletBuffer sets (wavelet.cc:283-343), so output
// files are byte-identical to the reference's.
#include "cubelet_io.h"

#include <cstdio>
#include <cstring>

namespace wl {
namespace {

void put_varint(std::string &o, uint64_t v) {
  while (v >= 0x80) { o.push_back((char)((v & 0x7f) | 0x80)); v >>= 7; }
  o.push_back((char)v);
}
void put_tag(std::string &o, int f, int w) { put_varint(o, ((uint64_t)f << 3) | (uint64_t)w); }
void put_int(std::string &o, int f, int64_t v) { put_tag(o, f, 0); put_varint(o, (uint64_t)v); }
void put_f32(std::string &o, int f, float x) {
  put_tag(o, f, 5);
  uint32_t u; memcpy(&u, &x, 4);
  for (int i = 0; i < 4; i++) o.push_back((char)((u >> (8 * i)) & 0xff));
}
void put_bytes(std::string &o, int f, const std::string &b) {
  put_tag(o, f, 2); put_varint(o, b.size()); o += b;
}

struct In {
  const uint8_t *p, *e;
  bool ok = true;
  In(const void *d, size_t n) : p((const uint8_t *)d), e((const uint8_t *)d + n) {}
  bool more() const { return ok && p < e; }
  uint64_t varint() {
    uint64_t v = 0;
    for (int sh = 0;; sh += 7) {
      if (p >= e || sh > 63) { ok = false; return 0; }
      uint8_t c = *p++;
      v |= (uint64_t)(c & 0x7f) << sh;
      if (!(c & 0x80)) return v;
    }
  }
  uint32_t fixed32() {
    if (e - p < 4) { ok = false; return 0; }
    uint32_t v = p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24);
    p += 4;
    return v;
  }
  float f32() { uint32_t u = fixed32(); float f; memcpy(&f, &u, 4); return f; }
  In sub() {
    uint64_t n = varint();
    if (!ok || (uint64_t)(e - p) < n) { ok = false; return In(p, 0); }
    In r(p, (size_t)n);
    p += n;
    return r;
  }
  void skip(int w) {
    if (w == 0) varint();
    else if (w == 1) { if (e - p < 8) ok = false; else p += 8; }
    else if (w == 2) sub();
    else if (w == 5) fixed32();
    else ok = false;
  }
};

std::string encode_params(const CubeMeta &m) {
  std::string o;
  put_int(o, 1, m.steps[0]);
  put_int(o, 2, m.steps[1]);
  put_int(o, 3, m.steps[2]);
  put_int(o, 4, m.wavelet);
  put_f32(o, 6, m.threshold_fraction);
  put_f32(o, 7, m.threshold_value);
  put_int(o, 8, m.bin_count);
  put_int(o, 9, m.pb_quant_alg);
  if (m.pb_quant_alg == kPbUniform || m.pb_quant_alg == kPbLog) {
    put_f32(o, 10, m.quant_max_value);
  } else {
    if (!m.boundaries.empty()) {
      std::string b;
      for (float f : m.boundaries) { uint32_t u; memcpy(&u, &f, 4); for (int i = 0; i < 4; i++) b.push_back((char)((u >> (8 * i)) & 0xff)); }
      put_bytes(o, 11, b);
    }
    if (!m.values.empty()) {
      std::string b;
      for (float f : m.values) { uint32_t u; memcpy(&u, &f, 4); for (int i = 0; i < 4; i++) b.push_back((char)((u >> (8 * i)) & 0xff)); }
      put_bytes(o, 12, b);
    }
  }
  if (!m.decode.empty()) {
    std::string b;
    for (int32_t v : m.decode) put_varint(b, (uint64_t)(int64_t)v);
    put_bytes(o, 13, b);
  }
  put_int(o, 14, m.original_size[0]);
  put_int(o, 15, m.original_size[1]);
  put_int(o, 16, m.original_size[2]);
  if (m.original_data_type > 0) put_int(o, 17, m.original_data_type);
  put_int(o, 18, m.transform_2d ? 1 : 0);  // transform_2d
  if (m.dup_key >= 0) put_int(o, 19, m.dup_key);
  if (m.dup_value >= 0) put_int(o, 20, m.dup_value);
  return o;
}

bool decode_params(In r, CubeMeta &m) {
  bool have[21] = {false};
  while (r.more()) {
    uint64_t tag = r.varint();
    int f = (int)(tag >> 3), w = (int)(tag & 7);
    if (f > 0 && f < 21) have[f] = true;
    switch (f) {
      case 1: m.steps[0] = (int32_t)r.varint(); break;
      case 2: m.steps[1] = (int32_t)r.varint(); break;
      case 3: m.steps[2] = (int32_t)r.varint(); break;
      case 4: m.wavelet = (int)r.varint(); break;
      case 6: m.threshold_fraction = r.f32(); break;
      case 7: m.threshold_value = r.f32(); break;
      case 8: m.bin_count = (int32_t)r.varint(); break;
      case 9: m.pb_quant_alg = (int)r.varint(); break;
      case 10: m.quant_max_value = r.f32(); break;
      case 11: case 12: {
        std::vector<float> &v = f == 11 ? m.boundaries : m.values;
        if (w == 2) { In s = r.sub(); while (s.more()) v.push_back(s.f32()); if (!s.ok) return false; }
        else v.push_back(r.f32());
        break;
      }
      case 13:
        if (w == 2) { In s = r.sub(); while (s.more()) m.decode.push_back((int32_t)s.varint()); if (!s.ok) return false; }
        else m.decode.push_back((int32_t)r.varint());
        break;
      case 14: m.original_size[0] = (int)r.varint(); break;
      case 15: m.original_size[1] = (int)r.varint(); break;
      case 16: m.original_size[2] = (int)r.varint(); break;
      case 17: m.original_data_type = (int)r.varint(); break;
      case 18: m.transform_2d = r.varint() != 0; break;
      case 19: m.dup_key = (int32_t)r.varint(); break;
      case 20: m.dup_value = (int32_t)r.varint(); break;
      default: r.skip(w);
    }
  }
  if (!have[14]) { m.original_size[0] = m.original_size[1] = m.original_size[2] = 0; }
  return r.ok && have[1] && have[2] && have[3] && have[4] && have[8];
}

}  // namespace

std::string encode_meta(const CubeMeta &m, uint64_t data_file_offset) {
  std::string o;
  put_int(o, 1, m.width);
  put_int(o, 2, m.height);
  put_int(o, 3, m.depth);
  put_int(o, 4, m.offset[0]);
  put_int(o, 5, m.offset[1]);
  put_int(o, 6, m.offset[2]);
  put_int(o, 7, m.data_type);
  put_int(o, 8, (int64_t)m.byte_count);
  put_int(o, 9, m.compressed ? 2 : 0);
  if (data_file_offset > 0) put_int(o, 13, (int64_t)data_file_offset);
  if (m.compressed) put_bytes(o, 14, encode_params(m));
  if (m.maximum_value > 0) put_int(o, 15, m.maximum_value);
  return o;
}

bool decode_meta(const void *buf, size_t n, CubeMeta &m) {
  In r(buf, n);
  bool have[16] = {false};
  while (r.more()) {
    uint64_t tag = r.varint();
    int f = (int)(tag >> 3), w = (int)(tag & 7);
    if (f > 0 && f < 16) have[f] = true;
    switch (f) {
      case 1: m.width = (int)r.varint(); break;
      case 2: m.height = (int)r.varint(); break;
      case 3: m.depth = (int)r.varint(); break;
      case 4: m.offset[0] = (int)r.varint(); break;
      case 5: m.offset[1] = (int)r.varint(); break;
      case 6: m.offset[2] = (int)r.varint(); break;
      case 7: m.data_type = (int)r.varint(); break;
      case 8: m.byte_count = r.varint(); break;
      case 9: m.compressed = r.varint() == 2; break;
      case 14: { In s = r.sub(); if (!r.ok || !decode_params(s, m)) return false; break; }
      case 15: m.maximum_value = (int32_t)r.varint(); break;
      default: r.skip(w);
    }
  }
  return r.ok && have[1] && have[2] && have[3] && have[7] && have[8];
}

std::string encode_file(const std::vector<CubeMeta> &metas,
                        const std::vector<const std::string *> &datas, bool footer) {
  std::string out(64, '\0');
  memcpy(&out[0], kCubeHeader, strlen(kCubeHeader));
  std::string index;
  for (size_t i = 0; i < metas.size(); i++) {
    CubeMeta m = metas[i];
    m.byte_count = datas[i]->size();
    std::string enc = encode_meta(m, 0);
    uint32_t n = (uint32_t)enc.size();
    out.append((const char *)&n, 4);
    out += enc;
    const uint64_t off = out.size();
    out += *datas[i];
    put_bytes(index, 5, encode_meta(m, off));
  }
  if (footer) {
    int32_t eof = -1;
    out.append((const char *)&eof, 4);
    out += index;
    int32_t n = (int32_t)index.size();
    out.append((const char *)&n, 4);
    out += "cube";
  }
  return out;
}

bool decode_file(const std::string &buf, std::vector<CubeMeta> &metas,
                 std::vector<std::string> &datas, std::string &err) {
  if (buf.size() < 64 || memcmp(buf.data(), kCubeHeader, strlen(kCubeHeader)) != 0) {
    err = "not a cubelet file";
    return false;
  }
  size_t pos = 64;
  while (pos + 4 <= buf.size()) {
    uint32_t n;
    memcpy(&n, buf.data() + pos, 4);
    pos += 4;
    if (n == 0xFFFFFFFFu) break;
    if (pos + n > buf.size()) { err = "truncated cubelet metadata"; return false; }
    CubeMeta m;
    if (!decode_meta(buf.data() + pos, n, m)) { err = "malformed cubelet metadata"; return false; }
    pos += n;
    if (pos + m.byte_count > buf.size()) { err = "truncated cubelet data"; return false; }
    datas.emplace_back(buf.data() + pos, (size_t)m.byte_count);
    pos += m.byte_count;
    metas.push_back(std::move(m));
  }
  return true;
}

bool read_whole_file(const char *path, std::string &out) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  bool ok = n <= 0 || fread(&out[0], 1, (size_t)n, f) == (size_t)n;
  fclose(f);
  return ok;
}

bool write_whole_file(const char *path, const std::string &data) {
  FILE *f = fopen(path, "wb");
  if (!f) return false;
  bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
  ok = (fclose(f) == 0) && ok;
  return ok;
}

}  // namespace wl
