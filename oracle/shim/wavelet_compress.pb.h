// Test-oracle support only (never linked into the product library).
//
// Hand-written proto2 classes for the three messages of the reference schema
// wavelet_compress.proto (CompressionParametersBuffer :7-77, CubeletBuffer
// :83-158, CubeletIndexBuffer :163-174).  protoc and libprotobuf are absent on
// this machine, so this header stands in for the generated
// wavelet_compress.pb.h that wavelet.h:11 and cubelet_file.h:8 include.  It
// implements the public proto2 wire format: fields are written in field-number
// order, scalars as varints (int32 sign-extended to 64 bits), floats as
// little-endian fixed32, repeated scalars packed, sub-messages length-
// delimited; optional fields are written only when set.  Only the accessors
// that the reference sources call are provided.
#ifndef WL_ORACLE_SHIM_WAVELET_COMPRESS_PB_H
#define WL_ORACLE_SHIM_WAVELET_COMPRESS_PB_H

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <google/protobuf/stubs/common.h>

namespace wl_pbshim {

// ---- encoding --------------------------------------------------------------
inline void put_varint(std::string &out, uint64_t v) {
  while (v >= 0x80) { out.push_back((char)((v & 0x7f) | 0x80)); v >>= 7; }
  out.push_back((char)v);
}
inline void put_tag(std::string &out, int field, int wire) {
  put_varint(out, ((uint64_t)field << 3) | (uint64_t)wire);
}
inline void put_i32(std::string &out, int field, int32_t v) {
  put_tag(out, field, 0); put_varint(out, (uint64_t)(int64_t)v);
}
inline void put_u32(std::string &out, int field, uint32_t v) {
  put_tag(out, field, 0); put_varint(out, v);
}
inline void put_u64(std::string &out, int field, uint64_t v) {
  put_tag(out, field, 0); put_varint(out, v);
}
inline void put_fixed32_raw(std::string &out, uint32_t v) {
  for (int i = 0; i < 4; i++) out.push_back((char)((v >> (8 * i)) & 0xff));
}
inline void put_float(std::string &out, int field, float f) {
  uint32_t v; memcpy(&v, &f, 4);
  put_tag(out, field, 5); put_fixed32_raw(out, v);
}
inline void put_bytes(std::string &out, int field, const std::string &b) {
  put_tag(out, field, 2); put_varint(out, b.size()); out += b;
}
inline void put_packed_floats(std::string &out, int field,
                              const std::vector<float> &v) {
  if (v.empty()) return;
  std::string body;
  for (float f : v) { uint32_t u; memcpy(&u, &f, 4); put_fixed32_raw(body, u); }
  put_bytes(out, field, body);
}
inline void put_packed_i32(std::string &out, int field,
                           const std::vector<int32_t> &v) {
  if (v.empty()) return;
  std::string body;
  for (int32_t x : v) put_varint(body, (uint64_t)(int64_t)x);
  put_bytes(out, field, body);
}

// ---- decoding --------------------------------------------------------------
struct Reader {
  const uint8_t *p, *end;
  bool ok;
  Reader(const void *d, int n) : p((const uint8_t*)d), end((const uint8_t*)d + n), ok(true) {}
  bool more() const { return ok && p < end; }
  uint64_t varint() {
    uint64_t v = 0; int shift = 0;
    while (true) {
      if (p >= end || shift > 63) { ok = false; return 0; }
      uint8_t b = *p++;
      v |= (uint64_t)(b & 0x7f) << shift;
      if (!(b & 0x80)) break;
      shift += 7;
    }
    return v;
  }
  uint32_t fixed32() {
    if (end - p < 4) { ok = false; return 0; }
    uint32_t v = (uint32_t)p[0] | ((uint32_t)p[1] << 8) |
                 ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    p += 4; return v;
  }
  float f32() { uint32_t u = fixed32(); float f; memcpy(&f, &u, 4); return f; }
  Reader sub() {
    uint64_t n = varint();
    if (!ok || (uint64_t)(end - p) < n) { ok = false; return Reader(p, 0); }
    Reader r(p, (int)n); p += n; return r;
  }
  void skip(int wire) {
    switch (wire) {
      case 0: varint(); break;
      case 1: if (end - p < 8) ok = false; else p += 8; break;
      case 2: sub(); break;
      case 5: fixed32(); break;
      default: ok = false;
    }
  }
};

// read one element (or a packed run) of a repeated float field
inline void read_floats(Reader &r, int wire, std::vector<float> &v) {
  if (wire == 2) { Reader s = r.sub(); while (s.more()) v.push_back(s.f32()); if (!s.ok) r.ok = false; }
  else if (wire == 5) v.push_back(r.f32());
  else r.ok = false;
}
inline void read_i32s(Reader &r, int wire, std::vector<int32_t> &v) {
  if (wire == 2) { Reader s = r.sub(); while (s.more()) v.push_back((int32_t)s.varint()); if (!s.ok) r.ok = false; }
  else if (wire == 0) v.push_back((int32_t)r.varint());
  else r.ok = false;
}

}  // namespace wl_pbshim

enum CompressionParametersBuffer_WaveletAlgorithm {
  CompressionParametersBuffer_WaveletAlgorithm_HAAR = 1,
  CompressionParametersBuffer_WaveletAlgorithm_CDF97 = 2,
  CompressionParametersBuffer_WaveletAlgorithm_CDF53 = 3
};
enum CompressionParametersBuffer_QuantizationAlgorithm {
  CompressionParametersBuffer_QuantizationAlgorithm_LOG = 1,
  CompressionParametersBuffer_QuantizationAlgorithm_UNIFORM = 2,
  CompressionParametersBuffer_QuantizationAlgorithm_LLOYD = 3
};
enum CubeletBuffer_DataType {
  CubeletBuffer_DataType_UINT8 = 1,
  CubeletBuffer_DataType_INT32 = 2,
  CubeletBuffer_DataType_FLOAT32 = 3
};
enum CubeletBuffer_CompressionAlgorithm {
  CubeletBuffer_CompressionAlgorithm_NONE = 0,
  CubeletBuffer_CompressionAlgorithm_ZLIB = 1,
  CubeletBuffer_CompressionAlgorithm_WAVELET = 2
};

#define WL_PB_OPT(type, name, dflt)                                        \
 private: type name##_ = dflt; bool has_##name##_ = false;                  \
 public:                                                                   \
  type name() const { return name##_; }                                    \
  bool has_##name() const { return has_##name##_; }                        \
  void set_##name(type v) { name##_ = v; has_##name##_ = true; }

#define WL_PB_REP(type, name)                                              \
 private: std::vector<type> name##_;                                       \
 public:                                                                   \
  int name##_size() const { return (int)name##_.size(); }                  \
  type name(int i) const { return name##_[i]; }                            \
  void add_##name(type v) { name##_.push_back(v); }

class CompressionParametersBuffer : public google::protobuf::Message {
 public:
  typedef CompressionParametersBuffer_WaveletAlgorithm WaveletAlgorithm;
  typedef CompressionParametersBuffer_QuantizationAlgorithm QuantizationAlgorithm;
  WL_PB_OPT(uint32_t, original_width, 0)
  WL_PB_OPT(uint32_t, original_height, 0)
  WL_PB_OPT(uint32_t, original_depth, 0)
  WL_PB_OPT(CubeletBuffer_DataType, original_data_type, CubeletBuffer_DataType_UINT8)
  WL_PB_OPT(int32_t, wavelet_transform_steps_x, 0)
  WL_PB_OPT(int32_t, wavelet_transform_steps_y, 0)
  WL_PB_OPT(int32_t, wavelet_transform_steps_z, 0)
  WL_PB_OPT(CompressionParametersBuffer_WaveletAlgorithm, wavelet_algorithm,
            CompressionParametersBuffer_WaveletAlgorithm_CDF97)
  WL_PB_OPT(bool, transform_2d, false)
  WL_PB_OPT(float, threshold_fraction, 0.0f)
  WL_PB_OPT(float, threshold_value, 0.0f)
  WL_PB_OPT(int32_t, quant_bin_count, 0)
  WL_PB_OPT(CompressionParametersBuffer_QuantizationAlgorithm, quantization_algorithm,
            CompressionParametersBuffer_QuantizationAlgorithm_LOG)
  WL_PB_OPT(float, quant_max_value, 0.0f)
  WL_PB_REP(float, quant_bin_boundaries)
  WL_PB_REP(float, quant_bin_values)
  WL_PB_REP(int32_t, huffman_decode_table)
  WL_PB_OPT(int32_t, huffman_dup_key, 0)
  WL_PB_OPT(int32_t, huffman_dup_value, 0)

 public:
  std::string encode() const {
    using namespace wl_pbshim;
    std::string o;
    if (has_wavelet_transform_steps_x_) put_i32(o, 1, wavelet_transform_steps_x_);
    if (has_wavelet_transform_steps_y_) put_i32(o, 2, wavelet_transform_steps_y_);
    if (has_wavelet_transform_steps_z_) put_i32(o, 3, wavelet_transform_steps_z_);
    if (has_wavelet_algorithm_) put_i32(o, 4, (int32_t)wavelet_algorithm_);
    if (has_threshold_fraction_) put_float(o, 6, threshold_fraction_);
    if (has_threshold_value_) put_float(o, 7, threshold_value_);
    if (has_quant_bin_count_) put_i32(o, 8, quant_bin_count_);
    if (has_quantization_algorithm_) put_i32(o, 9, (int32_t)quantization_algorithm_);
    if (has_quant_max_value_) put_float(o, 10, quant_max_value_);
    put_packed_floats(o, 11, quant_bin_boundaries_);
    put_packed_floats(o, 12, quant_bin_values_);
    put_packed_i32(o, 13, huffman_decode_table_);
    if (has_original_width_) put_u32(o, 14, original_width_);
    if (has_original_height_) put_u32(o, 15, original_height_);
    if (has_original_depth_) put_u32(o, 16, original_depth_);
    if (has_original_data_type_) put_i32(o, 17, (int32_t)original_data_type_);
    if (has_transform_2d_) put_u32(o, 18, transform_2d_ ? 1 : 0);
    if (has_huffman_dup_key_) put_i32(o, 19, huffman_dup_key_);
    if (has_huffman_dup_value_) put_i32(o, 20, huffman_dup_value_);
    return o;
  }
  bool decode(wl_pbshim::Reader r) {
    while (r.more()) {
      uint64_t tag = r.varint();
      int field = (int)(tag >> 3), wire = (int)(tag & 7);
      switch (field) {
        case 1: set_wavelet_transform_steps_x((int32_t)r.varint()); break;
        case 2: set_wavelet_transform_steps_y((int32_t)r.varint()); break;
        case 3: set_wavelet_transform_steps_z((int32_t)r.varint()); break;
        case 4: set_wavelet_algorithm((CompressionParametersBuffer_WaveletAlgorithm)r.varint()); break;
        case 6: set_threshold_fraction(r.f32()); break;
        case 7: set_threshold_value(r.f32()); break;
        case 8: set_quant_bin_count((int32_t)r.varint()); break;
        case 9: set_quantization_algorithm((CompressionParametersBuffer_QuantizationAlgorithm)r.varint()); break;
        case 10: set_quant_max_value(r.f32()); break;
        case 11: wl_pbshim::read_floats(r, wire, quant_bin_boundaries_); break;
        case 12: wl_pbshim::read_floats(r, wire, quant_bin_values_); break;
        case 13: wl_pbshim::read_i32s(r, wire, huffman_decode_table_); break;
        case 14: set_original_width((uint32_t)r.varint()); break;
        case 15: set_original_height((uint32_t)r.varint()); break;
        case 16: set_original_depth((uint32_t)r.varint()); break;
        case 17: set_original_data_type((CubeletBuffer_DataType)r.varint()); break;
        case 18: set_transform_2d(r.varint() != 0); break;
        case 19: set_huffman_dup_key((int32_t)r.varint()); break;
        case 20: set_huffman_dup_value((int32_t)r.varint()); break;
        default: r.skip(wire);
      }
    }
    return r.ok && has_wavelet_transform_steps_x_ && has_wavelet_transform_steps_y_ &&
           has_wavelet_transform_steps_z_ && has_wavelet_algorithm_ && has_quant_bin_count_;
  }
  int ByteSize() const override { return (int)encode().size(); }
  bool SerializeToArray(void *data, int size) const override {
    std::string s = encode();
    if ((int)s.size() > size) return false;
    memcpy(data, s.data(), s.size());
    return true;
  }
  bool ParseFromArray(const void *data, int size) override {
    *this = CompressionParametersBuffer();
    return decode(wl_pbshim::Reader(data, size));
  }
};

class CubeletBuffer : public google::protobuf::Message {
 public:
  WL_PB_OPT(uint32_t, width, 0)
  WL_PB_OPT(uint32_t, height, 0)
  WL_PB_OPT(uint32_t, depth, 0)
  WL_PB_OPT(uint32_t, x_offset, 0)
  WL_PB_OPT(uint32_t, y_offset, 0)
  WL_PB_OPT(uint32_t, z_offset, 0)
  WL_PB_OPT(CubeletBuffer_DataType, data_type, CubeletBuffer_DataType_UINT8)
  WL_PB_OPT(int32_t, maximum_value, 0)
  WL_PB_OPT(uint32_t, byte_count, 0)
  WL_PB_OPT(CubeletBuffer_CompressionAlgorithm, compression_algorithm,
            CubeletBuffer_CompressionAlgorithm_NONE)
  WL_PB_OPT(uint32_t, checksum, 0)
  WL_PB_OPT(std::string, data_file_name, std::string())
  WL_PB_OPT(uint32_t, data_file_index, 0)
  WL_PB_OPT(uint64_t, data_file_offset, 0)

 private:
  CompressionParametersBuffer compression_parameters_;
  bool has_compression_parameters_ = false;

 public:
  const CompressionParametersBuffer &compression_parameters() const {
    return compression_parameters_;
  }
  CompressionParametersBuffer *mutable_compression_parameters() {
    has_compression_parameters_ = true;
    return &compression_parameters_;
  }
  bool has_compression_parameters() const { return has_compression_parameters_; }

  std::string encode() const {
    using namespace wl_pbshim;
    std::string o;
    if (has_width_) put_u32(o, 1, width_);
    if (has_height_) put_u32(o, 2, height_);
    if (has_depth_) put_u32(o, 3, depth_);
    if (has_x_offset_) put_u32(o, 4, x_offset_);
    if (has_y_offset_) put_u32(o, 5, y_offset_);
    if (has_z_offset_) put_u32(o, 6, z_offset_);
    if (has_data_type_) put_i32(o, 7, (int32_t)data_type_);
    if (has_byte_count_) put_u32(o, 8, byte_count_);
    if (has_compression_algorithm_) put_i32(o, 9, (int32_t)compression_algorithm_);
    if (has_checksum_) put_u32(o, 10, checksum_);
    if (has_data_file_name_) put_bytes(o, 11, data_file_name_);
    if (has_data_file_index_) put_u32(o, 12, data_file_index_);
    if (has_data_file_offset_) put_u64(o, 13, data_file_offset_);
    if (has_compression_parameters_) put_bytes(o, 14, compression_parameters_.encode());
    if (has_maximum_value_) put_i32(o, 15, maximum_value_);
    return o;
  }
  bool decode(wl_pbshim::Reader r) {
    while (r.more()) {
      uint64_t tag = r.varint();
      int field = (int)(tag >> 3), wire = (int)(tag & 7);
      switch (field) {
        case 1: set_width((uint32_t)r.varint()); break;
        case 2: set_height((uint32_t)r.varint()); break;
        case 3: set_depth((uint32_t)r.varint()); break;
        case 4: set_x_offset((uint32_t)r.varint()); break;
        case 5: set_y_offset((uint32_t)r.varint()); break;
        case 6: set_z_offset((uint32_t)r.varint()); break;
        case 7: set_data_type((CubeletBuffer_DataType)r.varint()); break;
        case 8: set_byte_count((uint32_t)r.varint()); break;
        case 9: set_compression_algorithm((CubeletBuffer_CompressionAlgorithm)r.varint()); break;
        case 10: set_checksum((uint32_t)r.varint()); break;
        case 11: { wl_pbshim::Reader s = r.sub(); set_data_file_name(std::string((const char*)s.p, s.end - s.p)); break; }
        case 12: set_data_file_index((uint32_t)r.varint()); break;
        case 13: set_data_file_offset(r.varint()); break;
        case 14: {
          wl_pbshim::Reader s = r.sub();
          if (!mutable_compression_parameters()->decode(s)) return false;
          break;
        }
        case 15: set_maximum_value((int32_t)r.varint()); break;
        default: r.skip(wire);
      }
    }
    return r.ok && has_width_ && has_height_ && has_depth_ && has_data_type_ && has_byte_count_;
  }
  int ByteSize() const override { return (int)encode().size(); }
  bool SerializeToArray(void *data, int size) const override {
    std::string s = encode();
    if ((int)s.size() > size) return false;
    memcpy(data, s.data(), s.size());
    return true;
  }
  bool ParseFromArray(const void *data, int size) override {
    *this = CubeletBuffer();
    return decode(wl_pbshim::Reader(data, size));
  }
};

class CubeletIndexBuffer : public google::protobuf::Message {
 public:
  WL_PB_OPT(uint32_t, width, 0)
  WL_PB_OPT(uint32_t, height, 0)
  WL_PB_OPT(uint32_t, depth, 0)

 private:
  std::vector<std::string> data_files_;
  std::vector<CubeletBuffer> cubelets_;

 public:
  CubeletBuffer *add_cubelets() { cubelets_.emplace_back(); return &cubelets_.back(); }
  void clear_cubelets() { cubelets_.clear(); }
  int cubelets_size() const { return (int)cubelets_.size(); }
  const CubeletBuffer &cubelets(int i) const { return cubelets_[i]; }

  std::string encode() const {
    using namespace wl_pbshim;
    std::string o;
    if (has_width_) put_u32(o, 1, width_);
    if (has_height_) put_u32(o, 2, height_);
    if (has_depth_) put_u32(o, 3, depth_);
    for (const std::string &f : data_files_) put_bytes(o, 4, f);
    for (const CubeletBuffer &c : cubelets_) put_bytes(o, 5, c.encode());
    return o;
  }
  int ByteSize() const override { return (int)encode().size(); }
  bool SerializeToArray(void *data, int size) const override {
    std::string s = encode();
    if ((int)s.size() > size) return false;
    memcpy(data, s.data(), s.size());
    return true;
  }
  bool ParseFromArray(const void *data, int size) override {
    *this = CubeletIndexBuffer();
    wl_pbshim::Reader r(data, size);
    while (r.more()) {
      uint64_t tag = r.varint();
      int field = (int)(tag >> 3), wire = (int)(tag & 7);
      switch (field) {
        case 1: set_width((uint32_t)r.varint()); break;
        case 2: set_height((uint32_t)r.varint()); break;
        case 3: set_depth((uint32_t)r.varint()); break;
        case 4: { wl_pbshim::Reader s = r.sub(); data_files_.push_back(std::string((const char*)s.p, s.end - s.p)); break; }
        case 5: { wl_pbshim::Reader s = r.sub(); if (!add_cubelets()->decode(s)) return false; break; }
        default: r.skip(wire);
      }
    }
    return r.ok;
  }
};

#undef WL_PB_OPT
#undef WL_PB_REP

#endif
