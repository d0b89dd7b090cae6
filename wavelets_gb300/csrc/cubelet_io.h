// .cube container codec (reference cubelet_file.h:17-45, wavelet_compress.proto).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "wlgpu.h"

namespace wl {

constexpr const char *kCubeHeader = "SCU cubelets 1.0\n";
// CubeletBuffer.DataType / CompressionParametersBuffer enums on the wire
constexpr int kPbUint8 = 1, kPbInt32 = 2, kPbFloat32 = 3;
constexpr int kPbLog = 1, kPbUniform = 2, kPbLloyd = 3;

// CubeletBuffer + CompressionParametersBuffer fields used by this path.
struct CubeMeta {
  int width = 0, height = 0, depth = 0;
  int offset[3] = {0, 0, 0};    // position in the parent volume (x, y, z)
  int data_type = 0;            // wire DataType
  uint64_t byte_count = 0;
  int32_t maximum_value = 0;
  bool compressed = false;
  // compression parameters (compressed cubelets only)
  int steps[3] = {0, 0, 0};
  int wavelet = 2;
  bool transform_2d = false;
  float threshold_fraction = 0, threshold_value = 0;
  int bin_count = 0;
  int pb_quant_alg = kPbLog;
  float quant_max_value = 0;
  std::vector<float> boundaries, values;
  std::vector<int32_t> decode;
  int original_size[3] = {0, 0, 0};
  int original_data_type = 0;
  int dup_key = -1, dup_value = -1;
};

std::string encode_meta(const CubeMeta &m, uint64_t data_file_offset);
bool decode_meta(const void *buf, size_t n, CubeMeta &m);
std::string encode_file(const std::vector<CubeMeta> &metas,
                        const std::vector<const std::string *> &datas, bool footer);
bool decode_file(const std::string &buf, std::vector<CubeMeta> &metas,
                 std::vector<std::string> &datas, std::string &err);
bool read_whole_file(const char *path, std::string &out);
// conversions between a compressed cubelet's metadata and a wl_result
// (engine.cpp); meta_to_result points the result's arrays into m and words
wl_status result_to_meta(const wl_result *r, CubeMeta &m);
void meta_to_result(CubeMeta &m, const std::string &words, wl_result &r);
// a page-locked staging buffer of the context, kept across calls (engine.cpp)
char *ctx_staging(wl_ctx *ctx, int slot, size_t bytes);
bool write_whole_file(const char *path, const std::string &data);

}  // namespace wl
