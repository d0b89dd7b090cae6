// Test-oracle support only: never shipped, never measured.
//
// Glue around the UNMODIFIED reference CPU path (compiled from the reference
// sources by oracle/ref/Makefile).  It runs the same stages as the reference
// driver compressFile (test_compress_cpu.cc:68-184) by calling the reference's
// own functions, and additionally
//   * writes the transform output (the coefficients, in the reference's
//     rotated Z-X-Y order) and the quantized bins as raw files, and
//   * can replace the transform output with coefficients read from a file, so
//     the reference's threshold / quantizer / Huffman stages can be fed the
//     coefficients another implementation produced.
//
// usage: ref_dump [reference flags] <in.cube> <out.cube> <dumpdir> [coeffs.f32]
//   dumpdir receives coeffs.f32, bins.i32 and stats.txt.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "test_compress_common.h"
#include "test_compress_cpu.h"
#include "thresh_cpu.h"
#include "quant.h"

using namespace scu_wavelet;

static bool write_raw(const std::string &path, const void *p, size_t n) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = fwrite(p, 1, n, f) == n;
  fclose(f);
  return ok;
}

int main(int argc, char **argv) {
  Options opt;
  int next;
  if (!parseOptions(argc, argv, opt, next)) return 1;
  QUIET = true;
  opt.quiet = true;
  if (argc - next < 3) {
    fprintf(stderr, "usage: ref_dump [flags] in.cube out.cube dumpdir [coeffs.f32]\n");
    return 1;
  }
  const char *inPath = argv[next], *outPath = argv[next + 1];
  std::string dumpDir = argv[next + 2];
  const char *coeffPath = (argc - next >= 4) ? argv[next + 3] : NULL;

  WaveletCompressionParam param = opt.param;
  Cube inputData;
  CubeFloat data;
  CubeInt quantizedData;
  CubeletStreamReader reader;

  if (!readData(inPath, &inputData, &data, &reader, &param)) return 1;
  if (!waveletTransform(data, param, false, false)) return 1;
  data.param = param;

  if (coeffPath) {
    FILE *f = fopen(coeffPath, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", coeffPath); return 1; }
    size_t n = fread(data.data(), sizeof(float), data.count(), f);
    fclose(f);
    if ((int)n != data.count()) { fprintf(stderr, "short coefficient file\n"); return 1; }
  }
  write_raw(dumpDir + "/coeffs.f32", data.data(), sizeof(float) * data.count());

  const int count = data.count();
  float maxVal, minVal, *sortedAbs = NULL;
  int nonzeroCount;
  param.thresholdValue = thresh_cpu(&data, param.thresholdFraction,
                                    &nonzeroCount, &maxVal, &minVal, &sortedAbs);
  float maxAbsVal = sortedAbs[count - 1];
  float *nonzeroData = sortedAbs + count - nonzeroCount;

  int zeroBin;
  if (!quantize(data, quantizedData, maxAbsVal, param, nonzeroData,
                nonzeroCount, minVal, maxVal, &zeroBin)) return 1;
  quantizedData.param = param;
  if (!opt.doCompressZeros) zeroBin = -1;
  write_raw(dumpDir + "/bins.i32", quantizedData.data(), sizeof(int) * count);

  FILE *s = fopen((dumpDir + "/stats.txt").c_str(), "w");
  if (s) {
    fprintf(s, "size %d %d %d\n", data.size.x, data.size.y, data.size.z);
    fprintf(s, "steps %d %d %d\n", param.transformSteps.x, param.transformSteps.y,
            param.transformSteps.z);
    fprintf(s, "threshold %a\nmin %a\nmax %a\nmaxabs %a\n", param.thresholdValue,
            minVal, maxVal, maxAbsVal);
    fprintf(s, "nonzero %d\nzerobin %d\n", nonzeroCount, zeroBin);
    fprintf(s, "boundaries %d\n", (int)param.binBoundaries.size());
    for (float b : param.binBoundaries) fprintf(s, "%a\n", b);
    fprintf(s, "values %d\n", (int)param.binValues.size());
    for (float v : param.binValues) fprintf(s, "%a\n", v);
    fclose(s);
  }
  delete[] sortedAbs;

  CubeletStreamWriter writer;
  if (!writer.open(outPath)) return 1;
  if (!writeQuantData(writer, &quantizedData, opt, NULL, NULL, zeroBin)) return 1;
  writer.close(true);
  return 0;
}
