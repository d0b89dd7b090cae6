// wl_compress: the reference's command line on the GPU library.
//
//   wl_compress [opts] <input file> <output file>
//
// Flags and defaults follow parseOptions / printHelp
// (test_compress_common.cc:35-192): -d, -steps, -thresh, -qcount, -wave,
// -qalg, -noz, -2d, -opt, -err, -q, -v; -exact selects the reference float
// order for the CDF 9/7 transform (bit-identical output files).  -err prints
// the reference's error line after compressing (test_compress_cpu.cc:150-157).
// Flags of the reference that only print diagnostics (-pb, -enc, -bq, -aq)
// are rejected with a message rather than silently ignored.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "wlgpu.h"

static void help() {
  fprintf(stderr,
          "\n  wl_compress [opts] <input file> <output file>\n"
          "  Options:\n"
          "    -d : decompress (default is to compress)\n"
          "    -steps <n> : # of wavelet transform steps (default = -1)\n"
          "    -thresh <n> : proportion of data to be eliminated in threshold cutoff\n"
          "                  Must be between [0..1]. (default = 0.500)\n"
          "    -qcount <n> : # of bins into which data is quantized (default=256)\n"
          "    -wave <wavelet> : haar or cdf97 (default = cdf97)\n"
          "    -qalg <algorithm> : uniform, log, or lloyd (default = log)\n"
          "    -noz : disable compression of long strings of zeros\n"
          "    -2d : rather than 3d transform, do 2d transform at each layer\n"
          "    -opt : print the threshold / bin count sweep (8-bit input; no output)\n"
          "    -err : compute error metrics\n"
          "    -exact : CDF9/7 in the reference's float order\n"
          "    -q : be quiet\n\n");
  exit(1);
}

int main(int argc, char **argv) {
  wl_params p;
  wl_params_default(&p);
  bool decompress = false, quiet = false, optimize = false, errors = false;
  int i = 1;
  for (; i < argc && argv[i][0] == '-'; i++) {
    const char *a = argv[i];
    auto need = [&]() -> const char * {
      if (++i >= argc) help();
      return argv[i];
    };
    if (!strcmp(a, "-d")) decompress = true;
    else if (!strcmp(a, "-q")) quiet = true;
    else if (!strcmp(a, "-v")) {}
    else if (!strcmp(a, "-noz")) p.compress_zeros = 0;
    else if (!strcmp(a, "-exact")) p.exact_transform = 1;
    else if (!strcmp(a, "-2d")) p.transform_2d = 1;
    else if (!strcmp(a, "-opt")) optimize = true;
    else if (!strcmp(a, "-err")) errors = true;
    else if (!strcmp(a, "-steps")) {
      const char *v = need();
      int x = 1, y = 1, z = 1;
      int k = sscanf(v, "%d,%d,%d", &x, &y, &z);
      if (k == 1) { p.steps[0] = p.steps[1] = p.steps[2] = x; }
      else if (k == 2) { p.steps[0] = x; p.steps[1] = y; p.steps[2] = 0; }
      else if (k == 3) { p.steps[0] = x; p.steps[1] = y; p.steps[2] = z; }
      else { fprintf(stderr, "Invalid # of wavelet transform steps: \"%s\"\n", v); return 1; }
    } else if (!strcmp(a, "-thresh")) {
      const char *v = need();
      if (sscanf(v, "%f", &p.threshold_fraction) != 1 || p.threshold_fraction < 0 ||
          p.threshold_fraction > 1) {
        fprintf(stderr, "Invalid threshold proportion: \"%s\"\n", v);
        return 1;
      }
    } else if (!strcmp(a, "-qcount")) {
      const char *v = need();
      if (sscanf(v, "%d", &p.bin_count) != 1 || p.bin_count < 1) {
        fprintf(stderr, "Invalid # quantize bins: \"%s\"\n", v);
        return 1;
      }
    } else if (!strcmp(a, "-wave")) {
      const char *v = need();
      if (!strcmp(v, "haar")) p.wavelet = WL_HAAR;
      else if (!strcmp(v, "cdf97")) p.wavelet = WL_CDF97;
      else { fprintf(stderr, "Invalid wavelet: \"%s\"\n", v); return 1; }
    } else if (!strcmp(a, "-qalg")) {
      const char *v = need();
      if (!strcmp(v, "uniform")) p.quant_alg = WL_UNIFORM;
      else if (!strcmp(v, "log")) p.quant_alg = WL_LOG;
      else if (!strcmp(v, "lloyd")) p.quant_alg = WL_LLOYD;
      else { fprintf(stderr, "Invalid quantize algorithm: \"%s\"\n", v); return 1; }
    } else {
      fprintf(stderr, "Unrecognized option: \"%s\"\n", a);
      return 1;
    }
  }
  if (argc - i != 2) help();
  wl_ctx *ctx = nullptr;
  if (wl_init(0, &ctx) != WL_OK) {
    fprintf(stderr, "no CUDA device\n");
    return 1;
  }
  auto t0 = std::chrono::steady_clock::now();
  if (optimize && !decompress) {
    // the reference's plotAll table (optimize.cc:96-122); no output file
    int n = 0;
    wl_status st = wl_optimize_file(ctx, argv[i], &p, nullptr, 0, &n);
    wl_opt_point *pts = st == WL_OK ? new wl_opt_point[n] : nullptr;
    if (st == WL_OK) st = wl_optimize_file(ctx, argv[i], &p, pts, n, &n);
    if (st != WL_OK) {
      fprintf(stderr, "error: %s\n", wl_last_error(ctx));
      delete[] pts;
      wl_destroy(ctx);
      return 1;
    }
    printf("Threshold\tBins\tsize\tpSNR\n");
    for (int k = 0; k < n; k++)
      printf("%.3f\t%d\t%d\t%.6g\n", pts[k].threshold_fraction, pts[k].bin_count,
             pts[k].size_bytes, pts[k].psnr);
    delete[] pts;
    wl_destroy(ctx);
    return 0;
  }
  wl_status st = decompress ? wl_decompress_file(ctx, argv[i], argv[i + 1])
                            : wl_compress_file(ctx, argv[i], argv[i + 1], &p);
  auto t1 = std::chrono::steady_clock::now();
  if (st != WL_OK) {
    fprintf(stderr, "error: %s\n", wl_last_error(ctx));
    wl_destroy(ctx);
    return 1;
  }
  if (errors && !decompress) {
    // computeErrorRates after quantizing (test_compress_cpu.cc:150-157)
    wl_error_stats es;
    st = wl_error_metrics_file(ctx, argv[i], argv[i + 1], &es);
    if (st != WL_OK) {
      fprintf(stderr, "error: %s\n", wl_last_error(ctx));
      wl_destroy(ctx);
      return 1;
    }
    if (es.count == 0)
      fprintf(stderr, "Cannot compute error rates: no maximum possible input value set.\n");
    printf("Mean squared error: %.3f, relative error: %g, peak SNR: %.3f\n", es.mse,
           es.relative_error, es.psnr);
  }
  if (!quiet) {
    printf("Total: %.2f ms\n", std::chrono::duration<double, std::milli>(t1 - t0).count());
  }
  wl_destroy(ctx);
  return 0;
}
