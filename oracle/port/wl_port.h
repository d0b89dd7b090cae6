/* Test oracle (CPU restatement of the reference compression path).
 *
 * This library is TEST INFRASTRUCTURE: the parity tests, the smoke check and
 * the benchmark's CPU-baseline leg call it as the checker / baseline.  The
 * product (libwlgpu) never links or calls it.
 *
 * It restates, in plain C++, the reference's CPU path exactly as the reference
 * computes it (same float operation order, no fused multiply-add, same
 * tie-breaking), so its outputs are bit-identical to the reference's
 * test_compress_cpu.  Each function cites the reference file:line it follows.
 * Pinned against the reference itself: tests/golden holds outputs of the
 * reference built from its own sources (oracle/ref/Makefile).
 */
#ifndef WL_PORT_H
#define WL_PORT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* reference enums (wavelet.h:25-46) */
enum { ORC_HAAR = 1, ORC_CDF97 = 2 };
enum { ORC_UNIFORM = 1, ORC_LOG = 2, ORC_LLOYD = 3 };
enum { ORC_UINT8 = 1, ORC_INT32 = 2, ORC_FLOAT32 = 3 };

/* Result of the post-transform stages for one cubelet. */
typedef struct {
  float threshold, min_value, max_value, max_abs;
  int nonzero_count, zero_bin;       /* zero_bin = -1 when zero runs are off */
  int bin_count, quant_alg;
  int n_boundaries, n_values;        /* codebook (Lloyd) sizes */
  int n_words;                       /* Huffman stream length in 32-bit words */
  int n_decode;                      /* decode table length (ints) */
  int longest_code;                  /* bits */
  int dup_key, dup_value;            /* -1 when unused */
} orc_result;

/* Error metrics of the first compressed cubelet of comp_path against the
 * first uncompressed cubelet of orig_path (computeErrorRates,
 * test_compress_common.cc:587-694; ErrorAccumulator,
 * test_compress_common.h:90-160): sums = {sum a, sum a*a, sum |a-b|,
 * sum |a-b|^2}, getters = {average, L1, L2, MSE, PSNR, relative error}.
 * count = 0 when no maximum possible value is known (non-8-bit input without
 * maximum_value).  Returns 0 on success. */
int orc_error_metrics(const char *orig_path, const char *comp_path, double sums[4],
                      long long *count, float getters[6]);

/* Run the reference's command line (test_compress_cpu.cc:37-65) in-process:
 * same flags, same .cube output.  Returns 0 on success. */
int orc_main(int argc, const char **argv);

/* Forward 3-D transform of a padded float volume stored x-fastest
 * (X*Y*Z floats); writes the rotated Z-X-Y result (dwt_cpu.cc:943-965,
 * haar_3d :624-635; all-zero steps skip the rotation, test_compress_common.cc:496). */
int orc_forward(const float *in, int X, int Y, int Z, int sx, int sy, int sz,
                int wavelet, float *out);

/* Inverse of orc_forward: input in the rotated layout of a padded X*Y*Z
 * volume, output x-fastest (dwt_cpu.cc:966-983, haar_3d :636-645). */
int orc_inverse(const float *in, int X, int Y, int Z, int sx, int sy, int sz,
                int wavelet, float *out);

/* Threshold, quantize and Huffman-encode n coefficients (the second half of
 * compressFile, test_compress_cpu.cc:97-172).  bins_out (n ints), words_out
 * (words_cap words), decode_out (decode_cap ints), hist_out (bin_count+1
 * counts: the Huffman frequency table including the zero-run symbol),
 * boundaries_out / values_out (bin_count floats each) may be NULL.
 * Returns 0 on success, 1 if a buffer is too small. */
int orc_encode(const float *coeffs, int n, float threshold_fraction,
               int bin_count, int quant_alg, int compress_zeros,
               orc_result *res, int *bins_out, uint32_t *words_out,
               int words_cap, int *decode_out, int decode_cap,
               int64_t *hist_out, float *boundaries_out, float *values_out);

/* Quantize with given parameters (createQuantizer + quantizeRow,
 * test_compress_common.cc:1025-1039).  For Lloyd, boundaries/values hold
 * bin_count-1 / bin_count entries. */
int orc_quantize(const float *coeffs, int n, int quant_alg, int bin_count,
                 float threshold, float max_abs, const float *boundaries,
                 const float *values, int *bins_out);

/* Huffman-encode given bins exactly as the reference does after quantizing
 * (initHuffman + huffScan + computeHuffmanCoding + encodeToStream,
 * test_compress_common.cc:953-1022, huffman.cc:42-97, huffman.h:242-296).
 * zero_bin < 0 disables zero-run tokens.  hist_out: bin_count+1 counts. */
int orc_huffman_encode(const int *bins, int n, int bin_count, int zero_bin,
                       orc_result *res, uint32_t *words_out, int words_cap,
                       int *decode_out, int decode_cap, int64_t *hist_out);

/* Dequantize bins (dequantize, test_compress_common.cc:567-584). */
int orc_dequantize(const int *bins, int n, int quant_alg, int bin_count,
                   float threshold, float max_abs, const float *values,
                   float *out);

/* Decode a Huffman stream with the reference's table walk
 * (HuffmanDecoder::decodeFromStream, huffman.h:96-131).  Returns the number of
 * values decoded. */
int orc_huffman_decode(const uint32_t *words, int n_words, const int *table,
                       int n_table, int dup_key, int dup_value, int *out, int n);

/* Whole-cubelet compress of a raw volume (x fastest) of the given dtype:
 * pad, transform, encode.  Writes the compressed .cube to out_path.  Used as
 * the timed CPU baseline.  Returns 0 on success. */
int orc_compress_volume(const void *data, int dtype, int X, int Y, int Z,
                        int sx, int sy, int sz, int wavelet,
                        float threshold_fraction, int bin_count, int quant_alg,
                        int compress_zeros, const char *out_path,
                        orc_result *res);

#ifdef __cplusplus
}
#endif
#endif
