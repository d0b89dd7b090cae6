/* libwlgpu: GB300 (sm_103a) cubelet compression behind a C ABI.
 *
 * Drop-in for the reference's cubelet compression path
 * (transform -> threshold -> quantize -> count -> Huffman, and its inverse).
 * The entry points replace these reference interfaces:
 *
 *   wl_compress_file / wl_decompress_file
 *       test_compress_cpu / test_compress_gpu command line
 *       (compressFile test_compress_cpu.cc:68-184, test_compress_gpu.cu:150-436;
 *        decompressFile test_compress_cpu.cc:187-241): first uncompressed
 *       cubelet of a .cube file in, one compressed cubelet out, same bytes.
 *   wl_compress_cubelet
 *       readData .. writeQuantData for one in-memory cubelet
 *       (test_compress_common.h:173-248; waveletTransform :492,
 *        thresh_cpu thresh_cpu.cc:80, quantize test_compress_cpu.cc:244,
 *        writeQuantData test_compress_common.cc:198).
 *   wl_decompress_cubelet
 *       readQuantData + dequantize + inverse waveletTransform +
 *       translateCubeDataToOriginal (test_compress_common.cc:850, :567, :492, :699).
 *   wl_compress_batch
 *       no reference counterpart: many cubelets per launch (the reference
 *       compresses one cubelet per process, test_compress_common.cc:296-302).
 *
 * Conventions: every call returns a wl_status and never exits the process
 * (the reference prints and exit(1)s on CUDA errors, cucheck.h:9-21);
 * wl_last_error() describes the last failure on a context.  One context per
 * host thread; a context owns one CUDA stream and its device workspace.
 */
#ifndef WLGPU_H
#define WLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  WL_OK = 0,
  WL_EINVAL = 1,    /* bad argument or unsupported parameter */
  WL_ENOMEM = 2,    /* device or host allocation failed / budget exceeded */
  WL_ETIMEOUT = 3,  /* a bounded wait ran out */
  WL_EFORMAT = 4,   /* malformed .cube file or compressed stream */
  WL_ECUDA = 5,     /* CUDA runtime error */
  WL_EIO = 6        /* file open/read/write failed */
} wl_status;

/* element types; U8, I32 and F32 are the reference's (wavelet.h:41-46) */
typedef enum { WL_U8 = 1, WL_I32 = 2, WL_F32 = 3, WL_U16 = 4 } wl_dtype;
typedef enum { WL_HAAR = 1, WL_CDF97 = 2 } wl_wavelet;            /* wavelet.h:33-38 */
typedef enum { WL_UNIFORM = 1, WL_LOG = 2, WL_LLOYD = 3 } wl_quant; /* wavelet.h:25-30 */

/* Compression parameters (WaveletCompressionParam, wavelet.h:221-295, with the
 * command-line defaults of wavelet.h:48-53). */
typedef struct {
  int steps[3];             /* x, y, z; -1 = ceil(log2(axis length)) */
  int wavelet;              /* wl_wavelet */
  float threshold_fraction; /* fraction of coefficients set to the zero bin */
  int bin_count;            /* 2..4096 */
  int quant_alg;            /* wl_quant */
  int compress_zeros;       /* 1 = zero-run Huffman tokens (reference default) */
  int lloyd_iters;          /* Lloyd iterations on the |coefficient| histogram */
  int exact_transform;      /* 1 = reference float operation order (filter bank);
                               0 = lifting (default) */
  int transform_2d;         /* 1 = -2d: a 2-D transform of every z layer
                               (test_compress_common.cc:519-541); x and y step
                               counts below 1 mean the maximum, z steps only
                               pad; the stored order stays x fastest */
} wl_params;

/* Fill p with the reference's defaults. */
void wl_params_default(wl_params *p);

/* One compressed cubelet: metadata of the CubeletBuffer /
 * CompressionParametersBuffer messages (wavelet_compress.proto) plus the
 * Huffman words.  Arrays are owned by the library; release with wl_result_free. */
typedef struct {
  int size[3];              /* stored (rotated Z-X-Y) size: width, height, depth */
  int original_size[3];
  int original_dtype;       /* wl_dtype of the input */
  int steps[3];             /* after clamping */
  int wavelet, quant_alg, bin_count;
  float threshold_fraction;
  float threshold_value;
  float max_value;          /* largest |coefficient| (quant_max_value) */
  float min_coef, max_coef; /* signed extremes as the reference tracks them */
  int zero_bin;
  int dup_key, dup_value;   /* -1 when zero-run tokens are off */
  int longest_code;         /* bits */
  int n_words;              /* Huffman stream length, 32-bit words */
  uint32_t *words;
  int n_decode;             /* Huffman decode table length (ints) */
  int32_t *decode;
  int n_boundaries, n_values; /* codebook (Lloyd only) */
  float *boundaries, *values;
  void *owner;              /* library-internal: shared storage of the arrays
                               (NULL: each array is its own malloc block) */
  int transform_2d;         /* 2-D mode: size is the padded (x, y, z), not rotated */
} wl_result;

void wl_result_free(wl_result *r);
/* wl_result_free on each of r[0..n). */
void wl_results_free(wl_result *r, int n);

typedef struct wl_ctx wl_ctx;

/* Create a context on CUDA device `device`. */
wl_status wl_init(int device, wl_ctx **ctx);
void wl_destroy(wl_ctx *ctx);
const char *wl_last_error(const wl_ctx *ctx);

/* Compress one cubelet.  data points to X*Y*Z elements (x fastest) of dtype;
 * it may be host or device memory (data_on_device).  out is filled and owns
 * its arrays. */
wl_status wl_compress_cubelet(wl_ctx *ctx, const void *data, int dtype,
                              const int size[3], int data_on_device,
                              const wl_params *params, wl_result *out);

/* A batch entry for wl_compress_batch. */
typedef struct {
  const void *data;         /* X*Y*Z elements, x fastest */
  int dtype;
  int size[3];
  wl_params params;
  /* Elements between consecutive rows (y) and slices (z) of the source; 0
   * means dense (X and X*Y).  A sub-volume of a larger array -- a cubelet of
   * a split volume (cube split, cubelet_convert.cc:424-562) -- is passed in
   * place this way, without copying it out first. */
  long long row_pitch, slice_pitch;
} wl_cubelet;

/* Compress n cubelets of any sizes/dtypes/parameters in one pass of batched
 * launches.  data_on_device: all inputs are device pointers. */
wl_status wl_compress_batch(wl_ctx *ctx, const wl_cubelet *items, int n,
                            int data_on_device, wl_result *outs);

/* Decompress: inverse of wl_compress_cubelet.  out receives
 * original_size elements of out_dtype (WL_U8 clamps and truncates like the
 * reference's floatToByte; WL_I32 rounds (int)(f+0.5f); WL_U16 rounds and
 * clamps to 0..65535; WL_F32 as is). */
wl_status wl_decompress_cubelet(wl_ctx *ctx, const wl_result *in, int out_dtype,
                                void *out, int out_on_device);

/* Decompress n cubelets in one pass of batched launches (every stream decoded
 * by one set of decoder launches, one dequantization launch, the inverse
 * transform in concurrent launch groups).  out_dtypes: per cubelet (NULL =
 * each one's original type); outs[i]: original_size elements of that type,
 * all host or all device memory (outs_on_device).  Results are those of
 * wl_decompress_cubelet on each. */
wl_status wl_decompress_batch(wl_ctx *ctx, const wl_result *in, int n, const int *out_dtypes,
                              void *const *outs, int outs_on_device);

/* The transform alone (waveletTransform, test_compress_common.cc:492-564).
 * Forward: data (X*Y*Z elements of dtype, x fastest) is padded by repeating
 * edge values to a multiple of 2^steps per axis and transformed; coeffs
 * receives the padded element count of floats in the stored Z-X-Y order and
 * stored_size the stored (rotated) width, height, depth.  Inverse: coeffs in
 * that order back to original_size elements of out_dtype. */
wl_status wl_forward_transform(wl_ctx *ctx, const void *data, int dtype,
                               const int size[3], const wl_params *params,
                               float *coeffs, size_t coeffs_cap,
                               int stored_size[3]);
wl_status wl_inverse_transform(wl_ctx *ctx, const float *coeffs,
                               const int stored_size[3], const int steps[3],
                               int wavelet, const int original_size[3],
                               int out_dtype, void *out);

/* Command-line equivalents: read the first uncompressed cubelet of in_path,
 * write a .cube with one compressed cubelet (no footer, like the reference);
 * decompress writes the restored cubelet with a footer. */
wl_status wl_compress_file(wl_ctx *ctx, const char *in_path,
                           const char *out_path, const wl_params *params);
wl_status wl_decompress_file(wl_ctx *ctx, const char *in_path,
                             const char *out_path);

/* Serialize one compressed cubelet as a complete .cube file image
 * (header + length + CubeletBuffer + words), as the reference writes it.
 * *buf is malloc'ed; free with wl_free. */
wl_status wl_encode_cube(const wl_result *r, int footer, uint8_t **buf,
                         size_t *len);
void wl_free(void *p);

/* Per-stage device timings (milliseconds, CUDA events on the context's
 * stream) of the last compress call: transform, select, quantize+count,
 * Huffman build, encode, total device time. */
wl_status wl_last_timings(const wl_ctx *ctx, float out[6]);

/* Page-locked host inputs: mode 0 (default) reads them in place from the
 * first transform pass over the host link (fastest for one call at a time);
 * mode 1 copies them into device memory with the copy engine first, leaving
 * the SMs free for work of other contexts meanwhile (lanes whose batches
 * overlap).  Results are identical. */
wl_status wl_set_host_input_mode(wl_ctx *ctx, int mode);

/* Cap the device workspace a context holds (its grow-only buffers) at
 * `bytes` (0, the default: no cap), for hosts that give the library a fixed
 * memory budget.  A call that would need more fails with WL_ENOMEM before
 * anything is freed or launched, and the context stays usable.  Buffers
 * already held above a new, lower cap are kept until they must grow.
 * wl_memory_held: the bytes held now. */
wl_status wl_set_memory_limit(wl_ctx *ctx, size_t bytes);
size_t wl_memory_held(const wl_ctx *ctx);

/* high = 1: the context's streams get the device's greatest scheduling
 * priority, so its kernels are scheduled ahead of pending blocks of other
 * contexts' kernels (the serving loop's express lanes); 0: the default.
 * Call it while the context is idle. */
wl_status wl_set_stream_priority(wl_ctx *ctx, int high);

/* Synchronize the context's stream. */
wl_status wl_sync(wl_ctx *ctx);

/* ---- Serving -------------------------------------------------------------
 * No reference counterpart (the reference compresses one file per process).
 * A server runs a request loop over several lanes, each a context (stream and
 * buffers) driven by its own host thread: compress and decompress requests of
 * any size are admitted as they arrive, requests of one kind waiting together
 * are batched onto the next free lane (continuous batching), and batches on
 * different lanes overlap on the GPU.  Admission counts the device memory
 * every lane holds (its grow-only workspace, or the estimate of its running
 * batch if larger) against the memory budget, and a batch that needs its lane
 * to grow waits unless the device has that much memory free
 * (cudaMemGetInfo); a request larger than the whole budget runs alone once
 * nothing else is in flight.  Compress inputs may be device, page-locked or pageable
 * host pointers; they, and a decompress request's input and output, must stay
 * valid until the request is waited for. */
enum { WL_REQ_COMPRESS = 1, WL_REQ_DECOMPRESS = 2 };

typedef struct {
  int lanes;                /* concurrent batches on the device (default 2) */
  size_t memory_budget;     /* device working bytes admitted at once (default 16 GiB) */
  int max_batch;            /* requests per batch (default 1024) */
  int stage_host_inputs;    /* 1 (default): lanes copy page-locked host inputs
                               with the copy engine (wl_set_host_input_mode 1),
                               so one lane's transfer overlaps another's
                               compute; 0: lanes read them in place */
  size_t max_batch_bytes;   /* input (compress) or output (decompress) bytes of
                               one batch; a larger request runs alone (0, the
                               default: no cap) */
  int express_lanes;        /* lanes that take only requests of at most
                               small_request_bytes, so small requests do not
                               wait behind large ones (default 0) */
  size_t small_request_bytes; /* the express lanes' limit (default 4 MiB) */
  int express_priority;     /* 1: express lanes on the device's highest-priority
                               streams (wl_set_stream_priority); default 0 */
} wl_serve_config;

typedef struct {
  int kind;                 /* WL_REQ_COMPRESS or WL_REQ_DECOMPRESS */
  wl_cubelet cubelet;       /* compress: the input */
  const wl_result *compressed; /* decompress: the input */
  int out_dtype;            /* decompress: output element type */
  void *out;                /* decompress: original_size elements of out_dtype */
  int out_on_device;
} wl_request;

typedef struct {
  int status;               /* wl_status of the request */
  double queue_ms;          /* submit -> its batch started */
  double service_ms;        /* batch start -> done */
  double total_ms;          /* submit -> done */
  int batch_size;           /* requests in the batch that served it */
  int lane;
} wl_request_info;

typedef struct wl_server wl_server;

void wl_serve_config_default(wl_serve_config *cfg);
wl_status wl_serve_create(int device, const wl_serve_config *cfg, wl_server **out);
/* Queue a request; *ticket identifies it for wl_serve_wait. */
wl_status wl_serve_submit(wl_server *srv, const wl_request *req, unsigned long long *ticket);
/* Queue n requests back to back (nothing else between them in the queue),
 * so that a free lane can take them as one batch; tickets[i] for reqs[i].
 * Either all are queued or none (a request that fails validation queues
 * nothing). */
wl_status wl_serve_submit_batch(wl_server *srv, const wl_request *reqs, int n,
                                unsigned long long *tickets);
/* wl_serve_wait on each of tickets[0..n) with no time limit; outs[i]
 * (compress requests) and statuses[i] (may be NULL) receive each result.
 * Returns WL_OK when every request succeeded, else the first failure. */
wl_status wl_serve_wait_batch(wl_server *srv, const unsigned long long *tickets, int n,
                              wl_result *outs, wl_status *statuses);
/* Wait up to timeout_ms (0 polls, negative waits without limit).  Returns
 * WL_ETIMEOUT while the request is pending; otherwise the request's own
 * status, fills *info (may be NULL) and, for compress, *out (owns its arrays;
 * release with wl_result_free), and retires the ticket. */
wl_status wl_serve_wait(wl_server *srv, unsigned long long ticket, int timeout_ms,
                        wl_result *out, wl_request_info *info);
const char *wl_serve_last_error(const wl_server *srv);
/* Finishes the running batches; requests still queued fail with WL_EINVAL. */
void wl_serve_destroy(wl_server *srv);

/* Device memory helpers for callers that keep inputs resident on the GPU. */
void *wl_device_alloc(size_t bytes);
void wl_device_free(void *p);
wl_status wl_copy_to_device(void *dst, const void *src, size_t bytes);
wl_status wl_copy_to_host(void *dst, const void *src, size_t bytes);

/* Number of kernels the last compress/decompress call launched, and the
 * device time (ms, CUDA events on the context's stream) of each kernel
 * group: 0 dwt x pass, 1 dwt y pass, 2 dwt z pass, 3 select, 4 quantizer
 * set-up + Lloyd, 5 quantize + count, 6 zero-run join, 7 Huffman build,
 * 8 encode (count, scan, pack).  Per-group events are recorded only while
 * profiling is on (wl_set_profiling); they add a little launch overhead. */
int wl_last_launch_count(const wl_ctx *ctx);
wl_status wl_set_profiling(wl_ctx *ctx, int on);
wl_status wl_kernel_timings(const wl_ctx *ctx, float out[9]);

/* ---- Whole containers -------------------------------------------------------
 * Every cubelet of a .cube file compressed into a new .cube file (or every
 * compressed cubelet restored), in order, with the index footer
 * (cubelet_file.cc:303-327) and each cubelet's x/y/z offset kept.  The
 * reference compresses only the first cubelet of a file per run
 * (test_compress_common.cc:296-302).  Reading, GPU work and writing overlap:
 * a reader thread fills one of two page-locked buffers of batch_bytes
 * (0 = 256 MiB) while the GPU compresses the other as one batch, and a writer
 * thread appends finished batches.  Cubelets already in the target form are
 * copied unchanged.  16-bit data travels in .cube files as INT32, as the
 * reference stores it. */
typedef struct {
  int cubelets;                 /* written */
  int copied;                   /* of those, copied unchanged */
  unsigned long long bytes_in;  /* cubelet data read */
  unsigned long long bytes_out; /* cubelet data written */
  double seconds;               /* wall time of the call */
  double read_seconds, compute_seconds, write_seconds; /* busy time per stage */
} wl_container_stats;
wl_status wl_compress_container(wl_ctx *ctx, const char *in_path, const char *out_path,
                                const wl_params *params, size_t batch_bytes,
                                wl_container_stats *stats);
wl_status wl_decompress_container(wl_ctx *ctx, const char *in_path, const char *out_path,
                                  size_t batch_bytes, wl_container_stats *stats);

/* ---- Parameter sweep (-opt) -----------------------------------------------
 * The reference's -opt (optimizeParameters -> plotAll, optimize.cc:96-133;
 * testParameters optimize_cpu.cc:47-130), on the GPU: for every threshold
 * fraction f = 0.50, 0.51, ... < 0.999 (float steps of 0.01) and bin count
 * b = 100, (int)(b * 1.1), ... <= 2000, log quantization of the cubelet's
 * coefficients with the threshold at sorted |c| index (int)(count * f):
 * size_bytes = the Huffman-coded size as the reference counts it
 * (totalEncodedLengthBytes, huffman.cc:241-251: the code bits of every token,
 * zero-run tokens with their 3 length bits, in 32-bit words) and
 * psnr = 10 log10(255^2 / mse) of the restored 8-bit cubelet against the
 * input (computeErrorRatesAfterDequant, test_compress_common.cc:616-694).
 * 8-bit input only, like the reference (test_compress_cpu.cc:106-114); the
 * transform follows params (steps, wavelet, exact_transform, transform_2d)
 * and compress_zeros selects zero-run tokens.  *n_points receives the number
 * of grid points (1600); points may be NULL to ask for it.  Difference: a
 * threshold whose sorted |c| is exactly 0 is taken as 1e-16, as the
 * compression path does (the reference's sweep would use 0). */
typedef struct {
  float threshold_fraction;
  int bin_count;
  int size_bytes;
  float psnr;
} wl_opt_point;
wl_status wl_optimize(wl_ctx *ctx, const void *data, const int size[3], int data_on_device,
                      const wl_params *params, wl_opt_point *points, int cap, int *n_points);
/* The same on the first uncompressed cubelet of a .cube file (the
 * reference's `test_compress_cpu -opt in out`, which writes no output). */
wl_status wl_optimize_file(wl_ctx *ctx, const char *in_path, const wl_params *params,
                           wl_opt_point *points, int cap, int *n_points);

/* ---- Tile autotuner ------------------------------------------------------
 * No reference counterpart (the reference's GPU transform has fixed block
 * shapes, dwt_gpu.cu).  The column-tile transform runs the rows of each size
 * class -- pass (0 forward x, 1 forward y, 2 forward z, 3 inverse z,
 * 4 inverse y, 5 inverse x), element type of the pass's global side (0 u8,
 * 1 u16, 2 i32, 3 f32; +4 for 8/16-bit input read from page-locked host
 * memory) and row-length class k (rows of 2^(k-1)+1 .. 2^k elements) -- in
 * tiles of 32, 64 or 128 rows worked by four or eight warps: the warps that
 * share 32 rows split every lifting level into warps x 32 / rows segments
 * (a 128-row tile of four warps sweeps each row whole).  wl_autotune times
 * every shape that fits on a synthetic batch of about 2^24 elements per
 * class on ctx's device (rows up to max_len elements, 0 = 512; reps timed
 * launches per candidate, 0 = 5) and keeps the fastest in a process-wide
 * table that every context uses from its next call.  Untuned classes use
 * 128-row tiles for rows of up to 64 elements and 32-row tiles above, four
 * warps.  The shape changes speed only: every shape does the same
 * arithmetic on every element, so results are bit-identical.
 *
 * The table as text (wl_tune_export; *len = bytes without the NUL, buf may be
 * NULL to ask for the length): one line per tuned class,
 * "pass type class rows warps t0 t1 t2 t3 t4 t5" with the measured
 * microseconds per launch of the shapes 32x4, 64x4, 128x4, 32x8, 64x8, 128x8
 * (0 = not measured).  wl_tune_import reads the same lines (the times are
 * optional); wl_tune_reset returns every class to the default. */
wl_status wl_autotune(wl_ctx *ctx, int max_len, int reps);
wl_status wl_tune_export(char *buf, size_t cap, size_t *len);
wl_status wl_tune_import(const char *text);
void wl_tune_reset(void);

/* ---- CUDA graphs ---------------------------------------------------------
 * mode 1 (default): a batch whose geometry (count, element types, sizes,
 * pitches, parameters, kind of input memory) repeats the previous call's is
 * captured as a CUDA graph, and every later call with that geometry replays
 * it (up to 4 geometries per context); input addresses and per-call tables
 * reach the graph through page-locked upload buffers, so results are those
 * of the direct launches.  Batches that never repeat (serving) launch
 * directly and pay no capture.  mode 0: always launch directly.
 * wl_graph_stats: {direct segment runs, captures, replays, failed captures};
 * a failed capture turns graphs off for the context and wl_graph_error
 * names the reason. */
wl_status wl_set_graph_mode(wl_ctx *ctx, int mode);

/* Bit-packer slices per 4096-element chunk (no reference counterpart): the
 * Huffman tokens of a chunk are packed by `slices` lanes (1, 2, 4, 8, 16 or
 * 32) that each take a contiguous share.  0 (default): the smallest count
 * that gives the launch at least 16 warps per SM.  The packed bits do not
 * depend on it. */
wl_status wl_set_encode_slices(wl_ctx *ctx, int slices);
wl_status wl_graph_stats(const wl_ctx *ctx, long long out[4]);
const char *wl_graph_error(const wl_ctx *ctx);

/* Threshold selection that allocates nothing.  This entry point has no
 * counterpart in the reference.  It is for callers that may not call
 * cudaMalloc: code running while a stream is being captured (allocation is
 * illegal there), hosts that give the library a fixed memory budget or their
 * own pool, and real-time loops that must not wait on the allocator.
 *
 * coeffs: n transform coefficients in device memory.  out: 5 floats in
 * device memory, written on `stream` (a cudaStream_t; NULL = default
 * stream): threshold (the k-th smallest |c|, k = (int)(fraction * n), 0
 * replaced by 1e-16), smallest and largest coefficient (tracked like the
 * reference, starting from FLT_MAX / FLT_MIN), largest and second largest |c|
 * -- the same values wl_compress_cubelet reports for those coefficients.
 * The call only enqueues work; it does not synchronize.
 *
 * Scratch lives in a static device array of about 272 KB that every GPU that
 * loads this library keeps until the process exits.  n is limited to
 * WL_NOALLOC_MAX_ELEMENTS (larger n returns WL_EINVAL).  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress) for
 * that device, so make the first call on each device before any stream
 * capture.  Every call shares the one array and clears what must start at
 * zero; calls whose work overlaps on the GPU (other streams, other host
 * threads) race and must be serialized by the caller.  The looked-up address
 * is kept for the life of the process: after cudaDeviceReset on a device the
 * library must be unloaded and loaded again before this entry point is used
 * on that device.  A launch that fails returns WL_ECUDA; an error left pending
 * by earlier, unrelated CUDA work is neither reported nor cleared. */
#define WL_NOALLOC_MAX_ELEMENTS (64LL * 1024 * 1024)
wl_status wl_select_threshold_noalloc(const float *coeffs, long long n,
                                      float fraction, void *stream, float *out);

/* ---- Error metrics (-err) -------------------------------------------------
 * The reference's -err (computeErrorRates / computeErrorRatesAfterDequant,
 * test_compress_common.cc:587-694; ErrorAccumulator,
 * test_compress_common.h:90-160): the compressed cubelet is restored on the
 * device and compared with its original element by element.  Each pair adds
 * (in double) a, a*a, |a-b| and |a-b|^2 with the products and the difference
 * taken in float, a being the original value and b the restored value as the
 * reference converts it: 8-bit clamped to 0..255 and truncated, 32-bit and
 * 16-bit integers (int)(f + 0.5f), float32 (int)f (a quirk of the reference,
 * kept).  max_possible is the PSNR peak: <= 0 means 255 for 8-bit data; other
 * types without a positive maximum get no metrics (count 0 and zeros, as the
 * reference prints "Cannot compute error rates").  The float fields are the
 * reference's getters: average = sum|d| / count, l1 = sum|d|,
 * l2 = sqrt(sum d^2), mse = sum d^2 / count, psnr = 10 log10(max^2 / mse)
 * (0 when mse is 0), relative_error = sum d^2 / sum a^2. */
typedef struct {
  long long count;
  float average_error, l1, l2, mse, psnr, relative_error;
  double sum_value, sum_value_squared, sum_diff, sum_diff_squared;
} wl_error_stats;
wl_status wl_error_metrics(wl_ctx *ctx, const wl_result *compressed, const void *original,
                           int original_dtype, int original_on_device, float max_possible,
                           wl_error_stats *out);
/* The same for files: the first uncompressed cubelet of original_path (its
 * maximum_value field is the PSNR peak) against the first compressed cubelet
 * of compressed_path. */
wl_status wl_error_metrics_file(wl_ctx *ctx, const char *original_path,
                                const char *compressed_path, wl_error_stats *out);

/* Page-locked host memory for inputs and outputs of the host-pointer entry
 * points (copies from it overlap with device work). */
void *wl_host_alloc(size_t bytes);
void wl_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
