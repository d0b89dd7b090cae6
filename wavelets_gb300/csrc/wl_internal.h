// Internal declarations shared by the libwlgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "wlgpu.h"

namespace wl {

__host__ __device__ inline int clz32(unsigned x) {
#ifdef __CUDA_ARCH__
  return __clz(x);
#else
  return __builtin_clz(x);
#endif
}

constexpr int kMaxBins = 4096;          // bins per cubelet (kernel tables)
constexpr int kMaxSymbols = kMaxBins + 1;
constexpr int kChunk = 4096;            // elements per quantize/encode chunk
constexpr int kChunkThreads = 256;
constexpr int kSelectBins = 4096;       // radix-select digit histogram
constexpr int kLloydBins = 4096;        // |coefficient| histogram for Lloyd
constexpr int kCandSlices = 64;        // CTAs per cubelet over its threshold candidates
constexpr int kLutCells = 4096;         // Lloyd bin lookup: cells of the float order key
constexpr int kLutStride = kLutCells + 8;  // per-cubelet table stride (16-byte rows)
constexpr int kQuantGroup = 8;          // chunks per select / quantize / encode CTA
// Bit packer: a chunk's tokens are split into F slices (F a power of two,
// 1..32), one lane each; a CTA of kEncThreads lanes packs kEncThreads / F
// consecutive chunks of one cubelet (four warps: few CTAs, so kernels of
// another stream still find CTA slots on the SMs).  Short slices keep many warps in flight (a lane's tokens are a
// serial chain): measured on a 512-cubelet batch (92 K chunks), the encode
// stage (per-slice bit counts, scans, packer) took 0.79, 0.76, 0.60, 0.52,
// 0.50 and 0.52 ms for F = 1, 2, 4, 8, 16, 32.
// F = 16 unless the launch would then have fewer lanes than one full wave of
// a 152-SM GB300 (2048 per SM); small batches take 32.
constexpr int kEncThreads = 128;
constexpr long long kEncFullWave = 152LL * 2048;
inline int enc_slices(long long chunks) { return chunks * 16 >= kEncFullWave ? 16 : 32; }
constexpr int kTileBudget = 16384;      // floats of shared memory per DWT tile
constexpr int kMaxAxis = 16384;         // longest padded axis (one row per tile)

// One pass of the separable transform over one cubelet, as seen by the
// row kernel.  Rows are flattened r = b + B*a; row (a,b) of the input starts
// at in + a*inSA + b*inSB (contiguous along c); element (a,b,c) of the
// output goes to out + a*outSA + b*outSB + c*outSC.
// A Huffman token: symbol (bin, or binCount = the zero-run key) in bits 0-12,
// the zero-run length code v (run of 2^(v+3)) in bits 13-15.
__host__ __device__ inline uint16_t make_token(int sym, int v) {
  return (uint16_t)(sym | (v << 13));
}

// Tokens of a zero-bin run [s, e) that start inside [w0, w1), in order
// (HuffmanDup::dupCount / Huffman::dupEncodeString, huffman.h:31-57,
// 278-296: greedy runs of 1024, then the largest power of two >= 8 while
// more than 8 remain, then single zero-bin tokens).  Calls f(token).  At
// most 19 tokens start in a window of kChunk elements.
template <class F>
__host__ __device__ inline void run_tokens(long long s, long long e, long long w0,
                                           long long w1, int dupKey, int dupV, F f) {
  const long long L = e - s;
  const long long q = L >> 10;
  long long j0 = 0;
  if (w0 > s) j0 = (w0 - s + 1023) >> 10;
  for (long long j = j0; j < q; j++) {
    const long long pos = s + (j << 10);
    if (pos >= w1) break;
    f(make_token(dupKey, 7));
  }
  long long pos = s + (q << 10);
  int r = (int)(L - (q << 10));
  while (r > 8) {
    int lg = 31 - clz32(r);
    if (pos >= w0 && pos < w1) f(make_token(dupKey, lg - 3));
    pos += 1 << lg;
    r -= 1 << lg;
  }
  long long a = pos > w0 ? pos : w0, z = pos + r < w1 ? pos + r : w1;
  for (long long x = a; x < z; x++) f(make_token(dupV, 0));
}

// Number of tokens of a zero-bin run of length L (the same split as
// run_tokens): runs of 1024, then one token per set bit of the remainder at
// or above 8 -- except that a last 8 left over is coded as 8 single tokens.
__host__ __device__ inline int run_token_count(long long L) {
  const int q = (int)(L >> 10), r = (int)(L & 1023);
  const int hi = r & ~7, lo = r & 7;
#ifdef __CUDA_ARCH__
  int big = __popc(hi >> 4);
#else
  int big = __builtin_popcount(hi >> 4);
#endif
  if (hi & 8) return q + big + (lo > 0 ? 1 + lo : 8);
  return q + big + lo;
}

struct CubeletState;

struct PassDesc {
  const void *in;
  void *out;
  long long inSA, inSB;
  long long inSC;                   // input element stride (column-tile kernel)
  long long outSA, outSB, outSC;
  int L;          // row length (padded)
  int B;          // rows per 'a'
  int rows;       // total rows (A*B)
  int T;          // rows per tile (power of two)
  int tiles;
  int steps;
  int wavelet;    // WL_HAAR / WL_CDF97
  int exact;      // reference float order (filter bank) instead of lifting
  int clampL, clampB, clampA;  // forward load: source sizes (REPEAT padding)
  int cropL, cropB, cropA;     // inverse store: destination sizes (crop)
  int vecLoad;                 // source is page-locked host memory: 16-byte row loads
  // last forward pass of a compression (row-register z pass): also gather the
  // first radix-select digit histogram and the extremes of the values it
  // writes into these (null: no statistics)
  unsigned *selHist;
  CubeletState *selState;
};

// Per-cubelet state written by the kernels and read back by the host.
struct CubeletState {
  // select
  unsigned minOrd, maxOrd;       // order-preserving encodings of min/max
  unsigned absMax, absMax2;      // bits of the two largest |c|
  unsigned prefix;               // radix-select prefix of the threshold bits
  unsigned long long rank;       // remaining rank inside the prefix bucket
  float threshold;
  float minVal, maxVal, maxAbs, maxAbs2;
  // quantizer
  int zeroBin;
  int dupValue;                  // -1 when zero runs are off
  float negScale, negOffset, posScale, posOffset;  // uniform
  // quantizer tables: Lloyd boundary/value counts; log table layout
  int nBounds, nValues;
  int lowBin, highNeg, nPos, nNeg;
  // Huffman
  unsigned long long totalBits;
  long long wordsBase;           // word offset of this cubelet in the packed output
  long long metaBase;            // int offset of its decode table (+ codebook) in the packed metadata
  int nWords;
  int longest;
  int nDecode;
  int nLeaves;
  int error;                     // nonzero: kernel-side failure code
  int pad_;
  // threshold bucket candidates, compacted into the cubelet's own region of
  // the second coefficient buffer (free once the transform is done)
  unsigned candCount;
  // Lloyd histogram bins: bin = (bits(|c|) - lloydBase) >> lloydShift for
  // threshold < |c| <= the Lloyd range top (bits lloydHiBits)
  unsigned lloydBase, lloydHiBits;
  int lloydShift;
  int lloydDeferred;             // 1: the compaction pass cannot tell; separate pass
  int pad2_;
};

// Everything a kernel needs about one cubelet of a batch.
struct CubeletDev {
  long long n;            // padded element count
  long long coefOff;      // float offset of the coefficients
  long long chunkBase;    // first global chunk index
  long long wordsOff;     // word offset of the Huffman output
  long long wordsCap;     // capacity in words
  int nChunks;
  int binCount;
  int quantAlg;
  int compressZeros;
  float frac;
  int lloydIters;
  int tableOff;           // offset into per-cubelet quantizer tables (floats)
  int nTable;             // entries in the table (log: boundaries; lloyd: boundaries)
  int groupBase;          // first quantize group (kQuantGroup chunks per group)
  int encBase;            // first bit-packer CTA (kEncThreads / F chunks per CTA)
  int selFused;           // 1: the last transform pass gathered the first select
                          // digit and the extremes (no stand-alone first pass)
};

// Device workspace for one batch.
struct DevBatch {
  int n;                          // cubelets
  CubeletDev *cub;                // [n]
  CubeletState *state;            // [n]
  float *coef;                    // coefficients (ping)
  float *coef2;                   // second buffer (pong)
  uint16_t *tok;                  // Huffman tokens, one slot of kChunk per chunk
  int *chunkTok;                  // tokens stored per chunk by quantize
  int2 *chunkSpan;                // per chunk: first token slot, token count
                                  // (with the zero-run tokens at its edges)
  unsigned *selHist;              // [n][kSelectBins]
  float *lloydHist;               // [n][kLloydBins][2] (count, sum)
  float *qtable;                  // quantizer tables
  uint16_t *qlut;                 // [n][kLutStride] Lloyd boundaries below each key cell
  float *dqtable;                 // dequant values [n][binCount]
  unsigned long long *hist;       // [n][kMaxSymbols] Huffman counts
  int4 *chunkRun;                 // per chunk: lead, trail, allZero, len
  long long *chunkRunCtx;         // per chunk: start of incoming run, end of outgoing run (2 each)
  unsigned long long *chunkBits;  // per chunk bit count / offset
  unsigned long long *codes;      // [n][kMaxSymbols] code bits
  uint8_t *codeLen;               // [n][kMaxSymbols]
  int *decode;                    // [n][4*kMaxSymbols]
  uint32_t *words;                // Huffman output
  long long *chunkPrefix;         // [n+1] chunk prefix (== cub[i].chunkBase)
  int *chunkCub;                  // [totalChunks] cubelet of every chunk
  int *groupCub;                  // [totalGroups] cubelet of every quantize group
  long long totalGroups;
  int *encCub;                    // [totalEnc] cubelet of every bit-packer CTA
  long long totalEnc;
  int encF;                       // bit-packer slices per chunk
  unsigned *sliceOff;             // [totalChunks][32] bit offset of each slice in its chunk
  int4 *logHdr;                   // [n] log table layout from the host
  int *meta;                      // packed decode tables and Lloyd codebooks
  long long totalChunks;
};

// launchers (dwt.cu)
// Raise a kernel's dynamic shared-memory limit to at least `bytes`.  The
// limit is per kernel and process-wide; it only ever grows here, so a launch
// on one host thread cannot be undercut by a smaller setting from another.
void raise_smem_limit(const void *func, int bytes);
template <class F> inline void raise_smem_limit(F *func, int bytes) {
  raise_smem_limit(reinterpret_cast<const void *>(func), bytes);
}

void launch_dwt_pass(const PassDesc *d_passes, const int *d_tilePrefix,
                     int nPasses, int totalTiles, int smemBytes, int inType,
                     int outType, bool inverse, cudaStream_t s);
int dwt_tile_rows(int L, bool exact);
int dwt_smem_bytes(int L, int T, bool exact);
// column-tile passes (dwt_cols.cu): lifting / Haar, rows up to kColsMaxL
constexpr int kColsMaxL = 512;
void launch_dwt_cols(const PassDesc *d_passes, const int *d_tilePrefix, int nPasses, int tiles,
                     int smem, int rows, int warps, int inType, int outType, bool inverse,
                     bool vecLoad,
                     cudaStream_t s);
int dwt_cols_tile_rows(int L);               // default tile height for rows of L
int dwt_cols_smem_bytes(int L, int rows);
bool dwt_cols_rows_fit(int L, int rows);      // rows in {32, 64, 128} and smem fits
// row-register forward passes (dwt_rows.cu): float rows contiguous on both
// sides, L a power of two in 16 .. 256, 1 <= steps <= log2 L
bool dwt_rowreg_fits(int L, int steps);
// rows per block; sel: the last pass, which also gathers the select
// statistics of the values it writes (PassDesc::selHist), several row rounds
// per block
int dwt_rowreg_rows_per_block(int L, bool sel = false);
void launch_dwt_rowreg(const PassDesc *d_passes, const int *d_tilePrefix, int nPasses, int blocks,
                       int L, bool sel, cudaStream_t s);
// the same with the rows read from any element type (REPEAT clamp) and
// stored through a shared-memory tile to an output where consecutive rows
// are neighbours (forward x and y passes)
// the inverse of the in-place pass (the first inverse pass, z)
void launch_dwt_rowreg_inv(const PassDesc *d_passes, const int *d_tilePrefix, int nPasses,
                           int blocks, int L, cudaStream_t s);
int dwt_rowreg_t_rows_per_block(int L);
// inverse y and x passes (rows strided in the input, neighbouring rows
// neighbours in memory): rows through a shared-memory tile of
// dwt_rowreg_t_rows_per_block(L) rows, out to outType (the x pass: rows
// contiguous in the output, cropped) or back through the tile (the y pass)
void launch_dwt_rowreg_inv_t(const PassDesc *d_passes, const int *d_tilePrefix, int nPasses,
                             int blocks, int L, int outType, cudaStream_t s);
void launch_dwt_rowreg_t(const PassDesc *d_passes, const int *d_tilePrefix, int nPasses,
                         int blocks, int L, int inType, cudaStream_t s);

// ---- column-tile heights per size class (tune.cpp) ----
enum TuneKind { kTuneFwdX, kTuneFwdY, kTuneFwdZ, kTuneInvZ, kTuneInvY, kTuneInvX, kTuneKinds };
int tune_type_index(int dtype, bool vec);
// tile shape (rows, warps) for rows of up to L elements: the tuned entry,
// else the default
struct TileShape {
  int rows, warps;
};
constexpr int kTileShapes = 6;  // candidates: rows 32/64/128 x warps 4/8
constexpr TileShape kTileShape[kTileShapes] = {{32, 4}, {64, 4}, {128, 4},
                                               {32, 8}, {64, 8}, {128, 8}};
TileShape tuned_cols_shape(int kind, int typeIdx, int L);
void set_tuned_cols_shape(int kind, int typeIdx, int cls, TileShape t,
                          const float us[kTileShapes]);
unsigned tune_version();  // changes whenever the table does

// launchers (select.cu)
// per-cubelet select state (extremes from FLT_MAX / FLT_MIN); runs before the
// transform, whose last pass may gather the first digit
void launch_select_init(DevBatch &b, cudaStream_t s);
// pass0: run the stand-alone first digit pass for the cubelets whose last
// transform pass did not gather it (CubeletDev::selFused == 0)
void launch_select(DevBatch &b, const float *coef, bool pass0, cudaStream_t s);

// launchers (quant.cu)
void launch_quant_params(DevBatch &b, cudaStream_t s);
void launch_lloyd(DevBatch &b, const float *coef, int maxBins, cudaStream_t s);
// sum of squared differences of two u8 arrays into *out (opt.cu)
void launch_sq_err_u8(const uint8_t *a, const uint8_t *b, long long n, unsigned long long *out,
                      cudaStream_t s);
void launch_quantize(DevBatch &b, const float *coef, int maxTable, int maxSymbols,
                     cudaStream_t s);
void launch_runs(DevBatch &b, cudaStream_t s);

// error metrics (errors.cu): per-CTA double sums {a, a*a, |d|, d*d} of the
// original (dtype) against the restored floats, blocks = err_sums_blocks(n)
int err_sums_blocks(long long n);
void launch_err_sums(const void *orig, int dtype, const float *rest, long long n, double *part,
                     int blocks, cudaStream_t s);

// launchers (huffman.cu)
void launch_huffman_build(DevBatch &b, int maxSymbols, cudaStream_t s);
void launch_encode(DevBatch &b, int maxSymbols, cudaStream_t s);
void launch_pack_meta(DevBatch &b, cudaStream_t s);

// GPU Huffman decoding (decode.cu)
size_t decode_workspace_bytes(long long nWords);
// batched decoding (decode.cu)
struct DecodeItem {
  const uint32_t *words;  // device
  long long nWords;
  const int *table;       // device
  int nTable;
  int dupKey, dupValue, binCount;
  long long n;            // elements
  int *out;               // device bins
  // instead of bins: the dequantized values dq[bin] (binCount entries)
  float *fout = nullptr;
  const float *dq = nullptr;
};
inline long long decode_subsequences(long long nWords) {
  const long long k = (nWords * 32 + 1023) / 1024;
  return k > 0 ? k : 1;
}
size_t decode_batch_workspace_bytes(int n, long long totalSub);
// n floats at out set to v, for many ranges in one launch (blocks of
// kFillBlock elements; blockBase = the range's first block)
constexpr int kFillBlock = 4096;
struct FillItem {
  float *out;  // 16-byte aligned
  long long n;
  float v;
  long long blockBase;
};
void launch_fill_batch(const FillItem *items, int nItems, long long totalBlocks, cudaStream_t s);
int decode_streams(const DecodeItem *items, int n, void *ws, int *hostFlags, long long *hostTotals,
                   cudaStream_t s);
int decode_stream(const uint32_t *words, long long nWords, const int *table, int nTable,
                  int dupKey, int dupValue, int binCount, long long n, int *out, void *ws,
                  int *hostFlags, cudaStream_t s);
void fill_value(int *out, long long n, int v, cudaStream_t s);

// host-side exact log-quantizer tables (quant_host.cpp)
struct LogTable {
  std::vector<float> bounds;   // see quant_host.cpp for the layout
  int lowBin, highNeg, nPos, nNeg;
  float negScale, negOffset, posScale, posOffset;
};
void log_quant_table(int binCount, float threshold, float maxVal, LogTable &t);
void dequant_values(int quantAlg, int binCount, float threshold, float maxVal,
                    const float *codebookValues, float *out);

}  // namespace wl
