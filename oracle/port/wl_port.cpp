// Test oracle: CPU restatement of the reference compression path.
//
// TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); the
// product library never links it.  Every routine restates the reference's
// algorithm with the same float operation order (compile with
// -ffp-contract=off), so results are bit-identical to the reference's
// test_compress_cpu; tests/golden pins this against the reference itself.
#include "wl_port.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "wavelet_compress.pb.h"  // oracle/shim: proto2 messages

namespace {

// ---------------------------------------------------------------- filters
// 9/7 analysis and synthesis taps as the reference stores them: double
// literals rounded to float (dwt_cpu.cc:15-43).
const float kLo[5] = {(float).85269867900940, (float).377402855612650,
                      (float)-.110624404418420, (float)-.02384946501938,
                      (float).037828455506995};
const float kHi[4] = {(float)-.788485616405660, (float).418092273222210,
                      (float).040689417609558, (float)-.064538882628938};
const float kSynLo[4] = {(float).788485616405660, (float).377402855612650,
                         (float)-.040689417609558, (float)-.02384946501938};
const float kSynHi[5] = {(float)-.85269867900940, (float).418092273222210,
                         (float).110624404418420, (float)-.064538882628938,
                         (float)-.037828455506995};
const float kInvSqrt2 = 0.70710678118654752440f;  // dwt_cpu.cc:11

// Whole-sample mirror index with repeated folding (dwt_cpu.h:162-176).
inline int mirror(int i, int n) {
  if (i < 0) i = -i;
  while (i >= n) {
    i = n * 2 - i - 2;
    if (i < 0) i = -i;
  }
  return i;
}

// One row, `steps` CDF9/7 analysis levels (dwt_cpu.cc:682-739).
void cdf97_row(float *data, int len, int steps, float *tmp) {
  int n = len;
  for (int s = 0; s < steps; s++, n /= 2) {
    int lo = 0, hi = n / 2;
    for (int i = 0; i < n; i += 2) {
      float sum = kLo[0] * data[i];
      for (int k = 1; k <= 4; k++)
        sum += kLo[k] * (data[mirror(i + k, n)] + data[mirror(i - k, n)]);
      tmp[lo++] = sum;
      int j = i + 1;
      sum = kHi[0] * data[j];
      for (int k = 1; k <= 3; k++)
        sum += kHi[k] * (data[mirror(j + k, n)] + data[mirror(j - k, n)]);
      tmp[hi++] = sum;
    }
    memcpy(data, tmp, sizeof(float) * n);
  }
}

// One row, `steps` CDF9/7 synthesis levels (dwt_cpu.cc:756-799).
void cdf97_inv_row(float *data, int len, int steps, float *tmp) {
  int n = len >> (steps - 1);
  for (int s = 0; s < steps; s++, n *= 2) {
    int half = n >> 1;
    for (int j = 0; j < half; j++) {
      tmp[2 * j] = data[j];
      tmp[2 * j + 1] = data[half + j];
    }
    for (int i = 0; i < n; i += 2) {
      data[i] = tmp[i] * kSynLo[0];
      for (int k = 1; k <= 3; k++)
        data[i] += (tmp[mirror(i + k, n)] + tmp[mirror(i - k, n)]) * kSynLo[k];
      int j = i + 1;
      data[j] = tmp[j] * kSynHi[0];
      for (int k = 1; k <= 4; k++)
        data[j] += (tmp[mirror(j + k, n)] + tmp[mirror(j - k, n)]) * kSynHi[k];
    }
  }
}

// Haar analysis (dwt_cpu.cc:139-170).
void haar_row(float *data, int len, int steps, float *tmp) {
  unsigned n = (unsigned)len;
  while (n > 1 && steps > 0) {
    int half = n >> 1;
    steps--;
    for (int i = 0; i < half; i++) {
      tmp[half + i] = (data[2 * i] - data[2 * i + 1]) * kInvSqrt2;
      tmp[i] = (data[2 * i] + data[2 * i + 1]) * kInvSqrt2;
    }
    memcpy(data, tmp, sizeof(float) * n);
    n = half;
  }
}

// Haar synthesis (dwt_cpu.cc:174-203).
void haar_inv_row(float *data, int len, int steps, float *tmp) {
  int n = len >> (steps - 1);
  while (n <= len) {
    int half = n >> 1;
    for (int i = 0; i < half; i++) {
      tmp[2 * i] = kInvSqrt2 * (data[i] + data[half + i]);
      tmp[2 * i + 1] = kInvSqrt2 * (data[i] - data[half + i]);
    }
    memcpy(data, tmp, sizeof(float) * n);
    n <<= 1;
  }
}

// Apply a row routine to every x-row of a W*H*D cube (CubeNum::visitRows,
// wavelet.h:604-611).
template <class F>
void each_row(float *v, int W, int H, int D, int steps, F f) {
  if (steps <= 0) return;
  std::vector<float> tmp(W);
  for (long r = 0; r < (long)H * D; r++) f(v + r * (long)W, W, steps, tmp.data());
}

// 2-D transpose of a width x height row-major matrix (transpose2dInternal,
// wavelet.h:650-692; data movement only).
void transpose2d(const float *src, float *dst, long width, long height) {
  for (long y = 0; y < height; y++)
    for (long x = 0; x < width; x++) dst[x * height + y] = src[y * width + x];
}

// ---------------------------------------------------------------- quantizers
// QuantUniform (quant.h:189-293).
struct QUniform {
  int binCount;
  float threshold, maxVal, negOffset, posOffset, negScale, negInvScale,
      posScale, posInvScale;
  void init(int b, float t, float m) {
    binCount = b; threshold = t; maxVal = m;
    int negBinCount = (binCount - 1) / 2;
    negScale = (negBinCount - 1) / (maxVal - threshold);
    int posBinCount = binCount / 2;
    posScale = (posBinCount - 1) / (maxVal - threshold);
    negInvScale = negScale == 0 ? 0 : 1 / negScale;
    posInvScale = posScale == 0 ? 0 : 1 / posScale;
    negOffset = 1 - threshold * negScale;
    posOffset = 1 - threshold * posScale;
  }
  int quant(float x) const {
    int zeroBin = (binCount - 1) >> 1;
    if (x < 0) {
      if (x >= -threshold) return zeroBin;
      x = x * negScale - negOffset;
      int bin = (int)x + zeroBin;
      return bin < 0 ? 0 : bin;
    }
    if (x <= threshold) return zeroBin;
    x = x * posScale + posOffset + zeroBin;
    if (x > binCount - 1) return binCount - 1;
    return (int)x;
  }
  float dequant(int x) const {
    int zeroBin = (binCount - 1) >> 1;
    if (x < zeroBin) return (x - 0.5f + negOffset - zeroBin) * negInvScale;
    if (x > zeroBin) return (x + 0.5f - posOffset - zeroBin) * posInvScale;
    return 0;
  }
};

// QuantLog (quant.h:326-439).
struct QLog {
  int binCount;
  float threshold, negScale, negInvScale, negOffset, posScale, posInvScale,
      posOffset;
  void init(int b, float t, float maxVal) {
    binCount = b; threshold = t;
    int negBinCount = (binCount - 1) / 2;
    negScale = (negBinCount - 1) / logf(maxVal / threshold);
    negInvScale = 1 / negScale;
    negOffset = 1 - negScale * logf(threshold);
    int posBinCount = binCount / 2;
    posScale = (posBinCount - 1) / logf(maxVal / threshold);
    posInvScale = 1 / posScale;
    posOffset = 1 - posScale * logf(threshold);
  }
  int quant(float x) const {
    int zeroBin = (binCount - 1) >> 1;
    if (x < 0) {
      x = -x;
      if (x <= threshold) return zeroBin;
      x = zeroBin - negScale * logf(x) - negOffset;
      if (x < 0) return 0;
      return (int)(x + 0.5f);
    }
    if (x <= threshold) return zeroBin;
    x = zeroBin + posScale * logf(x) + posOffset;
    if (x >= binCount) return binCount - 1;
    return (int)(x + 0.5f);
  }
  float dequant(int x) const {
    int zeroBin = (binCount - 1) >> 1;
    float sign, invScale, offset;
    if (x < zeroBin) { sign = -1; offset = negOffset; invScale = negInvScale; }
    else { sign = 1; offset = posOffset; invScale = posInvScale; }
    if (x == zeroBin) return 0;
    return sign * expf((sign * (x - zeroBin) - offset) * invScale);
  }
};

// QuantCodebook::quant (quant.h:515-526): lower_bound with the special case
// for values at or above the last boundary.
int codebook_quant(float x, const std::vector<float> &bnd) {
  if (x >= bnd.back()) return (int)bnd.size();
  return (int)(std::lower_bound(bnd.begin(), bnd.end(), x) - bnd.begin());
}

// Lloyd's algorithm (Octave/LloydsAlgorithm/src/c++/lloyds.cpp:30-141).
void lloyd(const float *points, unsigned psize, float *codebook, unsigned csize,
           float *partition, float stop_criteria) {
  std::vector<float> sum(csize, 0.0f);
  std::vector<unsigned> count(csize, 0);
  for (unsigned i = 0; i + 1 < csize; i++)
    partition[i] = (codebook[i] + codebook[i + 1]) / 2;
  float pmax = points[0], pmin = points[0];
  float dist = 0, reldist;
  for (unsigned i = 0; i < psize; i++) {
    float p = points[i];
    pmax = (p > pmax) ? p : pmax;
    pmin = (p < pmin) ? p : pmin;
    float d = fabsf(p - codebook[0]), mn = d;
    unsigned idx = 0;
    for (unsigned j = 1; j < csize; j++) {
      d = fabsf(p - codebook[j]);
      if (d < mn) { idx = j; mn = d; }
    }
    sum[idx] += p;
    count[idx]++;
    dist += codebook[idx] - p;
  }
  dist /= psize;
  reldist = fabsf(dist);
  while (reldist > stop_criteria) {
    for (unsigned i = 0; i < csize; i++) {
      if (count[i] != 0) { codebook[i] = sum[i] / count[i]; count[i] = 0; }
      else if (i == 0) codebook[i] = (partition[0] + pmin) / 2;
      else if (i == csize - 1) codebook[i] = (partition[i - 1] + pmax) / 2;
      else codebook[i] = (partition[i - 1] + partition[i]) / 2;
      sum[i] = 0;
    }
    for (unsigned i = 0; i < psize; i++) {
      for (unsigned j = 0; j + 1 < csize; j++) {
        float p = points[i];
        if (p >= codebook[j] && p < codebook[j + 1]) {
          count[j]++;
          sum[j] += p;
          break;
        }
      }
    }
    for (unsigned i = 0; i + 1 < csize; i++) {
      if (count[i] != 0) { partition[i] = sum[i] / count[i]; count[i] = 0; }
      else partition[i] = (codebook[i] + codebook[i + 1]) / 2;
      sum[i] = 0;
    }
    reldist = dist;
    dist = 0;
    for (unsigned i = 0; i < psize; i++) {
      float p = points[i];
      float d = fabsf(p - codebook[0]), mn = d;
      unsigned idx = 0;
      for (unsigned j = 1; j < csize; j++) {
        d = fabsf(p - codebook[j]);
        if (d < mn) { idx = j; mn = d; }
      }
      sum[idx] += p;
      count[idx]++;
      dist += codebook[idx] - p;
    }
    dist /= psize;
    reldist = fabsf(reldist - dist);
  }
}

// computeLloydQuantization (test_compress_cpu.cc:404-459) with
// initialLloydCodebook (test_compress_common.cc:749-779) and
// setBinsFromCodebook (:784-846).
void lloyd_bins(const float *nonzero, int count, int binCount, float minVal,
                float maxVal, float thresholdValue, std::vector<float> &bnd,
                std::vector<float> &vals) {
  int cbs = (binCount - 1) / 2;
  float maxAbsVal = nonzero[count - 2];
  std::vector<float> cb(cbs);
  float logScale = logf(maxAbsVal / thresholdValue) / cbs;
  for (int i = 0; i < cbs; i++) cb[i] = thresholdValue * expf(i * logScale);
  std::vector<float> part(cbs > 1 ? cbs - 1 : 1);
  lloyd(nonzero, count - 1, cb.data(), cbs, part.data(), 10e-7f);

  bnd.clear();
  vals.clear();
  if ((binCount & 1) == 0 && fabsf(minVal) > maxVal) {
    vals.push_back(minVal);
    bnd.push_back((minVal + -cb[cbs - 1]) / 2);
  }
  vals.push_back(-cb[cbs - 1]);
  for (int i = cbs - 2; i >= 0; i--) {
    bnd.push_back((-cb[i] + -cb[i + 1]) / 2);
    vals.push_back(-cb[i]);
  }
  bnd.push_back(-thresholdValue);
  vals.push_back(0);
  bnd.push_back(thresholdValue);
  for (int i = 0; i < cbs - 1; i++) {
    vals.push_back(cb[i]);
    bnd.push_back((cb[i] + cb[i + 1]) / 2);
  }
  vals.push_back(cb[cbs - 1]);
  if ((binCount & 1) == 0 && maxVal >= fabsf(minVal)) {
    vals.push_back(maxVal);
    bnd.push_back((maxVal + cb[cbs - 1]) / 2);
  }
}

// ---------------------------------------------------------------- Huffman
const int kDupMin = 8;  // HuffmanDup::dupMinimumLength (huffman.h:17-27)

// HuffmanDup::dupFindLongest (huffman.h:31-42)
unsigned dup_longest(int length) {
  if (length >= (1 << (7 + 3))) return 7;
  unsigned enc = 0, el = kDupMin;
  while (length >= (int)(el << 1)) { enc++; el <<= 1; }
  return enc;
}

struct HuffTree {
  int S = 0;                       // symbols (bin_count, +1 with the dup key)
  std::vector<int64_t> count;      // per node
  std::vector<int> left, right;    // -1 for leaves
  int root = -1;
  std::vector<int> len;            // per symbol code length
  std::vector<uint64_t> code;      // per symbol, bit d = branch at depth d
  std::vector<int> decode;         // BFS decode table
  int longest = 0;

  // Huffman::computeHuffmanCoding (huffman.cc:42-97): min count first, ties
  // to the larger node index (CompareHuffmanNode, huffman.cc:9-18).
  void build(const std::vector<int64_t> &counts) {
    S = (int)counts.size();
    count.assign(2 * S, 0);
    left.assign(2 * S, -1);
    right.assign(2 * S, -1);
    for (int i = 0; i < S; i++) count[i] = counts[i];
    auto cmp = [this](int a, int b) {
      if (count[a] == count[b]) return a < b;
      return count[a] > count[b];
    };
    std::priority_queue<int, std::vector<int>, decltype(cmp)> q(cmp);
    for (int i = 0; i < S; i++)
      if (counts[i] > 0) q.push(i);
    int next = S;
    while (q.size() > 1) {
      int a = q.top(); q.pop();
      int b = q.top(); q.pop();
      left[next] = a; right[next] = b;
      count[next] = count[a] + count[b];
      q.push(next++);
    }
    root = q.empty() ? -1 : q.top();
    len.assign(S, 0);
    code.assign(S, 0);
    longest = 0;
    if (root >= 0) assign(root, 0, 0);
    // BFS decode table (computeDecodeTable / orderNodes, huffman.cc:177-228)
    decode.clear();
    if (root < 0) return;
    std::vector<int> order{root};
    std::vector<int> id(2 * S, -1);
    for (size_t h = 0; h < order.size(); h++) {
      int nd = order[h];
      id[nd] = (int)h;
      if (left[nd] >= 0) { order.push_back(left[nd]); order.push_back(right[nd]); }
    }
    decode.resize(2 * order.size());
    for (size_t i = 0; i < order.size(); i++) {
      int nd = order[i];
      if (left[nd] < 0) { decode[2 * i] = 0; decode[2 * i + 1] = nd; }
      else { decode[2 * i] = id[left[nd]]; decode[2 * i + 1] = id[right[nd]]; }
    }
  }
  // computeEncodedBits (huffman.cc:147-174): left = 0, right = 1, root first
  void assign(int nd, int depth, uint64_t bits) {
    if (left[nd] < 0) {
      len[nd] = depth; code[nd] = bits;
      if (depth > longest) longest = depth;
      return;
    }
    assign(left[nd], depth + 1, bits);
    assign(right[nd], depth + 1, bits | (depth < 64 ? (1ull << depth) : 0));
  }
};

// LSB-first 32-bit word stream (BitStreamWriter, bit_stream.h:60-162).
struct BitWriter {
  std::vector<uint32_t> words;
  uint64_t acc = 0;
  int nbits = 0;
  void write(uint64_t bits, int n) {  // n <= 32 per call
    if (n <= 0) return;
    if (n < 64) bits &= (1ull << n) - 1;
    acc |= bits << nbits;
    nbits += n;
    while (nbits >= 32) {
      words.push_back((uint32_t)acc);
      acc >>= 32;
      nbits -= 32;
    }
  }
  void write_code(uint64_t code, int n) {
    while (n > 32) { write(code & 0xffffffffu, 32); code >>= 32; n -= 32; }
    write(code, n);
  }
  void flush() {
    if (nbits > 0) { words.push_back((uint32_t)acc); acc = 0; nbits = 0; }
  }
};

// Decomposition of a run of the zero bin into dup tokens and singles
// (HuffmanDup::dupCount huffman.h:46-57, dupEncodeString :278-296).
template <class Tok, class Single>
void run_tokens(int length, Tok tok, Single single) {
  while (length > kDupMin) {
    unsigned e = dup_longest(length);
    length -= 1 << (e + 3);
    tok(e);
  }
  while (length > 0) { single(); length--; }
}

// ---------------------------------------------------------------- .cube IO
const char kHeaderLine[] = "SCU cubelets 1.0\n";

bool write_cube_file(const char *path, const std::vector<CubeletBuffer> &metas,
                     const std::vector<std::string> &datas, bool footer) {
  FILE *f = fopen(path, "wb");
  if (!f) return false;
  char header[64];
  memset(header, 0, sizeof header);
  memcpy(header, kHeaderLine, sizeof(kHeaderLine) - 1);
  fwrite(header, 1, 64, f);
  CubeletIndexBuffer index;
  for (size_t i = 0; i < metas.size(); i++) {
    std::string m = metas[i].encode();
    uint32_t n = (uint32_t)m.size();
    fwrite(&n, 4, 1, f);
    fwrite(m.data(), 1, n, f);
    CubeletBuffer *e = index.add_cubelets();
    *e = metas[i];
    e->set_data_file_offset((uint64_t)ftell(f));
    fwrite(datas[i].data(), 1, datas[i].size(), f);
  }
  if (footer) {
    int32_t eof = -1;
    fwrite(&eof, 4, 1, f);
    std::string idx = index.encode();
    fwrite(idx.data(), 1, idx.size(), f);
    int32_t n = (int32_t)idx.size();
    fwrite(&n, 4, 1, f);
    fwrite("cube", 1, 4, f);
  }
  bool ok = !ferror(f);
  fclose(f);
  return ok;
}

struct ReadCube {
  CubeletBuffer meta;
  std::string data;
};

bool read_cube_file(const char *path, std::vector<ReadCube> &out) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  char header[64];
  if (fread(header, 1, 64, f) != 64 || strcmp(header, kHeaderLine) != 0) {
    fclose(f);
    return false;
  }
  while (true) {
    uint32_t n;
    if (fread(&n, 4, 1, f) != 1 || n == 0xFFFFFFFFu) break;
    std::string m(n, '\0');
    if (fread(&m[0], 1, n, f) != n) break;
    ReadCube rc;
    if (!rc.meta.ParseFromArray(m.data(), (int)n)) break;
    rc.data.resize(rc.meta.byte_count());
    if (rc.meta.byte_count() &&
        fread(&rc.data[0], 1, rc.data.size(), f) != rc.data.size())
      break;
    out.push_back(rc);
  }
  fclose(f);
  return true;
}

int ceil_log2(unsigned x) {  // dwt_cpu.cc:60-78
  if (x == 0) return 0;
  int n = 0;
  unsigned v = x - 1;
  while (v) { n++; v >>= 1; }
  return n;
}

int padded_length(int len, int steps) {  // dwt_padded_length, dwt_cpu.cc:212-219
  int mod = 1 << steps;
  return mod * ((len - 1) / mod + 1);
}

// Everything the encoder produces for one cubelet.
struct Encoded {
  orc_result r;
  std::vector<int> bins;
  std::vector<uint32_t> words;
  std::vector<int> decode;
  std::vector<int64_t> hist;
  std::vector<float> bnd, vals;
};

void huffman_part(Encoded &e, int n, int binCount, int zeroBin);

// Threshold + quantize + Huffman (test_compress_cpu.cc:97-172).
void encode_coeffs(const float *c, int n, float frac, int binCount, int qalg,
                   int compressZeros, Encoded &e) {
  memset(&e.r, 0, sizeof e.r);
  // thresh_cpu(CubeFloat*) (thresh_cpu.cc:80-109): min starts at FLT_MAX and
  // max at FLT_MIN (the smallest positive float), both updated independently.
  std::vector<float> a(n);
  float mn = FLT_MAX, mx = FLT_MIN;
  for (int i = 0; i < n; i++) {
    a[i] = fabsf(c[i]);
    if (c[i] < mn) mn = c[i];
    if (c[i] > mx) mx = c[i];
  }
  std::sort(a.begin(), a.end());
  int k = (int)(frac * n);
  if (k >= n) k = n - 1;  // frac == 1 reads past the array in the reference
  float thr = a[k];
  if (thr == 0) thr = 1e-16;
  int nonzero = n - k - 1;
  float maxAbs = a[n - 1];
  e.r.threshold = thr; e.r.min_value = mn; e.r.max_value = mx;
  e.r.max_abs = maxAbs; e.r.nonzero_count = nonzero;
  e.r.bin_count = binCount; e.r.quant_alg = qalg;

  // quantize (test_compress_cpu.cc:244-295)
  e.bins.resize(n);
  int zeroBin;
  if (qalg == ORC_UNIFORM) {
    QUniform q; q.init(binCount, thr, maxAbs);
    zeroBin = q.quant(0);
    for (int i = 0; i < n; i++) e.bins[i] = q.quant(c[i]);
  } else if (qalg == ORC_LOG) {
    QLog q; q.init(binCount, thr, maxAbs);
    zeroBin = q.quant(0);
    for (int i = 0; i < n; i++) e.bins[i] = q.quant(c[i]);
  } else {
    lloyd_bins(a.data() + n - nonzero, nonzero, binCount, mn, mx, thr, e.bnd, e.vals);
    zeroBin = codebook_quant(0, e.bnd);
    for (int i = 0; i < n; i++) e.bins[i] = codebook_quant(c[i], e.bnd);
  }
  if (!compressZeros) zeroBin = -1;
  e.r.zero_bin = zeroBin;
  e.r.n_boundaries = (int)e.bnd.size();
  e.r.n_values = (int)e.vals.size();
  huffman_part(e, n, binCount, zeroBin);
}

// huffScan + tree + encodeToStream on e.bins (test_compress_common.cc:953-1022)
void huffman_part(Encoded &e, int n, int binCount, int zeroBin) {
  // huffScan (test_compress_common.cc:901-921) with the dup value set when
  // zero runs are on (initHuffman :960-994)
  int dupValue = (zeroBin >= 0 && zeroBin < binCount) ? zeroBin : -1;
  std::vector<int64_t> counts(binCount, 0);
  int64_t dupCount = 0;
  int run = 0;
  auto flush_run = [&]() {
    run_tokens(run, [&](unsigned) { dupCount++; }, [&]() { counts[dupValue]++; });
    run = 0;
  };
  for (int i = 0; i < n; i++) {
    if (e.bins[i] == dupValue) { run++; continue; }
    if (run > 0) flush_run();
    counts[e.bins[i]]++;
  }
  if (run > 0) flush_run();
  std::vector<int64_t> sym = counts;
  if (dupValue >= 0) sym.push_back(dupCount);
  e.hist = counts;
  e.hist.push_back(dupValue >= 0 ? dupCount : 0);

  HuffTree t;
  t.build(sym);
  e.decode = t.decode;
  e.r.longest_code = t.longest;

  // encodeToStream (huffman.h:242-265)
  BitWriter w;
  const int dupKey = binCount;
  for (int i = 0; i < n; i++) {
    int v = e.bins[i];
    if (v == dupValue) {
      int L = 1;
      while (i + L < n && e.bins[i + L] == dupValue) L++;
      run_tokens(L,
                 [&](unsigned enc) {
                   w.write_code(t.code[dupKey], t.len[dupKey]);
                   w.write(enc, 3);
                 },
                 [&]() { w.write_code(t.code[dupValue], t.len[dupValue]); });
      i += L - 1;
    } else {
      w.write_code(t.code[v], t.len[v]);
    }
  }
  w.flush();
  e.words = w.words;
  e.r.n_words = (int)w.words.size();
  e.r.n_decode = (int)e.decode.size();
  e.r.dup_key = dupValue >= 0 ? dupKey : -1;
  e.r.dup_value = dupValue;
}

// CubeletBuffer + CompressionParametersBuffer for a compressed cubelet,
// as Cube::copyToCubeletBuffer fills them (wavelet.cc:283-343).
CubeletBuffer compressed_meta(const Encoded &e, int Xr, int Yr, int Zr,
                              int ox, int oy, int oz, int odt, int sx, int sy,
                              int sz, int wavelet, float frac, bool two_d) {
  CubeletBuffer m;
  m.set_width(Xr); m.set_height(Yr); m.set_depth(Zr);
  m.set_x_offset(0); m.set_y_offset(0); m.set_z_offset(0);
  m.set_data_type(CubeletBuffer_DataType_INT32);
  m.set_compression_algorithm(CubeletBuffer_CompressionAlgorithm_WAVELET);
  m.set_byte_count((uint32_t)(e.words.size() * 4));
  CompressionParametersBuffer *p = m.mutable_compression_parameters();
  p->set_original_width(ox); p->set_original_height(oy); p->set_original_depth(oz);
  p->set_original_data_type((CubeletBuffer_DataType)odt);
  p->set_wavelet_transform_steps_x(sx);
  p->set_wavelet_transform_steps_y(sy);
  p->set_wavelet_transform_steps_z(sz);
  p->set_wavelet_algorithm((CompressionParametersBuffer_WaveletAlgorithm)wavelet);
  p->set_transform_2d(two_d);
  p->set_threshold_fraction(frac);
  p->set_threshold_value(e.r.threshold);
  p->set_quant_bin_count(e.r.bin_count);
  int q = e.r.quant_alg;
  p->set_quantization_algorithm(
      q == ORC_UNIFORM ? CompressionParametersBuffer_QuantizationAlgorithm_UNIFORM
      : q == ORC_LOG   ? CompressionParametersBuffer_QuantizationAlgorithm_LOG
                       : CompressionParametersBuffer_QuantizationAlgorithm_LLOYD);
  if (q == ORC_UNIFORM || q == ORC_LOG) {
    p->set_quant_max_value(e.r.max_abs);
  } else {
    for (float b : e.bnd) p->add_quant_bin_boundaries(b);
    for (float v : e.vals) p->add_quant_bin_values(v);
  }
  for (int d : e.decode) p->add_huffman_decode_table(d);
  if (e.r.dup_value >= 0) p->set_huffman_dup_value(e.r.dup_value);
  if (e.r.dup_key >= 0) p->set_huffman_dup_key(e.r.dup_key);
  return m;
}

// Read + pad a raw volume into floats (readData, translateCubeDataToFloat
// and padData: test_compress_common.cc:269-488).
template <class T>
void load_padded(const T *src, int X, int Y, int Z, int Xp, int Yp, int Zp,
                 std::vector<float> &v) {
  v.assign((size_t)Xp * Yp * Zp, 0.0f);
  for (int z = 0; z < Zp; z++)
    for (int y = 0; y < Yp; y++) {
      int zs = z < Z ? z : Z - 1, ys = y < Y ? y : Y - 1;
      const T *row = src + ((size_t)zs * Y + ys) * X;
      float *dst = v.data() + ((size_t)z * Yp + y) * Xp;
      for (int x = 0; x < Xp; x++) dst[x] = (float)row[x < X ? x : X - 1];
    }
}

void forward3d(std::vector<float> &v, int X, int Y, int Z, int sx, int sy,
               int sz, int wavelet) {
  if (sx == 0 && sy == 0 && sz == 0) return;
  auto row = [wavelet](float *d, int len, int s, float *t) {
    if (wavelet == ORC_HAAR) haar_row(d, len, s, t); else cdf97_row(d, len, s, t);
  };
  std::vector<float> t(v.size());
  each_row(v.data(), X, Y, Z, sx, row);
  transpose2d(v.data(), t.data(), X, (long)Y * Z);  // xyz -> yzx
  v.swap(t);
  each_row(v.data(), Y, Z, X, sy, row);
  transpose2d(v.data(), t.data(), Y, (long)Z * X);  // yzx -> zxy
  v.swap(t);
  each_row(v.data(), Z, X, Y, sz, row);
}

void inverse3d(std::vector<float> &v, int X, int Y, int Z, int sx, int sy,
               int sz, int wavelet) {
  if (sx == 0 && sy == 0 && sz == 0) return;
  auto row = [wavelet](float *d, int len, int s, float *t) {
    if (wavelet == ORC_HAAR) haar_inv_row(d, len, s, t); else cdf97_inv_row(d, len, s, t);
  };
  std::vector<float> t(v.size());
  each_row(v.data(), Z, X, Y, sz, row);
  transpose2d(v.data(), t.data(), (long)Z * X, Y);  // zxy -> yzx
  v.swap(t);
  each_row(v.data(), Y, Z, X, sy, row);
  transpose2d(v.data(), t.data(), (long)Y * Z, X);  // yzx -> xyz
  v.swap(t);
  each_row(v.data(), X, Y, Z, sx, row);
}

// 2-D transform of every z layer of a W x H x D cube (-2d; waveletTransform
// test_compress_common.cc:519-541 -> cdf97_2d / haar_2d, dwt_cpu.cc:811-864 and
// :495-547): step counts below 1 or above the maximum become the maximum
// (ceilLog2 of the padded length); a layer whose padded size does not suit
// those counts is left untransformed (the reference reports it and returns).
// Rows along x, a transpose, rows along y, a transpose back: the layout
// stays x fastest.
void transform2d(std::vector<float> &v, int W, int H, int D, int sx, int sy, int wavelet,
                 bool inverse) {
  if (sx < 1 || sx > ceil_log2(W)) sx = ceil_log2(W);
  if (sy < 1 || sy > ceil_log2(H)) sy = ceil_log2(H);
  if ((W & ((1 << sx) - 1)) || (H & ((1 << sy) - 1))) return;
  auto fwd = [wavelet](float *d, int len, int s, float *t) {
    if (wavelet == ORC_HAAR) haar_row(d, len, s, t); else cdf97_row(d, len, s, t);
  };
  auto inv = [wavelet](float *d, int len, int s, float *t) {
    if (wavelet == ORC_HAAR) haar_inv_row(d, len, s, t); else cdf97_inv_row(d, len, s, t);
  };
  std::vector<float> t((size_t)W * H);
  for (int z = 0; z < D; z++) {
    float *layer = v.data() + (size_t)z * W * H;
    if (!inverse) {
      each_row(layer, W, H, 1, sx, fwd);
      transpose2d(layer, t.data(), W, H);  // [y][x] -> [x][y]
      each_row(t.data(), H, W, 1, sy, fwd);
      transpose2d(t.data(), layer, H, W);  // back to [y][x]
    } else {
      transpose2d(layer, t.data(), W, H);
      each_row(t.data(), H, W, 1, sy, inv);
      transpose2d(t.data(), layer, H, W);
      each_row(layer, W, H, 1, sx, inv);
    }
  }
}

int compress_common(const void *data, int dtype, int X, int Y, int Z, int sx,
                    int sy, int sz, int wavelet, float frac, int binCount,
                    int qalg, int compressZeros, const char *out_path,
                    orc_result *res, bool two_d = false) {
  // setWaveletSteps (test_compress_common.cc:362-374)
  int mx = ceil_log2(X), my = ceil_log2(Y), mz = ceil_log2(Z);
  if (sx < 0 || sx > mx) sx = mx;
  if (sy < 0 || sy > my) sy = my;
  if (sz < 0 || sz > mz) sz = mz;
  int Xp = padded_length(X, sx), Yp = padded_length(Y, sy), Zp = padded_length(Z, sz);
  std::vector<float> v;
  if (dtype == ORC_UINT8) load_padded((const uint8_t *)data, X, Y, Z, Xp, Yp, Zp, v);
  else if (dtype == ORC_INT32) load_padded((const int32_t *)data, X, Y, Z, Xp, Yp, Zp, v);
  else load_padded((const float *)data, X, Y, Z, Xp, Yp, Zp, v);
  const bool any = !(sx == 0 && sy == 0 && sz == 0);
  if (!two_d) forward3d(v, Xp, Yp, Zp, sx, sy, sz, wavelet);
  else if (any) transform2d(v, Xp, Yp, Zp, sx, sy, wavelet, false);
  Encoded e;
  encode_coeffs(v.data(), (int)v.size(), frac, binCount, qalg, compressZeros, e);
  if (res) *res = e.r;
  if (!out_path) return 0;
  bool rotated = any && !two_d;
  CubeletBuffer m = compressed_meta(e, rotated ? Zp : Xp, rotated ? Xp : Yp,
                                    rotated ? Yp : Zp, X, Y, Z, dtype, sx, sy,
                                    sz, wavelet, frac, two_d);
  std::string words((const char *)e.words.data(), e.words.size() * 4);
  return write_cube_file(out_path, {m}, {words}, false) ? 0 : 1;
}

// A compressed cubelet's dequantized, inverse-transformed floats in the
// padded x-fastest layout (Xp x Yp x Zp): readQuantData + dequantize +
// inverse waveletTransform (test_compress_cpu.cc:187-220).
struct Restored {
  std::vector<float> v;
  int Xp = 0, Yp = 0, Zp = 0;
  int ox = 0, oy = 0, oz = 0, odt = ORC_FLOAT32;
};

int restore_floats(const ReadCube *rc, Restored &R) {
  const CompressionParametersBuffer &p = rc->meta.compression_parameters();
  int W = rc->meta.width(), H = rc->meta.height(), D = rc->meta.depth();
  long n = (long)W * H * D;
  std::vector<int> table(p.huffman_decode_table_size());
  for (size_t i = 0; i < table.size(); i++) table[i] = p.huffman_decode_table((int)i);
  std::vector<int> bins(n);
  int dk = p.has_huffman_dup_key() ? p.huffman_dup_key() : -1;
  int dv = p.has_huffman_dup_value() ? p.huffman_dup_value() : -1;
  int got = orc_huffman_decode((const uint32_t *)rc->data.data(),
                               (int)(rc->data.size() / 4), table.data(),
                               (int)table.size(), dk, dv, bins.data(), (int)n);
  if (got != n) return 1;
  int qalg = p.quantization_algorithm() == CompressionParametersBuffer_QuantizationAlgorithm_UNIFORM ? ORC_UNIFORM
             : p.quantization_algorithm() == CompressionParametersBuffer_QuantizationAlgorithm_LOG ? ORC_LOG
                                                                                                : ORC_LLOYD;
  std::vector<float> vals(p.quant_bin_values_size());
  for (size_t i = 0; i < vals.size(); i++) vals[i] = p.quant_bin_values((int)i);
  std::vector<float> v(n);
  orc_dequantize(bins.data(), (int)n, qalg, p.quant_bin_count(), p.threshold_value(),
                 p.quant_max_value(), vals.data(), v.data());
  int sx = p.wavelet_transform_steps_x(), sy = p.wavelet_transform_steps_y(),
      sz = p.wavelet_transform_steps_z();
  const bool any = !(sx == 0 && sy == 0 && sz == 0), two_d = p.transform_2d();
  bool rotated = any && !two_d;
  int Xp = rotated ? H : W, Yp = rotated ? D : H, Zp = rotated ? W : D;
  if (!two_d) inverse3d(v, Xp, Yp, Zp, sx, sy, sz, p.wavelet_algorithm());
  else if (any) transform2d(v, Xp, Yp, Zp, sx, sy, p.wavelet_algorithm(), true);
  R.v.swap(v);
  R.Xp = Xp; R.Yp = Yp; R.Zp = Zp;
  R.ox = p.original_width(); R.oy = p.original_height(); R.oz = p.original_depth();
  R.odt = p.has_original_data_type() ? p.original_data_type() : ORC_FLOAT32;
  return 0;
}

const ReadCube *first_compressed(const std::vector<ReadCube> &cubes) {
  for (auto &c : cubes)
    if (c.meta.data_type() == CubeletBuffer_DataType_INT32 &&
        c.meta.compression_algorithm() == CubeletBuffer_CompressionAlgorithm_WAVELET)
      return &c;
  return nullptr;
}

// Decompress the first compressed INT32 cubelet of in_path to out_path
// (decompressFile, test_compress_cpu.cc:187-241).
int decompress_file(const char *in_path, const char *out_path) {
  std::vector<ReadCube> cubes;
  if (!read_cube_file(in_path, cubes)) return 1;
  const ReadCube *rc = first_compressed(cubes);
  if (!rc) return 1;
  Restored R;
  if (restore_floats(rc, R)) return 1;
  const std::vector<float> &v = R.v;
  const int Xp = R.Xp, Yp = R.Yp, ox = R.ox, oy = R.oy, oz = R.oz, odt = R.odt;
  // translateCubeDataToOriginal (test_compress_common.cc:699-746), cropped to
  // the original size when written
  std::string out;
  for (int z = 0; z < oz; z++)
    for (int y = 0; y < oy; y++)
      for (int x = 0; x < ox; x++) {
        float f = v[((size_t)z * Yp + y) * Xp + x];
        if (odt == ORC_UINT8) {
          unsigned char b = f <= 0 ? 0 : (f >= 255 ? 255 : (unsigned char)f);
          out.push_back((char)b);
        } else if (odt == ORC_INT32) {
          int32_t iv = (int)(f + 0.5f);
          out.append((const char *)&iv, 4);
        } else {
          out.append((const char *)&f, 4);
        }
      }
  CubeletBuffer m;
  m.set_width(ox); m.set_height(oy); m.set_depth(oz);
  m.set_x_offset(0); m.set_y_offset(0); m.set_z_offset(0);
  m.set_data_type((CubeletBuffer_DataType)odt);
  m.set_compression_algorithm(CubeletBuffer_CompressionAlgorithm_NONE);
  m.set_byte_count((uint32_t)out.size());
  return write_cube_file(out_path, {m}, {out}, true) ? 0 : 1;
}

// ErrorAccumulator (test_compress_common.h:90-160): sums in double of float
// values, products and differences.
struct ErrAcc {
  double sumValue = 0, sumValueSquared = 0, sumDiff = 0, sumDiffSquared = 0;
  float maxValue = 0;
  long long count = 0;
  void add(float a, float b) {
    sumValue += a;
    sumValueSquared += a * a;
    float diff = fabsf(a - b);
    sumDiff += diff;
    sumDiffSquared += diff * diff;
    count++;
  }
};

// computeErrorRatesAfterDequant (test_compress_common.cc:616-694): the
// original cubelet against the restored floats, converted the way the
// reference compares each type.  Returns false (nothing accumulated) when no
// maximum possible value is known for a non-8-bit input.
bool error_rates(const ReadCube &orig, const Restored &R, ErrAcc &acc) {
  const int dt = orig.meta.data_type();
  const int maxPossible = orig.meta.has_maximum_value() ? orig.meta.maximum_value() : 0;
  if (dt == ORC_UINT8) acc.maxValue = maxPossible > 0 ? (float)maxPossible : 255.f;
  else if (maxPossible > 0) acc.maxValue = (float)maxPossible;
  else return false;
  const int W = orig.meta.width(), H = orig.meta.height(), D = orig.meta.depth();
  for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++) {
      const float *row = R.v.data() + ((size_t)z * R.Yp + y) * R.Xp;
      const size_t o = ((size_t)z * H + y) * W;
      for (int x = 0; x < W; x++) {
        if (dt == ORC_UINT8) {
          const float f = row[x];
          unsigned char b = f <= 0 ? 0 : (f >= 255 ? 255 : (unsigned char)f);
          acc.add((unsigned char)orig.data[o + x], b);
        } else if (dt == ORC_INT32) {
          int32_t a;
          memcpy(&a, orig.data.data() + 4 * (o + x), 4);
          acc.add((float)a, (float)(int)(row[x] + 0.5f));
        } else {
          float a;
          memcpy(&a, orig.data.data() + 4 * (o + x), 4);
          acc.add(a, (float)(int)row[x]);
        }
      }
    }
  return true;
}

const ReadCube *first_uncompressed(const std::vector<ReadCube> &cubes) {
  for (auto &c : cubes)
    if (c.meta.compression_algorithm() != CubeletBuffer_CompressionAlgorithm_WAVELET) return &c;
  return nullptr;
}

// The getters of ErrorAccumulator: average, L1, L2, MSE, PSNR, relative.
void err_getters(const ErrAcc &e, float g[6]) {
  g[0] = e.count ? (float)(e.sumDiff / e.count) : 0.f;
  g[1] = (float)e.sumDiff;
  g[2] = (float)sqrt(e.sumDiffSquared);
  g[3] = e.count ? (float)(e.sumDiffSquared / e.count) : 0.f;
  const float mse = g[3];
  g[4] = (e.maxValue == 0 || mse == 0) ? 0.f : (float)(10 * log10(e.maxValue * e.maxValue / mse));
  g[5] = e.sumValueSquared == 0 ? 0.f : (float)(e.sumDiffSquared / e.sumValueSquared);
}

int error_metrics_files(const char *orig_path, const char *comp_path, ErrAcc &acc,
                        bool &computed) {
  std::vector<ReadCube> oc, cc;
  if (!read_cube_file(orig_path, oc) || !read_cube_file(comp_path, cc)) return 1;
  const ReadCube *o = first_uncompressed(oc), *c = first_compressed(cc);
  if (!o || !c) return 1;
  Restored R;
  if (restore_floats(c, R)) return 1;
  computed = error_rates(*o, R, acc);
  return 0;
}

}  // namespace

extern "C" {

int orc_error_metrics(const char *orig_path, const char *comp_path, double sums[4],
                      long long *count, float getters[6]) {
  ErrAcc acc;
  bool computed = false;
  if (error_metrics_files(orig_path, comp_path, acc, computed)) return 1;
  sums[0] = acc.sumValue;
  sums[1] = acc.sumValueSquared;
  sums[2] = acc.sumDiff;
  sums[3] = acc.sumDiffSquared;
  *count = acc.count;
  err_getters(acc, getters);
  return 0;
}

int orc_forward(const float *in, int X, int Y, int Z, int sx, int sy, int sz,
                int wavelet, float *out) {
  std::vector<float> v(in, in + (size_t)X * Y * Z);
  forward3d(v, X, Y, Z, sx, sy, sz, wavelet);
  memcpy(out, v.data(), v.size() * sizeof(float));
  return 0;
}

int orc_inverse(const float *in, int X, int Y, int Z, int sx, int sy, int sz,
                int wavelet, float *out) {
  std::vector<float> v(in, in + (size_t)X * Y * Z);
  inverse3d(v, X, Y, Z, sx, sy, sz, wavelet);
  memcpy(out, v.data(), v.size() * sizeof(float));
  return 0;
}

int orc_encode(const float *coeffs, int n, float frac, int binCount, int qalg,
               int compressZeros, orc_result *res, int *bins_out,
               uint32_t *words_out, int words_cap, int *decode_out,
               int decode_cap, int64_t *hist_out, float *bnd_out,
               float *vals_out) {
  Encoded e;
  encode_coeffs(coeffs, n, frac, binCount, qalg, compressZeros, e);
  if (res) *res = e.r;
  if (bins_out) memcpy(bins_out, e.bins.data(), sizeof(int) * n);
  if (hist_out) memcpy(hist_out, e.hist.data(), sizeof(int64_t) * e.hist.size());
  if (bnd_out && !e.bnd.empty()) memcpy(bnd_out, e.bnd.data(), sizeof(float) * e.bnd.size());
  if (vals_out && !e.vals.empty()) memcpy(vals_out, e.vals.data(), sizeof(float) * e.vals.size());
  if (words_out) {
    if ((int)e.words.size() > words_cap) return 1;
    memcpy(words_out, e.words.data(), 4 * e.words.size());
  }
  if (decode_out) {
    if ((int)e.decode.size() > decode_cap) return 1;
    memcpy(decode_out, e.decode.data(), sizeof(int) * e.decode.size());
  }
  return 0;
}

int orc_huffman_encode(const int *bins, int n, int binCount, int zeroBin,
                       orc_result *res, uint32_t *words_out, int words_cap,
                       int *decode_out, int decode_cap, int64_t *hist_out) {
  Encoded e;
  memset(&e.r, 0, sizeof e.r);
  e.bins.assign(bins, bins + n);
  e.r.bin_count = binCount;
  e.r.zero_bin = zeroBin;
  huffman_part(e, n, binCount, zeroBin);
  if (res) *res = e.r;
  if (hist_out) memcpy(hist_out, e.hist.data(), sizeof(int64_t) * e.hist.size());
  if (words_out) {
    if ((int)e.words.size() > words_cap) return 1;
    memcpy(words_out, e.words.data(), 4 * e.words.size());
  }
  if (decode_out) {
    if ((int)e.decode.size() > decode_cap) return 1;
    memcpy(decode_out, e.decode.data(), sizeof(int) * e.decode.size());
  }
  return 0;
}

int orc_quantize(const float *c, int n, int qalg, int binCount, float thr,
                 float maxAbs, const float *bnd, const float *vals,
                 int *out) {
  (void)vals;
  if (qalg == ORC_UNIFORM) {
    QUniform q; q.init(binCount, thr, maxAbs);
    for (int i = 0; i < n; i++) out[i] = q.quant(c[i]);
  } else if (qalg == ORC_LOG) {
    QLog q; q.init(binCount, thr, maxAbs);
    for (int i = 0; i < n; i++) out[i] = q.quant(c[i]);
  } else {
    std::vector<float> b(bnd, bnd + binCount - 1);
    for (int i = 0; i < n; i++) out[i] = codebook_quant(c[i], b);
  }
  return 0;
}

int orc_dequantize(const int *bins, int n, int qalg, int binCount, float thr,
                   float maxAbs, const float *vals, float *out) {
  if (qalg == ORC_UNIFORM) {
    QUniform q; q.init(binCount, thr, maxAbs);
    for (int i = 0; i < n; i++) out[i] = q.dequant(bins[i]);
  } else if (qalg == ORC_LOG) {
    QLog q; q.init(binCount, thr, maxAbs);
    for (int i = 0; i < n; i++) out[i] = q.dequant(bins[i]);
  } else {
    for (int i = 0; i < n; i++) out[i] = vals[bins[i]];
  }
  return 0;
}

int orc_huffman_decode(const uint32_t *words, int n_words, const int *table,
                       int n_table, int dup_key, int dup_value, int *out,
                       int n) {
  // BitStreamReader semantics (bit_stream.h:216-311): reading past the last
  // word yields zero bits; decoding stops when no word is left at the start
  // of a symbol.
  long total = (long)n_words * 32, pos = 0;
  int i = 0;
  auto bit = [&](long p) -> unsigned {
    return p < total ? (words[p >> 5] >> (p & 31)) & 1u : 0u;
  };
  // A one-node tree gives its only symbol a zero-length code
  // (computeEncodedBits, huffman.cc:147-160).  The reference's table walk
  // indexes past such a table (undefined behaviour); decode it as what the
  // encoder wrote: every token is that symbol, and a zero-run token still
  // carries its 3 length bits.
  if (n_table == 2 && table[0] == 0) {
    int v = table[1];
    if (v != dup_key) {
      for (; i < n; i++) out[i] = v;
      return i;
    }
    while (i < n && pos + 3 <= total) {
      unsigned e = bit(pos) | (bit(pos + 1) << 1) | (bit(pos + 2) << 2);
      pos += 3;
      int L = 1 << (e + 3);
      while (L-- > 0 && i < n) out[i++] = dup_value;
    }
    return i;
  }
  while (i < n) {
    if (pos >= total) return i;
    int node = 0;
    while (true) {
      unsigned b = bit(pos++);
      int nx = table[node + b] * 2;
      if (nx < 0 || nx + 1 >= n_table) return i;
      node = nx;
      if (table[node] == 0) break;
    }
    int v = table[node + 1];
    if (v == dup_key) {
      unsigned e = 0;
      for (int k = 0; k < 3; k++) e |= bit(pos++) << k;
      int L = 1 << (e + 3);
      while (L-- > 0 && i < n) out[i++] = dup_value;
    } else {
      out[i++] = v;
    }
  }
  return i;
}

int orc_compress_volume(const void *data, int dtype, int X, int Y, int Z,
                        int sx, int sy, int sz, int wavelet, float frac,
                        int binCount, int qalg, int compressZeros,
                        const char *out_path, orc_result *res) {
  return compress_common(data, dtype, X, Y, Z, sx, sy, sz, wavelet, frac,
                         binCount, qalg, compressZeros, out_path, res);
}

// Command line with the reference's flags (parseOptions,
// test_compress_common.cc:73-192): -d -steps -thresh -qcount -wave -qalg
// -noz -2d -q (other reference flags are accepted and ignored).
int orc_main(int argc, const char **argv) {
  bool decompress = false, zeros = true, two_d = false, errors = false;
  int sx = -1, sy = -1, sz = -1, bins = 256, wave = ORC_CDF97, qalg = ORC_LOG;
  float frac = 0.5f;
  int i = 1;
  for (; i < argc && argv[i][0] == '-'; i++) {
    std::string a = argv[i];
    if (a == "-d") decompress = true;
    else if (a == "-noz") zeros = false;
    else if (a == "-2d") two_d = true;
    else if (a == "-err") errors = true;
    else if (a == "-q" || a == "-v" || a == "-pb" || a == "-enc") {}
    else if (i + 1 < argc && a == "-steps") {
      int x = 1, y = 1, z = 1;
      int k = sscanf(argv[++i], "%d,%d,%d", &x, &y, &z);
      if (k == 1) { sx = sy = sz = x; }
      else if (k == 2) { sx = x; sy = y; sz = 0; }
      else if (k == 3) { sx = x; sy = y; sz = z; }
      else return 1;
    } else if (i + 1 < argc && a == "-thresh") {
      if (sscanf(argv[++i], "%f", &frac) != 1 || frac < 0 || frac > 1) return 1;
    } else if (i + 1 < argc && a == "-qcount") {
      if (sscanf(argv[++i], "%d", &bins) != 1 || bins < 1) return 1;
    } else if (i + 1 < argc && a == "-wave") {
      std::string w = argv[++i];
      if (w == "haar") wave = ORC_HAAR; else if (w == "cdf97") wave = ORC_CDF97; else return 1;
    } else if (i + 1 < argc && a == "-qalg") {
      std::string q = argv[++i];
      if (q == "uniform") qalg = ORC_UNIFORM;
      else if (q == "log") qalg = ORC_LOG;
      else if (q == "lloyd") qalg = ORC_LLOYD;
      else return 1;
    } else if (i + 1 < argc && (a == "-bq" || a == "-aq")) {
      i++;
    } else {
      return 1;
    }
  }
  if (argc - i != 2) return 1;
  const char *in = argv[i], *out = argv[i + 1];
  if (decompress) return decompress_file(in, out);
  std::vector<ReadCube> cubes;
  if (!read_cube_file(in, cubes)) return 1;
  for (auto &c : cubes) {
    if (c.meta.compression_algorithm() == CubeletBuffer_CompressionAlgorithm_WAVELET) continue;
    int dt = c.meta.data_type();
    int rc = compress_common(c.data.data(), dt, c.meta.width(), c.meta.height(),
                             c.meta.depth(), sx, sy, sz, wave, frac, bins, qalg,
                             zeros, out, nullptr, two_d);
    if (rc == 0 && errors) {
      // computeErrorRates after quantizing (test_compress_cpu.cc:150-157)
      ErrAcc acc;
      bool computed = false;
      if (error_metrics_files(in, out, acc, computed)) return 1;
      if (!computed)
        fprintf(stderr, "Cannot compute error rates: no maximum possible input value set.\n");
      float g[6];
      err_getters(acc, g);
      printf("Mean squared error: %.3f, relative error: %g, peak SNR: %.3f\n", g[3], g[5], g[4]);
      fflush(stdout);
    }
    return rc;
  }
  return 1;
}

}  // extern "C"
