// Huffman decoding on the device for streams without any index (files the
// reference wrote decode too).
//
// Reference: HuffmanDecoder::decodeFromStream (huffman.h:96-131) walks the
// breadth-first decode table bit by bit; a zero-run key is followed by 3
// length bits and expands to 2^(v+3) copies of the zero bin.
//
// The stream is cut into subsequences of kSubBits bits.  Phase 1: every
// subsequence is decoded speculatively from its first bit until the decoder
// crosses into the next subsequence; it records where that happens (its exit,
// a token boundary) and how many elements it produced.  Huffman codes
// resynchronise after a few tokens, so the exit rarely depends on where the
// decoding started.  Rounds: a subsequence whose start differs from its
// predecessor's exit is decoded again from that exit; rounds repeat until no
// start changes (each round fixes at least the first wrong subsequence).
// The first kSync token boundaries of every speculative decode are kept, so a
// later round stops as soon as it lands on one of them: from there on its
// tokens are the speculative ones, and the exit and element count follow
// from the record (without it every subsequence would be decoded again,
// since a speculative start is almost never a token boundary).
// Then an exclusive scan of the element counts gives every subsequence its
// output offset, and a last pass decodes again and writes the elements (the
// bins, or for batched decompression their dequantized values, where zero-bin
// runs were set beforehand and are only skipped).  A 12-bit lookup table
// resolves most codes in one step; each thread reads its stream through a
// window of three words in registers.
#include <cstring>
#include <vector>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kSubBits = 1024;
constexpr int kSync = 8;  // token boundaries kept per speculative decode
constexpr int kLutBits = 12;
constexpr int kThreads = 256;

struct DecCub {
  const uint32_t *words;
  long long nWords;
  const int *table;
  int nTable;
  int dupKey, dupValue;
  int binCount;
  long long n;        // elements
  int *out;           // bins
  float *fout = nullptr;  // or the dequantized values dq[bin]
  const float *dq = nullptr;
  long long subBase;  // first subsequence
  long long nSub;
  int lutOff;
};

__device__ __forceinline__ int find_cub(const DecCub *c, int n, long long sub) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (c[mid].subBase <= sub) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// LUT entry: bit 31 leaf; leaf: bits 16-23 code length, bits 0-15 symbol;
// not a leaf: bits 0-30 node offset in the decode table after kLutBits bits
__global__ void build_lut_kernel(const DecCub *cubs, unsigned *lut) {
  const DecCub c = cubs[blockIdx.x];
  unsigned *L = lut + (size_t)c.lutOff;
  for (int p = threadIdx.x; p < (1 << kLutBits); p += blockDim.x) {
    if (c.nTable == 2) {  // one node: a zero-length code
      L[p] = 0x80000000u | (unsigned)c.table[1];
      continue;
    }
    int node = 0;
    unsigned e = 0;
    bool leaf = false;
    for (int d = 0; d < kLutBits; d++) {
      const int bit = (p >> d) & 1;
      const int nx = c.table[node + bit] * 2;
      if (nx < 0 || nx + 1 >= c.nTable) { e = 0x80000000u | (0xffu << 16) | 0xffffu; leaf = true; break; }
      node = nx;
      if (c.table[node] == 0) {
        e = 0x80000000u | ((unsigned)(d + 1) << 16) | (unsigned)c.table[node + 1];
        leaf = true;
        break;
      }
    }
    L[p] = leaf ? e : (unsigned)node;
  }
}

// Decode one token at bit p.  Returns bits consumed (0 = malformed), sets the
// element count and the value.
// Three stream words from word i on (zero past the end), moved on a word at a
// time as the bit position advances (it never goes back): a token loads a
// word only when it crosses into the next one.
struct Window {
  const uint32_t *w;
  long long nw, i;
  unsigned a, b, c;
  __device__ unsigned ld(long long k) const { return k < nw ? w[k] : 0u; }
  __device__ void init(const uint32_t *words, long long n, long long p) {
    w = words;
    nw = n;
    i = p >> 5;
    a = ld(i);
    b = ld(i + 1);
    c = ld(i + 2);
  }
  // 64 bits of the stream from bit p (p >= 32 i), as peek64
  __device__ unsigned long long peek(long long p) {
    const long long k = p >> 5;
    while (i < k) {
      a = b;
      b = c;
      c = ld(i + 3);
      i++;
    }
    // bits o .. o + 63 of c:b:a, as two 32-bit funnel shifts (o = 0 included)
    const unsigned o = (unsigned)(p & 31);
    const unsigned lo = __funnelshift_r(a, b, o), hi = __funnelshift_r(b, c, o);
    return lo | ((unsigned long long)hi << 32);
  }
};

__device__ __forceinline__ int decode_token(const DecCub &c, const unsigned *L, Window &win,
                                            long long p, int &count, int &value) {
  const unsigned long long b0 = win.peek(p);  // bits p .. p + 63
  unsigned long long bits = b0;
  const unsigned e = L[bits & ((1u << kLutBits) - 1)];
  int len, sym;
  if (e & 0x80000000u) {
    len = (e >> 16) & 0xff;
    sym = e & 0xffff;
    if (len == 0xff) return 0;
  } else {
    int node = (int)e;
    len = kLutBits;
    bits >>= kLutBits;
    while (true) {
      const int nx = c.table[node + (int)(bits & 1)] * 2;
      bits >>= 1;
      len++;
      if (nx < 0 || nx + 1 >= c.nTable || len > 60) return 0;
      node = nx;
      if (c.table[node] == 0) break;
    }
    sym = c.table[node + 1];
  }
  if (sym == c.dupKey && c.dupKey >= 0) {
    // the 3 length bits follow the code; len <= 60, so they are in b0
    const unsigned v = (unsigned)((b0 >> len) & 7u);
    count = 1 << (v + 3);
    value = c.dupValue;
    return len + 3;
  }
  count = 1;
  value = sym;
  return len > 0 ? len : -1;  // -1: zero-length code (one-symbol stream)
}

// Decode tokens from `start` until the position reaches `limit`; returns the
// exit position and the number of elements.
__device__ long long decode_span(const DecCub &c, const unsigned *L, long long start, long long limit,
                                 long long &elems, bool &bad) {
  long long p = start, e = 0;
  const long long total = c.nWords * 32;
  Window win;
  win.init(c.words, c.nWords, p);
  while (p < limit && p < total) {
    int cnt, val;
    const int used = decode_token(c, L, win, p, cnt, val);
    if (used <= 0) { bad = true; break; }
    p += used;
    e += cnt;
  }
  elems = e;
  return p;
}

// Speculative decode of subsequence i from its first bit, keeping the first
// kSync token boundaries: rec[k * totalSub + i] = (boundary - start) | (elements
// before it << 16), all ones where the subsequence ends first (a boundary is at
// most kSync * 61 bits and 8192 elements past the start).
__device__ long long decode_span_rec(const DecCub &c, const unsigned *L, long long start,
                                     long long limit, long long &elems, bool &bad,
                                     unsigned *rec, long long stride) {
  long long p = start, e = 0;
  const long long total = c.nWords * 32;
  Window win;
  win.init(c.words, c.nWords, p);
#pragma unroll
  for (int k = 0; k < kSync; k++) {
    unsigned r = ~0u;
    if (!bad && p < limit && p < total) {
      int cnt, val;
      const int used = decode_token(c, L, win, p, cnt, val);
      if (used <= 0) {
        bad = true;
      } else {
        p += used;
        e += cnt;
        r = (unsigned)(p - start) | ((unsigned)e << 16);
      }
    }
    rec[k * stride] = r;
  }
  while (!bad && p < limit && p < total) {
    int cnt, val;
    const int used = decode_token(c, L, win, p, cnt, val);
    if (used <= 0) { bad = true; break; }
    p += used;
    e += cnt;
  }
  elems = e;
  return p;
}

// Decode from a true token boundary s (s >= s0, the speculative start) until
// the position meets a boundary of the speculative decode (then its exit x0
// and element count e0 hold, less the elements it produced before that
// boundary) or the subsequence ends.
__device__ long long decode_span_sync(const DecCub &c, const unsigned *L, long long s,
                                      long long limit, long long s0, long long x0, long long e0,
                                      const unsigned *rec, long long stride, long long &elems,
                                      bool &bad) {
  long long p = s, e = 0;
  const long long total = c.nWords * 32;
  int k = -1;                 // speculative boundary below or at p: k = -1 is s0
  long long bk = s0, ck = 0;  // its position and the elements before it
  Window win;
  win.init(c.words, c.nWords, p);
  for (;;) {
    while (bk < p && k + 1 < kSync) {
      const unsigned r = rec[(k + 1) * stride];
      if (r == ~0u) break;
      k++;
      bk = s0 + (r & 0xffffu);
      ck = r >> 16;
    }
    if (bk == p) {  // on the speculative path from here
      elems = e + (e0 - ck);
      return x0;
    }
    if (!(p < limit && p < total)) break;
    int cnt, val;
    const int used = decode_token(c, L, win, p, cnt, val);
    if (used <= 0) { bad = true; break; }
    p += used;
    e += cnt;
  }
  elems = e;
  return p;
}

__global__ void spec_kernel(const DecCub *cubs, int nCub, const unsigned *lut, long long totalSub,
                            long long *start, long long *exitPos, long long *elems, int *flags,
                            int round, unsigned *rec, long long *spec0) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= totalSub) return;
  const int ci = find_cub(cubs, nCub, i);
  const DecCub c = cubs[ci];
  const long long local = i - c.subBase;
  const long long s0 = local * kSubBits, limit = (local + 1) * kSubBits;
  bool bad = false;
  long long e, x;
  if (round == 0) {
    start[i] = s0;
    x = decode_span_rec(c, lut + c.lutOff, s0, limit, e, bad, rec + i, totalSub);
    spec0[2 * i] = x;
    spec0[2 * i + 1] = e;
  } else {
    if (local == 0) {  // always starts right; carry its exit to this round's buffer
      exitPos[2 * i + (round & 1)] = exitPos[2 * i + ((round - 1) & 1)];
      return;
    }
    const long long s = exitPos[2 * (i - 1) + ((round - 1) & 1)];
    if (s == start[i]) {
      exitPos[2 * i + (round & 1)] = exitPos[2 * i + ((round - 1) & 1)];
      return;
    }
    atomicAdd(&flags[0], 1);
    start[i] = s;
    x = decode_span_sync(c, lut + c.lutOff, s, limit, s0, spec0[2 * i], spec0[2 * i + 1],
                         rec + i, totalSub, e, bad);
  }
  exitPos[2 * i + (round & 1)] = x;
  elems[i] = e;
  if (bad) atomicAdd(&flags[1], 1);
}

// per cubelet exclusive scan of element counts (one CTA per cubelet)
__global__ void __launch_bounds__(1024) elem_scan_kernel(const DecCub *cubs, long long *elems,
                                                         long long *totalOut) {
  __shared__ long long sh[32];
  const DecCub c = cubs[blockIdx.x];
  long long carry = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (long long seg = 0; seg < c.nSub; seg += 1024) {
    const long long j = seg + threadIdx.x;
    const long long v = j < c.nSub ? elems[c.subBase + j] : 0;
    long long inc = v;
    for (int off = 1; off < 32; off <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += t;
    }
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    long long before = 0, tot = 0;
    for (int k = 0; k < 32; k++) { if (k < w) before += sh[k]; tot += sh[k]; }
    if (j < c.nSub) elems[c.subBase + j] = carry + before + inc - v;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) totalOut[blockIdx.x] = carry;
}

__global__ void write_kernel(const DecCub *cubs, int nCub, const unsigned *lut, long long totalSub,
                             const long long *start, const long long *exitPos, const long long *offs,
                             int lastRound) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= totalSub) return;
  const int ci = find_cub(cubs, nCub, i);
  const DecCub c = cubs[ci];
  const unsigned *L = lut + c.lutOff;
  const long long limit = exitPos[2 * i + (lastRound & 1)];
  long long p = start[i], o = offs[i];
  const long long total = c.nWords * 32;
  Window win;
  win.init(c.words, c.nWords, p);
  if (c.fout) {
    // dequantized on the way.  With zero runs the output already holds the
    // zero bin's value everywhere (launch_fill_batch), so only the other
    // values are written; runs and single zero-bin tokens just move on.
    float *F = c.fout;
    if (c.dupValue >= 0) {
      // prefilled: a zero-run token or a single zero-bin token only moves on,
      // every other token is one value (only the zero-run key counts more
      // than one element)
      while (p < limit && p < total && o < c.n) {
        int cnt, val;
        const int used = decode_token(c, L, win, p, cnt, val);
        if (used <= 0) break;
        p += used;
        if (val != c.dupValue) F[o] = c.dq[min(max(val, 0), c.binCount - 1)];
        o = min(o + cnt, c.n);
      }
      return;
    }
    while (p < limit && p < total && o < c.n) {
      int cnt, val;
      const int used = decode_token(c, L, win, p, cnt, val);
      if (used <= 0) break;
      p += used;
      const float fv = c.dq[min(max(val, 0), c.binCount - 1)];
      const long long e = min(o + cnt, c.n);
      for (; o < e; o++) F[o] = fv;
    }
    return;
  }
  while (p < limit && p < total && o < c.n) {
    int cnt, val;
    const int used = decode_token(c, L, win, p, cnt, val);
    if (used <= 0) break;
    p += used;
    for (int k = 0; k < cnt && o < c.n; k++) c.out[o++] = val;
  }
}

// Fallback when rounds do not converge (codes that never resynchronise, e.g.
// all of one length): one thread per cubelet fixes its subsequences in order.
__global__ void seq_fix_kernel(const DecCub *cubs, const unsigned *lut, long long *start,
                               long long *exitPos, long long *elems, int buf, int *flags) {
  const DecCub c = cubs[blockIdx.x];
  for (long long j = 1; j < c.nSub; j++) {
    const long long i = c.subBase + j;
    const long long s = exitPos[2 * (i - 1) + buf];
    if (s == start[i]) continue;
    start[i] = s;
    bool bad = false;
    long long e;
    exitPos[2 * i + buf] = decode_span(c, lut + c.lutOff, s, (j + 1) * kSubBits, e, bad);
    elems[i] = e;
    if (bad) atomicAdd(&flags[1], 1);
  }
}

__global__ void fill_kernel(int *out, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = v;
}

}  // namespace

// Decode n streams at once (the DecCub records and scratch in ws: see
// decode_batch_workspace_bytes).  Streams are the items with a real tree
// (items whose table is one node are filled by the caller).  Returns 0 on
// success, 1 when a stream is malformed or holds fewer elements than its
// cubelet, -1 on a CUDA error; bad[i] (host, may be NULL) marks the items.
// per subsequence: start, two exits, element count (32 bytes), the
// speculative exit and count (16) and its kSync boundaries (4 each)
constexpr size_t kSubBytes = 48 + 4 * kSync;

size_t decode_batch_workspace_bytes(int n, long long totalSub) {
  return (size_t)n * sizeof(DecCub) + 256 + (size_t)n * 4096 * 4 + (size_t)totalSub * kSubBytes +
         (size_t)n * 8 + 64 + 256;
}

int decode_streams(const DecodeItem *items, int n, void *ws, int *hostFlags,
                   long long *hostTotals, cudaStream_t s) {
  if (n <= 0) return 0;
  std::vector<DecCub> cs(n);
  long long totalSub = 0;
  for (int i = 0; i < n; i++) {
    const DecodeItem &it = items[i];
    DecCub &c = cs[i];
    const long long nSub = (it.nWords * 32 + kSubBits - 1) / kSubBits > 0
                               ? (it.nWords * 32 + kSubBits - 1) / kSubBits : 1;
    c.words = it.words; c.nWords = it.nWords; c.table = it.table; c.nTable = it.nTable;
    c.dupKey = it.dupKey; c.dupValue = it.dupValue; c.binCount = it.binCount; c.n = it.n;
    c.out = it.out; c.fout = it.fout; c.dq = it.dq;
    c.subBase = totalSub; c.nSub = nSub; c.lutOff = i * 4096;
    totalSub += nSub;
  }
  char *p = static_cast<char *>(ws);
  DecCub *dc = reinterpret_cast<DecCub *>(p);
  p += ((size_t)n * sizeof(DecCub) + 255) & ~(size_t)255;
  unsigned *lut = reinterpret_cast<unsigned *>(p); p += (size_t)n * 4096 * 4;
  long long *start = reinterpret_cast<long long *>(p); p += totalSub * 8;
  long long *exitPos = reinterpret_cast<long long *>(p); p += totalSub * 16;
  long long *elems = reinterpret_cast<long long *>(p); p += totalSub * 8;
  long long *spec0 = reinterpret_cast<long long *>(p); p += totalSub * 16;
  unsigned *rec = reinterpret_cast<unsigned *>(p); p += totalSub * 4 * kSync;
  long long *total = reinterpret_cast<long long *>(p); p += (size_t)n * 8;
  int *flags = reinterpret_cast<int *>(p);
  if (cudaMemcpyAsync(dc, cs.data(), (size_t)n * sizeof(DecCub), cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return -1;
  build_lut_kernel<<<n, 1024, 0, s>>>(dc, lut);
  const unsigned grid = (unsigned)((totalSub + kThreads - 1) / kThreads);
  constexpr int kRounds = 6;
  int round = 0;
  cudaMemsetAsync(flags, 0, 8, s);
  spec_kernel<<<grid, kThreads, 0, s>>>(dc, n, lut, totalSub, start, exitPos, elems, flags, 0,
                                        rec, spec0);
  bool converged = false;
  for (round = 1; round <= kRounds; round++) {
    cudaMemsetAsync(flags, 0, 4, s);
    spec_kernel<<<grid, kThreads, 0, s>>>(dc, n, lut, totalSub, start, exitPos, elems, flags,
                                          round, rec, spec0);
    cudaMemcpyAsync(hostFlags, flags, 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    if (hostFlags[0] == 0) { converged = true; break; }
  }
  if (!converged) {
    round = kRounds;
    seq_fix_kernel<<<n, 1, 0, s>>>(dc, lut, start, exitPos, elems, round & 1, flags);
    cudaMemcpyAsync(hostFlags, flags, 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  }
  if (hostFlags[1]) return 1;
  elem_scan_kernel<<<n, 1024, 0, s>>>(dc, elems, total);
  cudaMemcpyAsync(hostTotals, total, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  for (int i = 0; i < n; i++)
    if (hostTotals[i] < items[i].n) return 1;  // fewer values than the cubelet holds
  write_kernel<<<grid, kThreads, 0, s>>>(dc, n, lut, totalSub, start, exitPos, elems, round);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Decode one stream (device words/table) into n ints at out.  Synchronizes
// the stream between rounds.  Returns 0 on success, 1 malformed stream,
// -1 CUDA error.  Scratch comes from `ws` (decode_workspace_bytes).  A
// one-node table whose symbol is not the zero-run key codes every element
// with zero bits: fill_value() handles that case.
size_t decode_workspace_bytes(long long nWords) {
  const long long nSub = (nWords * 32 + kSubBits - 1) / kSubBits + 1;
  return (size_t)nSub * kSubBytes + 4096 * 4 + 256 + 64;
}

int decode_stream(const uint32_t *words, long long nWords, const int *table, int nTable,
                  int dupKey, int dupValue, int binCount, long long n, int *out, void *ws,
                  int *hostFlags, cudaStream_t s) {
  const long long nSub = (nWords * 32 + kSubBits - 1) / kSubBits > 0
                             ? (nWords * 32 + kSubBits - 1) / kSubBits : 1;
  char *p = static_cast<char *>(ws);
  DecCub *dc = reinterpret_cast<DecCub *>(p); p += 256;
  unsigned *lut = reinterpret_cast<unsigned *>(p); p += 4096 * 4;
  long long *start = reinterpret_cast<long long *>(p); p += nSub * 8;
  long long *exitPos = reinterpret_cast<long long *>(p); p += nSub * 16;
  long long *elems = reinterpret_cast<long long *>(p); p += nSub * 8;
  long long *spec0 = reinterpret_cast<long long *>(p); p += nSub * 16;
  unsigned *rec = reinterpret_cast<unsigned *>(p); p += nSub * 4 * kSync;
  long long *total = reinterpret_cast<long long *>(p); p += 8;
  int *flags = reinterpret_cast<int *>(p);
  DecCub c{};  // bins out (fout stays null)
  c.words = words; c.nWords = nWords; c.table = table; c.nTable = nTable;
  c.dupKey = dupKey; c.dupValue = dupValue; c.binCount = binCount; c.n = n; c.out = out;
  c.subBase = 0; c.nSub = nSub; c.lutOff = 0;
  if (cudaMemcpyAsync(dc, &c, sizeof c, cudaMemcpyHostToDevice, s) != cudaSuccess) return -1;
  build_lut_kernel<<<1, 1024, 0, s>>>(dc, lut);
  const unsigned grid = (unsigned)((nSub + kThreads - 1) / kThreads);
  constexpr int kRounds = 6;
  int round = 0;
  cudaMemsetAsync(flags, 0, 8, s);
  spec_kernel<<<grid, kThreads, 0, s>>>(dc, 1, lut, nSub, start, exitPos, elems, flags, 0, rec,
                                        spec0);
  bool converged = false;
  for (round = 1; round <= kRounds; round++) {
    cudaMemsetAsync(flags, 0, 4, s);
    spec_kernel<<<grid, kThreads, 0, s>>>(dc, 1, lut, nSub, start, exitPos, elems, flags, round,
                                          rec, spec0);
    cudaMemcpyAsync(hostFlags, flags, 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    if (hostFlags[0] == 0) { converged = true; break; }
  }
  if (!converged) {
    round = kRounds;
    seq_fix_kernel<<<1, 1, 0, s>>>(dc, lut, start, exitPos, elems, round & 1, flags);
    cudaMemcpyAsync(hostFlags, flags, 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  }
  if (hostFlags[1]) return 1;
  elem_scan_kernel<<<1, 1024, 0, s>>>(dc, elems, total);
  cudaMemcpyAsync(hostFlags + 2, total, 8, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  long long got;
  memcpy(&got, hostFlags + 2, 8);
  if (got < n) return 1;  // the reference stops with fewer values than the cubelet holds
  write_kernel<<<grid, kThreads, 0, s>>>(dc, 1, lut, nSub, start, exitPos, elems, round);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void __launch_bounds__(256) fill_batch_kernel(const FillItem *__restrict__ items,
                                                         int nItems) {
  int lo = 0, hi = nItems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].blockBase <= (long long)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const FillItem it = items[lo];
  const long long b0 = ((long long)blockIdx.x - it.blockBase) * kFillBlock;
  const long long e = min(b0 + kFillBlock, it.n);
  const float4 v4 = make_float4(it.v, it.v, it.v, it.v);
  // b0 is a multiple of kFillBlock, so whole float4 words up to the end
  for (long long i = b0 + 4 * threadIdx.x; i + 4 <= e; i += 4 * 256)
    *reinterpret_cast<float4 *>(it.out + i) = v4;
  const long long tail = b0 + ((e - b0) & ~3LL);
  if (threadIdx.x < e - tail) it.out[tail + threadIdx.x] = it.v;
}

void launch_fill_batch(const FillItem *items, int nItems, long long totalBlocks, cudaStream_t s) {
  if (nItems > 0 && totalBlocks > 0)
    fill_batch_kernel<<<(unsigned)totalBlocks, 256, 0, s>>>(items, nItems);
}

void fill_value(int *out, long long n, int v, cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  fill_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, s>>>(out, n, v);
}

}  // namespace wl
