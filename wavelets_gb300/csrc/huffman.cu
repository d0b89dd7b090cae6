// Huffman coding on the device: exact tree construction, code assignment and
// decode table per cubelet, then a parallel bit packer.
//
// Tree (Huffman::computeHuffmanCoding, huffman.cc:42-97): the reference pops
// the two nodes of smallest count from a priority queue ordered by
// (count, node address) with ties going to the LARGER node index
// (CompareHuffmanNode, huffman.cc:9-18); the first popped becomes the 0
// branch.  Leaves are symbol indices 0..S-1 (S = bins, +1 for the zero-run
// key), merged nodes are numbered from S upward.  Here the leaves are sorted
// by (count asc, index desc) and merged nodes wait in a queue of equal-count
// groups; merged counts never decrease, so the group at the front holds the
// smallest merged count and its newest node is the one the reference pops
// next.  On equal counts a merged node beats a leaf (it has the larger index).
// Codes are root-first, bit d of the code word = branch taken at depth d
// (computeEncodedBits :147-174), the decode table lists nodes breadth first
// as (left id, right id) or (0, symbol) (computeDecodeTable :177-228).
//
// Packing (Huffman::encodeToStream, huffman.h:242-296; BitStreamWriter
// bit_stream.h:60-162): every coefficient yields zero or one token -- its own
// code, a single zero-bin code, or at the first element of a dup chunk the
// zero-run key code followed by 3 length bits.  Token lengths are summed per
// 4096-element chunk, chunk offsets are scanned per cubelet, and each chunk
// ORs its tokens into a shared-memory copy of its words; words wholly inside
// a chunk are stored directly, the two edge words are ORed into global memory.
#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int kPer = kChunk / kThreads;
constexpr int INF = 0x7fffffff;
constexpr int kMaxCodeBits = 58;  // + 3 dup bits fits 61 bits -> at most 3 words

__device__ __forceinline__ int find_cubelet(const long long *prefix, int n, long long c) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---- tree -------------------------------------------------------------------
struct BuildSmem {
  unsigned long long *keys;  // sorted leaves, later codes of all nodes
  short *lch, *rch;          // children of merged node (id - S)
  unsigned long long *icnt;  // counts of merged nodes
  short *gs, *ge;            // equal-count groups of the merged-node queue
  short *istack;             // merged-node storage of the groups
  unsigned char *depth;      // per node
  short *bfs, *bfsId;        // breadth-first order / position
};

__host__ __device__ inline size_t build_smem_bytes(int S) {
  int P = 1;
  while (P < S) P <<= 1;
  const size_t nodes = 2 * (size_t)S;
  size_t b = 0;
  b += (size_t)(P > (int)nodes ? P : nodes) * 8;  // keys / codes
  b += 2 * (size_t)S * 2;                         // lch, rch
  b += (size_t)S * 8;                             // icnt
  b += 2 * (size_t)S * 2;                         // gs, ge
  b += (size_t)S * 2;                             // istack
  b += nodes;                                     // depth
  b += 2 * nodes * 2;                             // bfs, bfsId
  return (b + 15) & ~(size_t)15;
}

__global__ void __launch_bounds__(1024) huffman_build_kernel(DevBatch b) {
  extern __shared__ unsigned long long hsm[];
  __shared__ int nLeaves;
  const int ci = blockIdx.x;
  const CubeletDev cd = b.cub[ci];
  CubeletState *st = b.state + ci;
  const int dupV = st->dupValue;
  const int S = cd.binCount + (dupV >= 0 ? 1 : 0);
  int P = 1;
  while (P < S) P <<= 1;
  const int nodesMax = 2 * S;

  BuildSmem m;
  char *p = reinterpret_cast<char *>(hsm);
  m.keys = reinterpret_cast<unsigned long long *>(p); p += (size_t)(P > nodesMax ? P : nodesMax) * 8;
  m.icnt = reinterpret_cast<unsigned long long *>(p); p += (size_t)S * 8;
  m.lch = reinterpret_cast<short *>(p); p += (size_t)S * 2;
  m.rch = reinterpret_cast<short *>(p); p += (size_t)S * 2;
  m.gs = reinterpret_cast<short *>(p); p += (size_t)S * 2;
  m.ge = reinterpret_cast<short *>(p); p += (size_t)S * 2;
  m.istack = reinterpret_cast<short *>(p); p += (size_t)S * 2;
  m.bfs = reinterpret_cast<short *>(p); p += (size_t)nodesMax * 2;
  m.bfsId = reinterpret_cast<short *>(p); p += (size_t)nodesMax * 2;
  m.depth = reinterpret_cast<unsigned char *>(p);

  const unsigned long long *cnt = b.hist + (size_t)ci * kMaxSymbols;
  if (threadIdx.x == 0) nLeaves = 0;
  __syncthreads();
  // leaves with a nonzero count, key = count:51 | (8191 - symbol):13
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    const unsigned long long c = (i == cd.binCount) ? cnt[cd.binCount] : cnt[i];
    if (c > 0) {
      const int slot = atomicAdd(&nLeaves, 1);
      m.keys[slot] = (c << 13) | (unsigned long long)(8191 - i);
    }
  }
  __syncthreads();
  const int nL = nLeaves;
  for (int i = nL + threadIdx.x; i < P; i += blockDim.x) m.keys[i] = ~0ull;
  __syncthreads();
  // bitonic sort, ascending
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = m.keys[i], c = m.keys[l];
          const bool up = (i & k) == 0;
          if ((a > c) == up) { m.keys[i] = c; m.keys[l] = a; }
        }
      }
      __syncthreads();
    }
  }

  if (threadIdx.x == 0) {
    int err = 0;
    // ---- merge (single thread, O(S)) ----
    int lf = 0;                 // next leaf
    int gF = 0, gL = -1;        // active groups gF..gL
    int top = 0;                // next free istack slot
    int next = S;               // next merged node id
    int root = -1;
    int remaining = nL;
    auto popNode = [&](unsigned long long &count) -> int {
      const bool haveLeaf = lf < nL;
      const bool haveInt = gF <= gL;
      bool takeInt = false;
      unsigned long long ic = 0;
      if (haveInt) ic = m.icnt[m.istack[m.gs[gF]] - S];
      if (haveInt && haveLeaf) takeInt = ic <= (m.keys[lf] >> 13);
      else takeInt = haveInt;
      if (takeInt) {
        const int id = m.istack[m.ge[gF] - 1];
        m.ge[gF]--;
        if (m.ge[gF] == m.gs[gF]) gF++;
        count = ic;
        return id;
      }
      const unsigned long long key = m.keys[lf++];
      count = key >> 13;
      return 8191 - (int)(key & 8191ull);
    };
    while (remaining > 1) {
      unsigned long long ca, cb2;
      const int a = popNode(ca);
      const int c = popNode(cb2);
      const int id = next++;
      const unsigned long long sum = ca + cb2;
      m.lch[id - S] = (short)a;
      m.rch[id - S] = (short)c;
      m.icnt[id - S] = sum;
      if (gF <= gL && m.icnt[m.istack[m.gs[gL]] - S] == sum) {
        m.istack[m.ge[gL]++] = (short)id;
        top = m.ge[gL];
      } else {
        gL++;
        if (gL < gF) gF = gL;
        m.gs[gL] = (short)top;
        m.ge[gL] = (short)(top + 1);
        m.istack[top++] = (short)id;
      }
      remaining--;
    }
    if (nL == 1) root = 8191 - (int)(m.keys[0] & 8191ull);
    else if (nL > 1) root = next - 1;
    const int nInternal = next - S;

    // ---- depths and codes (parents are created after their children) ----
    unsigned long long *code = m.keys;  // reuse: codes per node id
    const int nodes = S + nInternal;
    for (int i = 0; i < nodes; i++) { m.depth[i] = 0; code[i] = 0; }
    int longest = 0;
    for (int j = nInternal - 1; j >= 0; j--) {
      const int id = S + j;
      const int d = m.depth[id];
      const int l = m.lch[j], r = m.rch[j];
      m.depth[l] = (unsigned char)(d + 1);
      m.depth[r] = (unsigned char)(d + 1);
      code[l] = code[id];
      code[r] = code[id] | (d < 64 ? (1ull << d) : 0ull);
      if (d + 1 > longest) longest = d + 1;
    }
    if (longest > kMaxCodeBits) err = 2;

    // ---- decode table, breadth first ----
    int *dec = b.decode + (size_t)ci * 4 * kMaxSymbols;
    int nb = 0;
    if (root >= 0) {
      m.bfs[nb++] = (short)root;
      for (int h = 0; h < nb; h++) {
        const int nd = m.bfs[h];
        m.bfsId[nd] = (short)h;
        if (nd >= S) {
          m.bfs[nb++] = m.lch[nd - S];
          m.bfs[nb++] = m.rch[nd - S];
        }
      }
      for (int h = 0; h < nb; h++) {
        const int nd = m.bfs[h];
        if (nd >= S) {
          dec[2 * h] = m.bfsId[m.lch[nd - S]];
          dec[2 * h + 1] = m.bfsId[m.rch[nd - S]];
        } else {
          dec[2 * h] = 0;
          dec[2 * h + 1] = nd;
        }
      }
    }
    st->nDecode = 2 * nb;
    st->longest = longest;
    st->nLeaves = nL;
    if (err) st->error = err;
  }
  __syncthreads();
  // code table for the encoder
  unsigned long long *gcode = b.codes + (size_t)ci * kMaxSymbols;
  uint8_t *glen = b.codeLen + (size_t)ci * kMaxSymbols;
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    gcode[i] = m.keys[i];
    glen[i] = m.depth[i];
  }
}

// ---- tokens -----------------------------------------------------------------
struct TokCtx {
  const uint8_t *len;             // smem copy of code lengths
  const unsigned long long *code; // smem copy of codes (may be null when counting)
  int dupV, dupKey;
  long long chunkStart;           // cubelet coordinate of chunk element 0
  long long runIn, runOut;        // run entering / leaving the chunk
};

// Token of element at cubelet position P inside a zero-bin run [s, e).
// Returns the token length (0 = element is covered by an earlier dup token);
// bits receive the token bits when code != null.
__device__ __forceinline__ int run_token(long long P, long long s, long long e, const TokCtx &t,
                                         unsigned long long &bits) {
  const long long o = P - s, L = e - s;
  const long long q = L / 1024;
  int dupE = -1;
  if (o < q * 1024) {
    if ((o & 1023) == 0) dupE = 7;
    else return 0;
  } else {
    int r = (int)(L - q * 1024);
    int oo = (int)(o - q * 1024);
    int pos = 0;
    while (r > 8) {
      int p2 = 8, e2 = 0;
      while ((p2 << 1) <= r) { p2 <<= 1; e2++; }
      if (oo == pos) { dupE = e2; break; }
      if (oo < pos + p2) return 0;
      pos += p2;
      r -= p2;
    }
  }
  if (dupE >= 0) {
    const int l = t.len[t.dupKey];
    if (t.code) bits = t.code[t.dupKey] | ((unsigned long long)dupE << l);
    return l + 3;
  }
  if (t.code) bits = t.code[t.dupV];
  return t.len[t.dupV];
}

// Token lengths (and bits) for this thread's kPer elements.  Collective over
// the block (uses two block-wide scans).
__device__ void thread_tokens(const int (&bins)[kPer], int p0, int len, const TokCtx &t,
                              int (&tl)[kPer], unsigned long long (&tb)[kPer],
                              int *wFirst, int *wLast) {
  const int dupV = t.dupV;
  int first = INF, last = -1;
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    const int p = p0 + k;
    if (p < len && bins[k] != dupV) {
      if (first == INF) first = p;
      last = p;
    }
  }
  int nextNZ = INF, prevNZ = -1;
  if (dupV >= 0) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incMin = first, incMax = last;
    for (int off = 1; off < 32; off <<= 1) {
      int vmin = __shfl_down_sync(0xffffffffu, incMin, off);
      int vmax = __shfl_up_sync(0xffffffffu, incMax, off);
      if (lane + off < 32) incMin = min(incMin, vmin);
      if (lane >= off) incMax = max(incMax, vmax);
    }
    if (lane == 0) wFirst[w] = incMin;
    if (lane == 31) wLast[w] = incMax;
    __syncthreads();
    nextNZ = __shfl_down_sync(0xffffffffu, incMin, 1);
    if (lane == 31) nextNZ = INF;
    prevNZ = __shfl_up_sync(0xffffffffu, incMax, 1);
    if (lane == 0) prevNZ = -1;
    for (int v = w + 1; v < kThreads / 32; v++) nextNZ = min(nextNZ, wFirst[v]);
    for (int v = 0; v < w; v++) prevNZ = max(prevNZ, wLast[v]);
    __syncthreads();
  }
  // walk: last non-zero position seen so far (chunk coordinates)
  int lastNZ = prevNZ;
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    const int p = p0 + k;
    tl[k] = 0;
    tb[k] = 0;
    if (p >= len) continue;
    const int v = bins[k];
    if (v != dupV) {
      tl[k] = t.len[v];
      if (t.code) tb[k] = t.code[v];
      lastNZ = p;
      continue;
    }
    // run start
    const long long s = lastNZ < 0 ? t.runIn : t.chunkStart + lastNZ + 1;
    // run end: next non-zero position after p
    int nz = INF;
    for (int k2 = k + 1; k2 < kPer; k2++)
      if (p0 + k2 < len && bins[k2] != dupV) { nz = p0 + k2; break; }
    if (nz == INF) nz = nextNZ;
    const long long e = (nz == INF || nz >= len) ? t.runOut : t.chunkStart + nz;
    unsigned long long bits = 0;
    tl[k] = run_token(t.chunkStart + p, s, e, t, bits);
    tb[k] = bits;
  }
}

__device__ __forceinline__ void load_bins(const uint16_t *src, int p0, int len, int dupV,
                                          int (&bins)[kPer]) {
  if (p0 + kPer <= len) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + p0);
#pragma unroll
    for (int k = 0; k < kPer / 8; k++) {
      const uint4 v = s4[k];
      bins[8 * k + 0] = v.x & 0xffff; bins[8 * k + 1] = v.x >> 16;
      bins[8 * k + 2] = v.y & 0xffff; bins[8 * k + 3] = v.y >> 16;
      bins[8 * k + 4] = v.z & 0xffff; bins[8 * k + 5] = v.z >> 16;
      bins[8 * k + 6] = v.w & 0xffff; bins[8 * k + 7] = v.w >> 16;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kPer; k++) bins[k] = (p0 + k < len) ? src[p0 + k] : dupV;
  }
}

// block sum of unsigned long long (256 threads)
__device__ __forceinline__ unsigned long long block_sum(unsigned long long v, unsigned long long *sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  unsigned long long t = 0;
  for (int i = 0; i < kThreads / 32; i++) t += sh[i];
  __syncthreads();
  return t;
}

// exclusive block scan (256 threads)
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *sh, unsigned &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned inc = v;
  for (int off = 1; off < 32; off <<= 1) {
    unsigned t = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += t;
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  unsigned before = 0;
  total = 0;
  for (int i = 0; i < kThreads / 32; i++) {
    if (i < w) before += sh[i];
    total += sh[i];
  }
  __syncthreads();
  return before + inc - v;
}

__device__ __forceinline__ void setup_ctx(const DevBatch &b, long long chunk, int ci,
                                          const CubeletDev &cd, TokCtx &t, uint8_t *sLen,
                                          unsigned long long *sCode) {
  const CubeletState *st = b.state + ci;
  t.dupV = st->dupValue;
  t.dupKey = cd.binCount;
  t.chunkStart = (chunk - cd.chunkBase) * (long long)kChunk;
  t.runIn = t.dupV >= 0 ? b.chunkRunCtx[2 * chunk] : 0;
  t.runOut = t.dupV >= 0 ? b.chunkRunCtx[2 * chunk + 1] : 0;
  const int S = cd.binCount + 1;
  for (int i = threadIdx.x; i < S; i += kThreads) {
    sLen[i] = b.codeLen[(size_t)ci * kMaxSymbols + i];
    if (sCode) sCode[i] = b.codes[(size_t)ci * kMaxSymbols + i];
  }
  t.len = sLen;
  t.code = sCode;
}

__global__ void __launch_bounds__(kThreads) encode_count_kernel(DevBatch b) {
  __shared__ uint8_t sLen[kMaxSymbols + 3];
  __shared__ int wFirst[kThreads / 32], wLast[kThreads / 32];
  __shared__ unsigned long long sh[kThreads / 32];
  const long long chunk = blockIdx.x;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletDev cd = b.cub[ci];
  TokCtx t;
  setup_ctx(b, chunk, ci, cd, t, sLen, nullptr);
  __syncthreads();
  const int len = (int)min((long long)kChunk, cd.n - t.chunkStart);
  const int p0 = threadIdx.x * kPer;
  int bins[kPer];
  load_bins(b.bins + cd.coefOff + t.chunkStart, p0, len, t.dupV, bins);
  int tl[kPer];
  unsigned long long tb[kPer];
  thread_tokens(bins, p0, len, t, tl, tb, wFirst, wLast);
  unsigned long long s = 0;
#pragma unroll
  for (int k = 0; k < kPer; k++) s += tl[k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) b.chunkBits[chunk] = s;
}

// per cubelet: exclusive scan of the chunk bit counts
__global__ void __launch_bounds__(1024) encode_scan_kernel(DevBatch b) {
  __shared__ unsigned long long sh[64];
  const int ci = blockIdx.x;
  const CubeletDev cd = b.cub[ci];
  CubeletState *st = b.state + ci;
  unsigned long long carry = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int seg = 0; seg < cd.nChunks; seg += 1024) {
    const int c = seg + threadIdx.x;
    const unsigned long long v = c < cd.nChunks ? b.chunkBits[cd.chunkBase + c] : 0;
    unsigned long long inc = v;
    for (int off = 1; off < 32; off <<= 1) {
      unsigned long long t = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += t;
    }
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    unsigned long long before = 0, total = 0;
    for (int i = 0; i < 32; i++) {
      if (i < w) before += sh[i];
      total += sh[i];
    }
    if (c < cd.nChunks) b.chunkBits[cd.chunkBase + c] = carry + before + inc - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    st->totalBits = carry;
    const unsigned long long words = (carry + 31) / 32;
    st->nWords = (int)words;
    if ((long long)words > cd.wordsCap) st->error = 4;
  }
}

// packed word offset of every cubelet (one thread; n is small)
__global__ void cubelet_offsets_kernel(DevBatch b) {
  long long off = 0;
  for (int i = 0; i < b.n; i++) {
    CubeletState *st = b.state + i;
    st->wordsBase = off;
    off += st->error ? 0 : st->nWords;
  }
}

// zero the first and last word of every chunk (the words chunks share)
__global__ void encode_zero_kernel(DevBatch b) {
  const long long chunk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (chunk >= b.totalChunks) return;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletState *st = b.state + ci;
  if (st->error) return;
  const unsigned long long off = b.chunkBits[chunk];
  const unsigned long long end = (chunk + 1 < b.cub[ci].chunkBase + b.cub[ci].nChunks)
                                     ? b.chunkBits[chunk + 1] : st->totalBits;
  if (end == off) return;
  uint32_t *w = b.words + st->wordsBase;
  w[off >> 5] = 0;
  w[(end - 1) >> 5] = 0;
}

constexpr int kMaxChunkWords = (kChunk * (kMaxCodeBits + 3) + 31) / 32 + 2;

__global__ void __launch_bounds__(kThreads) encode_write_kernel(DevBatch b) {
  __shared__ uint8_t sLen[kMaxSymbols + 3];
  __shared__ unsigned long long sCode[kMaxSymbols];
  __shared__ int wFirst[kThreads / 32], wLast[kThreads / 32];
  __shared__ unsigned shs[kThreads / 32];
  extern __shared__ uint32_t sw[];
  const long long chunk = blockIdx.x;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  if (st->error) return;
  TokCtx t;
  setup_ctx(b, chunk, ci, cd, t, sLen, sCode);
  const unsigned long long chunkOff = b.chunkBits[chunk];
  const unsigned long long chunkEnd = (chunk + 1 < cd.chunkBase + cd.nChunks)
                                          ? b.chunkBits[chunk + 1] : st->totalBits;
  const int shift = (int)(chunkOff & 31);
  const int nW = (int)((shift + (chunkEnd - chunkOff) + 31) >> 5);
  for (int i = threadIdx.x; i < nW; i += kThreads) sw[i] = 0;
  __syncthreads();
  const int len = (int)min((long long)kChunk, cd.n - t.chunkStart);
  const int p0 = threadIdx.x * kPer;
  int bins[kPer];
  load_bins(b.bins + cd.coefOff + t.chunkStart, p0, len, t.dupV, bins);
  int tl[kPer];
  unsigned long long tb[kPer];
  thread_tokens(bins, p0, len, t, tl, tb, wFirst, wLast);
  unsigned mine = 0;
#pragma unroll
  for (int k = 0; k < kPer; k++) mine += tl[k];
  unsigned total;
  unsigned pos = block_excl_scan(mine, shs, total) + shift;
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    int l = tl[k];
    if (!l) continue;
    unsigned long long v = tb[k];
    unsigned p = pos;
    pos += l;
    // up to 61 bits starting anywhere in a word: at most 3 words
    while (l > 0) {
      const int o = p & 31;
      const int take = min(l, 32 - o);
      const unsigned chunkBits = (unsigned)(v & ((take == 32) ? 0xffffffffull : ((1ull << take) - 1)));
      atomicOr(&sw[p >> 5], chunkBits << o);
      v >>= take;
      p += take;
      l -= take;
    }
  }
  __syncthreads();
  uint32_t *gw = b.words + st->wordsBase + (chunkOff >> 5);
  for (int i = threadIdx.x; i < nW; i += kThreads) {
    if (i == 0 || i == nW - 1) {
      if (sw[i]) atomicOr(&gw[i], sw[i]);
    } else {
      gw[i] = sw[i];
    }
  }
}

}  // namespace

void launch_huffman_build(DevBatch &b, int maxSymbols, cudaStream_t s) {
  const size_t smem = build_smem_bytes(maxSymbols);
  cudaFuncSetAttribute(huffman_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  huffman_build_kernel<<<b.n, 1024, smem, s>>>(b);
}

void launch_encode(DevBatch &b, cudaStream_t s) {
  const unsigned chunks = (unsigned)b.totalChunks;
  encode_count_kernel<<<chunks, kThreads, 0, s>>>(b);
  encode_scan_kernel<<<b.n, 1024, 0, s>>>(b);
  cubelet_offsets_kernel<<<1, 1, 0, s>>>(b);
  encode_zero_kernel<<<(chunks + 255) / 256, 256, 0, s>>>(b);
  const int smem = kMaxChunkWords * 4;
  cudaFuncSetAttribute(encode_write_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  encode_write_kernel<<<chunks, kThreads, smem, s>>>(b);
}

}  // namespace wl
