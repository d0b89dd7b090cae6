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
// 4096-element chunk, chunk offsets are scanned per cubelet, and lanes pack
// slices of a chunk's tokens in registers (the bit packer below).
#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kMaxCodeBits = 58;  // + 3 dup bits fits 61 bits -> at most 3 words

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

// 256 threads: the merge, depths and decode table are one thread's work, so a
// small CTA lets every cubelet of a large batch build at once (eight CTAs per
// SM) instead of waiting for a second wave.
constexpr int kBuildThreads = 256;
__global__ void __launch_bounds__(kBuildThreads) huffman_build_kernel(DevBatch b) {
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
// A chunk's tokens, in stream order, are slots [span.x, span.x + span.y) of
// its token slot: the zero-run tokens entering it, its stored tokens and the
// zero-run tokens leaving it (quantize_kernel and runs_kernel put them there).

// ---- bit packer -------------------------------------------------------------
// A chunk's tokens are cut into F slices of ceil(n / F) tokens (F from
// enc_slices, per launch); lane s of the chunk's F lanes packs slice s, and a
// CTA of kEncThreads lanes takes kEncThreads / F consecutive chunks of one
// cubelet.  The bit
// counter sums each slice's code lengths and places the slices inside their
// chunk with an F-lane exclusive scan; the packer starts each slice at its
// chunk's offset (from the per-cubelet scan) plus that place.  A lane keeps
// its bits in a 64-bit register and stores whole words: words wholly inside
// its slice are stored directly, its first and last word (which it may share
// with neighbouring slices) are OR-ed in.  A word shared
// by slices of one chunk is zeroed by the lane whose slice starts in it,
// before any lane of the chunk ORs (the chunk's lanes are one warp); the
// chunk's first and last words, shared with neighbouring chunks, were zeroed
// by encode_zero_kernel.  Tokens are read with 16-byte loads: a slot starts
// at a multiple of 128 bytes and holds kChunk tokens, so the aligned blocks
// around a slice stay inside its chunk's slot.

// code bits (below kMaxCodeBits) and length (above) of one symbol
constexpr unsigned long long kCodeMask = (1ull << kMaxCodeBits) - 1;

// f(token, table entry) for tokens [a, e) of a slot, in order.  In a block
// of eight tokens that all lie in [a, e) the table entries are read before
// any is used; in the blocks at the ends only the tokens inside [a, e) are
// looked up (the other slots hold other slices' tokens or stale values).
template <class T, class Fn>
__device__ __forceinline__ void for_tokens(const uint16_t *slot, int a, int e, const T *tab,
                                           Fn &&f) {
  if (a >= e) return;
  const uint4 *p = reinterpret_cast<const uint4 *>(slot) + (a >> 3);
  const uint4 *pe = reinterpret_cast<const uint4 *>(slot) + ((e + 7) >> 3);
  for (int i = a & ~7; p < pe; p++, i += 8) {
    const uint4 q = *p;
    const unsigned w[4] = {q.x, q.y, q.z, q.w};
    if (i >= a && i + 8 <= e) {
      unsigned t[8];
      T en[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        t[k] = (w[k >> 1] >> (16 * (k & 1))) & 0xffffu;
        en[k] = tab[t[k] & 0x1fff];
      }
#pragma unroll
      for (int k = 0; k < 8; k++) f(t[k], en[k]);
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        if (i + k >= a && i + k < e) {
          const unsigned t = (w[k >> 1] >> (16 * (k & 1))) & 0xffffu;
          f(t, tab[t & 0x1fff]);
        }
      }
    }
  }
}

// Slice geometry shared by the bit counter and the packer: chunk `cl` of the
// cubelet (within its CTA's run), slice `sub` of it, tokens [t0, t1) of the
// chunk's token list.
struct SliceAt {
  int cl, sub, t0, t1;
  bool ok;        // the chunk exists
  long long chunk;
  int2 span;      // first token slot, token count
};
__device__ __forceinline__ SliceAt slice_at(const DevBatch &b, const CubeletDev &cd, int lgF) {
  SliceAt r;
  const int lane = threadIdx.x;
  r.cl = (((int)blockIdx.x - cd.encBase) << (7 - lgF)) + (lane >> lgF);
  r.sub = lane & ((1 << lgF) - 1);
  r.ok = r.cl < cd.nChunks;
  r.chunk = cd.chunkBase + r.cl;
  r.span = r.ok ? b.chunkSpan[r.chunk] : make_int2(0, 0);
  const int m = (r.span.y + (1 << lgF) - 1) >> lgF;
  r.t0 = min(r.span.y, r.sub * m);
  r.t1 = min(r.span.y, r.t0 + m);
  return r;
}

// Bits of every slice: lane s of a chunk's F lanes sums its tokens' code
// lengths, an F-lane exclusive scan places the slice inside the chunk
// (sliceOff), and the chunk's last lane writes the chunk's bit count.
__global__ void __launch_bounds__(kEncThreads) encode_count_kernel(DevBatch b) {
  extern __shared__ uint8_t sLen[];
  const int ci = b.encCub[blockIdx.x];
  const CubeletDev cd = b.cub[ci];
  const int lgF = __ffs(b.encF) - 1, F = 1 << lgF;
  const int dupKey = cd.binCount, S = cd.binCount + 1;
  for (int i = threadIdx.x; i < S; i += kEncThreads) sLen[i] = b.codeLen[(size_t)ci * kMaxSymbols + i];
  __syncthreads();
  const SliceAt sl = slice_at(b, cd, lgF);
  unsigned mine = 0;  // at most kChunk tokens of at most 61 bits
  if (sl.ok) {
    const uint16_t *slot = b.tok + cd.coefOff + (long long)sl.cl * kChunk;
    for_tokens(slot, sl.span.x + sl.t0, sl.span.x + sl.t1, sLen, [&](unsigned t, uint8_t l) {
      mine += l + ((int)(t & 0x1fff) == dupKey ? 3u : 0u);
    });
  }
  unsigned inc = mine;
  for (int d = 1; d < F; d <<= 1) {
    const unsigned x = __shfl_up_sync(0xffffffffu, inc, d, F);
    if (sl.sub >= d) inc += x;
  }
  if (sl.ok) {
    b.sliceOff[sl.chunk * 32 + sl.sub] = inc - mine;
    if (sl.sub == F - 1) b.chunkBits[sl.chunk] = inc;
  }
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

// packed word and metadata offsets of every cubelet: exclusive scans over
// the cubelets, 1024 at a time
__global__ void __launch_bounds__(1024) cubelet_offsets_kernel(DevBatch b) {
  __shared__ long long sw[32], sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long carryW = 0, carryM = 0;
  for (int base = 0; base < b.n; base += 1024) {
    const int i = base + threadIdx.x;
    long long vw = 0, vm = 0;
    if (i < b.n) {
      const CubeletState *st = b.state + i;
      vw = st->error ? 0 : st->nWords;
      vm = st->nDecode + (b.cub[i].quantAlg == WL_LLOYD ? st->nBounds + st->nValues : 0);
    }
    long long iw = vw, im = vm;
    for (int off = 1; off < 32; off <<= 1) {
      const long long tw = __shfl_up_sync(0xffffffffu, iw, off);
      const long long tm = __shfl_up_sync(0xffffffffu, im, off);
      if (lane >= off) { iw += tw; im += tm; }
    }
    if (lane == 31) { sw[w] = iw; sm[w] = im; }
    __syncthreads();
    long long bw = 0, bm = 0, tw = 0, tm = 0;
    for (int v = 0; v < 32; v++) {
      if (v < w) { bw += sw[v]; bm += sm[v]; }
      tw += sw[v];
      tm += sm[v];
    }
    if (i < b.n) {
      CubeletState *st = b.state + i;
      st->wordsBase = carryW + bw + iw - vw;
      st->metaBase = carryM + bm + im - vm;
    }
    carryW += tw;
    carryM += tm;
    __syncthreads();
  }
}

// decode table and Lloyd codebook of every cubelet into one buffer
__global__ void pack_meta_kernel(DevBatch b) {
  const int ci = blockIdx.x;
  const CubeletState *st = b.state + ci;
  const CubeletDev cd = b.cub[ci];
  int *m = b.meta + st->metaBase;
  const int *dec = b.decode + (size_t)ci * 4 * kMaxSymbols;
  for (int i = threadIdx.x; i < st->nDecode; i += blockDim.x) m[i] = dec[i];
  if (cd.quantAlg == WL_LLOYD) {
    const float *bnd = b.qtable + cd.tableOff;
    const float *val = b.dqtable + (size_t)ci * kMaxBins;
    for (int i = threadIdx.x; i < st->nBounds; i += blockDim.x)
      m[st->nDecode + i] = __float_as_int(bnd[i]);
    for (int i = threadIdx.x; i < st->nValues; i += blockDim.x)
      m[st->nDecode + st->nBounds + i] = __float_as_int(val[i]);
  }
}

// zero the first and last word of every chunk (the words chunks share)
__global__ void encode_zero_kernel(DevBatch b) {
  const long long chunk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (chunk >= b.totalChunks) return;
  const int ci = b.chunkCub[chunk];
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

__global__ void __launch_bounds__(kEncThreads, 8) encode_write_kernel(DevBatch b) {
  extern __shared__ unsigned long long sTab[];  // code | length << kMaxCodeBits
  const int ci = b.encCub[blockIdx.x];
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  if (st->error) return;
  const int lane = threadIdx.x;
  const int lgF = __ffs(b.encF) - 1, F = 1 << lgF;
  const int dupKey = cd.binCount, S = cd.binCount + 1;
  {
    const unsigned long long *gc = b.codes + (size_t)ci * kMaxSymbols;
    const uint8_t *gl = b.codeLen + (size_t)ci * kMaxSymbols;
    for (int i = lane; i < S; i += kEncThreads)
      sTab[i] = (gc[i] & kCodeMask) | ((unsigned long long)gl[i] << kMaxCodeBits);
  }
  __syncthreads();
  const SliceAt sl = slice_at(b, cd, lgF);
  unsigned long long off = 0, end = 0;
  if (sl.ok) {
    off = b.chunkBits[sl.chunk];
    end = sl.cl + 1 < cd.nChunks ? b.chunkBits[sl.chunk + 1] : st->totalBits;
  }
  // the slice's first bit and bit count
  const unsigned rel = sl.ok ? b.sliceOff[sl.chunk * 32 + sl.sub] : 0u;
  unsigned nxt = __shfl_down_sync(0xffffffffu, rel, 1, F);
  if (sl.sub == F - 1) nxt = (unsigned)(end - off);
  const unsigned long long sb = nxt - rel, pos = off + rel;
  const uint16_t *slot = b.tok + cd.coefOff + (long long)sl.cl * kChunk;
  uint32_t *gw = b.words + st->wordsBase;
  const bool any = sl.ok && sb > 0;
  if (any && F > 1) {
    const unsigned long long fw = pos >> 5;
    if (fw > (off >> 5) && fw < ((end - 1) >> 5)) gw[fw] = 0;
  }
  __syncwarp();
  if (!any) return;
  unsigned long long w = pos >> 5;
  const unsigned long long wFirst = w;
  unsigned long long acc = 0;  // bit 0 = bit 0 of word w
  int bits = (int)(pos & 31);
  for_tokens(slot, sl.span.x + sl.t0, sl.span.x + sl.t1, sTab,
             [&](unsigned t, unsigned long long e) {
    const int sym = t & 0x1fff;
    int l = (int)(e >> kMaxCodeBits);
    unsigned long long v = e & kCodeMask;
    if (sym == dupKey) {
      v |= (unsigned long long)(t >> 13) << l;
      l += 3;
    }
    // the common case: at most 32 bits, one OR into the accumulator (bits <
    // 32 here, and a code has no bits above its length)
    if (l <= 32) {
      acc |= v << bits;
      bits += l;
      if (bits >= 32) {
        if (w == wFirst) atomicOr(&gw[w], (unsigned)acc);
        else gw[w] = (unsigned)acc;
        w++;
        acc >>= 32;
        bits -= 32;
      }
      return;
    }
    // up to 61 bits, appended at most 32 at a time
    while (l > 0) {
      const int take = l < 32 ? l : 32;
      acc |= (v & ((1ull << take) - 1)) << bits;
      bits += take;
      v >>= take;
      l -= take;
      if (bits >= 32) {
        if (w == wFirst) atomicOr(&gw[w], (unsigned)acc);
        else gw[w] = (unsigned)acc;
        w++;
        acc >>= 32;
        bits -= 32;
      }
    }
  });
  if (bits > 0) atomicOr(&gw[w], (unsigned)acc);
}

}  // namespace

void launch_huffman_build(DevBatch &b, int maxSymbols, cudaStream_t s) {
  const size_t smem = build_smem_bytes(maxSymbols);
  raise_smem_limit(huffman_build_kernel, (int)smem);
  huffman_build_kernel<<<b.n, kBuildThreads, smem, s>>>(b);
}

void launch_pack_meta(DevBatch &b, cudaStream_t s) { pack_meta_kernel<<<b.n, 256, 0, s>>>(b); }

void launch_encode(DevBatch &b, int maxSymbols, cudaStream_t s) {
  const unsigned chunks = (unsigned)b.totalChunks;
  encode_count_kernel<<<(unsigned)b.totalEnc, kEncThreads, (maxSymbols + 15) & ~15, s>>>(b);
  encode_scan_kernel<<<b.n, 1024, 0, s>>>(b);
  cubelet_offsets_kernel<<<1, 1024, 0, s>>>(b);
  encode_zero_kernel<<<(chunks + 255) / 256, 256, 0, s>>>(b);
  const int smem = maxSymbols * (int)sizeof(unsigned long long);
  raise_smem_limit(encode_write_kernel, smem);
  encode_write_kernel<<<(unsigned)b.totalEnc, kEncThreads, smem, s>>>(b);
}

}  // namespace wl
