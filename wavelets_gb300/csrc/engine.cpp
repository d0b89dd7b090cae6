// libwlgpu engine: context, device workspace, batch planning and the C ABI.
//
// One call compresses a batch of cubelets of any sizes, dtypes and
// parameters with a fixed sequence of batched launches on the context's
// stream: transform (one launch per axis; the x pass once per input dtype),
// radix select, quantizer set-up, Lloyd (if any cubelet uses it), quantize +
// count, zero-run join, Huffman build, encode.  Cubelets that use the log
// quantizer need one host round trip after the select (their bin boundaries
// are computed with the host's logf, quant_host.cpp).  Device memory is a set
// of grow-only buffers owned by the context and reused across calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <map>
#include <unordered_map>
#include <mutex>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#include "cubelet_io.h"
#include "wl_internal.h"

using namespace wl;

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
};

int ceil_log2_int(int v) {
  int k = 0;
  while ((1 << k) < v) k++;
  return k;
}

// Per-cubelet plan computed on the host.
struct Plan {
  const void *data;
  int dtype;
  int X, Y, Z;
  wl_params p;
  int sx, sy, sz;
  int Xp, Yp, Zp;
  long long n;
  long long inOff;     // bytes into the input staging buffer (host inputs)
  long long coefOff;   // elements
  long long chunkBase;
  int nChunks;
  long long wordsCap;
  int tableOff;
  bool identity;       // all steps zero: no transform, no axis rotation
  bool cols;           // transform runs on the column-tile kernel
  bool two_d;          // -2d: x and y levels of every z layer, no rotation
  int sx2, sy2;        // 2-D mode: x / y levels actually applied
  long long pitchY, pitchZ;  // source elements between rows / slices
};

// Column-tile kernel for every lifting / Haar cubelet whose padded axes fit
// its tile; exact-order CDF 9/7 and longer rows use the row-cooperative one.
bool use_cols(int Xp, int Yp, int Zp, bool identity, const wl_params &p) {
  if (identity || (p.exact_transform && p.wavelet == WL_CDF97)) return false;
  return Xp <= kColsMaxL && Yp <= kColsMaxL && Zp <= kColsMaxL;
}

// Launch groups of one transform phase, keyed by (kernel, source type, row
// length class): a launch's shared memory is sized for its longest row, so
// rows of very different lengths go to different launches.
using PassGroups = std::map<int, std::vector<PassDesc>>;
int group_key(bool cols, int dtype, int L, bool vec = false) {
  return ((vec ? 1 : 0) << 13) | ((cols ? 1 : 0) << 12) | (dtype << 8) |
         (cols ? ceil_log2_int(L) : 0);
}
// row-register passes: one group per row length (and source type for the
// passes stored through a tile)
int rowreg_key(int L) { return (1 << 20) | L; }
int rowreg_t_key(int dtype, int L) { return (1 << 21) | (dtype << 16) | L; }
int rowreg_inv_key(int L) { return (1 << 23) | L; }
int rowreg_inv_t_key(int outType, int L) { return (1 << 24) | (outType << 16) | L; }
enum RegKind { kRegNone, kRegInPlace, kRegTile, kRegInvInPlace, kRegInvTile };

// ---- result storage ------------------------------------------------------------
// The arrays of all results of one compression call live in one page-locked
// slab that the device copies into directly (no host-side copy).  Every
// result holds a reference; the slab returns to a process-wide pool when the
// last one is released.
struct ResultSlab {
  std::atomic<int> refs{0};
  char *base = nullptr;
  size_t cap = 0;
};

class SlabPool {
 public:
  ResultSlab *acquire(size_t bytes) {
    {
      std::lock_guard<std::mutex> g(mu_);
      int bi = -1;
      for (int i = 0; i < (int)free_.size(); i++)
        if (free_[i]->cap >= bytes && (bi < 0 || free_[i]->cap < free_[bi]->cap)) bi = i;
      if (bi >= 0) {
        ResultSlab *s = free_[bi];
        free_.erase(free_.begin() + bi);
        return s;
      }
    }
    ResultSlab *s = new ResultSlab;
    // power-of-two sizes from 1 MiB, so that freed slabs fit later requests
    size_t cap = (size_t)1 << 20;
    while (cap < bytes) cap <<= 1;
    if (cudaHostAlloc(reinterpret_cast<void **>(&s->base), cap, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      return nullptr;
    }
    s->cap = cap;
    return s;
  }
  void release(ResultSlab *s) {
    std::lock_guard<std::mutex> g(mu_);
    free_.push_back(s);
    while (free_.size() > kKeep) {
      ResultSlab *o = free_.front();
      free_.erase(free_.begin());
      cudaFreeHost(o->base);
      delete o;
    }
  }

 private:
  static constexpr size_t kKeep = 16;  // free slabs kept for reuse
  std::mutex mu_;
  std::vector<ResultSlab *> free_;
};

// Host worker threads shared by every context (the log quantizer's boundary
// tables): started once, kept for the life of the process, so that a call
// does not pay for creating threads.  run(n, f) calls f(i) for i in [0, n)
// on the caller and the workers (about one per 8 items; fewer than 16 items
// run on the caller alone) and returns when all are done; calls from several
// host threads share the workers.
class HostPool {
 public:
  HostPool() {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int n = std::min(hw, 16) - 1;
    for (int i = 0; i < n; i++) threads_.emplace_back([this] { loop(); });
  }
  void run(int n, const std::function<void(int)> &f) {
    if (n <= 0) return;
    if (n < kMinShared) {  // a few items: on the caller, no thread woken
      for (int i = 0; i < n; i++) f(i);
      return;
    }
    auto job = std::make_shared<Job>();
    job->f = &f;
    job->n = n;
    if (!threads_.empty()) {
      std::lock_guard<std::mutex> g(mu_);
      jobs_.push_back(job);
      // wake about one worker per 8 items
      const int wake = std::min<int>((int)threads_.size(), (n + 7) / 8 - 1);
      for (int k = 0; k < wake; k++) cv_.notify_one();
    }
    work(*job);
    std::unique_lock<std::mutex> lk(job->mu);
    job->cv.wait(lk, [&] { return job->done == job->n; });
  }

 private:
  static constexpr int kMinShared = 16;  // fewer items run on the caller
  struct Job {
    const std::function<void(int)> *f = nullptr;
    int n = 0;
    std::atomic<int> next{0};
    int done = 0;
    std::mutex mu;
    std::condition_variable cv;
  };
  static void work(Job &j) {
    int k, mine = 0;
    while ((k = j.next.fetch_add(1)) < j.n) {
      (*j.f)(k);
      mine++;
    }
    if (mine) {
      std::lock_guard<std::mutex> g(j.mu);
      j.done += mine;
      if (j.done == j.n) j.cv.notify_all();
    }
  }
  void loop() {
    for (;;) {
      std::shared_ptr<Job> j;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !jobs_.empty(); });
        j = jobs_.front();
        if (j->next.load() >= j->n) {  // nothing left to take: retire it
          jobs_.pop_front();
          continue;
        }
      }
      work(*j);
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<Job>> jobs_;
  std::vector<std::thread> threads_;
};

// never destroyed: its threads live until the process exits
HostPool &host_pool() {
  static HostPool *p = new HostPool;
  return *p;
}

// never destroyed: results may be released during process teardown
SlabPool &slab_pool() {
  static SlabPool *p = new SlabPool;
  return *p;
}

int dtype_size(int dt) {
  switch (dt) {
    case WL_U8: return 1;
    case WL_U16: return 2;
    case WL_I32: return 4;
    case WL_F32: return 4;
    default: return 0;
  }
}

int ceil_log2(unsigned x) {  // ceilLog2 (dwt_cpu.cc:75-78)
  if (x == 0) return 0;
  int n = 0;
  unsigned v = x - 1;
  while (v) { n++; v >>= 1; }
  return n;
}

int padded_length(int len, int steps) {  // dwt_padded_length (dwt_cpu.cc:212-219)
  int mod = 1 << steps;
  return mod * ((len - 1) / mod + 1);
}

}  // namespace

namespace wl {
void raise_smem_limit(const void *func, int bytes) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> *limits = new std::unordered_map<const void *, int>;
  std::lock_guard<std::mutex> g(mu);
  int &cur = (*limits)[func];
  if (bytes <= cur) return;
  if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
    cur = bytes;
  else
    cudaGetLastError();  // the launch reports the error
}
}  // namespace wl

namespace {
// A captured compression of one batch geometry: the launch sequence, grids
// and kernel arguments are functions of the geometry (key) and of the
// context's buffers (gen); what changes from call to call -- input
// addresses, thresholds' host tables -- travels through the page-locked
// upload block and tables that the graph's copy nodes read at launch time.
struct GraphEntry {
  std::vector<long long> key;
  unsigned long long gen = 0;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int launches[2] = {0, 0};  // kernels in each segment
  unsigned long long lastUse = 0;
};
constexpr size_t kGraphCache = 4;
}  // namespace

struct wl_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  DevBuf input, coef, coef2, bins, tokCount, state, selHist, lloydHist, qtable, dqtable, qlut,
      hist, chunkRun, chunkRunCtx, chunkBits, chunkCub, groupCub, encCub, sliceOff, codes, codeLen, decode, chunkSpan,
      words, passes, logHdr, outbuf, decWords, decTable, decWs, meta, optIn, optOut, optErr,
      errIn, errRest, errPart;
  HostBuf hState, hDecode, hPasses, hTab, hLogHdr, hPrefix, hIn, hVals, hFlags;
  HostBuf hStage[2];  // staging buffers of the container pipeline
  // CUDA graphs: 0 = off, 1 = capture a batch geometry seen twice in a row
  // and replay it from then on
  int graphMode = 1;
  int stageHost = 0;  // copy page-locked inputs with the copy engine
  bool capturing = false;
  unsigned long long gen = 0;  // bumped whenever a buffer is reallocated
  unsigned long long useClock = 0;
  std::vector<GraphEntry> graphs;
  std::vector<long long> lastKey;
  unsigned long long lastGen = ~0ull;
  long long graphStats[4] = {0, 0, 0, 0};  // direct runs, captures, replays, capture failures
  std::string graphErr;
  cudaEvent_t ev[7] = {};
  // side streams for the independent launch groups of one transform phase
  static constexpr int kSide = 3;
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork = nullptr, join[kSide] = {};
  // second half of a large batch: its own stream, started when the first
  // half's transform has finished (halfT), joined back at the end (halfJ)
  cudaStream_t stream2 = nullptr;
  cudaEvent_t halfT = nullptr, halfJ = nullptr;
  cudaStream_t side2[kSide] = {};  // the second half's side streams
  cudaEvent_t fork2 = nullptr, join2[kSide] = {};
  int splitMode = 1;  // 1: split large batches into two staggered halves
  int encSlices = 0;  // bit-packer slices per chunk; 0: from the batch size
  float timings[6] = {0, 0, 0, 0, 0, 0};
  bool profiling = false;
  cudaEvent_t pev[10] = {};
  float ktimes[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int launches = 0;
  size_t devBytes = 0;     // device workspace held (grow-only buffers)
  size_t memLimit = 0;     // wl_set_memory_limit (0: none)
};

namespace {

wl_status fail(wl_ctx *c, wl_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return s;
}

#define CU(expr)                                                               \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return fail(ctx, WL_ECUDA, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

wl_status ensure(wl_ctx *ctx, DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return WL_OK;
  size_t want = bytes + bytes / 4;
  if (ctx->memLimit) {
    // the context's workspace cap: grow to what is needed, no slack, and
    // fail before freeing anything
    const size_t others = ctx->devBytes - b.cap;
    if (others + bytes > ctx->memLimit)
      return fail(ctx, WL_ENOMEM, "device workspace limit of %zu bytes reached (%zu held, %zu "
                  "more needed)", ctx->memLimit, ctx->devBytes, bytes - b.cap);
    if (others + want > ctx->memLimit) want = bytes;
  }
  if (b.p) cudaFree(b.p);
  ctx->devBytes -= b.cap;
  b.p = nullptr;
  b.cap = 0;
  ctx->gen++;
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ENOMEM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
  }
  b.cap = want;
  ctx->devBytes += want;
  return WL_OK;
}

wl_status ensure_host(wl_ctx *ctx, HostBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return WL_OK;
  if (b.p) cudaFreeHost(b.p);
  b.p = nullptr;
  b.cap = 0;
  ctx->gen++;
  size_t want = bytes + bytes / 4;
  cudaError_t e = cudaMallocHost(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, WL_ENOMEM, "cudaMallocHost(%zu) failed: %s", want, cudaGetErrorString(e));
  }
  b.cap = want;
  return WL_OK;
}

#define TRY(expr)                          \
  do {                                     \
    wl_status s_ = (expr);                 \
    if (s_ != WL_OK) return s_;            \
  } while (0)

template <class T> T *P(DevBuf &b) { return static_cast<T *>(b.p); }

// An event record on the context's stream; during graph capture an event
// node, so that replays record it too.
inline cudaError_t record(wl_ctx *ctx, cudaEvent_t e) {
  return ctx->capturing ? cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal)
                        : cudaEventRecord(e, ctx->stream);
}

// kernel-group boundary for the optional per-group timings
inline void mark(wl_ctx *ctx, int i) {
  if (ctx->profiling) record(ctx, ctx->pev[i]);
}
template <class T> T *H(HostBuf &b) { return static_cast<T *>(b.p); }

void drop_graph(GraphEntry &g) {
  for (cudaGraphExec_t &x : g.exec)
    if (x) {
      cudaGraphExecDestroy(x);
      x = nullptr;
    }
}

// The cached graph of this batch geometry, a new (empty) entry when the
// geometry repeats the previous call's, else null: batches that never repeat
// (serving) run directly and pay no capture.
GraphEntry *graph_for(wl_ctx *ctx, std::vector<long long> &&key) {
  // entries of reallocated buffers can never match again
  for (size_t i = 0; i < ctx->graphs.size();) {
    if (ctx->graphs[i].gen != ctx->gen) {
      drop_graph(ctx->graphs[i]);
      ctx->graphs.erase(ctx->graphs.begin() + i);
    } else {
      i++;
    }
  }
  for (GraphEntry &g : ctx->graphs)
    if (g.key == key) {
      g.lastUse = ++ctx->useClock;
      return &g;
    }
  const bool repeat = ctx->lastGen == ctx->gen && ctx->lastKey == key;
  if (!repeat) {
    ctx->lastKey = std::move(key);
    ctx->lastGen = ctx->gen;
    return nullptr;
  }
  if (ctx->graphs.size() >= kGraphCache) {
    size_t lru = 0;
    for (size_t i = 1; i < ctx->graphs.size(); i++)
      if (ctx->graphs[i].lastUse < ctx->graphs[lru].lastUse) lru = i;
    drop_graph(ctx->graphs[lru]);
    ctx->graphs.erase(ctx->graphs.begin() + lru);
  }
  ctx->graphs.emplace_back();
  GraphEntry &g = ctx->graphs.back();
  g.key = std::move(key);
  g.gen = ctx->gen;
  g.lastUse = ++ctx->useClock;
  return &g;
}

// Run one segment of device work: directly, by replaying its graph, or by
// capturing the graph first.  A capture that fails turns graphs off for the
// context (the reason is kept) and the segment runs directly.
template <class F> wl_status run_segment(wl_ctx *ctx, GraphEntry *ge, int seg, F &&enqueue) {
  cudaStream_t s = ctx->stream;
  if (!ge || !ctx->graphMode) {
    ctx->graphStats[0]++;
    return enqueue();
  }
  if (ge->exec[seg]) {
    ctx->graphStats[2]++;
    ctx->launches += ge->launches[seg];
    CU(cudaGraphLaunch(ge->exec[seg], s));
    return WL_OK;
  }
  CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  ctx->capturing = true;
  const int launches = ctx->launches;
  const wl_status st = enqueue();
  ctx->capturing = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (st == WL_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge->exec[seg], g, 0);
  if (g) cudaGraphDestroy(g);
  if (st == WL_OK && e == cudaSuccess) {
    ctx->graphStats[1]++;
    ge->launches[seg] = ctx->launches - launches;
    CU(cudaGraphLaunch(ge->exec[seg], s));
    return WL_OK;
  }
  // capture failed: nothing was enqueued; run the segment directly
  ge->exec[seg] = nullptr;
  cudaGetLastError();
  ctx->graphStats[3]++;
  ctx->graphErr = st != WL_OK ? ctx->err : cudaGetErrorString(e);
  ctx->graphMode = 0;
  ctx->launches = launches;
  ctx->graphStats[0]++;
  return enqueue();
}

wl_status check_params(wl_ctx *ctx, const wl_params &p) {
  if (p.wavelet != WL_HAAR && p.wavelet != WL_CDF97)
    return fail(ctx, WL_EINVAL, "unknown wavelet %d", p.wavelet);
  if (p.quant_alg != WL_UNIFORM && p.quant_alg != WL_LOG && p.quant_alg != WL_LLOYD)
    return fail(ctx, WL_EINVAL, "unknown quantization algorithm %d", p.quant_alg);
  if (p.bin_count < 2 || p.bin_count > kMaxBins)
    return fail(ctx, WL_EINVAL, "bin count %d outside 2..%d", p.bin_count, kMaxBins);
  if (!(p.threshold_fraction >= 0.f && p.threshold_fraction <= 1.f))
    return fail(ctx, WL_EINVAL, "threshold fraction %g outside [0,1]", p.threshold_fraction);
  if (p.quant_alg == WL_LLOYD && p.bin_count < 3)
    return fail(ctx, WL_EINVAL, "Lloyd quantization needs at least 3 bins");
  return WL_OK;
}

// Build PassDescs for one cubelet's forward transform.
// Column-tile layouts: x pass [raw x-y-z] -> z-y-x, y pass z-y-x -> z-x-y,
// z pass z-x-y in place (a-b-c lists axes from fastest to slowest).  Rows
// are numbered so that neighbouring rows are neighbours in memory on every
// side whose element stride is not 1.
// selHist / selState: the cubelet's select histogram and state; a z pass on
// the row-register kernel, the last pass, gathers the first select digit and
// the extremes into them.  Returns true when it does.
bool forward_passes_cols(const Plan &pl, const void *in, bool hostIn, float *coef, float *coef2,
                         PassGroups &xs, PassGroups &ys, PassGroups &zs,
                         unsigned *selHist = nullptr, CubeletState *selState = nullptr) {
  const int big = 0x7fffffff;
  const long long Xp = pl.Xp, Yp = pl.Yp, Zp = pl.Zp;
  float *o = coef + pl.coefOff;
  float *o2 = coef2 + pl.coefOff;
  PassDesc d;
  memset(&d, 0, sizeof d);
  d.cropL = d.cropB = d.cropA = big;
  d.wavelet = pl.p.wavelet;
  // x pass: rows (a = y, b = z) of the source, REPEAT padding by clamping,
  // to z-y-x (z fastest): consecutive rows are neighbours in the output
  d.in = in;
  d.vecLoad = hostIn ? 1 : 0;
  d.inSA = pl.pitchY; d.inSB = pl.pitchZ; d.inSC = 1;
  d.clampL = pl.X; d.clampA = pl.Y; d.clampB = pl.Z;
  d.L = pl.Xp; d.B = pl.Zp; d.rows = (int)(Yp * Zp);
  d.out = o2;
  d.outSA = Zp; d.outSB = 1; d.outSC = Zp * Yp;
  d.steps = pl.sx;
  if (dwt_rowreg_fits(d.L, d.steps)) {
    d.T = dwt_rowreg_t_rows_per_block(d.L); d.tiles = (d.rows + d.T - 1) / d.T;
    xs[rowreg_t_key(pl.dtype, d.L)].push_back(d);
  } else {
    d.T = dwt_cols_tile_rows(d.L); d.tiles = (d.rows + d.T - 1) / d.T;
    xs[group_key(true, pl.dtype, d.L, hostIn && dtype_size(pl.dtype) < 4)].push_back(d);
  }
  // y pass: rows (a = x, b = z) of z-y-x -> z-x-y (column tiles: rows that
  // are neighbours in memory on both sides)
  PassDesc e = d;
  e.clampL = e.clampB = e.clampA = big;
  e.vecLoad = 0;
  e.in = o2;
  e.inSA = Zp * Yp; e.inSB = 1; e.inSC = Zp;
  e.L = pl.Yp; e.B = pl.Zp; e.rows = (int)(Zp * Xp);
  e.out = o;
  e.outSA = Zp; e.outSB = 1; e.outSC = Zp * Xp;
  e.steps = pl.sy;
  e.T = dwt_cols_tile_rows(e.L); e.tiles = (e.rows + e.T - 1) / e.T;
  ys[group_key(true, WL_F32, e.L)].push_back(e);
  if (pl.sz == 0) return false;
  // z pass: rows (a = y, b = x) of z-x-y, in place
  PassDesc f = e;
  f.in = o;
  f.inSA = Zp * Xp; f.inSB = Zp; f.inSC = 1;
  f.L = pl.Zp; f.B = pl.Xp; f.rows = (int)(Xp * Yp);
  f.out = o;
  f.outSA = Zp * Xp; f.outSB = Zp; f.outSC = 1;
  f.steps = pl.sz;
  if (dwt_rowreg_fits(f.L, f.steps)) {
    f.selHist = selHist;
    f.selState = selState;
    f.T = dwt_rowreg_rows_per_block(f.L, selHist != nullptr);
    f.tiles = (f.rows + f.T - 1) / f.T;
    zs[rowreg_key(f.L)].push_back(f);
    return selHist != nullptr;
  }
  f.T = dwt_cols_tile_rows(f.L); f.tiles = (f.rows + f.T - 1) / f.T;
  zs[group_key(true, WL_F32, f.L)].push_back(f);
  return false;
}

// 2-D mode (cdf97_2d / haar_2d, dwt_cpu.cc:811-864 and :495-547): x and y
// step counts below 1 or above the maximum become the maximum for the padded
// length; false when the padded size does not suit them (the reference then
// leaves the layers untransformed).
bool twod_steps(int Xp, int Yp, int sx, int sy, int &sx2, int &sy2) {
  const int mx = ceil_log2((unsigned)Xp), my = ceil_log2((unsigned)Yp);
  sx2 = (sx < 1 || sx > mx) ? mx : sx;
  sy2 = (sy < 1 || sy > my) ? my : sy;
  return Xp % (1 << sx2) == 0 && Yp % (1 << sy2) == 0;
}

// 2-D mode passes (both kernels): x pass raw x-y-z (REPEAT clamp) -> coef2 in
// [z][x][y] (y fastest), y pass [z][x][y] -> coef in [z][y][x], the stored
// order (x fastest).  Both read rows contiguous in memory.
void forward_passes_2d(const Plan &pl, const void *in, bool hostIn, float *coef, float *coef2,
                       PassGroups &xs, PassGroups &ys) {
  const int big = 0x7fffffff;
  const long long Xp = pl.Xp, Yp = pl.Yp, Zp = pl.Zp;
  const bool exact = pl.p.exact_transform && pl.p.wavelet == WL_CDF97;
  PassDesc d;
  memset(&d, 0, sizeof d);
  d.cropL = d.cropB = d.cropA = big;
  d.wavelet = pl.p.wavelet;
  d.exact = pl.p.exact_transform;
  // x pass: rows (a = z, b = y) of the source
  d.in = in;
  d.vecLoad = pl.cols && hostIn ? 1 : 0;
  d.inSA = pl.pitchZ; d.inSB = pl.pitchY; d.inSC = 1;
  d.clampL = pl.X; d.clampA = pl.Z; d.clampB = pl.Y;
  d.L = pl.Xp; d.B = pl.Yp; d.rows = (int)(Yp * Zp);
  d.out = coef2 + pl.coefOff;
  d.outSA = Xp * Yp; d.outSB = 1; d.outSC = Yp;
  d.steps = pl.sx2;
  d.T = pl.cols ? dwt_cols_tile_rows(d.L) : dwt_tile_rows(d.L, exact);
  d.tiles = (d.rows + d.T - 1) / d.T;
  xs[group_key(pl.cols, pl.dtype, d.L, pl.cols && hostIn && dtype_size(pl.dtype) < 4)]
      .push_back(d);
  // y pass: rows (a = z, b = x) of [z][x][y]
  PassDesc e = d;
  e.clampL = e.clampA = e.clampB = big;
  e.vecLoad = 0;
  e.in = coef2 + pl.coefOff;
  e.inSA = Xp * Yp; e.inSB = Yp; e.inSC = 1;
  e.L = pl.Yp; e.B = pl.Xp; e.rows = (int)(Xp * Zp);
  e.out = coef + pl.coefOff;
  e.outSA = Xp * Yp; e.outSB = 1; e.outSC = Xp;
  e.steps = pl.sy2;
  e.T = pl.cols ? dwt_cols_tile_rows(e.L) : dwt_tile_rows(e.L, exact);
  e.tiles = (e.rows + e.T - 1) / e.T;
  ys[group_key(pl.cols, WL_F32, e.L)].push_back(e);
}

// Returns true when the last pass gathers the first select digit and the
// extremes (see forward_passes_cols).
bool forward_passes(const Plan &pl, const void *in, bool hostIn, float *coef, float *coef2,
                    PassGroups &xs, PassGroups &ys, PassGroups &zs, unsigned *selHist = nullptr,
                    CubeletState *selState = nullptr) {
  if (pl.two_d && !pl.identity) {
    forward_passes_2d(pl, in, hostIn, coef, coef2, xs, ys);
    return false;
  }
  if (pl.cols)
    return forward_passes_cols(pl, in, hostIn, coef, coef2, xs, ys, zs, selHist, selState);
  const int big = 0x7fffffff;
  const float *c = coef + pl.coefOff;
  float *o = coef + pl.coefOff;
  float *o2 = coef2 + pl.coefOff;
  const long long Xp = pl.Xp, Yp = pl.Yp, Zp = pl.Zp;
  PassDesc d;
  memset(&d, 0, sizeof d);
  d.cropL = d.cropB = d.cropA = big;
  // x pass: rows (z, y) of the source, REPEAT padding by clamping
  d.in = in;
  d.inSA = pl.pitchZ;
  d.inSB = pl.pitchY;
  d.inSC = 1;
  d.clampL = pl.X; d.clampB = pl.Y; d.clampA = pl.Z;
  d.L = pl.Xp; d.B = pl.Yp; d.rows = (int)(Yp * Zp);
  d.wavelet = pl.p.wavelet; d.exact = pl.p.exact_transform;
  if (pl.identity) {
    d.out = o;
    d.outSA = Xp * Yp; d.outSB = Xp; d.outSC = 1;
    d.steps = 0;
  } else {
    d.out = o2;                       // x-y-z -> y-z-x
    d.outSA = Yp; d.outSB = 1; d.outSC = Yp * Zp;
    d.steps = pl.sx;
  }
  d.T = dwt_tile_rows(d.L, d.exact && d.wavelet == WL_CDF97);
  d.tiles = (d.rows + d.T - 1) / d.T;
  xs[group_key(false, pl.dtype, d.L)].push_back(d);
  if (pl.identity) return false;
  // y pass: rows (x, z) of the y-z-x cube -> z-x-y
  PassDesc e;
  memset(&e, 0, sizeof e);
  e.cropL = e.cropB = e.cropA = big;
  e.clampL = e.clampB = e.clampA = big;
  e.in = o2;
  e.inSA = Zp * Yp; e.inSB = Yp; e.inSC = 1;
  e.L = pl.Yp; e.B = pl.Zp; e.rows = (int)(Zp * Xp);
  e.out = o;
  e.outSA = Zp; e.outSB = 1; e.outSC = Zp * Xp;
  e.steps = pl.sy; e.wavelet = pl.p.wavelet; e.exact = pl.p.exact_transform;
  e.T = dwt_tile_rows(e.L, e.exact && e.wavelet == WL_CDF97);
  e.tiles = (e.rows + e.T - 1) / e.T;
  ys[group_key(false, WL_F32, e.L)].push_back(e);
  if (pl.sz == 0) return false;
  // z pass: rows (y, x) of the z-x-y cube, in place
  PassDesc f = e;
  f.in = c;
  f.inSA = Xp * Zp; f.inSB = Zp;
  f.L = pl.Zp; f.B = pl.Xp; f.rows = (int)(Xp * Yp);
  f.out = o;
  f.outSA = Xp * Zp; f.outSB = Zp; f.outSC = 1;
  f.steps = pl.sz;
  f.T = dwt_tile_rows(f.L, f.exact && f.wavelet == WL_CDF97);
  f.tiles = (f.rows + f.T - 1) / f.T;
  zs[group_key(false, WL_F32, f.L)].push_back(f);
  return false;
}

// One launch of a transform pass group: its descriptors and tile prefix sit
// at `off` bytes into the context's upload block.
struct GroupLaunch {
  size_t off;
  int n, tiles, smem, rows, warps, inType, outType;
  bool inverse, cols, vec;
  int regL;  // row-register pass of rows of regL elements (0: another kernel)
  int regKind;  // which row-register kernel (RegKind)
  bool sel;     // in-place row-register pass gathering the select statistics
  // bytes a launch moves, for ordering concurrent groups
  double weight() const { return (double)tiles * (regL ? 4.0 * regL * rows : (double)smem); }
};

// Stage a group of passes (descriptors + tile prefix) at hoff of the host
// upload block and note its launch.  Column-tile groups take the tile shape
// of their size class from the tile table (kind: the pass) unless one is
// forced.
wl_status stage_group(wl_ctx *ctx, std::vector<PassDesc> g, size_t &hoff, int kind, int inType,
                      int outType, bool inverse, bool cols, bool vec,
                      std::vector<GroupLaunch> &out, const TileShape *force = nullptr,
                      int regL = 0, int regKind = kRegNone) {
  if (g.empty()) return WL_OK;
  const size_t n = g.size();
  const size_t bytes = n * sizeof(PassDesc) + (n + 1) * sizeof(int);
  if (hoff + bytes > ctx->hPasses.cap || hoff + bytes > ctx->passes.cap)
    return fail(ctx, WL_ENOMEM, "pass staging too small");
  int rows = 0, warps = 4;
  const bool sel = regKind == kRegInPlace && g[0].selHist != nullptr;
  for (const PassDesc &d : g)
    if ((d.selHist != nullptr) != sel)
      return fail(ctx, WL_EINVAL, "internal: mixed select-gathering passes in one group");
  if (regL) {
    rows = (regKind == kRegTile || regKind == kRegInvTile) ? dwt_rowreg_t_rows_per_block(regL)
                                                          : dwt_rowreg_rows_per_block(regL, sel);
    for (PassDesc &d : g) {
      d.T = rows;
      d.tiles = (d.rows + rows - 1) / rows;
    }
  } else if (cols) {
    int Lmax = 0;
    for (const PassDesc &d : g) Lmax = std::max(Lmax, d.L);
    const int gtype = kind == kTuneFwdX ? inType : kind == kTuneInvX ? outType : WL_F32;
    const TileShape t = force ? *force : tuned_cols_shape(kind, tune_type_index(gtype, vec), Lmax);
    rows = t.rows;
    warps = t.warps;
    for (PassDesc &d : g) {
      d.T = rows;
      d.tiles = (d.rows + rows - 1) / rows;
    }
  }
  char *h = H<char>(ctx->hPasses) + hoff;
  memcpy(h, g.data(), n * sizeof(PassDesc));
  int *tp = reinterpret_cast<int *>(h + n * sizeof(PassDesc));
  int tiles = 0, smem = 0;
  for (size_t i = 0; i < n; i++) {
    tp[i] = tiles;
    tiles += g[i].tiles;
    if (!regL)
      smem = std::max(smem, cols ? dwt_cols_smem_bytes(g[i].L, rows)
                                 : dwt_smem_bytes(g[i].L, g[i].T,
                                                  g[i].exact && g[i].wavelet == WL_CDF97));
  }
  tp[n] = tiles;
  out.push_back({hoff, (int)n, tiles, smem, rows, warps, inType, outType, inverse, cols, vec,
                 regL, regKind, sel});
  hoff += (bytes + 255) & ~(size_t)255;
  return WL_OK;
}

// Stage every group of one transform phase.
wl_status stage_groups(wl_ctx *ctx, const PassGroups &gs, size_t &hoff, int kind, int outType,
                       bool inverse, std::vector<GroupLaunch> &out) {
  for (const auto &kv : gs) {
    const bool regT = (kv.first >> 21) & 1;
    const int regL = regT || ((kv.first >> 20) & 1) ? kv.second[0].L : 0;
    const int regKind = regT ? kRegTile : regL ? kRegInPlace : kRegNone;
    const bool cols = !regL && ((kv.first >> 12) & 1), vec = !regL && ((kv.first >> 13) & 1);
    const int dt = regT ? (kv.first >> 16) & 15 : regL ? WL_F32 : (kv.first >> 8) & 15;
    TRY(stage_group(ctx, kv.second, hoff, kind, inverse ? WL_F32 : dt, outType, inverse, cols, vec,
                    out, nullptr, regL, regKind));
  }
  return WL_OK;
}

wl_status launch_one(wl_ctx *ctx, const GroupLaunch &l, cudaStream_t s) {
  const char *base = P<char>(ctx->passes);
  const PassDesc *dp = reinterpret_cast<const PassDesc *>(base + l.off);
  const int *dtp = reinterpret_cast<const int *>(base + l.off + l.n * sizeof(PassDesc));
  if (l.regKind == kRegTile)
    launch_dwt_rowreg_t(dp, dtp, l.n, l.tiles, l.regL, l.inType, s);
  else if (l.regKind == kRegInvInPlace)
    launch_dwt_rowreg_inv(dp, dtp, l.n, l.tiles, l.regL, s);
  else if (l.regKind == kRegInvTile)
    launch_dwt_rowreg_inv_t(dp, dtp, l.n, l.tiles, l.regL, l.outType, s);
  else if (l.regL)
    launch_dwt_rowreg(dp, dtp, l.n, l.tiles, l.regL, l.sel, s);
  else if (l.cols)
    launch_dwt_cols(dp, dtp, l.n, l.tiles, l.smem, l.rows, l.warps, l.inType, l.outType, l.inverse,
                    l.vec, s);
  else
    launch_dwt_pass(dp, dtp, l.n, l.tiles, l.smem, l.inType, l.outType, l.inverse, s);
  CU(cudaGetLastError());
  ctx->launches++;
  return WL_OK;
}

// Launch staged groups [a, b) whose descriptors are already on the device,
// in order on the context's stream.
wl_status launch_groups(wl_ctx *ctx, const std::vector<GroupLaunch> &ls, size_t a, size_t b) {
  for (size_t i = a; i < b; i++) TRY(launch_one(ctx, ls[i], ctx->stream));
  return WL_OK;
}

// Launch the groups [a, b) of one transform phase concurrently.  They touch
// disjoint cubelets, so they fork from the context's stream onto it and the
// side streams (largest first, dealt round-robin), and the phase joins back
// before anything later in the stream runs.  Small groups -- a few hundred
// tiles of short rows -- fill the SMs that a lone launch of them would leave
// idle.
wl_status launch_phase_on(wl_ctx *ctx, const std::vector<GroupLaunch> &ls, size_t a, size_t b,
                          cudaStream_t main, cudaStream_t *side, cudaEvent_t fork,
                          cudaEvent_t *join) {
  if (b - a <= 1 || !fork) {
    for (size_t i = a; i < b; i++) TRY(launch_one(ctx, ls[i], main));
    return WL_OK;
  }
  std::vector<size_t> order;
  for (size_t i = a; i < b; i++) order.push_back(i);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return ls[x].weight() > ls[y].weight();
  });
  const int nStreams = (int)std::min<size_t>(order.size(), wl_ctx::kSide + 1);
  CU(cudaEventRecord(fork, main));
  for (int k = 1; k < nStreams; k++) CU(cudaStreamWaitEvent(side[k - 1], fork, 0));
  for (size_t j = 0; j < order.size(); j++) {
    const int k = (int)(j % nStreams);
    TRY(launch_one(ctx, ls[order[j]], k ? side[k - 1] : main));
  }
  for (int k = 1; k < nStreams; k++) {
    CU(cudaEventRecord(join[k - 1], side[k - 1]));
    CU(cudaStreamWaitEvent(main, join[k - 1], 0));
  }
  return WL_OK;
}

wl_status launch_phase(wl_ctx *ctx, const std::vector<GroupLaunch> &ls, size_t a, size_t b) {
  if (b - a <= 1 || !ctx->fork) return launch_groups(ctx, ls, a, b);
  std::vector<size_t> order;
  for (size_t i = a; i < b; i++) order.push_back(i);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return ls[x].weight() > ls[y].weight();
  });
  const int nStreams = (int)std::min<size_t>(order.size(), wl_ctx::kSide + 1);
  CU(cudaEventRecord(ctx->fork, ctx->stream));
  for (int k = 1; k < nStreams; k++) CU(cudaStreamWaitEvent(ctx->side[k - 1], ctx->fork, 0));
  for (size_t j = 0; j < order.size(); j++) {
    const int k = (int)(j % nStreams);
    TRY(launch_one(ctx, ls[order[j]], k ? ctx->side[k - 1] : ctx->stream));
  }
  for (int k = 1; k < nStreams; k++) {
    CU(cudaEventRecord(ctx->join[k - 1], ctx->side[k - 1]));
    CU(cudaStreamWaitEvent(ctx->stream, ctx->join[k - 1], 0));
  }
  return WL_OK;
}

int pb_dtype(int dt) {  // data type as the reference stores it
  if (dt == WL_U8) return kPbUint8;
  if (dt == WL_F32) return kPbFloat32;
  return kPbInt32;  // I32 and U16 (16-bit data travels as INT32)
}

wl_status compress_impl(wl_ctx *ctx, const wl_cubelet *items, int n, int onDevice,
                        wl_result *outs, float *coefOut = nullptr, size_t coefCap = 0,
                        int *storedSize = nullptr) {
  if (n <= 0) return fail(ctx, WL_EINVAL, "empty batch");
  CU(cudaSetDevice(ctx->device));
  std::vector<Plan> plans(n);
  long long coefTotal = 0, chunkTotal = 0, inBytes = 0, wordsTotal = 0;
  int tableTotal = 0, maxS = 2, maxTable = 0, maxLloyd = 3;
  bool anyLog = false, anyLloyd = false;
  for (int i = 0; i < n; i++) {
    const wl_cubelet &it = items[i];
    Plan &pl = plans[i];
    TRY(check_params(ctx, it.params));
    if (!it.data) return fail(ctx, WL_EINVAL, "cubelet %d: null data", i);
    if (dtype_size(it.dtype) == 0) return fail(ctx, WL_EINVAL, "cubelet %d: bad dtype %d", i, it.dtype);
    pl.data = it.data;
    pl.dtype = it.dtype;
    pl.X = it.size[0]; pl.Y = it.size[1]; pl.Z = it.size[2];
    if (pl.X < 1 || pl.Y < 1 || pl.Z < 1)
      return fail(ctx, WL_EINVAL, "cubelet %d: empty size %dx%dx%d", i, pl.X, pl.Y, pl.Z);
    pl.pitchY = it.row_pitch ? it.row_pitch : pl.X;
    pl.pitchZ = it.slice_pitch ? it.slice_pitch : pl.pitchY * pl.Y;
    if (pl.pitchY < pl.X || pl.pitchZ < pl.pitchY * pl.Y)
      return fail(ctx, WL_EINVAL, "cubelet %d: pitches %lld, %lld smaller than its rows/slices",
                  i, pl.pitchY, pl.pitchZ);
    pl.p = it.params;
    // setWaveletSteps (test_compress_common.cc:362-374)
    int m;
    m = ceil_log2(pl.X); pl.sx = (pl.p.steps[0] < 0 || pl.p.steps[0] > m) ? m : pl.p.steps[0];
    m = ceil_log2(pl.Y); pl.sy = (pl.p.steps[1] < 0 || pl.p.steps[1] > m) ? m : pl.p.steps[1];
    m = ceil_log2(pl.Z); pl.sz = (pl.p.steps[2] < 0 || pl.p.steps[2] > m) ? m : pl.p.steps[2];
    pl.Xp = padded_length(pl.X, pl.sx);
    pl.Yp = padded_length(pl.Y, pl.sy);
    pl.Zp = padded_length(pl.Z, pl.sz);
    pl.identity = pl.sx == 0 && pl.sy == 0 && pl.sz == 0;
    pl.two_d = pl.p.transform_2d != 0;
    pl.sx2 = pl.sy2 = 0;
    if (pl.two_d) {
      if (!pl.identity && !twod_steps(pl.Xp, pl.Yp, pl.sx, pl.sy, pl.sx2, pl.sy2))
        pl.identity = true;  // the reference leaves such layers as they are
      pl.cols = !pl.identity && !(pl.p.exact_transform && pl.p.wavelet == WL_CDF97) &&
                pl.Xp <= kColsMaxL && pl.Yp <= kColsMaxL;
    } else {
      pl.cols = use_cols(pl.Xp, pl.Yp, pl.Zp, pl.identity, pl.p);
    }
    if (pl.Xp > kMaxAxis || pl.Yp > kMaxAxis || pl.Zp > kMaxAxis)
      return fail(ctx, WL_EINVAL, "cubelet %d: padded axis length above %d", i, kMaxAxis);
    pl.n = (long long)pl.Xp * pl.Yp * pl.Zp;
    if (pl.n > 0x7fffffffLL) return fail(ctx, WL_EINVAL, "cubelet %d too large", i);
    pl.inOff = inBytes;
    inBytes += ((long long)pl.X * pl.Y * pl.Z * dtype_size(pl.dtype) + 255) & ~255LL;
    pl.coefOff = coefTotal;
    coefTotal += (pl.n + 63) & ~63LL;
    pl.chunkBase = chunkTotal;
    pl.nChunks = (int)((pl.n + kChunk - 1) / kChunk);
    chunkTotal += pl.nChunks;
    // Huffman output bound: < log2(symbols)+1 bits per token plus 3 per dup token
    pl.wordsCap = pl.n / 2 + 64;
    wordsTotal += pl.wordsCap;
    pl.tableOff = tableTotal;
    tableTotal += ((2 * pl.p.bin_count + 2) + 63) & ~63;
    maxS = std::max(maxS, pl.p.bin_count + 1);
    if (pl.p.quant_alg == WL_LLOYD) maxTable = std::max(maxTable, pl.p.bin_count);
    if (pl.p.quant_alg == WL_LLOYD) maxLloyd = std::max(maxLloyd, pl.p.bin_count);
    if (pl.p.quant_alg == WL_LOG) maxTable = std::max(maxTable, 2 * pl.p.bin_count);
    if (pl.p.quant_alg == WL_LOG) anyLog = true;
    if (pl.p.quant_alg == WL_LLOYD) anyLloyd = true;
  }

  // ---- workspace ----
  TRY(ensure(ctx, ctx->coef, coefTotal * 4));
  TRY(ensure(ctx, ctx->coef2, coefTotal * 4));
  TRY(ensure(ctx, ctx->bins, (coefTotal + (long long)n * kChunk) * 2));
  TRY(ensure(ctx, ctx->tokCount, chunkTotal * sizeof(int)));
  TRY(ensure(ctx, ctx->state, n * sizeof(CubeletState)));
  TRY(ensure(ctx, ctx->chunkCub, chunkTotal * sizeof(int)));
  TRY(ensure(ctx, ctx->groupCub, chunkTotal * sizeof(int)));
  TRY(ensure(ctx, ctx->encCub, chunkTotal * sizeof(int)));
  TRY(ensure(ctx, ctx->sliceOff, chunkTotal * 32 * sizeof(unsigned)));
  TRY(ensure(ctx, ctx->selHist, (size_t)n * kSelectBins * 4));
  if (anyLloyd) TRY(ensure(ctx, ctx->lloydHist, (size_t)n * kLloydBins * 4));
  TRY(ensure(ctx, ctx->qtable, (size_t)tableTotal * 4));
  if (anyLloyd) TRY(ensure(ctx, ctx->qlut, (size_t)n * kLutStride * 2));
  TRY(ensure(ctx, ctx->dqtable, (size_t)n * kMaxBins * 4));
  TRY(ensure(ctx, ctx->hist, (size_t)n * kMaxSymbols * 8));
  TRY(ensure(ctx, ctx->chunkRun, chunkTotal * sizeof(int4)));
  TRY(ensure(ctx, ctx->chunkSpan, chunkTotal * sizeof(int2)));
  TRY(ensure(ctx, ctx->chunkRunCtx, chunkTotal * 2 * sizeof(long long)));
  TRY(ensure(ctx, ctx->chunkBits, chunkTotal * 8));
  TRY(ensure(ctx, ctx->codes, (size_t)n * kMaxSymbols * 8));
  TRY(ensure(ctx, ctx->codeLen, (size_t)n * kMaxSymbols));
  TRY(ensure(ctx, ctx->decode, (size_t)n * 4 * kMaxSymbols * 4));
  TRY(ensure(ctx, ctx->words, wordsTotal * 4));
  TRY(ensure(ctx, ctx->logHdr, n * sizeof(int4)));
  TRY(ensure(ctx, ctx->meta, (size_t)n * (4 * kMaxSymbols + 2 * kMaxBins) * 4));
  // upload block: cubelet records | chunk prefix | transform pass groups
  const size_t cubBytes = ((size_t)n * sizeof(CubeletDev) + 255) & ~(size_t)255;
  const size_t prefBytes = ((size_t)n * sizeof(long long) + 255) & ~(size_t)255;
  const size_t passBytes =
      cubBytes + prefBytes + (size_t)3 * n * (sizeof(PassDesc) + sizeof(int) + 260) + 4096;
  TRY(ensure(ctx, ctx->passes, passBytes));
  TRY(ensure_host(ctx, ctx->hPasses, passBytes));
  TRY(ensure_host(ctx, ctx->hState, n * sizeof(CubeletState)));
  TRY(ensure_host(ctx, ctx->hLogHdr, n * sizeof(int4)));
  if (anyLog) TRY(ensure_host(ctx, ctx->hTab, (size_t)tableTotal * 4));

  cudaStream_t s = ctx->stream;
  CU(cudaEventRecord(ctx->ev[0], s));

  // ---- inputs ----
  std::vector<const void *> dIn(n);
  std::vector<char> hostIn(n, 0);  // input read in place from page-locked host memory
  if (onDevice) {
    for (int i = 0; i < n; i++) dIn[i] = plans[i].data;
  } else {
    // Page-locked host inputs are read in place by the first transform pass
    // (the GPU reaches pinned memory directly) unless the context stages
    // them (then, like pageable ones, they are copied -- by the copy engine,
    // without staging, since they are page-locked); device (or managed)
    // pointers are used as they are.
    bool staged = false;
    for (int i = 0; i < n; i++) {
      cudaPointerAttributes attr;
      const bool known = cudaPointerGetAttributes(&attr, plans[i].data) == cudaSuccess;
      if (known && attr.type == cudaMemoryTypeHost && attr.devicePointer && !ctx->stageHost) {
        dIn[i] = attr.devicePointer;
        hostIn[i] = 1;
      } else if (known && (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged)) {
        dIn[i] = plans[i].data;
      } else {
        cudaGetLastError();
        dIn[i] = nullptr;
        staged = true;
      }
    }
    if (staged) TRY(ensure(ctx, ctx->input, inBytes));
    for (int i = 0; i < n; i++) {
      if (dIn[i]) continue;
      Plan &pl = plans[i];
      char *dst = P<char>(ctx->input) + pl.inOff;
      const size_t es = dtype_size(pl.dtype);
      if (pl.pitchY == pl.X && pl.pitchZ == (long long)pl.X * pl.Y) {
        CU(cudaMemcpyAsync(dst, pl.data, (size_t)pl.X * pl.Y * pl.Z * es,
                           cudaMemcpyHostToDevice, s));
      } else if (pl.pitchZ % pl.pitchY == 0) {
        // a sub-volume of a larger array (slices a whole number of rows
        // apart): gathered dense by one three-dimensional copy
        cudaMemcpy3DParms cp;
        memset(&cp, 0, sizeof cp);
        cp.srcPtr = make_cudaPitchedPtr(const_cast<void *>(pl.data), (size_t)pl.pitchY * es,
                                        (size_t)pl.X * es, (size_t)(pl.pitchZ / pl.pitchY));
        cp.dstPtr = make_cudaPitchedPtr(dst, (size_t)pl.X * es, (size_t)pl.X * es, (size_t)pl.Y);
        cp.extent = make_cudaExtent((size_t)pl.X * es, (size_t)pl.Y, (size_t)pl.Z);
        cp.kind = cudaMemcpyHostToDevice;
        CU(cudaMemcpy3DAsync(&cp, s));
        pl.pitchY = pl.X;
        pl.pitchZ = (long long)pl.X * pl.Y;
      } else {
        // other layouts: slice by slice
        for (int z = 0; z < pl.Z; z++)
          CU(cudaMemcpy2DAsync(dst + (size_t)z * pl.X * pl.Y * es, (size_t)pl.X * es,
                               static_cast<const char *>(pl.data) + (size_t)z * pl.pitchZ * es,
                               (size_t)pl.pitchY * es, (size_t)pl.X * es, pl.Y,
                               cudaMemcpyHostToDevice, s));
        pl.pitchY = pl.X;
        pl.pitchZ = (long long)pl.X * pl.Y;
      }
      dIn[i] = dst;
    }
  }

  // ---- halves ----
  // A large batch runs as two halves (cubelets [0, cut) and [cut, n), cut at
  // half of the padded elements) on two streams: the second half's transform
  // starts when the first half's has finished, so each half's latency-bound
  // steps (radix-select resolves, Lloyd solve, zero-run join, Huffman tree
  // build) run beside the other half's bulk passes.  Each half is a view of
  // the same buffers (per-cubelet and per-chunk arrays offset to its first
  // cubelet and chunk), so the results are those of one batch.
  int cut = n, nh = 1;
  if (ctx->splitMode && ctx->stream2 && !coefOut && !ctx->profiling && n >= 8 &&
      coefTotal >= (32LL << 20)) {
    long long acc = 0;
    for (int i = 0; i < n; i++) {
      acc += plans[i].n;
      if (2 * acc >= coefTotal) { cut = i + 1; break; }
    }
    cut = std::max(1, std::min(cut, n - 1));
    nh = 2;
  }
  const int hc0[3] = {0, cut, n};
  auto half_of = [&](int i) { return i < cut ? 0 : 1; };

  // ---- descriptors (host side of the upload block) ----
  CubeletDev *hc = H<CubeletDev>(ctx->hPasses);
  long long *hp = reinterpret_cast<long long *>(H<char>(ctx->hPasses) + cubBytes);
  long long groupTotal = 0, encTotal = 0;
  long long chunk0[2] = {0, 0}, group0[2] = {0, 0}, words0[2] = {0, 0}, enc0[2] = {0, 0};
  long long wordsAcc = 0;
  // bit-packer slices per chunk, from each half's chunk count
  int encF[2] = {1, 1};
  {
    long long halfChunks[2] = {0, 0};
    for (int i = 0; i < n; i++) halfChunks[half_of(i)] += plans[i].nChunks;
    for (int h = 0; h < nh; h++) encF[h] = ctx->encSlices ? ctx->encSlices : enc_slices(halfChunks[h]);
  }
  for (int i = 0; i < n; i++) {
    const Plan &pl = plans[i];
    const int h = half_of(i);
    if (i == hc0[h]) {
      chunk0[h] = pl.chunkBase;
      group0[h] = groupTotal;
      words0[h] = wordsAcc;
      enc0[h] = encTotal;
    }
    CubeletDev &c = hc[i];
    memset(&c, 0, sizeof c);
    c.n = pl.n;
    c.coefOff = pl.coefOff;
    c.chunkBase = pl.chunkBase - chunk0[h];
    c.wordsOff = 0;
    c.wordsCap = pl.wordsCap;
    c.nChunks = pl.nChunks;
    c.binCount = pl.p.bin_count;
    c.quantAlg = pl.p.quant_alg;
    c.compressZeros = pl.p.compress_zeros ? 1 : 0;
    c.frac = pl.p.threshold_fraction;
    c.lloydIters = pl.p.lloyd_iters > 0 ? pl.p.lloyd_iters : 20;
    c.tableOff = pl.tableOff;
    c.groupBase = (int)(groupTotal - group0[h]);
    groupTotal += (pl.nChunks + kQuantGroup - 1) / kQuantGroup;
    c.encBase = (int)(encTotal - enc0[h]);
    encTotal += ((long long)pl.nChunks * encF[h] + kEncThreads - 1) / kEncThreads;
    wordsAcc += pl.wordsCap;
    hp[i] = c.chunkBase;
  }

  DevBatch b;
  memset(&b, 0, sizeof b);
  b.n = n;
  b.cub = reinterpret_cast<CubeletDev *>(P<char>(ctx->passes));
  b.state = P<CubeletState>(ctx->state);
  b.coef = P<float>(ctx->coef);
  b.coef2 = P<float>(ctx->coef2);
  b.tok = P<uint16_t>(ctx->bins);
  b.chunkTok = P<int>(ctx->tokCount);
  b.selHist = P<unsigned>(ctx->selHist);
  b.lloydHist = P<float>(ctx->lloydHist);
  b.qtable = P<float>(ctx->qtable);
  b.qlut = P<uint16_t>(ctx->qlut);
  b.dqtable = P<float>(ctx->dqtable);
  b.hist = P<unsigned long long>(ctx->hist);
  b.chunkRun = P<int4>(ctx->chunkRun);
  b.chunkSpan = P<int2>(ctx->chunkSpan);
  b.chunkRunCtx = P<long long>(ctx->chunkRunCtx);
  b.chunkBits = P<unsigned long long>(ctx->chunkBits);
  b.codes = P<unsigned long long>(ctx->codes);
  b.codeLen = P<uint8_t>(ctx->codeLen);
  b.decode = P<int>(ctx->decode);
  b.words = P<uint32_t>(ctx->words);
  b.chunkPrefix = reinterpret_cast<long long *>(P<char>(ctx->passes) + cubBytes);
  b.chunkCub = P<int>(ctx->chunkCub);
  b.groupCub = P<int>(ctx->groupCub);
  b.totalGroups = groupTotal;
  b.encCub = P<int>(ctx->encCub);
  b.totalEnc = encTotal;
  b.encF = encF[0];
  b.sliceOff = P<unsigned>(ctx->sliceOff);
  b.logHdr = P<int4>(ctx->logHdr);
  b.meta = P<int>(ctx->meta);
  b.totalChunks = chunkTotal;
  constexpr long long kMetaPer = 4LL * kMaxSymbols + 2LL * kMaxBins;  // ints per cubelet
  DevBatch bh[2] = {b, b};
  if (nh == 2) {
    for (int h = 0; h < 2; h++) {
      DevBatch &v = bh[h];
      const int c0 = hc0[h];
      const long long ch = chunk0[h], g = group0[h];
      v.n = hc0[h + 1] - c0;
      v.cub += c0;
      v.state += c0;
      v.selHist += (size_t)c0 * kSelectBins;
      v.lloydHist += (size_t)c0 * kLloydBins;
      v.qlut += (size_t)c0 * kLutStride;
      v.dqtable += (size_t)c0 * kMaxBins;
      v.hist += (size_t)c0 * kMaxSymbols;
      v.codes += (size_t)c0 * kMaxSymbols;
      v.codeLen += (size_t)c0 * kMaxSymbols;
      v.decode += (size_t)c0 * 4 * kMaxSymbols;
      v.logHdr += c0;
      v.chunkPrefix += c0;
      v.chunkTok += ch;
      v.chunkSpan += ch;
      v.chunkRun += ch;
      v.chunkRunCtx += 2 * ch;
      v.chunkBits += ch;
      v.chunkCub += ch;
      v.groupCub += g;
      v.encCub += enc0[h];
      v.totalEnc = (h ? encTotal : enc0[1]) - enc0[h];
      v.encF = encF[h];
      v.sliceOff += ch * 32;
      v.words += words0[h];
      v.meta += c0 * kMetaPer;
      v.totalChunks = (h ? chunkTotal : chunk0[1]) - ch;
      v.totalGroups = (h ? groupTotal : group0[1]) - g;
    }
  }

  PassGroups xs[2], ys[2], zs[2];
  bool pass0[2] = {false, false};  // a cubelet needs the stand-alone first select pass
  for (int i = 0; i < n; i++) {
    const int h = half_of(i);
    const bool fused = forward_passes(plans[i], dIn[i], hostIn[i] != 0, b.coef, b.coef2, xs[h],
                                      ys[h], zs[h], b.selHist + (size_t)i * kSelectBins,
                                      b.state + i);
    hc[i].selFused = fused ? 1 : 0;
    pass0[h] |= !fused;
  }
  std::vector<GroupLaunch> gl;
  size_t hoff = cubBytes + prefBytes;
  size_t gb[2][4];  // per half: group index bounds of the x, y, z phases
  for (int h = 0; h < nh; h++) {
    gb[h][0] = gl.size();
    TRY(stage_groups(ctx, xs[h], hoff, kTuneFwdX, WL_F32, false, gl));
    gb[h][1] = gl.size();
    TRY(stage_groups(ctx, ys[h], hoff, kTuneFwdY, WL_F32, false, gl));
    gb[h][2] = gl.size();
    TRY(stage_groups(ctx, zs[h], hoff, kTuneFwdZ, WL_F32, false, gl));
    gb[h][3] = gl.size();
  }
  const size_t upBytes = hoff;
  cudaStream_t s2 = ctx->stream2;

  // ---- device work, in one or two segments (a host step between them
  // computes the log quantizer tables); each may run as a CUDA graph ----
  ctx->launches = 0;
  // everything after the select for half h on stream st
  auto post = [&](int h, cudaStream_t st) -> wl_status {
    DevBatch &v = bh[h];
    const bool first = h == 0;
    if (first) CU(record(ctx, ctx->ev[2]));
    launch_quant_params(v, st);
    ctx->launches += 1;
    if (anyLloyd) { launch_lloyd(v, v.coef, maxLloyd, st); ctx->launches += 3; }
    if (first) mark(ctx, 5);
    launch_quantize(v, v.coef, maxTable, maxS, st);
    if (first) mark(ctx, 6);
    launch_runs(v, st);
    ctx->launches += 2;
    if (first) mark(ctx, 7);
    CU(cudaGetLastError());
    if (first) CU(record(ctx, ctx->ev[3]));
    launch_huffman_build(v, maxS, st);
    ctx->launches += 1;
    if (first) mark(ctx, 8);
    CU(cudaGetLastError());
    if (first) CU(record(ctx, ctx->ev[4]));
    launch_encode(v, maxS, st);
    launch_pack_meta(v, st);
    ctx->launches += 6;
    if (first) mark(ctx, 9);
    CU(cudaGetLastError());
    if (first) CU(record(ctx, ctx->ev[5]));
    return WL_OK;
  };
  // the second half's stream joins the context's stream
  auto join = [&]() -> wl_status {
    if (nh == 2) {
      CU(cudaEventRecord(ctx->halfJ, s2));
      CU(cudaStreamWaitEvent(s, ctx->halfJ, 0));
    }
    return WL_OK;
  };
  auto quantize_to_end = [&]() -> wl_status {
    if (anyLog) {
      CU(cudaMemcpyAsync(ctx->qtable.p, ctx->hTab.p, (size_t)tableTotal * 4,
                         cudaMemcpyHostToDevice, s));
      CU(cudaMemcpyAsync(ctx->logHdr.p, ctx->hLogHdr.p, n * sizeof(int4), cudaMemcpyHostToDevice, s));
      if (nh == 2) {  // the second half starts once the tables are on the device
        CU(cudaEventRecord(ctx->halfT, s));
        CU(cudaStreamWaitEvent(s2, ctx->halfT, 0));
      }
    }
    TRY(post(0, s));
    if (nh == 2) TRY(post(1, s2));
    TRY(join());
    CU(cudaMemcpyAsync(ctx->hState.p, ctx->state.p, n * sizeof(CubeletState),
                       cudaMemcpyDeviceToHost, s));
    return WL_OK;
  };
  auto transform_select = [&]() -> wl_status {
    CU(cudaMemcpyAsync(ctx->passes.p, ctx->hPasses.p, upBytes, cudaMemcpyHostToDevice, s));
    CU(cudaMemsetAsync(ctx->state.p, 0, n * sizeof(CubeletState), s));
    CU(cudaMemsetAsync(ctx->selHist.p, 0, (size_t)n * kSelectBins * 4, s));
    CU(cudaMemsetAsync(ctx->hist.p, 0, (size_t)n * kMaxSymbols * 8, s));
    if (anyLloyd) CU(cudaMemsetAsync(ctx->lloydHist.p, 0, (size_t)n * kLloydBins * 4, s));
    launch_select_init(b, s);
    ctx->launches += 1;
    if (nh == 2) {  // the second half starts with the first
      CU(cudaEventRecord(ctx->halfT, s));
      CU(cudaStreamWaitEvent(s2, ctx->halfT, 0));
    }
    mark(ctx, 0);
    TRY(launch_phase(ctx, gl, gb[0][0], gb[0][1]));
    mark(ctx, 1);
    TRY(launch_phase(ctx, gl, gb[0][1], gb[0][2]));
    mark(ctx, 2);
    TRY(launch_phase(ctx, gl, gb[0][2], gb[0][3]));
    mark(ctx, 3);
    CU(record(ctx, ctx->ev[1]));
    if (nh == 2) {
      for (int ph = 0; ph < 3; ph++)
        TRY(launch_phase_on(ctx, gl, gb[1][ph], gb[1][ph + 1], s2, ctx->side2, ctx->fork2,
                            ctx->join2));
    }
    if (coefOut) return WL_OK;
    launch_select(bh[0], bh[0].coef, pass0[0], s);
    ctx->launches += pass0[0] ? 8 : 7;
    if (nh == 2) {
      launch_select(bh[1], bh[1].coef, pass0[1], s2);
      ctx->launches += pass0[1] ? 8 : 7;
    }
    CU(cudaGetLastError());
    mark(ctx, 4);
    if (anyLog) {
      TRY(join());
      CU(cudaMemcpyAsync(ctx->hState.p, ctx->state.p, n * sizeof(CubeletState),
                         cudaMemcpyDeviceToHost, s));
    } else {
      if (nh == 2) TRY(post(1, s2));
      TRY(post(0, s));
      TRY(join());
      CU(cudaMemcpyAsync(ctx->hState.p, ctx->state.p, n * sizeof(CubeletState),
                         cudaMemcpyDeviceToHost, s));
    }
    return WL_OK;
  };

  GraphEntry *ge = nullptr;
  if (ctx->graphMode && !coefOut) {
    // everything the captured launches depend on besides the upload block
    std::vector<long long> key;
    key.reserve(4 + (size_t)n * 18);
    key.push_back(n);
    key.push_back(onDevice | (ctx->profiling ? 2 : 0) | (nh == 2 ? 4 : 0));
    key.push_back((long long)tune_version());
    key.push_back(ctx->encSlices);
    for (int i = 0; i < n; i++) {
      const Plan &pl = plans[i];
      const wl_params &q = pl.p;
      uint32_t fb;
      memcpy(&fb, &q.threshold_fraction, 4);
      const long long v[] = {pl.dtype | (hostIn[i] << 8), pl.X, pl.Y, pl.Z, pl.pitchY, pl.pitchZ,
                             q.steps[0], q.steps[1], q.steps[2], q.wavelet, (long long)fb,
                             q.bin_count, q.quant_alg, q.compress_zeros, q.lloyd_iters,
                             q.exact_transform, q.transform_2d};
      key.insert(key.end(), v, v + sizeof v / sizeof v[0]);
    }
    ge = graph_for(ctx, std::move(key));
  }

  // ---- transform ----
  TRY(run_segment(ctx, ge, 0, transform_select));
  if (coefOut) {  // transform only: hand back the coefficients of cubelet 0
    const Plan &pl = plans[0];
    if ((size_t)pl.n > coefCap) return fail(ctx, WL_EINVAL, "coefficient buffer too small");
    CU(cudaMemcpyAsync(coefOut, b.coef + pl.coefOff, (size_t)pl.n * 4, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (pl.identity || pl.two_d) { storedSize[0] = pl.Xp; storedSize[1] = pl.Yp; storedSize[2] = pl.Zp; }
    else { storedSize[0] = pl.Zp; storedSize[1] = pl.Xp; storedSize[2] = pl.Yp; }
    return WL_OK;
  }

  // ---- log quantizer tables (host logf) ----
  if (anyLog) {
    CU(cudaStreamSynchronize(s));
    const CubeletState *hs = H<CubeletState>(ctx->hState);
    float *tab = H<float>(ctx->hTab);
    int4 *lh = H<int4>(ctx->hLogHdr);
    // one table per log cubelet, independent: spread over host threads
    std::vector<int> logIdx;
    for (int i = 0; i < n; i++) {
      lh[i] = make_int4(0, 0, 0, 0);
      if (plans[i].p.quant_alg == WL_LOG) logIdx.push_back(i);
    }
    std::atomic<int> bad{-1};
    const std::function<void(int)> one = [&](int k) {
      LogTable t;
      const int i = logIdx[k];
      log_quant_table(plans[i].p.bin_count, hs[i].threshold, hs[i].maxAbs, t);
      if (t.nPos + t.nNeg > 2 * plans[i].p.bin_count) {
        bad.store(i);
        return;
      }
      lh[i] = make_int4(t.lowBin, t.highNeg, t.nPos, t.nNeg);
      std::copy(t.bounds.begin(), t.bounds.end(), tab + plans[i].tableOff);
    };
    host_pool().run((int)logIdx.size(), one);
    if (bad.load() >= 0)
      return fail(ctx, WL_EINVAL, "cubelet %d: log quantizer degenerate (largest |c| ~ threshold)",
                  bad.load());
    TRY(run_segment(ctx, ge, 1, quantize_to_end));
  }

  // ---- results ----
  CU(cudaStreamSynchronize(s));
  const CubeletState *hs = H<CubeletState>(ctx->hState);
  long long hw0[3] = {0, 0, 0};  // words of each half, then their sum
  size_t hm0[3] = {0, 0, 0};     // packed metadata ints of each half
  for (int i = 0; i < n; i++) {
    if (hs[i].error)
      return fail(ctx, WL_EINVAL, "cubelet %d: device error %d (code too long or output overflow)",
                  i, hs[i].error);
    const int h = half_of(i);
    hw0[h] += hs[i].nWords;
    hm0[h] += hs[i].nDecode +
              (plans[i].p.quant_alg == WL_LLOYD ? hs[i].nBounds + hs[i].nValues : 0);
  }
  const long long totalWords = hw0[0] + hw0[1];
  const size_t metaInts = hm0[0] + hm0[1];
  // words, then the packed decode tables and codebooks, straight into the slab
  const size_t wordsBytes = ((size_t)totalWords * 4 + 15) & ~(size_t)15;
  ResultSlab *slab = slab_pool().acquire(wordsBytes + metaInts * 4 + 16);
  if (!slab) return fail(ctx, WL_ENOMEM, "cannot allocate %zu bytes of page-locked result storage",
                         wordsBytes + metaInts * 4 + 16);
  uint32_t *hw = reinterpret_cast<uint32_t *>(slab->base);
  int *hd = reinterpret_cast<int *>(slab->base + wordsBytes);
  const long long wAt[2] = {0, hw0[0]};
  const size_t mAt[2] = {0, hm0[0]};
  for (int h = 0; h < nh; h++) {
    if (hw0[h]) {
      const cudaError_t e = cudaMemcpyAsync(hw + wAt[h], bh[h].words, (size_t)hw0[h] * 4,
                                            cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) { slab_pool().release(slab); CU(e); }
    }
    if (hm0[h]) {
      const cudaError_t e = cudaMemcpyAsync(hd + mAt[h], bh[h].meta, hm0[h] * 4,
                                            cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) { slab_pool().release(slab); CU(e); }
    }
  }
  std::vector<size_t> decOff(n), cbOff(n, 0), wOff(n);
  for (int i = 0; i < n; i++) {
    const int h = half_of(i);
    decOff[i] = mAt[h] + (size_t)hs[i].metaBase;
    cbOff[i] = decOff[i] + hs[i].nDecode;
    wOff[i] = (size_t)(wAt[h] + hs[i].wordsBase);
  }
  {
    cudaError_t e = cudaEventRecord(ctx->ev[6], s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { slab_pool().release(slab); CU(e); }
  }
  slab->refs.store(n);

  float t[6];
  cudaEventElapsedTime(&t[0], ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&t[1], ctx->ev[1], ctx->ev[2]);
  cudaEventElapsedTime(&t[2], ctx->ev[2], ctx->ev[3]);
  cudaEventElapsedTime(&t[3], ctx->ev[3], ctx->ev[4]);
  cudaEventElapsedTime(&t[4], ctx->ev[4], ctx->ev[5]);
  cudaEventElapsedTime(&t[5], ctx->ev[0], ctx->ev[6]);
  memcpy(ctx->timings, t, sizeof t);
  if (ctx->profiling)
    for (int g = 0; g < 9; g++) cudaEventElapsedTime(&ctx->ktimes[g], ctx->pev[g], ctx->pev[g + 1]);

  for (int i = 0; i < n; i++) {
    const Plan &pl = plans[i];
    const CubeletState &st = hs[i];
    wl_result &r = outs[i];
    memset(&r, 0, sizeof r);
    r.transform_2d = pl.two_d ? 1 : 0;
    if (pl.identity || pl.two_d) { r.size[0] = pl.Xp; r.size[1] = pl.Yp; r.size[2] = pl.Zp; }
    else { r.size[0] = pl.Zp; r.size[1] = pl.Xp; r.size[2] = pl.Yp; }
    r.original_size[0] = pl.X; r.original_size[1] = pl.Y; r.original_size[2] = pl.Z;
    r.original_dtype = pl.dtype;
    r.steps[0] = pl.sx; r.steps[1] = pl.sy; r.steps[2] = pl.sz;
    r.wavelet = pl.p.wavelet;
    r.quant_alg = pl.p.quant_alg;
    r.bin_count = pl.p.bin_count;
    r.threshold_fraction = pl.p.threshold_fraction;
    r.threshold_value = st.threshold;
    r.max_value = st.maxAbs;
    r.min_coef = st.minVal;
    r.max_coef = st.maxVal;
    r.zero_bin = st.zeroBin;
    r.dup_value = st.dupValue;
    r.dup_key = st.dupValue >= 0 ? pl.p.bin_count : -1;
    r.longest_code = st.longest;
    r.owner = slab;
    r.n_words = st.nWords;
    r.words = hw + wOff[i];
    r.n_decode = st.nDecode;
    r.decode = hd + decOff[i];
    if (pl.p.quant_alg == WL_LLOYD) {
      r.n_boundaries = st.nBounds;
      r.n_values = st.nValues;
      r.boundaries = reinterpret_cast<float *>(hd + cbOff[i]);
      r.values = reinterpret_cast<float *>(hd + cbOff[i] + st.nBounds);
    }
  }
  return WL_OK;
}

// ---- decompression -----------------------------------------------------------
}  // namespace

// dequantize kernel launcher lives in dwt.cu
namespace wl {
void launch_dequant(const int *bins, const float *table, float *out, long long n, int nTable,
                    cudaStream_t s);
}

namespace {

// Column-tile inverse passes (the forward layouts in reverse): z in place on
// z-x-y (only with z levels), y z-x-y -> z-y-x into c2, x z-y-x -> x-y-z with
// the crop to the original size into dst.  Returns the pass count.
int inverse_passes_cols(int Xp, int Yp, int Zp, const int orig[3], const int steps[3],
                        int wavelet, float *c1, float *c2, void *dst, PassDesc *out) {
  const int big = 0x7fffffff;
  const int X = orig[0], Y = orig[1], Z = orig[2];
  auto mk = [&]() { PassDesc d; memset(&d, 0, sizeof d); d.cropL = d.cropB = d.cropA = big;
                    d.clampL = d.clampB = d.clampA = big; d.wavelet = wavelet; d.exact = 0;
                    d.inSC = 1; return d; };
  int np = 0;
  if (steps[2] > 0) {  // rows (a = y, b = x)
    PassDesc a = mk();
    a.in = c1; a.inSA = (long long)Zp * Xp; a.inSB = Zp; a.inSC = 1;
    a.out = c1; a.outSA = (long long)Zp * Xp; a.outSB = Zp; a.outSC = 1;
    a.L = Zp; a.B = Xp; a.rows = Xp * Yp; a.steps = steps[2];
    out[np++] = a;
  }
  PassDesc e = mk();  // rows (a = x, b = z)
  e.in = c1; e.inSA = Zp; e.inSB = 1; e.inSC = (long long)Zp * Xp;
  e.out = c2; e.outSA = (long long)Zp * Yp; e.outSB = 1; e.outSC = Zp;
  e.L = Yp; e.B = Zp; e.rows = Zp * Xp; e.steps = steps[1];
  out[np++] = e;
  PassDesc x = mk();  // rows (a = y, b = z)
  x.in = c2; x.inSA = Zp; x.inSB = 1; x.inSC = (long long)Zp * Yp;
  x.out = dst; x.outSA = X; x.outSB = (long long)X * Y; x.outSC = 1;
  x.cropL = X; x.cropA = Y; x.cropB = Z;
  x.L = Xp; x.B = Zp; x.rows = Yp * Zp; x.steps = steps[0];
  out[np++] = x;
  return np;
}

// Inverse transform of the coefficients already in ctx->coef (stored order)
// into out (original size, outType), then synchronize.
// Inverse transform passes of one cubelet, sorted into three phases that run
// in order (phase k of every cubelet of a batch may run concurrently):
// 0 the z levels, 1 the y levels (2-D mode: the x levels), 2 the last pass
// into the output with the crop and the element type (2-D mode: the y
// levels).  c1 holds the coefficients in the stored order, c2 is scratch of
// the same size, dst receives original_size elements of outType.  Groups are
// keyed like the forward ones, with the output type in the type field.
void inverse_passes(const int size[3], const int steps[3], int wavelet, const int original_size[3],
                    int outType, bool two_d, float *c1, float *c2, void *dst, PassGroups ph[3]) {
  bool identity = steps[0] == 0 && steps[1] == 0 && steps[2] == 0;
  const bool unrotated = identity || two_d;
  const int Xp = unrotated ? size[0] : size[1];
  const int Yp = unrotated ? size[1] : size[2];
  const int Zp = unrotated ? size[2] : size[0];
  int sx2 = 0, sy2 = 0;
  if (two_d && !identity && !twod_steps(Xp, Yp, steps[0], steps[1], sx2, sy2)) identity = true;
  const int X = original_size[0], Y = original_size[1], Z = original_size[2];
  const int big = 0x7fffffff;
  auto mk = [&]() { PassDesc d; memset(&d, 0, sizeof d); d.cropL = d.cropB = d.cropA = big;
                    d.clampL = d.clampB = d.clampA = big; d.wavelet = wavelet; d.exact = 0;
                    d.inSC = 1; return d; };
  auto put = [&](int phase, bool cols, const PassDesc &d) {
    ph[phase][group_key(cols, phase == 2 ? outType : WL_F32, d.L)].push_back(d);
  };
  wl_params wp;
  memset(&wp, 0, sizeof wp);
  wp.wavelet = wavelet;
  if (two_d && !identity) {
    // x levels first ([z][y][x] -> [z][x][y]), then y levels into the output
    // (the reference undoes y first; the 1-D transforms along different axes
    // commute, so this differs from its order only by float rounding), both
    // reading rows contiguous in memory
    const bool cols = Xp <= kColsMaxL && Yp <= kColsMaxL;
    PassDesc a = mk();
    a.in = c1; a.inSA = (long long)Xp * Yp; a.inSB = Xp; a.inSC = 1;
    a.out = c2; a.outSA = (long long)Xp * Yp; a.outSB = 1; a.outSC = Yp;
    a.L = Xp; a.B = Yp; a.rows = Yp * Zp; a.steps = sx2;
    a.T = dwt_tile_rows(a.L, false); a.tiles = (a.rows + a.T - 1) / a.T;
    put(1, cols, a);
    PassDesc b = mk();
    b.in = c2; b.inSA = (long long)Xp * Yp; b.inSB = Yp; b.inSC = 1;
    b.out = dst; b.outSA = (long long)X * Y; b.outSB = 1; b.outSC = X;
    b.cropL = Y; b.cropA = Z; b.cropB = X;
    b.L = Yp; b.B = Xp; b.rows = Xp * Zp; b.steps = sy2;
    b.T = dwt_tile_rows(b.L, false); b.tiles = (b.rows + b.T - 1) / b.T;
    put(2, cols, b);
  } else if (use_cols(Xp, Yp, Zp, identity, wp)) {
    PassDesc d[3];
    const int np = inverse_passes_cols(Xp, Yp, Zp, original_size, steps, wavelet, c1, c2, dst, d);
    for (int i = 0; i < np; i++) {
      const int phase = 3 - np + i;
      if (phase == 0 && dwt_rowreg_fits(d[i].L, d[i].steps))  // z rows in registers
        ph[0][rowreg_inv_key(d[i].L)].push_back(d[i]);
      else if (phase > 0 && dwt_rowreg_fits(d[i].L, d[i].steps))  // y, x: through a tile
        ph[phase][rowreg_inv_t_key(phase == 2 ? outType : WL_F32, d[i].L)].push_back(d[i]);
      else
        put(phase, true, d[i]);
    }
  } else {
    if (!identity) {
      // inverse z pass: z-x-y -> y-z-x
      PassDesc a = mk();
      a.in = c1; a.inSA = Zp; a.inSB = (long long)Xp * Zp;
      a.L = Zp; a.B = Yp; a.rows = Xp * Yp;
      a.out = c2; a.outSA = (long long)Yp * Zp; a.outSB = 1; a.outSC = Yp;
      a.steps = steps[2];
      a.T = dwt_tile_rows(a.L, false); a.tiles = (a.rows + a.T - 1) / a.T;
      put(0, false, a);
      // inverse y pass: y-z-x -> x-y-z
      PassDesc bq = mk();
      bq.in = c2; bq.inSA = Yp; bq.inSB = (long long)Zp * Yp;
      bq.L = Yp; bq.B = Xp; bq.rows = Zp * Xp;
      bq.out = c1; bq.outSA = (long long)Xp * Yp; bq.outSB = 1; bq.outSC = Xp;
      bq.steps = steps[1];
      bq.T = dwt_tile_rows(bq.L, false); bq.tiles = (bq.rows + bq.T - 1) / bq.T;
      put(1, false, bq);
    }
    // inverse x pass + crop + dtype
    PassDesc x = mk();
    x.in = c1; x.inSA = (long long)Yp * Xp; x.inSB = Xp;
    x.L = Xp; x.B = Yp; x.rows = Yp * Zp;
    x.out = dst; x.outSA = (long long)X * Y; x.outSB = X; x.outSC = 1;
    x.cropL = X; x.cropB = Y; x.cropA = Z;
    x.steps = identity ? 0 : steps[0];
    x.T = dwt_tile_rows(x.L, false); x.tiles = (x.rows + x.T - 1) / x.T;
    put(2, false, x);
  }
}

// Stage the three inverse phases (one upload) and launch them in order; the
// groups of a phase run concurrently.  pb receives the phase boundaries.
wl_status run_inverse_phases(wl_ctx *ctx, PassGroups ph[3]) {
  size_t hoff = 0, count = 0;
  for (int k = 0; k < 3; k++)
    for (const auto &kv : ph[k]) count += kv.second.size();
  const size_t need = count * (sizeof(PassDesc) + sizeof(int) + 260) + 4096;
  TRY(ensure(ctx, ctx->passes, need));
  TRY(ensure_host(ctx, ctx->hPasses, need));
  std::vector<GroupLaunch> gl;
  size_t bound[4] = {0, 0, 0, 0};
  const int kinds[3] = {kTuneInvZ, kTuneInvY, kTuneInvX};
  for (int k = 0; k < 3; k++) {
    for (const auto &kv : ph[k]) {
      if ((kv.first >> 24) & 1) {
        TRY(stage_group(ctx, kv.second, hoff, kinds[k], WL_F32, (kv.first >> 16) & 15, true, false,
                        false, gl, nullptr, kv.second[0].L, kRegInvTile));
        continue;
      }
      if ((kv.first >> 23) & 1) {
        TRY(stage_group(ctx, kv.second, hoff, kinds[k], WL_F32, WL_F32, true, false, false, gl,
                        nullptr, kv.second[0].L, kRegInvInPlace));
        continue;
      }
      const bool cols = (kv.first >> 12) & 1;
      const int outT = (kv.first >> 8) & 15;
      TRY(stage_group(ctx, kv.second, hoff, kinds[k], WL_F32, outT, true, cols, false, gl));
    }
    bound[k + 1] = gl.size();
  }
  CU(cudaMemcpyAsync(ctx->passes.p, ctx->hPasses.p, hoff, cudaMemcpyHostToDevice, ctx->stream));
  for (int k = 0; k < 3; k++) TRY(launch_phase(ctx, gl, bound[k], bound[k + 1]));
  return WL_OK;
}

wl_status inverse_impl(wl_ctx *ctx, const int size[3], const int steps[3], int wavelet,
                       const int original_size[3], int outType, void *out, int outOnDevice,
                       bool two_d = false) {
  cudaStream_t s = ctx->stream;
  const int X = original_size[0], Y = original_size[1], Z = original_size[2];
  const size_t outBytes = (size_t)X * Y * Z * dtype_size(outType);
  if (!outOnDevice) TRY(ensure(ctx, ctx->outbuf, outBytes));
  void *dst = outOnDevice ? out : ctx->outbuf.p;
  PassGroups ph[3];
  inverse_passes(size, steps, wavelet, original_size, outType, two_d, P<float>(ctx->coef),
                 P<float>(ctx->coef2), dst, ph);
  TRY(run_inverse_phases(ctx, ph));
  if (!outOnDevice) CU(cudaMemcpyAsync(out, dst, outBytes, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return WL_OK;
}

wl_status check_sizes(wl_ctx *ctx, const int size[3], const int steps[3], const int orig[3],
                      long long &n, bool two_d = false) {
  const bool unrotated = two_d || (steps[0] == 0 && steps[1] == 0 && steps[2] == 0);
  const int Xp = unrotated ? size[0] : size[1];
  const int Yp = unrotated ? size[1] : size[2];
  const int Zp = unrotated ? size[2] : size[0];
  for (int a = 0; a < 3; a++)
    if (steps[a] < 0 || steps[a] > 30) return fail(ctx, WL_EFORMAT, "bad step count");
  if (orig[0] < 1 || orig[1] < 1 || orig[2] < 1 || orig[0] > Xp || orig[1] > Yp || orig[2] > Zp)
    return fail(ctx, WL_EFORMAT, "inconsistent sizes");
  if (Xp % (1 << steps[0]) || Yp % (1 << steps[1]) || Zp % (1 << steps[2]))
    return fail(ctx, WL_EFORMAT, "size not padded for the step counts");
  n = (long long)Xp * Yp * Zp;
  return WL_OK;
}

// Checks of a compressed cubelet before decoding; n = its padded element count.
wl_status check_result(wl_ctx *ctx, const wl_result *r, int outType, long long &n) {
  if (!r) return fail(ctx, WL_EINVAL, "null argument");
  if (dtype_size(outType) == 0) return fail(ctx, WL_EINVAL, "bad output dtype %d", outType);
  TRY(check_sizes(ctx, r->size, r->steps, r->original_size, n, r->transform_2d != 0));
  if (r->size[0] > kMaxAxis || r->size[1] > kMaxAxis || r->size[2] > kMaxAxis)
    return fail(ctx, WL_EINVAL, "axis length above %d", kMaxAxis);
  if (r->bin_count < 2 || r->bin_count > kMaxBins) return fail(ctx, WL_EFORMAT, "bad bin count");
  if (r->n_decode < 2 || !r->decode) return fail(ctx, WL_EFORMAT, "empty Huffman decode table");
  if (r->n_words < 0 || (r->n_words > 0 && !r->words))
    return fail(ctx, WL_EFORMAT, "missing Huffman stream");
  if (r->dup_key >= 0 && (r->dup_value < 0 || r->dup_value >= r->bin_count))
    return fail(ctx, WL_EFORMAT, "zero-run value out of range");
  for (int i = 0; i < r->n_decode; i += 2) {  // every entry must be a node or a symbol
    const int a = r->decode[i], b = r->decode[i + 1];
    if (a == 0 ? (b < 0 || (b >= r->bin_count && b != r->dup_key))
               : (a < 0 || 2 * a >= r->n_decode || b < 0 || 2 * b >= r->n_decode))
      return fail(ctx, WL_EFORMAT, "corrupt Huffman decode table");
  }
  if (r->quant_alg == WL_LLOYD && (!r->values || r->n_values != r->bin_count))
    return fail(ctx, WL_EFORMAT, "codebook values missing");
  return WL_OK;
}

// one symbol coded with zero bits: every element is that symbol
bool single_symbol(const wl_result *r) {
  return r->n_decode == 2 && r->decode[0] == 0 && r->decode[1] != r->dup_key;
}

wl_status decompress_impl(wl_ctx *ctx, const wl_result *r, int outType, void *out, int outOnDevice) {
  CU(cudaSetDevice(ctx->device));
  if (!r || !out) return fail(ctx, WL_EINVAL, "null argument");
  long long n;
  TRY(check_result(ctx, r, outType, n));
  std::vector<float> dq(r->bin_count);
  if (r->quant_alg == WL_LLOYD && (!r->values || r->n_values != r->bin_count))
    return fail(ctx, WL_EFORMAT, "codebook values missing");
  dequant_values(r->quant_alg, r->bin_count, r->threshold_value, r->max_value, r->values, dq.data());
  const long long padded = (n + 63) & ~63LL;
  TRY(ensure(ctx, ctx->coef, padded * 4));
  TRY(ensure(ctx, ctx->coef2, padded * 4));
  TRY(ensure(ctx, ctx->bins, padded * 4));  // int bins for the dequant kernel
  TRY(ensure(ctx, ctx->dqtable, (size_t)kMaxBins * 4));
  TRY(ensure(ctx, ctx->decWords, (size_t)r->n_words * 4 + 16));
  TRY(ensure(ctx, ctx->decTable, (size_t)r->n_decode * 4 + 16));
  TRY(ensure(ctx, ctx->decWs, decode_workspace_bytes(r->n_words)));
  TRY(ensure_host(ctx, ctx->hFlags, 64));
  cudaStream_t s = ctx->stream;
  CU(cudaMemcpyAsync(ctx->decWords.p, r->words, (size_t)r->n_words * 4, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(ctx->decTable.p, r->decode, (size_t)r->n_decode * 4, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(ctx->dqtable.p, dq.data(), dq.size() * 4, cudaMemcpyHostToDevice, s));
  if (r->n_decode == 2 && r->decode[0] == 0 && r->decode[1] != r->dup_key) {
    fill_value(P<int>(ctx->bins), n, r->decode[1], s);  // one symbol, zero-length code
  } else {
    const int rc = decode_stream(P<uint32_t>(ctx->decWords), r->n_words, P<int>(ctx->decTable),
                                 r->n_decode, r->dup_key, r->dup_value, r->bin_count, n,
                                 P<int>(ctx->bins), ctx->decWs.p, H<int>(ctx->hFlags), s);
    if (rc < 0) return fail(ctx, WL_ECUDA, "decode failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (rc > 0) return fail(ctx, WL_EFORMAT, "corrupt Huffman stream");
  }
  ctx->launches = 1;
  launch_dequant(P<int>(ctx->bins), P<float>(ctx->dqtable), P<float>(ctx->coef), n,
                 r->bin_count, s);
  CU(cudaGetLastError());
  return inverse_impl(ctx, r->size, r->steps, r->wavelet, r->original_size, outType, out,
                      outOnDevice, r->transform_2d != 0);
}

// ---- error metrics (-err) ----------------------------------------------------------
// computeErrorRatesAfterDequant (test_compress_common.cc:616-694) with
// ErrorAccumulator (test_compress_common.h:90-160): the cubelet restored to
// floats on the device (the reference dequantizes its bins, which the
// lossless Huffman stream gives back exactly, and runs the inverse
// transform), compared there, the per-CTA sums added here in CTA order.
wl_status error_impl(wl_ctx *ctx, const wl_result *r, const void *orig, int odt, int origOnDevice,
                     float maxPossible, wl_error_stats *out) {
  if (!out) return fail(ctx, WL_EINVAL, "null argument");
  memset(out, 0, sizeof *out);
  if (!r || !orig) return fail(ctx, WL_EINVAL, "null argument");
  if (dtype_size(odt) == 0) return fail(ctx, WL_EINVAL, "bad original dtype %d", odt);
  if (odt == WL_U8 && !(maxPossible > 0)) maxPossible = 255.f;
  if (!(maxPossible > 0)) return WL_OK;  // nothing computed, like the reference
  const long long n = (long long)r->original_size[0] * r->original_size[1] * r->original_size[2];
  if (n <= 0) return fail(ctx, WL_EINVAL, "empty cubelet");
  const int blocks = err_sums_blocks(n);
  TRY(ensure(ctx, ctx->errRest, (size_t)n * 4));
  TRY(ensure(ctx, ctx->errPart, (size_t)blocks * 4 * sizeof(double)));
  TRY(decompress_impl(ctx, r, WL_F32, ctx->errRest.p, 1));
  cudaStream_t s = ctx->stream;
  const void *dOrig = orig;
  if (!origOnDevice) {
    TRY(ensure(ctx, ctx->errIn, (size_t)n * dtype_size(odt)));
    CU(cudaMemcpyAsync(ctx->errIn.p, orig, (size_t)n * dtype_size(odt), cudaMemcpyHostToDevice, s));
    dOrig = ctx->errIn.p;
  }
  launch_err_sums(dOrig, odt, P<float>(ctx->errRest), n, P<double>(ctx->errPart), blocks, s);
  CU(cudaGetLastError());
  std::vector<double> part((size_t)blocks * 4);
  CU(cudaMemcpyAsync(part.data(), ctx->errPart.p, part.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  double sv = 0, svv = 0, sd = 0, sdd = 0;
  for (int b = 0; b < blocks; b++) {
    sv += part[4 * b];
    svv += part[4 * b + 1];
    sd += part[4 * b + 2];
    sdd += part[4 * b + 3];
  }
  out->count = n;
  out->sum_value = sv;
  out->sum_value_squared = svv;
  out->sum_diff = sd;
  out->sum_diff_squared = sdd;
  // the reference's getters (float results)
  out->average_error = (float)(sd / n);
  out->l1 = (float)sd;
  out->l2 = (float)sqrt(sdd);
  out->mse = (float)(sdd / n);
  const float peak2 = maxPossible * maxPossible;
  out->psnr = out->mse == 0.f ? 0.f : (float)(10.0 * log10((double)(peak2 / out->mse)));
  out->relative_error = svv == 0 ? 0.f : (float)(sdd / svv);
  return WL_OK;
}

// ---- tile autotuner -------------------------------------------------------------
// For every size class of the column-tile transform -- pass (forward x / y / z,
// inverse z / y / x), element type of its global side, row-length class 2^k --
// time each tile shape that fits (32, 64 or 128 rows, four or eight warps) on
// a synthetic batch of about 2^24 elements on the device: blocks with the
// tuned axis 2^k long and the other two max(32, min(2^k, 2^((24-k)/2))) (cubes
// from 32 to 256, two 512 x 128 x 128 blocks at 512), CDF 9/7 with up to 3
// levels on the tuned axis.  The fastest shape goes into the process-wide tile
// table.  The forward x pass of 8- and 16-bit data is tuned twice, reading
// from device memory and from page-locked host memory.
wl_status autotune_impl(wl_ctx *ctx, int maxLen, int reps) {
  CU(cudaSetDevice(ctx->device));
  const long long kElems = 1LL << 24;
  TRY(ensure(ctx, ctx->coef, (kElems + 4096) * 4));
  TRY(ensure(ctx, ctx->coef2, (kElems + 4096) * 4));
  TRY(ensure(ctx, ctx->input, (kElems + 4096) * 4));
  TRY(ensure_host(ctx, ctx->hIn, (kElems + 4096) * 2));
  cudaStream_t s = ctx->stream;
  // finite, ordinary values in every element type
  CU(cudaMemsetAsync(ctx->input.p, 0x3c, (kElems + 4096) * 4, s));
  CU(cudaMemsetAsync(ctx->coef.p, 0x3c, (kElems + 4096) * 4, s));
  CU(cudaMemsetAsync(ctx->coef2.p, 0x3c, (kElems + 4096) * 4, s));
  memset(ctx->hIn.p, 0x3c, (kElems + 4096) * 2);
  void *hostDev = nullptr;
  CU(cudaHostGetDevicePointer(&hostDev, ctx->hIn.p, 0));
  std::vector<cudaEvent_t> ev(reps + 1);
  for (cudaEvent_t &e : ev) CU(cudaEventCreate(&e));
  struct EvGuard {
    std::vector<cudaEvent_t> &v;
    ~EvGuard() { for (cudaEvent_t e : v) if (e) cudaEventDestroy(e); }
  } guard{ev};
  float *c1 = P<float>(ctx->coef), *c2 = P<float>(ctx->coef2);

  for (int lg = 1; lg <= 9 && (1 << lg) <= maxLen; lg++) {
    const int L = 1 << lg;
    const int other = std::max(32, std::min(L, 1 << ((24 - lg) / 2)));
    const long long per = (long long)L * other * other;
    const int count = (int)std::max(1LL, kElems / per);
    const int steps = std::min(lg, 3);
    for (int kind = 0; kind < kTuneKinds; kind++) {
      // (element type, 16-byte host loads) of this pass's global side
      std::vector<std::pair<int, bool>> types;
      if (kind == kTuneFwdX)
        types = {{WL_U8, false}, {WL_U16, false}, {WL_I32, false}, {WL_F32, false},
                 {WL_U8, true}, {WL_U16, true}};
      else if (kind == kTuneInvX)
        types = {{WL_U8, false}, {WL_U16, false}, {WL_I32, false}, {WL_F32, false}};
      else
        types = {{WL_F32, false}};
      const int axis = kind <= kTuneFwdZ ? kind : kTuneInvX - kind;  // 0 x, 1 y, 2 z
      for (const auto &ty : types) {
        std::vector<PassDesc> g;
        for (int c = 0; c < count; c++) {
          Plan pl;
          memset(&pl, 0, sizeof pl);
          int dims[3] = {other, other, other};
          dims[axis] = L;
          pl.X = pl.Xp = dims[0]; pl.Y = pl.Yp = dims[1]; pl.Z = pl.Zp = dims[2];
          pl.sx = pl.sy = pl.sz = 0;
          (axis == 0 ? pl.sx : axis == 1 ? pl.sy : pl.sz) = steps;
          // the other axes get one level so that every pass exists
          if (axis != 0) pl.sx = 1;
          if (axis != 1) pl.sy = 1;
          if (axis != 2) pl.sz = 1;
          pl.dtype = ty.first;
          pl.p.wavelet = WL_CDF97;
          pl.pitchY = pl.X;
          pl.pitchZ = (long long)pl.X * pl.Y;
          pl.n = per;
          pl.coefOff = (long long)c * per;
          if (kind <= kTuneFwdZ) {
            const void *in = ty.second ? hostDev : ctx->input.p;
            PassGroups xs, ys, zs;
            forward_passes_cols(pl, in, ty.second, c1, c2, xs, ys, zs);
            PassGroups &ph = kind == kTuneFwdX ? xs : kind == kTuneFwdY ? ys : zs;
            for (auto &kv : ph) g.insert(g.end(), kv.second.begin(), kv.second.end());
          } else {
            const int orig[3] = {pl.X, pl.Y, pl.Z};
            const int st[3] = {pl.sx, pl.sy, pl.sz};
            PassDesc d[3];
            // every cubelet writes the same output block: timing only
            const int np = inverse_passes_cols(pl.Xp, pl.Yp, pl.Zp, orig, st, WL_CDF97,
                                               c1 + pl.coefOff, c2 + pl.coefOff,
                                               kind == kTuneInvX ? ctx->input.p : nullptr, d);
            g.push_back(d[np - 1 - (kTuneInvX - kind)]);
          }
        }
        if (g.empty()) continue;
        const size_t need = g.size() * (sizeof(PassDesc) + sizeof(int)) + 4096;
        TRY(ensure(ctx, ctx->passes, need));
        TRY(ensure_host(ctx, ctx->hPasses, need));
        const bool inv = kind >= kTuneInvZ;
        const int inType = inv ? WL_F32 : ty.first, outType = kind == kTuneInvX ? ty.first : WL_F32;
        float us[kTileShapes] = {0, 0, 0, 0, 0, 0};
        int best = -1;
        for (int ci = 0; ci < kTileShapes; ci++) {
          const TileShape cand = kTileShape[ci];
          if (!dwt_cols_rows_fit(L, cand.rows)) continue;
          std::vector<GroupLaunch> gl;
          size_t hoff = 0;
          TRY(stage_group(ctx, g, hoff, kind, inType, outType, inv, true, ty.second, gl, &cand));
          CU(cudaMemcpyAsync(ctx->passes.p, ctx->hPasses.p, hoff, cudaMemcpyHostToDevice, s));
          TRY(launch_groups(ctx, gl, 0, gl.size()));  // warm-up
          for (int r = 0; r < reps; r++) {
            CU(cudaEventRecord(ev[r], s));
            TRY(launch_groups(ctx, gl, 0, gl.size()));
          }
          CU(cudaEventRecord(ev[reps], s));
          CU(cudaEventSynchronize(ev[reps]));
          std::vector<float> t(reps);
          for (int r = 0; r < reps; r++) CU(cudaEventElapsedTime(&t[r], ev[r], ev[r + 1]));
          std::sort(t.begin(), t.end());
          us[ci] = t[reps / 2] * 1000.f;
          if (best < 0 || us[ci] < us[best]) best = ci;
        }
        if (best >= 0)
          set_tuned_cols_shape(kind, tune_type_index(ty.first, ty.second), lg, kTileShape[best], us);
      }
    }
  }
  CU(cudaStreamSynchronize(s));
  return WL_OK;
}

// ---- parameter sweep (-opt) ------------------------------------------------------
// optimizeParameters -> plotAll (optimize.cc:96-133): every threshold fraction
// 0.50, 0.51, ... (float steps) below 0.999 with every bin count 100, 110, ...
// ((int)(b * 1.1)) up to 2000, log quantization; each point's Huffman-coded
// size and the PSNR of the restored bytes.  A
// row of bin counts is one batched compression of the same device-resident
// cubelet; each point is then restored on the device and compared there.
wl_status optimize_impl(wl_ctx *ctx, const void *data, const int size[3], int onDevice,
                        const wl_params &base, wl_opt_point *pts, int cap, int *count) {
  std::vector<float> fracs;
  for (float f = .5f; f < .999f; f += 0.01f) fracs.push_back(f);
  std::vector<int> binsList;
  for (int b = 100; b <= 2000; b = (int)(b * 1.1)) binsList.push_back(b);
  const int total = (int)(fracs.size() * binsList.size());
  if (count) *count = total;
  if (!pts) return WL_OK;
  if (cap < total) return fail(ctx, WL_EINVAL, "room for %d points, %d needed", cap, total);
  TRY(check_params(ctx, base));
  CU(cudaSetDevice(ctx->device));
  const long long N = (long long)size[0] * size[1] * size[2];
  if (size[0] < 1 || size[1] < 1 || size[2] < 1) return fail(ctx, WL_EINVAL, "empty size");
  TRY(ensure(ctx, ctx->optIn, (size_t)N));
  TRY(ensure(ctx, ctx->optOut, (size_t)N));
  TRY(ensure(ctx, ctx->optErr, 16));
  cudaStream_t s = ctx->stream;
  CU(cudaMemcpyAsync(ctx->optIn.p, data, (size_t)N,
                     onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  const int m = (int)binsList.size();
  std::vector<wl_cubelet> items(m);
  std::vector<wl_result> outs(m);
  int k = 0;
  for (float f : fracs) {
    for (int i = 0; i < m; i++) {
      wl_cubelet &c = items[i];
      memset(&c, 0, sizeof c);
      c.data = ctx->optIn.p;
      c.dtype = WL_U8;
      c.size[0] = size[0]; c.size[1] = size[1]; c.size[2] = size[2];
      c.params = base;
      c.params.threshold_fraction = f;
      c.params.bin_count = binsList[i];
      c.params.quant_alg = WL_LOG;
    }
    TRY(compress_impl(ctx, items.data(), m, 1, outs.data()));
    wl_status st = WL_OK;
    for (int i = 0; i < m && st == WL_OK; i++) {
      st = decompress_impl(ctx, &outs[i], WL_U8, ctx->optOut.p, 1);
      if (st != WL_OK) break;
      launch_sq_err_u8(P<uint8_t>(ctx->optIn), P<uint8_t>(ctx->optOut), N,
                       P<unsigned long long>(ctx->optErr), s);
      unsigned long long sq = 0;
      cudaError_t e = cudaMemcpyAsync(&sq, ctx->optErr.p, 8, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) { st = fail(ctx, WL_ECUDA, "sweep error sum: %s", cudaGetErrorString(e)); break; }
      // ErrorAccumulator::getPeakSignalToNoiseRatio (test_compress_common.h:148-153)
      const float mse = (float)((double)sq / (double)N);
      wl_opt_point &pt = pts[k + i];
      pt.threshold_fraction = f;
      pt.bin_count = binsList[i];
      // totalEncodedLengthBytes (huffman.cc:241-251): every token's code,
      // dup tokens with their length bits, in 32-bit words -- the stream
      pt.size_bytes = outs[i].n_words * 4;
      pt.psnr = mse == 0.f ? 0.f : 10.f * log10f(255.f * 255.f / mse);
    }
    for (wl_result &r : outs) wl_result_free(&r);
    if (st != WL_OK) return st;
    k += m;
  }
  return WL_OK;
}

// Decompress n cubelets at once: one copy of all streams, decode tables and
// dequantization tables; every stream decoded by one set of decoder launches;
// one dequantization launch; the inverse transform as three phases of
// concurrent launch groups; the outputs copied back per cubelet.
wl_status decompress_batch_impl(wl_ctx *ctx, const wl_result *rs, int n, const int *outTypes,
                                void *const *outs, int outOnDevice) {
  CU(cudaSetDevice(ctx->device));
  if (n <= 0) return fail(ctx, WL_EINVAL, "empty batch");
  if (!rs || !outs) return fail(ctx, WL_EINVAL, "null argument");
  std::vector<long long> N(n), coefOff(n), wordsOff(n), tableOff(n), outOff(n);
  std::vector<int> ot(n);
  long long coefTotal = 0, wordsTotal = 0, tableTotal = 0, outTotal = 0, totalSub = 0;
  int nStreams = 0;
  // results whose words follow each other in memory (the results of one
  // compression call) keep that layout on the device: one copy per run
  auto follows = [&](int i) {
    return i > 0 && rs[i].words && rs[i - 1].words &&
           rs[i].words == rs[i - 1].words + rs[i - 1].n_words;
  };
  for (int i = 0; i < n; i++) {
    const wl_result *r = rs + i;
    ot[i] = outTypes ? outTypes[i] : r->original_dtype;
    if (!outs[i]) return fail(ctx, WL_EINVAL, "cubelet %d: null output", i);
    TRY(check_result(ctx, r, ot[i], N[i]));
    coefOff[i] = coefTotal;
    coefTotal += (N[i] + 63) & ~63LL;
    wordsOff[i] = follows(i) ? wordsOff[i - 1] + rs[i - 1].n_words : (wordsTotal + 3) & ~3LL;
    wordsTotal = wordsOff[i] + r->n_words;
    tableOff[i] = tableTotal;
    tableTotal += ((long long)r->n_decode + 3) & ~3LL;
    outOff[i] = outTotal;
    outTotal += ((long long)r->original_size[0] * r->original_size[1] * r->original_size[2] *
                     dtype_size(ot[i]) + 255) & ~255LL;
    if (!single_symbol(r)) {
      nStreams++;
      totalSub += decode_subsequences(r->n_words);
    }
  }
  const size_t decWsBytes = decode_batch_workspace_bytes(nStreams, totalSub);
  const size_t fillOff = (decWsBytes + 255) & ~(size_t)255;
  TRY(ensure(ctx, ctx->coef, (size_t)coefTotal * 4 + 256));
  TRY(ensure(ctx, ctx->coef2, (size_t)coefTotal * 4 + 256));
  TRY(ensure(ctx, ctx->bins, (size_t)coefTotal * 4 + 256));
  TRY(ensure(ctx, ctx->decWords, (size_t)wordsTotal * 4 + 16));
  TRY(ensure(ctx, ctx->decTable, (size_t)tableTotal * 4 + 16));
  TRY(ensure(ctx, ctx->dqtable, (size_t)n * kMaxBins * 4));
  TRY(ensure(ctx, ctx->decWs, fillOff + (size_t)n * sizeof(FillItem)));
  if (!outOnDevice) TRY(ensure(ctx, ctx->outbuf, (size_t)outTotal + 16));
  TRY(ensure_host(ctx, ctx->hDecode, (size_t)tableTotal * 4 + 16));
  TRY(ensure_host(ctx, ctx->hVals, (size_t)n * kMaxBins * 4 + (size_t)n * sizeof(FillItem)));
  TRY(ensure_host(ctx, ctx->hFlags, 64 + (size_t)n * 8));
  cudaStream_t s = ctx->stream;
  // decode tables and dequantization tables gathered into page-locked staging
  int *ht = H<int>(ctx->hDecode);
  float *hq = H<float>(ctx->hVals);
  // ranges set to one value before decoding: a single-symbol cubelet whole,
  // and the cubelets with zero runs to the zero bin's value (the decoder
  // then writes only the other values)
  FillItem *hfill = reinterpret_cast<FillItem *>(hq + (size_t)n * kMaxBins);
  int nFill = 0;
  long long fillBlocks = 0;
  std::vector<DecodeItem> items;
  items.reserve(nStreams);
  for (int i = 0; i < n; i++) {
    const wl_result *r = rs + i;
    memcpy(ht + tableOff[i], r->decode, (size_t)r->n_decode * 4);
    dequant_values(r->quant_alg, r->bin_count, r->threshold_value, r->max_value, r->values,
                   hq + (size_t)i * kMaxBins);
    const bool single = single_symbol(r);
    if (single || r->dup_value >= 0) {
      const int v = std::min(std::max(single ? r->decode[1] : r->dup_value, 0), r->bin_count - 1);
      hfill[nFill++] = FillItem{P<float>(ctx->coef) + coefOff[i], N[i],
                                hq[(size_t)i * kMaxBins + v], fillBlocks};
      fillBlocks += (N[i] + kFillBlock - 1) / kFillBlock;
    }
    if (!single) {
      DecodeItem it{P<uint32_t>(ctx->decWords) + wordsOff[i], r->n_words,
                    P<int>(ctx->decTable) + tableOff[i], r->n_decode, r->dup_key,
                    r->dup_value, r->bin_count, N[i], P<int>(ctx->bins) + coefOff[i]};
      it.fout = P<float>(ctx->coef) + coefOff[i];
      it.dq = P<float>(ctx->dqtable) + (size_t)i * kMaxBins;
      items.push_back(it);
    }
  }
  for (int i = 0; i < n;) {  // the words, run by run
    int j = i + 1;
    long long nw = rs[i].n_words;
    while (j < n && follows(j)) nw += rs[j++].n_words;
    if (nw)
      CU(cudaMemcpyAsync(P<uint32_t>(ctx->decWords) + wordsOff[i], rs[i].words, (size_t)nw * 4,
                         cudaMemcpyHostToDevice, s));
    i = j;
  }
  CU(cudaMemcpyAsync(ctx->decTable.p, ht, (size_t)tableTotal * 4, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(ctx->dqtable.p, hq, (size_t)n * kMaxBins * 4, cudaMemcpyHostToDevice, s));
  ctx->launches = 0;
  if (nFill) {
    FillItem *dfill = reinterpret_cast<FillItem *>(P<char>(ctx->decWs) + fillOff);
    CU(cudaMemcpyAsync(dfill, hfill, (size_t)nFill * sizeof(FillItem), cudaMemcpyHostToDevice, s));
    launch_fill_batch(dfill, nFill, fillBlocks, s);
    ctx->launches++;
  }
  if (!items.empty()) {
    int *hf = H<int>(ctx->hFlags);
    long long *totals = reinterpret_cast<long long *>(hf + 16);
    const int rc = decode_streams(items.data(), (int)items.size(), ctx->decWs.p, hf, totals, s);
    if (rc < 0) return fail(ctx, WL_ECUDA, "decode failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (rc > 0) return fail(ctx, WL_EFORMAT, "corrupt Huffman stream in the batch");
    ctx->launches += 5;
  }
  CU(cudaGetLastError());
  PassGroups ph[3];
  for (int i = 0; i < n; i++) {
    void *dst = outOnDevice ? outs[i] : (void *)(P<char>(ctx->outbuf) + outOff[i]);
    inverse_passes(rs[i].size, rs[i].steps, rs[i].wavelet, rs[i].original_size, ot[i],
                   rs[i].transform_2d != 0, P<float>(ctx->coef) + coefOff[i],
                   P<float>(ctx->coef2) + coefOff[i], dst, ph);
  }
  TRY(run_inverse_phases(ctx, ph));
  if (!outOnDevice)
    for (int i = 0; i < n; i++) {
      const wl_result *r = rs + i;
      const size_t bytes = (size_t)r->original_size[0] * r->original_size[1] *
                           r->original_size[2] * dtype_size(ot[i]);
      CU(cudaMemcpyAsync(outs[i], P<char>(ctx->outbuf) + outOff[i], bytes,
                         cudaMemcpyDeviceToHost, s));
    }
  CU(cudaStreamSynchronize(s));
  return WL_OK;
}

}  // namespace

namespace wl {
// A page-locked buffer of at least `bytes` owned by the context (grow-only,
// kept across calls), for the container pipeline's staging.
char *ctx_staging(wl_ctx *ctx, int slot, size_t bytes) {
  if (!ctx || slot < 0 || slot > 1) return nullptr;
  if (ensure_host(ctx, ctx->hStage[slot], bytes) != WL_OK) return nullptr;
  return H<char>(ctx->hStage[slot]);
}

wl_status result_to_meta(const wl_result *r, CubeMeta &m) {
  m.width = r->size[0]; m.height = r->size[1]; m.depth = r->size[2];
  m.transform_2d = r->transform_2d != 0;
  m.data_type = kPbInt32;
  m.compressed = true;
  m.steps[0] = r->steps[0]; m.steps[1] = r->steps[1]; m.steps[2] = r->steps[2];
  m.wavelet = r->wavelet;
  m.threshold_fraction = r->threshold_fraction;
  m.threshold_value = r->threshold_value;
  m.bin_count = r->bin_count;
  m.pb_quant_alg = r->quant_alg == WL_UNIFORM ? kPbUniform : r->quant_alg == WL_LOG ? kPbLog : kPbLloyd;
  m.quant_max_value = r->max_value;
  if (r->quant_alg == WL_LLOYD) {
    m.boundaries.assign(r->boundaries, r->boundaries + r->n_boundaries);
    m.values.assign(r->values, r->values + r->n_values);
  }
  m.decode.assign(r->decode, r->decode + r->n_decode);
  m.original_size[0] = r->original_size[0];
  m.original_size[1] = r->original_size[1];
  m.original_size[2] = r->original_size[2];
  m.original_data_type = pb_dtype(r->original_dtype);
  m.dup_key = r->dup_key;
  m.dup_value = r->dup_value;
  return WL_OK;
}

// A wl_result over a compressed cubelet's metadata and words (the arrays stay
// in m and words).
void meta_to_result(CubeMeta &m, const std::string &words, wl_result &r) {
  memset(&r, 0, sizeof r);
  r.size[0] = m.width; r.size[1] = m.height; r.size[2] = m.depth;
  r.original_size[0] = m.original_size[0];
  r.original_size[1] = m.original_size[1];
  r.original_size[2] = m.original_size[2];
  r.original_dtype = m.original_data_type == kPbUint8 ? WL_U8
                     : m.original_data_type == kPbInt32 ? WL_I32 : WL_F32;
  r.steps[0] = m.steps[0]; r.steps[1] = m.steps[1]; r.steps[2] = m.steps[2];
  r.wavelet = m.wavelet;
  r.transform_2d = m.transform_2d ? 1 : 0;
  r.quant_alg = m.pb_quant_alg == kPbUniform ? WL_UNIFORM : m.pb_quant_alg == kPbLog ? WL_LOG : WL_LLOYD;
  r.bin_count = m.bin_count;
  r.threshold_fraction = m.threshold_fraction;
  r.threshold_value = m.threshold_value;
  r.max_value = m.quant_max_value;
  r.dup_key = m.dup_key;
  r.dup_value = m.dup_value;
  r.n_words = (int)(words.size() / 4);
  r.words = (uint32_t *)const_cast<char *>(words.data());
  r.n_decode = (int)m.decode.size();
  r.decode = m.decode.data();
  r.n_values = (int)m.values.size();
  r.values = m.values.data();
  r.n_boundaries = (int)m.boundaries.size();
  r.boundaries = m.boundaries.data();
}
}  // namespace wl

namespace {

}  // namespace

// ============================================================== C ABI
extern "C" {

void wl_params_default(wl_params *p) {
  p->steps[0] = p->steps[1] = p->steps[2] = -1;
  p->wavelet = WL_CDF97;
  p->threshold_fraction = 0.5f;
  p->bin_count = 256;
  p->quant_alg = WL_LOG;
  p->compress_zeros = 1;
  p->lloyd_iters = 20;
  p->exact_transform = 0;
  p->transform_2d = 0;
}

void wl_result_free(wl_result *r) {
  if (!r) return;
  if (r->owner) {
    ResultSlab *s = static_cast<ResultSlab *>(r->owner);
    if (s->refs.fetch_sub(1) == 1) slab_pool().release(s);
  } else {
    free(r->words);
    free(r->decode);
    free(r->boundaries);
    free(r->values);
  }
  memset(r, 0, sizeof *r);
}

void wl_results_free(wl_result *r, int n) {
  if (!r) return;
  for (int i = 0; i < n; i++) wl_result_free(r + i);
}

wl_status wl_init(int device, wl_ctx **out) {
  if (!out) return WL_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return WL_ECUDA;
  }
  if (device < 0 || device >= count) return WL_EINVAL;
  wl_ctx *ctx = new wl_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return WL_ECUDA;
  }
  for (auto &e : ctx->ev) cudaEventCreate(&e);
  bool sideOk = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < wl_ctx::kSide && sideOk; k++)
    sideOk = cudaStreamCreateWithFlags(&ctx->side[k], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->join[k], cudaEventDisableTiming) == cudaSuccess;
  if (!sideOk) {  // phases then run in order on the context's stream
    cudaGetLastError();
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    ctx->fork = nullptr;
  }
  for (auto &e : ctx->pev) cudaEventCreate(&e);
  bool ok2 = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->halfT, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->halfJ, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->fork2, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < wl_ctx::kSide && ok2; k++)
    ok2 = cudaStreamCreateWithFlags(&ctx->side2[k], cudaStreamNonBlocking) == cudaSuccess &&
          cudaEventCreateWithFlags(&ctx->join2[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok2) {
    cudaGetLastError();  // batches then run as one
    ctx->splitMode = 0;
  }
  *out = ctx;
  return WL_OK;
}

void wl_destroy(wl_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf *dbs[] = {&ctx->input, &ctx->coef, &ctx->coef2, &ctx->bins, &ctx->tokCount,
                   &ctx->state,
                   &ctx->selHist, &ctx->lloydHist, &ctx->qtable, &ctx->dqtable, &ctx->qlut, &ctx->hist,
                   &ctx->chunkRun, &ctx->chunkRunCtx, &ctx->chunkBits, &ctx->chunkCub, &ctx->groupCub,
                   &ctx->encCub, &ctx->sliceOff,
                   &ctx->chunkSpan, &ctx->optIn, &ctx->optOut, &ctx->optErr,
                   &ctx->codes, &ctx->codeLen, &ctx->decode, &ctx->words, &ctx->passes,
                   &ctx->logHdr, &ctx->outbuf, &ctx->decWords, &ctx->decTable, &ctx->decWs,
                   &ctx->meta, &ctx->errIn, &ctx->errRest, &ctx->errPart};
  for (DevBuf *d : dbs) if (d->p) cudaFree(d->p);
  for (GraphEntry &g : ctx->graphs) drop_graph(g);
  HostBuf *hbs[] = {&ctx->hStage[0], &ctx->hStage[1], &ctx->hState, &ctx->hDecode, &ctx->hPasses,
                    &ctx->hTab, &ctx->hLogHdr, &ctx->hPrefix, &ctx->hIn, &ctx->hVals,
                    &ctx->hFlags};
  for (HostBuf *h : hbs) if (h->p) cudaFreeHost(h->p);
  for (auto &e : ctx->ev) if (e) cudaEventDestroy(e);
  for (auto &e : ctx->pev) if (e) cudaEventDestroy(e);
  for (int k = 0; k < wl_ctx::kSide; k++) {
    if (ctx->side[k]) cudaStreamDestroy(ctx->side[k]);
    if (ctx->join[k]) cudaEventDestroy(ctx->join[k]);
  }
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->stream2) {
    cudaStreamSynchronize(ctx->stream2);
    cudaStreamDestroy(ctx->stream2);
  }
  if (ctx->halfT) cudaEventDestroy(ctx->halfT);
  if (ctx->halfJ) cudaEventDestroy(ctx->halfJ);
  if (ctx->fork2) cudaEventDestroy(ctx->fork2);
  for (int k = 0; k < wl_ctx::kSide; k++) {
    if (ctx->side2[k]) cudaStreamDestroy(ctx->side2[k]);
    if (ctx->join2[k]) cudaEventDestroy(ctx->join2[k]);
  }
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *wl_last_error(const wl_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

wl_status wl_compress_cubelet(wl_ctx *ctx, const void *data, int dtype, const int size[3],
                              int onDevice, const wl_params *params, wl_result *out) {
  if (!ctx || !data || !size || !params || !out) return fail(ctx, WL_EINVAL, "null argument");
  wl_cubelet it;
  memset(&it, 0, sizeof it);
  it.data = data;
  it.dtype = dtype;
  it.size[0] = size[0]; it.size[1] = size[1]; it.size[2] = size[2];
  it.params = *params;
  return compress_impl(ctx, &it, 1, onDevice, out);
}

wl_status wl_compress_batch(wl_ctx *ctx, const wl_cubelet *items, int n, int onDevice,
                            wl_result *outs) {
  if (!ctx || !items || !outs) return fail(ctx, WL_EINVAL, "null argument");
  return compress_impl(ctx, items, n, onDevice, outs);
}

wl_status wl_decompress_cubelet(wl_ctx *ctx, const wl_result *in, int outType, void *out,
                                int outOnDevice) {
  if (!ctx) return WL_EINVAL;
  return decompress_impl(ctx, in, outType, out, outOnDevice);
}

wl_status wl_decompress_batch(wl_ctx *ctx, const wl_result *in, int n, const int *out_dtypes,
                              void *const *outs, int outs_on_device) {
  if (!ctx) return WL_EINVAL;
  return decompress_batch_impl(ctx, in, n, out_dtypes, outs, outs_on_device);
}

wl_status wl_encode_cube(const wl_result *r, int footer, uint8_t **buf, size_t *len) {
  if (!r || !buf || !len) return WL_EINVAL;
  CubeMeta m;
  result_to_meta(r, m);
  std::string words((const char *)r->words, (size_t)r->n_words * 4);
  std::string f = encode_file({m}, {&words}, footer != 0);
  *buf = (uint8_t *)malloc(f.size());
  if (!*buf) return WL_ENOMEM;
  memcpy(*buf, f.data(), f.size());
  *len = f.size();
  return WL_OK;
}

void wl_free(void *p) { free(p); }

wl_status wl_compress_file(wl_ctx *ctx, const char *inPath, const char *outPath,
                           const wl_params *params) {
  if (!ctx || !inPath || !outPath || !params) return fail(ctx, WL_EINVAL, "null argument");
  std::string buf, err;
  if (!read_whole_file(inPath, buf)) return fail(ctx, WL_EIO, "cannot read %s", inPath);
  std::vector<CubeMeta> metas;
  std::vector<std::string> datas;
  if (!decode_file(buf, metas, datas, err)) return fail(ctx, WL_EFORMAT, "%s: %s", inPath, err.c_str());
  // first uncompressed cubelet (readData, test_compress_common.cc:296-302)
  for (size_t i = 0; i < metas.size(); i++) {
    const CubeMeta &m = metas[i];
    if (m.compressed) continue;
    int dt = m.data_type == kPbUint8 ? WL_U8 : m.data_type == kPbInt32 ? WL_I32
             : m.data_type == kPbFloat32 ? WL_F32 : 0;
    if (!dt) return fail(ctx, WL_EFORMAT, "unknown data type %d", m.data_type);
    const size_t need = (size_t)m.width * m.height * m.depth * dtype_size(dt);
    if (datas[i].size() < need) return fail(ctx, WL_EFORMAT, "cubelet data truncated");
    int size[3] = {m.width, m.height, m.depth};
    wl_result r;
    TRY(wl_compress_cubelet(ctx, datas[i].data(), dt, size, 0, params, &r));
    CubeMeta om;
    result_to_meta(&r, om);
    std::string words((const char *)r.words, (size_t)r.n_words * 4);
    wl_result_free(&r);
    // the reference closes the compressed file without a footer
    // (test_compress_cpu.cc:174-175)
    if (!write_whole_file(outPath, encode_file({om}, {&words}, false)))
      return fail(ctx, WL_EIO, "cannot write %s", outPath);
    return WL_OK;
  }
  return fail(ctx, WL_EFORMAT, "No uncompressed cubelets in the input data.");
}

wl_status wl_error_metrics(wl_ctx *ctx, const wl_result *compressed, const void *original,
                           int original_dtype, int original_on_device, float max_possible,
                           wl_error_stats *out) {
  if (!ctx) return WL_EINVAL;
  CU(cudaSetDevice(ctx->device));
  return error_impl(ctx, compressed, original, original_dtype, original_on_device, max_possible,
                    out);
}

wl_status wl_error_metrics_file(wl_ctx *ctx, const char *origPath, const char *compPath,
                                wl_error_stats *out) {
  if (!ctx || !origPath || !compPath || !out) return fail(ctx, WL_EINVAL, "null argument");
  std::string ob, cb, err;
  if (!read_whole_file(origPath, ob)) return fail(ctx, WL_EIO, "cannot read %s", origPath);
  if (!read_whole_file(compPath, cb)) return fail(ctx, WL_EIO, "cannot read %s", compPath);
  std::vector<CubeMeta> om, cm;
  std::vector<std::string> od, cd;
  if (!decode_file(ob, om, od, err)) return fail(ctx, WL_EFORMAT, "%s: %s", origPath, err.c_str());
  if (!decode_file(cb, cm, cd, err)) return fail(ctx, WL_EFORMAT, "%s: %s", compPath, err.c_str());
  int oi = -1, ci = -1;
  for (size_t i = 0; i < om.size() && oi < 0; i++)
    if (!om[i].compressed) oi = (int)i;
  for (size_t i = 0; i < cm.size() && ci < 0; i++)
    if (cm[i].compressed) ci = (int)i;
  if (oi < 0) return fail(ctx, WL_EFORMAT, "No uncompressed cubelets in %s", origPath);
  if (ci < 0) return fail(ctx, WL_EFORMAT, "No compressed cubelets in %s", compPath);
  const CubeMeta &m = om[oi];
  const int dt = m.data_type == kPbUint8 ? WL_U8 : m.data_type == kPbInt32 ? WL_I32
                 : m.data_type == kPbFloat32 ? WL_F32 : 0;
  if (!dt) return fail(ctx, WL_EFORMAT, "unknown data type %d", m.data_type);
  if (od[oi].size() < (size_t)m.width * m.height * m.depth * dtype_size(dt))
    return fail(ctx, WL_EFORMAT, "cubelet data truncated");
  wl_result r;
  meta_to_result(cm[ci], cd[ci], r);
  if (r.original_size[0] != m.width || r.original_size[1] != m.height ||
      r.original_size[2] != m.depth)
    return fail(ctx, WL_EINVAL, "the compressed cubelet is %dx%dx%d, the original %dx%dx%d",
                r.original_size[0], r.original_size[1], r.original_size[2], m.width, m.height,
                m.depth);
  return wl_error_metrics(ctx, &r, od[oi].data(), dt, 0, (float)m.maximum_value, out);
}

wl_status wl_optimize_file(wl_ctx *ctx, const char *inPath, const wl_params *params,
                           wl_opt_point *points, int cap, int *n_points) {
  if (!ctx || !inPath || !params) return fail(ctx, WL_EINVAL, "null argument");
  std::string buf, err;
  if (!read_whole_file(inPath, buf)) return fail(ctx, WL_EIO, "cannot read %s", inPath);
  std::vector<CubeMeta> metas;
  std::vector<std::string> datas;
  if (!decode_file(buf, metas, datas, err)) return fail(ctx, WL_EFORMAT, "%s: %s", inPath, err.c_str());
  for (size_t i = 0; i < metas.size(); i++) {
    const CubeMeta &m = metas[i];
    if (m.compressed) continue;
    // the reference's sweep takes 8-bit data only (test_compress_cpu.cc:107)
    if (m.data_type != kPbUint8) return fail(ctx, WL_EINVAL, "-opt needs 8-bit data");
    if (datas[i].size() < (size_t)m.width * m.height * m.depth)
      return fail(ctx, WL_EFORMAT, "cubelet data truncated");
    int size[3] = {m.width, m.height, m.depth};
    return wl_optimize(ctx, datas[i].data(), size, 0, params, points, cap, n_points);
  }
  return fail(ctx, WL_EFORMAT, "No uncompressed cubelets in the input data.");
}

wl_status wl_decompress_file(wl_ctx *ctx, const char *inPath, const char *outPath) {
  if (!ctx || !inPath || !outPath) return fail(ctx, WL_EINVAL, "null argument");
  std::string buf, err;
  if (!read_whole_file(inPath, buf)) return fail(ctx, WL_EIO, "cannot read %s", inPath);
  std::vector<CubeMeta> metas;
  std::vector<std::string> datas;
  if (!decode_file(buf, metas, datas, err)) return fail(ctx, WL_EFORMAT, "%s: %s", inPath, err.c_str());
  // first compressed INT32 cubelet (readQuantData, test_compress_common.cc:850-862)
  for (size_t i = 0; i < metas.size(); i++) {
    CubeMeta &m = metas[i];
    if (!m.compressed || m.data_type != kPbInt32) continue;
    if (datas[i].size() % 4)
      return fail(ctx, WL_EFORMAT, "compressed data of %zu bytes is not a whole number of "
                  "32-bit words", datas[i].size());
    wl_result r;
    meta_to_result(m, datas[i], r);
    const int odt = r.original_dtype;
    if (r.original_size[0] == 0) {
      return fail(ctx, WL_EFORMAT, "compressed cubelet lacks its original size");
    }
    const size_t n = (size_t)r.original_size[0] * r.original_size[1] * r.original_size[2];
    std::string out(n * dtype_size(odt), '\0');
    TRY(decompress_impl(ctx, &r, odt, &out[0], 0));
    CubeMeta om;
    om.width = r.original_size[0]; om.height = r.original_size[1]; om.depth = r.original_size[2];
    om.data_type = pb_dtype(odt);
    if (!write_whole_file(outPath, encode_file({om}, {&out}, true)))
      return fail(ctx, WL_EIO, "cannot write %s", outPath);
    return WL_OK;
  }
  return fail(ctx, WL_EFORMAT, "No compressed cubelet found");
}

wl_status wl_forward_transform(wl_ctx *ctx, const void *data, int dtype, const int size[3],
                               const wl_params *params, float *coeffs, size_t cap,
                               int stored[3]) {
  if (!ctx || !data || !size || !params || !coeffs || !stored)
    return fail(ctx, WL_EINVAL, "null argument");
  wl_cubelet it;
  memset(&it, 0, sizeof it);
  it.data = data;
  it.dtype = dtype;
  it.size[0] = size[0]; it.size[1] = size[1]; it.size[2] = size[2];
  it.params = *params;
  wl_result dummy;
  return compress_impl(ctx, &it, 1, 0, &dummy, coeffs, cap, stored);
}

wl_status wl_inverse_transform(wl_ctx *ctx, const float *coeffs, const int stored[3],
                               const int steps[3], int wavelet, const int orig[3],
                               int outType, void *out) {
  if (!ctx || !coeffs || !stored || !steps || !orig || !out)
    return fail(ctx, WL_EINVAL, "null argument");
  CU(cudaSetDevice(ctx->device));
  if (dtype_size(outType) == 0) return fail(ctx, WL_EINVAL, "bad output dtype %d", outType);
  if (wavelet != WL_HAAR && wavelet != WL_CDF97) return fail(ctx, WL_EINVAL, "unknown wavelet");
  long long n;
  TRY(check_sizes(ctx, stored, steps, orig, n));
  if (stored[0] > kMaxAxis || stored[1] > kMaxAxis || stored[2] > kMaxAxis)
    return fail(ctx, WL_EINVAL, "axis length above %d", kMaxAxis);
  TRY(ensure(ctx, ctx->coef, n * 4 + 256));
  TRY(ensure(ctx, ctx->coef2, n * 4 + 256));
  CU(cudaMemcpyAsync(ctx->coef.p, coeffs, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  return inverse_impl(ctx, stored, steps, wavelet, orig, outType, out, 0);
}

wl_status wl_optimize(wl_ctx *ctx, const void *data, const int size[3], int data_on_device,
                      const wl_params *params, wl_opt_point *points, int cap, int *n_points) {
  if (!ctx || !data || !size || !params) return fail(ctx, WL_EINVAL, "null argument");
  return optimize_impl(ctx, data, size, data_on_device, *params, points, cap, n_points);
}

wl_status wl_autotune(wl_ctx *ctx, int max_len, int reps) {
  if (!ctx) return WL_EINVAL;
  if (max_len <= 0 || max_len > kColsMaxL) max_len = kColsMaxL;
  if (reps <= 0) reps = 5;
  if (reps > 64) reps = 64;
  return autotune_impl(ctx, max_len, reps);
}

wl_status wl_set_stream_priority(wl_ctx *ctx, int high) {
  if (!ctx) return WL_EINVAL;
  CU(cudaSetDevice(ctx->device));
  int least = 0, greatest = 0;
  CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  const int prio = high ? greatest : least;
  // new streams, once the old ones have drained (captured graphs are not
  // bound to a stream and stay valid)
  cudaStream_t ns = nullptr;
  CU(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
  cudaStream_t nside[wl_ctx::kSide] = {};
  for (int k = 0; k < wl_ctx::kSide; k++)
    if (ctx->side[k] &&
        cudaStreamCreateWithPriority(&nside[k], cudaStreamNonBlocking, prio) != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < k; j++) cudaStreamDestroy(nside[j]);
      cudaStreamDestroy(ns);
      return fail(ctx, WL_ECUDA, "cannot create a stream of priority %d", prio);
    }
  CU(cudaStreamSynchronize(ctx->stream));
  cudaStreamDestroy(ctx->stream);
  ctx->stream = ns;
  if (ctx->stream2) {
    cudaStream_t n2 = nullptr;
    if (cudaStreamCreateWithPriority(&n2, cudaStreamNonBlocking, prio) == cudaSuccess) {
      cudaStreamSynchronize(ctx->stream2);
      cudaStreamDestroy(ctx->stream2);
      ctx->stream2 = n2;
    } else {
      cudaGetLastError();
    }
  }
  for (int k = 0; k < wl_ctx::kSide; k++)
    if (ctx->side[k]) {
      cudaStreamSynchronize(ctx->side[k]);
      cudaStreamDestroy(ctx->side[k]);
      ctx->side[k] = nside[k];
    }
  return WL_OK;
}

wl_status wl_set_memory_limit(wl_ctx *ctx, size_t bytes) {
  if (!ctx) return WL_EINVAL;
  ctx->memLimit = bytes;
  return WL_OK;
}

size_t wl_memory_held(const wl_ctx *ctx) { return ctx ? ctx->devBytes : 0; }

wl_status wl_set_host_input_mode(wl_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return WL_EINVAL;
  ctx->stageHost = mode;
  return WL_OK;
}

wl_status wl_set_encode_slices(wl_ctx *ctx, int slices) {
  if (!ctx || slices < 0 || slices > 32 || (slices & (slices - 1))) return WL_EINVAL;
  ctx->encSlices = slices;
  return WL_OK;
}

wl_status wl_set_graph_mode(wl_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return WL_EINVAL;
  ctx->graphMode = mode;
  if (!mode) {
    for (GraphEntry &g : ctx->graphs) drop_graph(g);
    ctx->graphs.clear();
    ctx->lastKey.clear();
  }
  return WL_OK;
}

wl_status wl_graph_stats(const wl_ctx *ctx, long long out[4]) {
  if (!ctx || !out) return WL_EINVAL;
  for (int i = 0; i < 4; i++) out[i] = ctx->graphStats[i];
  return WL_OK;
}

const char *wl_graph_error(const wl_ctx *ctx) { return ctx ? ctx->graphErr.c_str() : ""; }

wl_status wl_last_timings(const wl_ctx *ctx, float out[6]) {
  if (!ctx || !out) return WL_EINVAL;
  memcpy(out, ctx->timings, sizeof ctx->timings);
  return WL_OK;
}

void *wl_device_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void wl_device_free(void *p) {
  if (p) cudaFree(p);
}

wl_status wl_copy_to_device(void *dst, const void *src, size_t bytes) {
  return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? WL_OK : WL_ECUDA;
}

wl_status wl_copy_to_host(void *dst, const void *src, size_t bytes) {
  return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? WL_OK : WL_ECUDA;
}

int wl_last_launch_count(const wl_ctx *ctx) { return ctx ? ctx->launches : 0; }

wl_status wl_set_profiling(wl_ctx *ctx, int on) {
  if (!ctx) return WL_EINVAL;
  ctx->profiling = on != 0;
  return WL_OK;
}

wl_status wl_kernel_timings(const wl_ctx *ctx, float out[9]) {
  if (!ctx || !out) return WL_EINVAL;
  memcpy(out, ctx->ktimes, sizeof ctx->ktimes);
  return WL_OK;
}

void *wl_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void wl_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

wl_status wl_sync(wl_ctx *ctx) {
  if (!ctx) return WL_EINVAL;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(ctx, WL_ECUDA, "%s", cudaGetErrorString(e));
  return WL_OK;
}

}  // extern "C"
