// Whole .cube containers: every cubelet of a file compressed (or restored)
// into a new file, with reading, GPU work and writing overlapped.
//
// The reference writes and reads containers one cubelet at a time
// (CubeletStreamWriter / CubeletStreamReader, cubelet_file.cc:153-327 and
// :330-540) and its compressor takes only the first cubelet of a file
// (readData, test_compress_common.cc:296-302).  Here three stages run at
// once: a reader thread parses the input stream (64-byte header, then per
// cubelet a 4-byte length, the CubeletBuffer message and the data) into one
// of two page-locked staging buffers; the calling thread compresses a full
// buffer as one batch (the GPU reads the cubelets in place) while the reader
// fills the other; a writer thread appends each finished batch's cubelets
// (length, message, Huffman words from the page-locked result block) and
// finally the index footer (0xFFFFFFFF, CubeletIndexBuffer, its length,
// "cube"; cubelet_file.cc:303-327) with every cubelet's data_file_offset.
// Cubelets that are already in the target form (compressed ones when
// compressing, uncompressed ones when restoring) are copied through
// unchanged; every cubelet keeps its x/y/z offset in the parent volume and
// its maximum value.
#include <cuda_runtime.h>

#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cubelet_io.h"
#include "wl_internal.h"
#include "wlgpu.h"

namespace {

using namespace wl;
using Clock = std::chrono::steady_clock;

double secs(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

template <class T> class Queue {
 public:
  void push(T v) {
    {
      std::lock_guard<std::mutex> g(mu_);
      q_.push_back(std::move(v));
    }
    cv_.notify_all();
  }
  // false once closed and drained
  bool pop(T &v) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return closed_ || !q_.empty(); });
    if (q_.empty()) return false;
    v = std::move(q_.front());
    q_.pop_front();
    return true;
  }
  void close() {
    {
      std::lock_guard<std::mutex> g(mu_);
      closed_ = true;
    }
    cv_.notify_all();
  }

 private:
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<T> q_;
  bool closed_ = false;
};

struct Item {
  CubeMeta meta;
  const char *staged = nullptr;  // data in a staging buffer, or null
  size_t bytes = 0;
  std::string own;               // data read outside the staging buffers
  long long fileOff = 0;         // where the data starts in the input file
  bool through = false;          // copied to the output unchanged
  // the cubelet's data (taken when used: `own` moves with the item)
  const char *data() const { return staged ? staged : own.data(); }
};

struct Batch {
  std::vector<Item> items;
  int buf = -1;  // staging buffer holding the data, -1 none
};

struct Done {
  std::vector<Item> items;
  std::vector<wl_result> res;          // per item (unused for copied items)
  std::vector<std::string> restored;   // restoring: per item output data
};

int wl_type(int pb) {
  return pb == kPbUint8 ? WL_U8 : pb == kPbInt32 ? WL_I32 : pb == kPbFloat32 ? WL_F32 : 0;
}
int elem_size(int pb) { return pb == kPbUint8 ? 1 : 4; }

// Page-locked double buffer shared by the reader and the compute stage (the
// context's, kept across calls: page-locking hundreds of MB per call would
// cost more than the transfers).
struct Staging {
  char *buf[2] = {nullptr, nullptr};
  size_t cap = 0;
  bool busy[2] = {false, false};
  std::mutex mu;
  std::condition_variable cv;
  bool init(wl_ctx *ctx, size_t bytes) {
    cap = bytes;
    for (int i = 0; i < 2; i++)
      if (!(buf[i] = ctx_staging(ctx, i, bytes))) return false;
    return true;
  }
  void acquire(int i) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return !busy[i]; });
    busy[i] = true;
  }
  void release(int i) {
    {
      std::lock_guard<std::mutex> g(mu);
      busy[i] = false;
    }
    cv.notify_all();
  }
};

struct Shared {
  std::mutex mu;
  std::string err;
  void fail(const std::string &e) {
    std::lock_guard<std::mutex> g(mu);
    if (err.empty()) err = e;
  }
  bool failed() {
    std::lock_guard<std::mutex> g(mu);
    return !err.empty();
  }
};

// Reader: parse the input container into batches.  restoring: compressed
// cubelets are the work (read into `own`), uncompressed ones are copied;
// compressing: uncompressed cubelets go to the staging buffers.  The
// metadata is parsed in order (the data is skipped); a batch's data is then
// read by several threads at once (pread at the known offsets), which moves
// a page-cached file several times faster than one thread.
struct ReadTask {
  long long off;
  char *dst;
  size_t bytes;
};

bool read_parallel(int fd, std::vector<ReadTask> &tasks) {
  if (tasks.empty()) return true;
  size_t total = 0;
  for (const ReadTask &t : tasks) total += t.bytes;
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nThreads = (int)std::min<size_t>({(size_t)std::min(hw, 8), tasks.size(),
                                               total / (1 << 20) + 1});
  // split into pieces of at most 8 MB so that one large cubelet spreads too
  std::vector<ReadTask> pieces;
  for (const ReadTask &t : tasks)
    for (size_t o = 0; o < t.bytes; o += (8 << 20))
      pieces.push_back({t.off + (long long)o, t.dst + o, std::min<size_t>(8 << 20, t.bytes - o)});
  std::atomic<size_t> next{0};
  std::atomic<bool> ok{true};
  auto work = [&]() {
    for (size_t k; (k = next.fetch_add(1)) < pieces.size();) {
      const ReadTask &t = pieces[k];
      size_t done = 0;
      while (done < t.bytes) {
        const ssize_t r = pread(fd, t.dst + done, t.bytes - done, (off_t)(t.off + done));
        if (r <= 0) { ok = false; return; }
        done += (size_t)r;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nThreads; i++) pool.emplace_back(work);
  work();
  for (std::thread &th : pool) th.join();
  tasks.clear();
  return ok.load();
}

void reader(FILE *f, bool restoring, Staging *st, size_t batchBytes, Queue<Batch> *out,
            Shared *sh, double *readSecs) {
  const Clock::time_point t0 = Clock::now();
  const int fd = fileno(f);
  Batch b;
  std::vector<ReadTask> tasks;
  int cur = 0;
  size_t used = 0;
  bool haveBuf = false;
  auto flush = [&]() {
    if (b.items.empty()) return;
    // `own` buffers are final now (no more pushes into this batch)
    for (Item &it : b.items)
      if (!it.staged && it.bytes) tasks.push_back({it.fileOff, &it.own[0], it.bytes});
    if (!read_parallel(fd, tasks)) sh->fail("truncated cubelet data");
    b.buf = haveBuf ? cur : -1;
    out->push(std::move(b));
    b = Batch();
    if (haveBuf) cur ^= 1;
    haveBuf = false;
    used = 0;
  };
  size_t batchWork = 0;
  long long pos = 64;
  for (;;) {
    if (sh->failed()) break;
    uint32_t len;
    if (fread(&len, 4, 1, f) != 1 || len == 0xFFFFFFFFu) break;
    std::string msg(len, '\0');
    if (len && fread(&msg[0], 1, len, f) != len) { sh->fail("truncated cubelet metadata"); break; }
    pos += 4 + (long long)len;
    Item it;
    if (!decode_meta(msg.data(), msg.size(), it.meta)) { sh->fail("malformed cubelet metadata"); break; }
    it.bytes = (size_t)it.meta.byte_count;
    it.fileOff = pos;
    if (fseeko(f, (off_t)it.bytes, SEEK_CUR) != 0) { sh->fail("truncated cubelet data"); break; }
    pos += (long long)it.bytes;
    const bool work = restoring ? it.meta.compressed : !it.meta.compressed;
    it.through = !work;
    if (work && !restoring) {
      const size_t need = (size_t)it.meta.width * it.meta.height * it.meta.depth *
                          elem_size(it.meta.data_type);
      if (!wl_type(it.meta.data_type) || it.bytes < need) { sh->fail("bad cubelet data"); break; }
      const size_t slot = (it.bytes + 255) & ~(size_t)255;
      if (slot <= st->cap) {
        if (haveBuf && used + slot > st->cap) flush();
        if (!haveBuf) {
          st->acquire(cur);
          haveBuf = true;
        }
        it.staged = st->buf[cur] + used;
        tasks.push_back({it.fileOff, const_cast<char *>(it.staged), it.bytes});
        used += slot;
      }
    }
    if (!it.staged) it.own.resize(it.bytes);  // filled at the batch's flush
    batchWork += it.bytes;
    b.items.push_back(std::move(it));
    // restoring: batches by input bytes (no staging buffers)
    if (restoring && batchWork >= batchBytes) {
      flush();
      batchWork = 0;
    }
    if (!restoring && !haveBuf && batchWork >= batchBytes) {
      flush();
      batchWork = 0;
    }
    if (!restoring && haveBuf && used >= st->cap) {
      flush();
      batchWork = 0;
    }
  }
  flush();
  out->close();
  *readSecs = secs(t0, Clock::now());
}

// Writer: header, the cubelets in order, the index footer.
void writer(FILE *f, bool restoring, Queue<Done> *in, Shared *sh, unsigned long long *bytesOut,
            int *written, int *through, double *writeSecs) {
  double busy = 0;
  char header[64] = {0};
  memcpy(header, kCubeHeader, strlen(kCubeHeader));
  bool ok = fwrite(header, 1, 64, f) == 64;
  unsigned long long off = 64;
  std::string index;
  Done d;
  while (in->pop(d)) {
    const Clock::time_point t0 = Clock::now();
    for (size_t i = 0; i < d.items.size() && ok; i++) {
      Item &it = d.items[i];
      CubeMeta m;
      const char *data;
      size_t bytes;
      if (it.through) {
        m = it.meta;
        data = it.data();
        bytes = it.bytes;
        (*through)++;
      } else if (!restoring) {
        const wl_result &r = d.res[i];
        result_to_meta(&r, m);
        m.offset[0] = it.meta.offset[0]; m.offset[1] = it.meta.offset[1];
        m.offset[2] = it.meta.offset[2];
        m.maximum_value = it.meta.maximum_value;
        data = reinterpret_cast<const char *>(r.words);
        bytes = (size_t)r.n_words * 4;
      } else {
        const CubeMeta &c = it.meta;
        m.width = c.original_size[0]; m.height = c.original_size[1]; m.depth = c.original_size[2];
        m.data_type = c.original_data_type ? c.original_data_type : kPbFloat32;
        m.offset[0] = c.offset[0]; m.offset[1] = c.offset[1]; m.offset[2] = c.offset[2];
        m.maximum_value = c.maximum_value;
        data = d.restored[i].data();
        bytes = d.restored[i].size();
      }
      m.byte_count = bytes;
      const std::string enc = encode_meta(m, 0);
      const uint32_t n = (uint32_t)enc.size();
      ok = fwrite(&n, 4, 1, f) == 1 && fwrite(enc.data(), 1, n, f) == n &&
           (bytes == 0 || fwrite(data, 1, bytes, f) == bytes);
      off += 4 + n;
      // CubeletIndexBuffer.cubelets (field 5, wavelet_compress.proto:173)
      // with data_file_offset
      const std::string ie = encode_meta(m, off);
      index.push_back((char)((5 << 3) | 2));
      for (uint64_t v = ie.size(); ; v >>= 7) {
        if (v < 0x80) { index.push_back((char)v); break; }
        index.push_back((char)((v & 0x7f) | 0x80));
      }
      index += ie;
      off += bytes;
      *bytesOut += bytes;
      (*written)++;
    }
    if (!restoring)
      for (wl_result &r : d.res) wl_result_free(&r);
    busy += secs(t0, Clock::now());
    if (!ok) sh->fail("write failed");
  }
  if (ok) {
    const int32_t eof = -1;
    const int32_t n = (int32_t)index.size();
    ok = fwrite(&eof, 4, 1, f) == 1 && fwrite(index.data(), 1, index.size(), f) == index.size() &&
         fwrite(&n, 4, 1, f) == 1 && fwrite("cube", 1, 4, f) == 4;
    if (!ok) sh->fail("write failed");
  }
  *writeSecs = busy;
}

wl_status run(wl_ctx *ctx, const char *inPath, const char *outPath, const wl_params *params,
              size_t batchBytes, bool restoring, wl_container_stats *stats) {
  if (!inPath || !outPath || (!restoring && !params)) return WL_EINVAL;
  if (batchBytes == 0) batchBytes = (size_t)256 << 20;
  const Clock::time_point t0 = Clock::now();
  FILE *fi = fopen(inPath, "rb");
  if (!fi) return WL_EIO;
  char header[64];
  if (fread(header, 1, 64, fi) != 64 || memcmp(header, kCubeHeader, strlen(kCubeHeader)) != 0) {
    fclose(fi);
    return WL_EFORMAT;
  }
  FILE *fo = fopen(outPath, "wb");
  if (!fo) {
    fclose(fi);
    return WL_EIO;
  }
  // the writer appends many small pieces (lengths, messages, words); one
  // writing thread with a large buffer measured faster than positioned
  // writes from several threads
  std::vector<char> obuf((size_t)16 << 20);
  setvbuf(fo, obuf.data(), _IOFBF, obuf.size());

  Staging st;
  if (!restoring && !st.init(ctx, batchBytes)) {
    fclose(fi);
    fclose(fo);
    return WL_ENOMEM;
  }
  Queue<Batch> work;
  Queue<Done> done;
  Shared sh;
  double readSecs = 0, writeSecs = 0, computeSecs = 0;
  unsigned long long bytesIn = 0, bytesOut = 0;
  int written = 0, through = 0;
  std::thread rt(reader, fi, restoring, &st, batchBytes, &work, &sh, &readSecs);
  std::thread wt(writer, fo, restoring, &done, &sh, &bytesOut, &written, &through, &writeSecs);
  wl_status status = WL_OK;
  Batch b;
  while (work.pop(b)) {
    const Clock::time_point c0 = Clock::now();
    Done d;
    d.res.resize(b.items.size());
    if (status == WL_OK && !sh.failed()) {
      if (!restoring) {
        std::vector<wl_cubelet> cs;
        std::vector<size_t> idx;
        for (size_t i = 0; i < b.items.size(); i++) {
          const Item &it = b.items[i];
          bytesIn += it.bytes;
          if (it.through) continue;
          wl_cubelet c;
          memset(&c, 0, sizeof c);
          c.data = it.data();
          c.dtype = wl_type(it.meta.data_type);
          c.size[0] = it.meta.width; c.size[1] = it.meta.height; c.size[2] = it.meta.depth;
          c.params = *params;
          cs.push_back(c);
          idx.push_back(i);
        }
        if (!cs.empty()) {
          std::vector<wl_result> rs(cs.size());
          status = wl_compress_batch(ctx, cs.data(), (int)cs.size(), 0, rs.data());
          if (status == WL_OK)
            for (size_t k = 0; k < idx.size(); k++) d.res[idx[k]] = rs[k];
        }
      } else {
        // every compressed cubelet of the batch restored by one batched call
        d.restored.resize(b.items.size());
        std::vector<wl_result> rs;
        std::vector<void *> outs;
        for (size_t i = 0; i < b.items.size(); i++) {
          Item &it = b.items[i];
          bytesIn += it.bytes;
          if (it.through) continue;
          wl_result r;
          meta_to_result(it.meta, it.own, r);
          if (r.original_size[0] <= 0 || r.original_size[1] <= 0 || r.original_size[2] <= 0) {
            status = WL_EFORMAT;
            break;
          }
          const size_t n = (size_t)r.original_size[0] * r.original_size[1] * r.original_size[2];
          d.restored[i].assign(n * (r.original_dtype == WL_U8 ? 1 : 4), '\0');
          rs.push_back(r);
          outs.push_back(&d.restored[i][0]);
        }
        if (status == WL_OK && !rs.empty())
          status = wl_decompress_batch(ctx, rs.data(), (int)rs.size(), nullptr, outs.data(), 0);
      }
    }
    if (b.buf >= 0) st.release(b.buf);  // the inputs were read before the call returned
    computeSecs += secs(c0, Clock::now());
    d.items = std::move(b.items);
    if (status != WL_OK) {
      sh.fail("compression failed");
      for (wl_result &r : d.res)
        if (r.owner || r.words) wl_result_free(&r);
      d.res.clear();
      continue;  // drain the reader
    }
    done.push(std::move(d));
  }
  done.close();
  rt.join();
  wt.join();
  fclose(fi);
  const bool closed = fclose(fo) == 0;
  if (status == WL_OK && sh.failed()) status = sh.err == "write failed" ? WL_EIO : WL_EFORMAT;
  if (status == WL_OK && !closed) status = WL_EIO;
  if (stats) {
    stats->cubelets = written;
    stats->copied = through;
    stats->bytes_in = bytesIn;
    stats->bytes_out = bytesOut;
    stats->seconds = secs(t0, Clock::now());
    stats->read_seconds = readSecs;
    stats->compute_seconds = computeSecs;
    stats->write_seconds = writeSecs;
  }
  return status;
}

}  // namespace

extern "C" {

wl_status wl_compress_container(wl_ctx *ctx, const char *in_path, const char *out_path,
                                const wl_params *params, size_t batch_bytes,
                                wl_container_stats *stats) {
  if (!ctx) return WL_EINVAL;
  return run(ctx, in_path, out_path, params, batch_bytes, false, stats);
}

wl_status wl_decompress_container(wl_ctx *ctx, const char *in_path, const char *out_path,
                                  size_t batch_bytes, wl_container_stats *stats) {
  if (!ctx) return WL_EINVAL;
  return run(ctx, in_path, out_path, nullptr, batch_bytes, true, stats);
}

}  // extern "C"
