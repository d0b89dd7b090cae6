// Process-wide table of column-tile shapes, filled by the tile autotuner.
//
// A size class is (pass, element type of the global side, row-length class):
// the pass is one of forward x / y / z and inverse z / y / x, the element type
// is the source type of the forward x pass (with or without 16-byte loads from
// host memory) or the destination type of the inverse x pass and float
// elsewhere, and row-length class k holds rows of 2^(k-1)+1 .. 2^k elements.
// An entry is a tile shape -- 32, 64 or 128 rows, four or eight warps -- or
// empty for the default.  Every shape does the same arithmetic on every
// element, so the table changes speed only, never results.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "wl_internal.h"
#include "wlgpu.h"

namespace wl {
namespace {

constexpr int kTypes = 8;     // 4 element types x (plain, 16-byte host loads)
constexpr int kClasses = 10;  // row-length classes 0..9 (up to 512 elements)

// rows | warps << 16, 0 = default
std::atomic<int> g_shape[kTuneKinds][kTypes][kClasses];
std::atomic<float> g_us[kTuneKinds][kTypes][kClasses][kTileShapes];
std::atomic<unsigned> g_version{1};

int row_class(int L) {
  int k = 0;
  while ((1 << k) < L) k++;
  return k;
}

bool valid_shape(int rows, int warps) {
  return (rows == 32 || rows == 64 || rows == 128) && (warps == 4 || warps == 8);
}

}  // namespace

int tune_type_index(int dtype, bool vec) {
  int t;
  switch (dtype) {
    case WL_U8: t = 0; break;
    case WL_U16: t = 1; break;
    case WL_I32: t = 2; break;
    default: t = 3; break;
  }
  return t + (vec ? 4 : 0);
}

TileShape tuned_cols_shape(int kind, int typeIdx, int L) {
  const int k = row_class(L);
  if (kind >= 0 && kind < kTuneKinds && typeIdx >= 0 && typeIdx < kTypes && k < kClasses) {
    const int v = g_shape[kind][typeIdx][k].load(std::memory_order_relaxed);
    const TileShape t{v & 0xffff, v >> 16};
    if (v && valid_shape(t.rows, t.warps) && dwt_cols_rows_fit(L, t.rows)) return t;
  }
  return TileShape{dwt_cols_tile_rows(L), 4};
}

void set_tuned_cols_shape(int kind, int typeIdx, int cls, TileShape t,
                          const float us[kTileShapes]) {
  if (kind < 0 || kind >= kTuneKinds || typeIdx < 0 || typeIdx >= kTypes || cls < 0 ||
      cls >= kClasses)
    return;
  g_shape[kind][typeIdx][cls].store(valid_shape(t.rows, t.warps) ? (t.rows | (t.warps << 16)) : 0,
                                    std::memory_order_relaxed);
  for (int c = 0; c < kTileShapes; c++) g_us[kind][typeIdx][cls][c].store(us ? us[c] : 0.f);
  g_version.fetch_add(1);
}

unsigned tune_version() { return g_version.load(); }

}  // namespace wl

using namespace wl;

extern "C" {

// One line per tuned class: "kind type class rows warps t0 .. t5" (times in
// microseconds per launch of the tuning batch for the six candidate shapes
// 32x4, 64x4, 128x4, 32x8, 64x8, 128x8; 0 where not measured).
wl_status wl_tune_export(char *buf, size_t cap, size_t *len) {
  std::string out;
  char line[256];
  for (int k = 0; k < kTuneKinds; k++)
    for (int t = 0; t < kTypes; t++)
      for (int c = 0; c < kClasses; c++) {
        const int v = g_shape[k][t][c].load();
        if (!v) continue;
        int n = snprintf(line, sizeof line, "%d %d %d %d %d", k, t, c, v & 0xffff, v >> 16);
        for (int i = 0; i < kTileShapes; i++)
          n += snprintf(line + n, sizeof line - n, " %.2f", g_us[k][t][c][i].load());
        snprintf(line + n, sizeof line - n, "\n");
        out += line;
      }
  if (len) *len = out.size();
  if (!buf) return WL_OK;
  if (cap < out.size() + 1) return WL_EINVAL;
  memcpy(buf, out.c_str(), out.size() + 1);
  return WL_OK;
}

wl_status wl_tune_import(const char *text) {
  if (!text) return WL_EINVAL;
  const char *p = text;
  while (*p) {
    const char *e = strchr(p, '\n');
    const std::string ln(p, e ? (size_t)(e - p) : strlen(p));
    p = e ? e + 1 : p + ln.size();
    int k, t, c, r, w;
    float us[kTileShapes] = {0, 0, 0, 0, 0, 0};
    const int got = sscanf(ln.c_str(), "%d %d %d %d %d %f %f %f %f %f %f", &k, &t, &c, &r, &w,
                           &us[0], &us[1], &us[2], &us[3], &us[4], &us[5]);
    if (got <= 0) continue;  // blank line
    if (got < 5 || k < 0 || k >= kTuneKinds || t < 0 || t >= kTypes || c < 0 || c >= kClasses ||
        !valid_shape(r, w))
      return WL_EFORMAT;
    set_tuned_cols_shape(k, t, c, TileShape{r, w}, us);
  }
  return WL_OK;
}

void wl_tune_reset(void) {
  for (int k = 0; k < kTuneKinds; k++)
    for (int t = 0; t < kTypes; t++)
      for (int c = 0; c < kClasses; c++) {
        g_shape[k][t][c].store(0);
        for (int i = 0; i < kTileShapes; i++) g_us[k][t][c][i].store(0.f);
      }
  g_version.fetch_add(1);
}

}  // extern "C"
