// Tuning parameters of the drivers: the thresholds and counts that choose
// between code paths and launch shapes (split tensor-core products or the
// native ones, the batched calls' streams and per-product CTA caps, the
// Newton-Schulz finish, the sign iteration's fixed step count, ...).
//
// Each parameter's value is, in order: the one set through
// mak_tuning_set (an autotuner's table, loaded by the caller), else the
// environment variable of the same name, else the built-in default (the
// values measured best on a GB300).  The kernels' tiles themselves are
// fixed at build time; these parameters decide which kernels run and how
// many run side by side.
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "internal.h"

namespace mak {

namespace {
struct Param {
  const char* name;
  double dflt;  // NAN: computed (per device) by tuning_default
  double lo, hi;
};
const Param kParams[TUNE_COUNT] = {
    {"MAK_BATCH_STREAMS", 32, 1, 32},
    {"MAK_BATCH_GEMM_CTAS", NAN, 8, 1024},  // default: a quarter of the SMs
    {"MAK_SIGN_FIXED_ITERS", 30, 4, 200},
    {"MAK_SPLIT_MIN_MNK", 4194304.0, 1, 1e15},  // 2^22
    {"MAK_GJ_SPLIT_MIN", 33554432.0, 1, 1e18},  // 2^25
    {"MAK_NS_FIXED_MIN_N", 256, 0, 1073741824.0},
    {"MAK_NS_FIXED_MAX_N", 1073741824.0, 0, 1073741824.0},
    {"MAK_QR_OUTER64_MAX_N", 0, 0, 1073741824.0},
    {"MAK_LOOKAHEAD_CTAS", 48, 8, 120},
    {"MAK_PANEL_HIER_C", 0, 0, 8},
    {"MAK_PANEL_PAIR", 1, 0, 1},
    {"MAK_OZ_MERGED", 1, 0, 1},
    {"MAK_OZ_NARROW", 1, 0, 1},
    {"MAK_LOOKAHEAD_TAIL_COLS", 4096, 0, 1073741824.0},
    {"MAK_LOOKAHEAD_TAIL_CTAS", 96, 8, 144},
    {"MAK_SMALL_QR_BYTES", 200704, 0, 229376},
    {"MAK_SMALL_POLAR_BYTES", 200704, 0, 229376},
    {"MAK_QR_PANEL_SPLIT", 1, 0, 1},
};

std::atomic<double> g_set[TUNE_COUNT];
double g_env[TUNE_COUNT];
std::once_flag g_init;

void init_tables() {
  for (int i = 0; i < TUNE_COUNT; i++) {
    g_set[i].store(NAN, std::memory_order_relaxed);
    g_env[i] = NAN;
    const char* e = getenv(kParams[i].name);
    if (e && *e) {
      const double x = atof(e);
      if (x >= kParams[i].lo && x <= kParams[i].hi) g_env[i] = x;
    }
  }
}

int find(const char* name) {
  if (name == nullptr) return -1;
  for (int i = 0; i < TUNE_COUNT; i++)
    if (strcmp(name, kParams[i].name) == 0) return i;
  return -1;
}
}  // namespace

double tuning(int id) {
  std::call_once(g_init, init_tables);
  const double s = g_set[id].load(std::memory_order_relaxed);
  if (!std::isnan(s)) return s;
  if (!std::isnan(g_env[id])) return g_env[id];
  if (!std::isnan(kParams[id].dflt)) return kParams[id].dflt;
  switch (id) {
    case TUNE_BATCH_GEMM_CTAS: return num_sms() / 4;
    default: return 0;
  }
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_tuning_set(const char* name, double value) {
  std::call_once(g_init, init_tables);
  const int i = find(name);
  if (i < 0) return -1;
  if (!std::isnan(value) && !(value >= kParams[i].lo && value <= kParams[i].hi)) return -2;
  g_set[i].store(value, std::memory_order_relaxed);  // NaN: back to env / default
  return 0;
}

int mak_tuning_get(const char* name, double* value) {
  const int i = find(name);
  if (i < 0) return -1;
  if (value == nullptr) return -2;
  *value = tuning(i);
  return 0;
}

const char* mak_tuning_name(int index) {
  return (index >= 0 && index < TUNE_COUNT) ? kParams[index].name : nullptr;
}

}  // extern "C"
