// Optional device-time accounting per kernel class (mak_profile_*).
//
// While enabled, every launch of an instrumented kernel class is bracketed
// by a pair of CUDA events recorded on the launching stream (no host
// synchronization); mak_profile_read() waits for the recorded events and
// sums their elapsed times.  This is how a benchmark measures the average
// duration of the dominant kernel live, inside its own timed region.
#include "mak_common.cuh"

#include <mutex>
#include <vector>

namespace mak {

namespace {
struct Rec {
  cudaEvent_t e0, e1;
  int kind;
  double work;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

ProfScope::ProfScope(cudaStream_t s, int k, double w) : st(s), kind(k), work(w) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_on) return;
  e0 = take_event();
  if (e0) cudaEventRecord(e0, st);
}

ProfScope::~ProfScope() {
  if (!e0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e1 = take_event();
  if (!e1) return;
  cudaEventRecord(e1, st);
  g_recs.push_back({e0, e1, kind, work});
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_profile_start(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_recs) {
    g_pool.push_back(r.e0);
    g_pool.push_back(r.e1);
  }
  g_recs.clear();
  g_on = true;
  return 0;
}

int mak_profile_stop(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_on = false;
  return 0;
}

int mak_profile_read(int kind, double* total_ms, double* total_work, uint64_t* launches) {
  std::lock_guard<std::mutex> lk(g_mu);
  double ms = 0.0, work = 0.0;
  uint64_t cnt = 0;
  for (auto& r : g_recs) {
    if (kind >= 0 && r.kind != kind) continue;
    if (cudaEventSynchronize(r.e1) != cudaSuccess) return MAK_ERR_CUDA;
    float t = 0.f;
    if (cudaEventElapsedTime(&t, r.e0, r.e1) != cudaSuccess) return MAK_ERR_CUDA;
    ms += t;
    work += r.work;
    cnt++;
  }
  if (total_ms) *total_ms = ms;
  if (total_work) *total_work = work;
  if (launches) *launches = cnt;
  return 0;
}

}  // extern "C"
