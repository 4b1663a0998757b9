// Launch counters and optional per-launch CUDA-event timing (adfwi_profile_* in the C ABI).
#include <atomic>
#include <mutex>
#include <string.h>
#include <vector>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"
#include "profile.cuh"

namespace adfwi {
namespace {

const char* kNames[kNumKernelClasses] = {"acoustic_fwd_step", "acoustic_adj_step", "elastic_fwd_step",
                                         "elastic_adj_step", "auxiliary"};

std::atomic<long long> g_launches[kNumKernelClasses];

struct Pending {
  int cls;
  cudaEvent_t a, b;
};

std::mutex g_mu;
bool g_timed = false;
std::vector<cudaEvent_t> g_pool;  // events reused across sessions
size_t g_used = 0;
std::vector<Pending> g_pending;
long long g_sess_launches[kNumKernelClasses];

cudaEvent_t take_event() {
  if (g_used == g_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    g_pool.push_back(e);
  }
  return g_pool[g_used++];
}

}  // namespace

int prof_before(int cls, cudaStream_t st) {
  g_launches[cls].fetch_add(1, std::memory_order_relaxed);
  std::lock_guard<std::mutex> lk(g_mu);
  g_sess_launches[cls]++;
  if (!g_timed) return -1;
  cudaEvent_t a = take_event(), b = take_event();
  if (!a || !b) return -1;
  cudaEventRecord(a, st);
  g_pending.push_back({cls, a, b});
  return (int)g_pending.size() - 1;
}

void prof_after(int cls, cudaStream_t st, int token) {
  (void)cls;
  if (token < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if ((size_t)token < g_pending.size()) cudaEventRecord(g_pending[token].b, st);
}

}  // namespace adfwi

using namespace adfwi;

extern "C" {

int adfwi_profile_start(int32_t timed) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_timed = timed != 0;
  g_used = 0;
  g_pending.clear();
  memset(g_sess_launches, 0, sizeof(g_sess_launches));
  return 0;
}

int adfwi_profile_stop(adfwi_kernel_stat* out, int32_t max_out, int32_t* n_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  double ms[kNumKernelClasses] = {0};
  long long timed_launches[kNumKernelClasses] = {0};
  for (const Pending& p : g_pending) {
    if (cudaEventSynchronize(p.b) != cudaSuccess) {
      set_error("profile: event synchronize failed");
      return kCudaError;
    }
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
      ms[p.cls] += t;
      timed_launches[p.cls]++;
    }
  }
  int n = 0;
  for (int c = 0; c < kNumKernelClasses && n < max_out; ++c) {
    if (g_sess_launches[c] == 0) continue;
    if (out) {
      strncpy(out[n].name, kNames[c], sizeof(out[n].name) - 1);
      out[n].name[sizeof(out[n].name) - 1] = '\0';
      out[n].launches = g_sess_launches[c];
      out[n].timed_launches = timed_launches[c];
      out[n].total_ms = ms[c];
    }
    ++n;
  }
  if (n_out) *n_out = n;
  g_timed = false;
  g_pending.clear();
  g_used = 0;
  return 0;
}

int64_t adfwi_launch_count(void) {
  long long s = 0;
  for (int c = 0; c < kNumKernelClasses; ++c) s += g_launches[c].load(std::memory_order_relaxed);
  return s;
}

}  // extern "C"
