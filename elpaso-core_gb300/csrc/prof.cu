// Launch counting and per-kernel-class device timing (see prof.cuh).
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "device.cuh"
#include "prof.cuh"

namespace elp {

namespace {
struct Pending {
  cudaEvent_t a, b;
  int cls;
  int level;
};
constexpr int kMaxLevels = 64;
thread_local int t_level = -1;
double g_level_ms[kMaxLevels][KC_COUNT];
bool levels_on() {
  static const bool v = getenv("ELP_PROF_LEVELS") != nullptr;
  return v;
}
std::atomic<int64_t> g_count[KC_COUNT];
std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
double g_ms[KC_COUNT];
int64_t g_timed[KC_COUNT];

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

void prof_count(int cls) { g_count[cls].fetch_add(1, std::memory_order_relaxed); }
void prof_set_level(int level) { t_level = levels_on() ? level : -1; }
bool prof_on() { return g_on.load(std::memory_order_relaxed); }

void prof_begin(cudaStream_t s, int cls, void** token) {
  std::lock_guard<std::mutex> lk(g_mu);
  Pending* p = new Pending{take_event(), take_event(), cls, t_level};
  cudaEventRecord(p->a, s);
  *token = p;
}

void prof_end(cudaStream_t s, void* token) {
  Pending* p = static_cast<Pending*>(token);
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEventRecord(p->b, s);
  g_pending.push_back(*p);
  delete p;
}

void prof_resolve() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& p : g_pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g_ms[p.cls] += ms;
      g_timed[p.cls] += 1;
      if (p.level >= 0 && p.level < kMaxLevels) g_level_ms[p.level][p.cls] += ms;
    }
    g_pool.push_back(p.a);
    g_pool.push_back(p.b);
  }
  g_pending.clear();
}

}  // namespace elp

using namespace elp;

extern "C" {

int elp_profile(int enable) {
  prof_resolve();
  std::lock_guard<std::mutex> lk(g_mu);
  for (int i = 0; i < KC_COUNT; ++i) {
    g_count[i].store(0);
    g_ms[i] = 0.0;
    g_timed[i] = 0;
  }
  for (int l = 0; l < kMaxLevels; ++l)
    for (int i = 0; i < KC_COUNT; ++i) g_level_ms[l][i] = 0.0;
  g_on.store(enable != 0);
  return ELP_OK;
}

int elp_profile_read(double* ms, int64_t* launches, int64_t* timed, int* n_classes) {
  prof_resolve();
  std::lock_guard<std::mutex> lk(g_mu);
  for (int i = 0; i < KC_COUNT; ++i) {
    if (ms) ms[i] = g_ms[i];
    if (launches) launches[i] = g_count[i].load();
    if (timed) timed[i] = g_timed[i];
  }
  if (n_classes) *n_classes = KC_COUNT;
  if (levels_on()) {
    for (int l = 0; l < kMaxLevels; ++l) {
      double tot = 0.0;
      for (int i = 0; i < KC_COUNT; ++i) tot += g_level_ms[l][i];
      if (tot == 0.0) continue;
      fprintf(stderr, "[elp levels] level %2d total %8.3f ms:", l, tot);
      for (int i = 0; i < KC_COUNT; ++i)
        if (g_level_ms[l][i] > 0.0) fprintf(stderr, " c%d=%.3f", i, g_level_ms[l][i]);
      fprintf(stderr, "\n");
    }
  }
  return ELP_OK;
}

}  // extern "C"
