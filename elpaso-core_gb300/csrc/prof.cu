// Launch counting and per-kernel-class device timing (see prof.cuh).
#include <mutex>
#include <vector>

#include "device.cuh"
#include "prof.cuh"

namespace elp {

namespace {
struct Pending {
  cudaEvent_t a, b;
  int cls;
};
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
bool prof_on() { return g_on.load(std::memory_order_relaxed); }

void prof_begin(cudaStream_t s, int cls, void** token) {
  std::lock_guard<std::mutex> lk(g_mu);
  Pending* p = new Pending{take_event(), take_event(), cls};
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
  return ELP_OK;
}

}  // extern "C"
