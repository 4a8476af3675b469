// Host-side fault injection for the failure-path tests (elp_fault_inject).
//
// Every fault is made on the host: a device allocation that reports
// cudaErrorMemoryAllocation without calling the allocator, a host allocation
// that throws std::bad_alloc, and a tensor-core launch whose producer is told
// to issue no copy, so that the MMA and epilogue waits of that one launch run
// out after a short bound with nothing in flight. No fault touches device
// memory or the GPU's state.
#include <atomic>
#include <new>

#include "device.cuh"

namespace elp {
namespace {
std::atomic<int> g_dev_alloc{0}, g_host_alloc{0}, g_tc_wait{0};

// counts down to the armed event: true exactly once, on the countdown-th call
bool take(std::atomic<int>& c) {
  int v = c.load(std::memory_order_relaxed);
  while (v > 0)
    if (c.compare_exchange_weak(v, v - 1)) return v == 1;
  return false;
}
}  // namespace

bool fault_device_alloc() { return take(g_dev_alloc); }
void fault_host_alloc_point() {
  if (take(g_host_alloc)) throw std::bad_alloc();
}
bool fault_tc_wait() { return take(g_tc_wait); }

}  // namespace elp

extern "C" int elp_fault_inject(int kind, int countdown) {
  using namespace elp;
  if (countdown < 0) { set_error("countdown must be >= 0"); return ELP_ERR_ARG; }
  switch (kind) {
    case ELP_FAULT_NONE: g_dev_alloc = 0; g_host_alloc = 0; g_tc_wait = 0; return ELP_OK;
    case ELP_FAULT_DEVICE_ALLOC: g_dev_alloc = countdown; return ELP_OK;
    case ELP_FAULT_HOST_ALLOC: g_host_alloc = countdown; return ELP_OK;
    case ELP_FAULT_TC_WAIT: g_tc_wait = countdown; return ELP_OK;
    default: set_error("unknown fault kind"); return ELP_ERR_ARG;
  }
}
