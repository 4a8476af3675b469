// Launch counting and per-kernel-class device timing.
//
// Every kernel launch of the library goes through PROF_LAUNCH, which counts
// it; when profiling is enabled (elp_profile), a CUDA event pair is recorded
// on the launching stream around it and the elapsed time is added to the
// kernel's class when the pair is resolved (at the next host sync point of
// the calling routine, prof_resolve).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

namespace elp {

enum KernelClass {
  KC_ASSEMBLE = 0, KC_DSCALE, KC_SCATTER, KC_PANEL, KC_BORDER, KC_UROW, KC_GEMM, KC_EXTEND_ADD,
  KC_FORWARD, KC_BACKWARD, KC_RESIDUAL, KC_NORMS, KC_RHS, KC_UPDATE, KC_VALUES, KC_GEMM_TC,
  KC_SPMV, KC_FWD_BORDER, KC_BWD_U12, KC_KRYLOV, KC_SCHUR_TC, KC_PACK,
  KC_COUNT
};

void prof_count(int cls);
bool prof_on();
void prof_begin(cudaStream_t s, int cls, void** token);
void prof_end(cudaStream_t s, void* token);
void prof_resolve();
// Tree level the calling thread's next launches belong to (-1: none). With
// ELP_PROF_LEVELS set and profiling on, prof_resolve also sums the device
// time per (level, class) and elp_profile_read prints that table to stderr.
void prof_set_level(int level);

struct ProfScope {
  void* tok = nullptr;
  cudaStream_t s;
  ProfScope(cudaStream_t st, int cls) : s(st) {
    prof_count(cls);
    if (prof_on()) prof_begin(st, cls, &tok);
  }
  ~ProfScope() {
    if (tok) prof_end(s, tok);
  }
};

#define PROF_LAUNCH(cls, stream, ...)         \
  do {                                        \
    ::elp::ProfScope ps_((stream), (cls));    \
    __VA_ARGS__;                              \
  } while (0)

}  // namespace elp
