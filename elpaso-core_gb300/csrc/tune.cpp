// Per-model tuning and the autotuner (elp_model_set_tuning / _get_tuning /
// _autotune, elp_group_autotune).
//
// The knobs change how a model is factorised, never what is computed:
//  - leaf: the nested-dissection leaf size (front count and sizes of the
//    lowest tree levels);
//  - schur_tile: 128 x 64 or 128 x 32 complex tiles of the converter kernel's
//    Schur update (levels not run by the packed kernel); narrow tiles give
//    more CTAs on short borders;
//  - pack_count / pack_minb: which levels run the packed-operand Schur kernel;
//  - lanes: how many workspace lanes a batch of 16+ frequencies is split over.
// The built-in defaults were measured on the coupled plate-cavity sweep; the
// autotuner measures instead: starting from the model's current tuning it
// tries each knob's values in turn (coordinate descent: leaf, tile, packed
// levels, lanes), keeping a value when the solve of the caller's frequencies
// gets faster. Every trial times real solves (the faster of two, after a
// warm-up call, since a changed tuning rebuilds workspaces or the symbolic
// phase).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <functional>
#include <limits>
#include <new>
#include <vector>

#include "device.cuh"
#include "numeric.cuh"
#include "symbolic.hpp"

using namespace elp;

namespace elp {

// A changed tuning invalidates the symbolic phase (leaf) or the workspaces.
void apply_tuning(Model& m, const Tuning& t) {
  const Tuning before = resolved_tuning(m);
  m.tune = t;
  const Tuning after = resolved_tuning(m);
  for (auto& w : m.ws) w.reset();
  for (auto& lane : m.ws_b)
    for (auto& w : lane) w.reset();
  if (after.leaf != before.leaf) {
    m.sym.reset();
    m.dsym.reset();
    m.analysed = false;
  } else if (m.sym && m.dsym) {
    m.dsym->pack_max = workspace_plan(m).pack_max;
  }
}

}  // namespace elp

namespace {

elp_tuning to_c(const Tuning& t) {
  elp_tuning c;
  c.leaf = t.leaf;
  c.schur_tile = t.schur_tile;
  c.pack_count = t.pack_count;
  c.pack_min_border = t.pack_minb;
  c.lanes = t.lanes;
  return c;
}

Tuning from_c(const elp_tuning& c) {
  Tuning t;
  t.leaf = c.leaf;
  t.schur_tile = c.schur_tile;
  t.pack_count = c.pack_count;
  t.pack_minb = c.pack_min_border;
  t.lanes = c.lanes;
  return t;
}

// seconds of a solve with tuning t: the faster of two timed solves after a
// warm-up solve (one timing alone let run-to-run noise pick between knobs a
// few percent apart), or infinity when a solve failed
double trial(Model& m, const Tuning& t, const std::function<int()>& run) {
  apply_tuning(m, t);
  int rc = run();
  if (rc && rc != ELP_ERR_NOCONV && rc != ELP_ERR_SINGULAR) return std::numeric_limits<double>::infinity();
  double best = std::numeric_limits<double>::infinity();
  for (int rep = 0; rep < 2; ++rep) {
    const auto t0 = std::chrono::steady_clock::now();
    rc = run();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc && rc != ELP_ERR_NOCONV && rc != ELP_ERR_SINGULAR) return std::numeric_limits<double>::infinity();
    best = std::min(best, s);
  }
  return best;
}

int autotune(Model& m, int n_omega, const std::function<int()>& run, elp_tuning* chosen, double* seconds,
             int* trials) {
  Tuning best = resolved_tuning(m);
  double best_s = trial(m, best, run);
  int n = 1;
  if (!(best_s < std::numeric_limits<double>::infinity())) {
    set_error("the solve with the current tuning failed");
    return ELP_ERR_ARG;
  }
  auto consider = [&](Tuning t) {
    const double s = trial(m, t, run);
    ++n;
    if (s < best_s) { best_s = s; best = t; }
  };
  const Tuning base = best;
  for (int leaf : {64, 128, 256})
    if (leaf != base.leaf) { Tuning t = best; t.leaf = leaf; consider(t); }
  { Tuning t = best; t.schur_tile = best.schur_tile == 64 ? 32 : 64; consider(t); }
  {  // packed-operand Schur levels off, or on every level that reaches 300 border rows
    Tuning t = best;
    if (best.pack_count > 0) { t.pack_count = 0; } else { t.pack_count = 300; t.pack_minb = 300; }
    consider(t);
  }
  if (n_omega >= 16)
    for (int lanes : {1, 2, 4})
      if (lanes != best.lanes) { Tuning t = best; t.lanes = lanes; consider(t); }
  apply_tuning(m, best);
  if (chosen) *chosen = to_c(best);
  if (seconds) *seconds = best_s;
  if (trials) *trials = n;
  return ELP_OK;
}

}  // namespace

#define GUARD_BEGIN try {
#define GUARD_END                                      \
  }                                                    \
  catch (const std::bad_alloc&) {                      \
    set_error("host allocation failed");               \
    return ELP_ERR_NOMEM;                              \
  }                                                    \
  catch (const std::exception& ex) {                   \
    set_error(std::string("exception: ") + ex.what()); \
    return ELP_ERR_ARG;                                \
  }

extern "C" {

int elp_model_set_tuning(elp_model* h, const elp_tuning* t) {
  GUARD_BEGIN
  if (!h || !t) { set_error("null argument"); return ELP_ERR_ARG; }
  if (t->schur_tile > 0 && t->schur_tile != 32 && t->schur_tile != 64) {
    set_error("schur_tile must be 32 or 64 (0 or negative: default)");
    return ELP_ERR_ARG;
  }
  if (t->lanes > 4) { set_error("at most 4 lanes"); return ELP_ERR_ARG; }
  apply_tuning(h->m, from_c(*t));
  return ELP_OK;
  GUARD_END
}

int elp_model_get_tuning(const elp_model* h, elp_tuning* t) {
  if (!h || !t) { set_error("null argument"); return ELP_ERR_ARG; }
  *t = to_c(resolved_tuning(h->m));
  return ELP_OK;
}

int elp_model_autotune(elp_model* h, const double* omegas, int n_omega, int precision, elp_tuning* chosen,
                       double* seconds, int* trials) {
  GUARD_BEGIN
  if (!h || !omegas || n_omega < 1 || n_omega > 64) { set_error("bad autotune arguments"); return ELP_ERR_ARG; }
  int rc = h->m.assembled ? ELP_OK : elp_model_assemble(h);
  if (rc) return rc;
  const int64_t n = h->m.n;
  DevBuf<double2> xd;
  ELP_CUDA(xd.alloc((size_t)n * n_omega));
  auto run = [&]() -> int {
    return elp_solve_device(h, omegas, n_omega, precision, nullptr, reinterpret_cast<double*>(xd.p), nullptr,
                            1e-10, nullptr);
  };
  return autotune(h->m, n_omega, run, chosen, seconds, trials);
  GUARD_END
}

int elp_group_autotune(elp_group* g, const double* omegas, int n_omega, int precision, elp_tuning* chosen,
                       double* seconds, int* trials) {
  GUARD_BEGIN
  if (!g || !omegas || n_omega < 1) { set_error("bad autotune arguments"); return ELP_ERR_ARG; }
  Model& m = group_model(g);
  int64_t total = 0;
  for (int k = 0; k < m.n_members; ++k) total += m.member_row_off[k + 1] - m.member_row_off[k];
  std::vector<double> x((size_t)2 * total * n_omega);
  auto run = [&]() -> int { return elp_group_solve(g, omegas, n_omega, precision, x.data(), nullptr, 1e-10); };
  return autotune(m, n_omega, run, chosen, seconds, trials);
  GUARD_END
}

int elp_group_set_tuning(elp_group* g, const elp_tuning* t) {
  GUARD_BEGIN
  if (!g || !t) { set_error("null argument"); return ELP_ERR_ARG; }
  apply_tuning(group_model(g), from_c(*t));
  return ELP_OK;
  GUARD_END
}

}  // extern "C"
