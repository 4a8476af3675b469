// Serving loop: frequency-sweep requests on resident models, continuous
// batching, admission by HBM budget.
//
// The reference runs one model per process and one frequency at a time
// (analysisfrequencybasic.cpp:101-242). Here a server keeps models resident
// (assembled value arrays + symbolic factorisation + per-model front
// workspace) and runs frequency work items:
//  - requests are split into frequencies; the frequencies waiting on one
//    model are packed into batches of up to `omega_batch` slots in arrival
//    order, so a request that arrives while another runs on the same model
//    joins the next batch (continuous batching, not a request queue);
//  - `max_inflight` worker threads, each with its own CUDA stream, run
//    batches of DIFFERENT models at the same time, so their work overlaps
//    on the device; a model is held by at most one worker at a time;
//  - a model's device memory (arrays + front workspace) is admitted against
//    `hbm_budget_bytes`; idle models' workspaces are released to admit
//    others, and a model that cannot fit alone fails its requests with
//    ELP_ERR_NOMEM;
//  - every slot of a batch is computed by the same kernels independently of
//    its neighbours (fixed summation orders, no atomics on values), so a
//    result does not depend on the batch it landed in.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device.cuh"
#include "numeric.cuh"

using namespace elp;


namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int model = 0;
  std::vector<double> omegas;
  double* x_out = nullptr;
  int next = 0;          // next frequency to schedule
  int done = 0;          // frequencies finished
  int status = ELP_OK;
  double max_res = 0.0;
  Clock::time_point arrival;
};

struct ModelSlot {
  elp_model* h = nullptr;
  bool busy = false;
  bool ready = false;            // assembled + analysed
  int64_t resident = 0;          // bytes charged against the budget
  std::deque<int64_t> queue;     // requests with unscheduled frequencies
};

// device bytes of a resident model: value arrays (VK, VM, per-group VK,
// col_idx, class, arena offsets) + per-row data + its solve workspace
int64_t model_bytes(const Model& m, int precision, int slots) {
  const int64_t groups = std::max<int64_t>(1, (int64_t)m.groups.size());
  int64_t b = m.nnz * (8 + 8 + 8 * (groups - 1) + 4 + 1 + 8) + m.n * 64;
  return b + workspace_bytes(m, precision, slots);
}

}  // namespace

struct elp_server {
  elp_server_config cfg;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<ModelSlot> models;
  std::unordered_map<int64_t, Request> reqs;
  std::deque<elp_request_result> done;
  std::vector<std::thread> workers;
  int64_t next_id = 1;
  int64_t resident = 0;
  bool stop = false;
  int device = 0;

  void finish_request(Request& r) {
    elp_request_result res;
    res.request_id = r.id;
    res.status = r.status;
    res.n_omega = (int)r.omegas.size();
    res.latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r.arrival).count();
    res.max_rel_residual = r.max_res;
    done.push_back(res);
    reqs.erase(r.id);
    cv_done.notify_all();
  }

  // picks the idle model whose oldest waiting request arrived first
  int pick_model() {
    int best = -1;
    Clock::time_point t0 = Clock::time_point::max();
    for (int i = 0; i < (int)models.size(); ++i) {
      ModelSlot& s = models[i];
      if (s.busy || s.queue.empty()) continue;
      const Request& r = reqs.at(s.queue.front());
      if (r.arrival < t0) { t0 = r.arrival; best = i; }
    }
    return best;
  }

  // makes room for `need` bytes by releasing idle models' workspaces
  bool admit(int mi, int64_t need) {
    ModelSlot& s = models[mi];
    if (s.resident >= need) return true;
    int64_t extra = need - s.resident;
    if (extra > cfg.hbm_budget_bytes) return false;
    for (int i = 0; i < (int)models.size() && resident + extra > cfg.hbm_budget_bytes; ++i) {
      ModelSlot& o = models[i];
      if (i == mi || o.busy || o.resident == 0 || !o.queue.empty()) continue;
      for (auto& w : o.h->m.ws) w.reset();
      for (auto& lw : o.h->m.ws_b)
        for (auto& w : lw) w.reset();
      resident -= o.resident;
      o.resident = 0;
    }
    if (resident + extra > cfg.hbm_budget_bytes) return false;
    resident += extra;
    s.resident = need;
    return true;
  }

  void worker() {
    cudaSetDevice(device);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    DevBuf<double2> xdev;
    std::vector<double2> xh;
    for (;;) {
      std::unique_lock<std::mutex> lk(mu);
      int mi = -1;
      cv_work.wait(lk, [&] { return stop || (mi = pick_model()) >= 0; });
      if (stop) break;
      ModelSlot& s = models[mi];
      s.busy = true;
      // build the batch: frequencies of waiting requests in arrival order
      struct Item { int64_t rid; int k; double w; };
      std::vector<Item> items;
      while (!s.queue.empty() && (int)items.size() < cfg.omega_batch) {
        Request& r = reqs.at(s.queue.front());
        while (r.next < (int)r.omegas.size() && (int)items.size() < cfg.omega_batch) {
          items.push_back({r.id, r.next, r.omegas[r.next]});
          r.next++;
        }
        if (r.next >= (int)r.omegas.size()) s.queue.pop_front();
      }
      Model& m = s.h->m;
      bool ready = s.ready;
      lk.unlock();

      int rc = ELP_OK;
      if (!ready) {
        rc = elp_model_assemble(s.h);
        if (!rc) rc = elp_model_analyse(s.h);
      }
      if (!rc) {
        lk.lock();
        s.ready = true;
        bool ok = admit(mi, model_bytes(m, cfg.precision, cfg.omega_batch));
        lk.unlock();
        if (!ok) { rc = ELP_ERR_NOMEM; set_error("model does not fit the HBM budget"); }
      }
      std::vector<elp_solve_info> info(items.size());
      const int64_t n = m.n;
      if (!rc) {
        std::vector<double> oms(items.size());
        for (size_t i = 0; i < items.size(); ++i) oms[i] = items[i].w;
        if (xdev.n < (size_t)n * items.size()) {
          if (xdev.alloc((size_t)n * cfg.omega_batch) != cudaSuccess) rc = ELP_ERR_NOMEM;
        }
        if (!rc) {
          // every batch uses the full slot count so the workspace is shaped once;
          // one lane: the loop already overlaps up to max_inflight batches, and
          // lane workspaces per model would double the allocations it admits
          rc = numeric_solve_batch(m, cfg.precision, oms.data(), (int)oms.size(), nullptr, xdev.p, info.data(),
                                   cfg.tol, st, 1);
          if (rc == ELP_ERR_NOCONV) rc = ELP_OK;  // reported per request through its residual
        }
        if (!rc || rc == ELP_ERR_NOCONV) {
          xh.resize((size_t)n * items.size());
          if (cudaMemcpyAsync(xh.data(), xdev.p, sizeof(double2) * xh.size(), cudaMemcpyDeviceToHost, st) !=
                  cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)
            rc = ELP_ERR_CUDA;
        }
      }
      if (rc && rc != ELP_ERR_NOMEM)  // the per-thread error text does not reach the caller's thread
        fprintf(stderr, "[elp server] batch of %zu frequencies on model %d failed (%d): %s\n", items.size(), mi, rc,
                get_error().c_str());
      lk.lock();
      for (size_t i = 0; i < items.size(); ++i) {
        auto it = reqs.find(items[i].rid);
        if (it == reqs.end()) continue;
        Request& r = it->second;
        if (rc) r.status = rc;
        else {
          memcpy(r.x_out + (size_t)items[i].k * 2 * n, xh.data() + i * n, sizeof(double2) * n);
          r.max_res = std::max(r.max_res, info[i].rel_residual);
          if (!(info[i].rel_residual <= cfg.tol)) r.status = ELP_ERR_NOCONV;
        }
        r.done++;
        if (r.done == (int)r.omegas.size()) finish_request(r);
      }
      s.busy = false;
      lk.unlock();
      cv_work.notify_all();
    }
    cudaStreamDestroy(st);
  }
};

extern "C" {

int elp_server_create(const elp_server_config* cfg, elp_server** out) {
  if (!cfg || !out) { set_error("null argument"); return ELP_ERR_ARG; }
  *out = nullptr;
  if (cfg->max_inflight < 1 || cfg->omega_batch < 1 || cfg->omega_batch > kMaxSlots || cfg->hbm_budget_bytes <= 0 ||
      (cfg->precision != ELP_FP64_PLAIN && cfg->precision != ELP_MIXED)) {
    set_error("invalid server configuration");
    return ELP_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device: this library has no CPU path");
    return ELP_ERR_CUDA;
  }
  elp_server* s = new elp_server();
  s->cfg = *cfg;
  if (!(s->cfg.tol > 0)) s->cfg.tol = 1e-10;
  cudaGetDevice(&s->device);
  for (int i = 0; i < cfg->max_inflight; ++i) s->workers.emplace_back([s] { s->worker(); });
  *out = s;
  return ELP_OK;
}

int elp_server_add_model(elp_server* s, elp_model* m, int* model_id) {
  if (!s || !m || !model_id) { set_error("null argument"); return ELP_ERR_ARG; }
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto& ms : s->models)
    if (ms.h == m) { set_error("model already registered"); return ELP_ERR_ARG; }
  ModelSlot ms;
  ms.h = m;
  ms.ready = m->m.assembled && m->m.analysed;
  s->models.push_back(ms);
  *model_id = (int)s->models.size() - 1;
  return ELP_OK;
}

int elp_server_submit(elp_server* s, int model_id, const double* omegas, int n_omega, double* x_out,
                      int64_t* request_id) {
  if (!s || !omegas || !x_out || n_omega <= 0) { set_error("bad request"); return ELP_ERR_ARG; }
  for (int i = 0; i < n_omega; ++i)
    if (!(omegas[i] > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  std::lock_guard<std::mutex> lk(s->mu);
  if (model_id < 0 || model_id >= (int)s->models.size()) { set_error("unknown model id"); return ELP_ERR_ARG; }
  Request r;
  r.id = s->next_id++;
  r.model = model_id;
  r.omegas.assign(omegas, omegas + n_omega);
  r.x_out = x_out;
  r.arrival = Clock::now();
  s->reqs[r.id] = r;
  s->models[model_id].queue.push_back(r.id);
  if (request_id) *request_id = r.id;
  s->cv_work.notify_one();
  return ELP_OK;
}

int elp_server_wait(elp_server* s, elp_request_result* result, double timeout_ms) {
  if (!s || !result) { set_error("null argument"); return ELP_ERR_ARG; }
  std::unique_lock<std::mutex> lk(s->mu);
  auto ready = [&] { return !s->done.empty(); };
  if (timeout_ms < 0) s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
    set_error("no request finished within the timeout");
    return ELP_ERR_TIMEOUT;
  }
  *result = s->done.front();
  s->done.pop_front();
  return ELP_OK;
}

int elp_server_destroy(elp_server* s) {
  if (!s) return ELP_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  return ELP_OK;
}

}  // extern "C"
