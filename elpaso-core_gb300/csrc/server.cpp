// Serving loop: frequency-sweep requests on resident models, continuous
// batching, admission by HBM budget.
//
// The reference runs one model per process and one frequency at a time
// (analysisfrequencybasic.cpp:101-242). Here a server keeps models resident
// (assembled value arrays + symbolic factorisation + front workspaces) and
// runs frequency work items:
//  - requests are split into frequencies; the frequencies waiting on one
//    model are packed into batches of up to `omega_batch` slots in arrival
//    order, so a request that arrives while another runs on the same model
//    joins the next batch (continuous batching, not a request queue);
//  - `max_inflight` worker threads, each with its own CUDA stream, run
//    batches at the same time, so their work overlaps on the device; a
//    model has up to kLanesPerModel workspace lanes, so while one worker
//    runs a long batch of a model, a second worker can start the model's
//    newer requests on another lane instead of waiting behind it;
//  - device memory is admitted against `hbm_budget_bytes` BEFORE it is
//    allocated: a model's resident arrays once (sized from the host model,
//    before assembly), and each lane's front workspace per batch (sized from
//    the host symbolic phase); a batch takes as many frequencies as the
//    budget leaves room for, idle models' workspaces are released to make
//    room, a batch that finds no room while other batches run waits for
//    them, and a model that cannot fit alone fails its requests with
//    ELP_ERR_NOMEM;
//  - model slots have stable addresses (models may be added while batches
//    run);
//  - every slot of a batch is computed by the same kernels independently of
//    its neighbours (fixed summation orders, no atomics on values), so a
//    result does not depend on the batch or lane it landed in.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device.cuh"
#include "numeric.cuh"

using namespace elp;


namespace {

using Clock = std::chrono::steady_clock;
constexpr int kLanesPerModel = 2;

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
  bool ready = false;            // assembled + analysed
  bool preparing = false;        // a worker is assembling / analysing it
  bool failed = false;           // its arrays do not fit the budget: requests fail with NOMEM
  int lanes_busy = 0;            // bit l: a worker runs a batch on workspace lane l
  int64_t array_bytes = 0;       // charged once, when the model is first prepared
  int64_t ws_bytes[kLanesPerModel] = {0, 0};  // charged per lane workspace
  int ws_slots[kLanesPerModel] = {0, 0};      // frequencies the lane's workspace holds
  int ws_store[kLanesPerModel] = {0, 0};      // its front store (FrontStore)
  std::deque<int64_t> queue;     // requests with unscheduled frequencies
};

}  // namespace

struct elp_server {
  elp_server_config cfg;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::unique_ptr<ModelSlot>> models;
  std::unordered_map<int64_t, Request> reqs;
  std::deque<elp_request_result> done;
  std::vector<std::thread> workers;
  int64_t next_id = 1;
  int64_t resident = 0;          // bytes charged against the budget
  int running = 0;               // batches on the device
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

  // fails every unscheduled frequency of model `mi` with `status`
  void fail_queue(int mi, int status) {
    ModelSlot& s = *models[mi];
    while (!s.queue.empty()) {
      auto it = reqs.find(s.queue.front());
      s.queue.pop_front();
      if (it == reqs.end()) continue;
      Request& r = it->second;
      r.status = status;
      r.done += (int)r.omegas.size() - r.next;
      r.next = (int)r.omegas.size();
      if (r.done == (int)r.omegas.size()) finish_request(r);
    }
  }

  // the model whose oldest waiting request arrived first, with a free lane;
  // a model being prepared is left to the worker preparing it
  int pick_model(int& lane) {
    int best = -1;
    Clock::time_point t0 = Clock::time_point::max();
    for (int i = 0; i < (int)models.size(); ++i) {
      ModelSlot& s = *models[i];
      if (s.queue.empty() || s.preparing) continue;
      if (!s.ready && s.lanes_busy) continue;
      int l = 0;
      while (l < kLanesPerModel && (s.lanes_busy >> l & 1)) ++l;
      if (l == kLanesPerModel) continue;
      const Request& r = reqs.at(s.queue.front());
      if (r.arrival < t0) { t0 = r.arrival; best = i; lane = l; }
    }
    return best;
  }

  // releases idle models' workspaces until `need` more bytes fit; returns
  // whether they do. Idle: no lane busy and nothing queued; with `queued`,
  // also models whose requests wait (their next batch makes its workspace
  // again) -- used when no batch runs, so that nothing else would free memory.
  bool make_room(int64_t need, int keep, bool queued = false) {
    for (int i = 0; i < (int)models.size() && resident + need > cfg.hbm_budget_bytes; ++i) {
      ModelSlot& o = *models[i];
      if (i == keep || o.lanes_busy || (!queued && !o.queue.empty())) continue;
      for (int l = 0; l < kLanesPerModel; ++l) {
        if (!o.ws_bytes[l]) continue;
        std::unique_ptr<Workspace>& W = l ? o.h->m.ws_b[cfg.precision][l - 1] : o.h->m.ws[cfg.precision];
        W.reset();
        resident -= o.ws_bytes[l];
        o.ws_bytes[l] = 0;
        o.ws_slots[l] = 0;
        o.ws_store[l] = STORE_FULL;
      }
    }
    return resident + need <= cfg.hbm_budget_bytes;
  }

  // frequencies a batch of model `mi` on `lane` may take (<= want), with the
  // lane's workspace charged for them (whole fronts where they fit, else the
  // compact factor store); 0 when no room is left now
  int admit_batch(int mi, int lane, int want, int& store, bool queued = false) {
    ModelSlot& s = *models[mi];
    const Model& m = s.h->m;
    store = s.ws_store[lane];
    if (s.ws_slots[lane] >= want) return want;  // the lane's workspace already holds them
    const int forced = forced_store();
    for (int S = want; S >= 1; S = S > 4 ? S / 2 : S - 1) {
      if (S <= s.ws_slots[lane]) return S;
      const int64_t full_bytes = workspace_bytes(m, cfg.precision, S, STORE_FULL);
      for (int st = STORE_FULL; st <= STORE_COMPACT; ++st) {
        if (forced >= 0 && st != forced) continue;
        const int64_t bytes = st == STORE_FULL ? full_bytes : workspace_bytes(m, cfg.precision, S, st);
        if (st == STORE_COMPACT && forced < 0 && bytes >= full_bytes) continue;  // no saving on small trees
        const int64_t extra = bytes - s.ws_bytes[lane];  // the old workspace is freed before the new one is made
        if (make_room(extra, mi, queued)) {
          resident += extra;
          s.ws_bytes[lane] = bytes;
          s.ws_slots[lane] = S;
          s.ws_store[lane] = st;
          store = st;
          return S;
        }
      }
    }
    return 0;
  }

  // host symbolic phase, admission of the resident arrays, then assembly and
  // device upload; false when the model failed
  bool prepare(std::unique_lock<std::mutex>& lk, int mi) {
    ModelSlot& s = *models[mi];
    elp_model* h = s.h;
    s.preparing = true;
    lk.unlock();
    int rc;
    try {
      rc = model_symbolic_host(h->m);
    } catch (const std::bad_alloc&) {
      set_error("host allocation failed");
      rc = ELP_ERR_NOMEM;
    } catch (const std::exception& e) {
      set_error(std::string("exception: ") + e.what());
      rc = ELP_ERR_ARG;
    }
    lk.lock();
    if (!rc) {
      const int64_t arrays = model_array_bytes(h->m);
      const int64_t one = workspace_bytes(h->m, cfg.precision, 1, forced_store() >= 0 ? forced_store() : STORE_COMPACT);
      if (arrays + one > cfg.hbm_budget_bytes) {
        rc = ELP_ERR_NOMEM;  // cannot run even alone
      } else if (!make_room(arrays, mi, running == 0)) {
        if (running == 0) {
          rc = ELP_ERR_NOMEM;  // other models' resident arrays hold the budget
        } else {
          // running batches free their workspaces when they end: prepared
          // again then (the symbolic phase is kept)
          s.preparing = false;
          return false;
        }
      } else {
        resident += arrays;
        s.array_bytes = arrays;
      }
    }
    if (!rc) {
      // workspaces the model made before it was registered: the server keeps
      // (and charges) the lanes it uses at its precision and releases the rest
      Model& m = h->m;
      for (int prec = 0; prec < 2; ++prec)
        for (int l = 0; l < 4; ++l) {
          std::unique_ptr<Workspace>& W = l ? m.ws_b[prec][l - 1] : m.ws[prec];
          if (!W) continue;
          if (prec != cfg.precision || l >= kLanesPerModel) { W.reset(); continue; }
          s.ws_slots[l] = W->slots;
          s.ws_store[l] = W->store;
          s.ws_bytes[l] = workspace_bytes(m, prec, W->slots, W->store);
          resident += s.ws_bytes[l];
        }
    }
    if (!rc) {
      lk.unlock();
      if (!h->m.assembled) rc = elp_model_assemble(h);
      if (!rc) rc = elp_model_analyse(h);
      lk.lock();
    }
    s.preparing = false;
    if (rc) {
      if (rc != ELP_ERR_NOMEM)
        fprintf(stderr, "[elp server] model %d could not be prepared (%d): %s\n", mi, rc, get_error().c_str());
      s.failed = true;
      fail_queue(mi, rc);
      return false;
    }
    s.ready = true;
    return true;
  }

  void worker() {
    cudaSetDevice(device);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      int mi = -1, lane = 0;
      cv_work.wait(lk, [&] { return stop || (mi = pick_model(lane)) >= 0; });
      if (stop) break;
      ModelSlot& s = *models[mi];
      if (s.failed) { fail_queue(mi, ELP_ERR_NOMEM); continue; }
      if (!s.ready) {
        if (!prepare(lk, mi)) {
          if (!s.failed) cv_work.wait(lk);  // no room yet: a running batch frees memory when it ends
          cv_work.notify_all();
          continue;
        }
        if (s.queue.empty() || (s.lanes_busy >> lane & 1)) { cv_work.notify_all(); continue; }
      }
      // batch size: waiting frequencies, capped by omega_batch and by the budget
      int waiting = 0;
      for (int64_t rid : s.queue) {
        const Request& r = reqs.at(rid);
        waiting += (int)r.omegas.size() - r.next;
        if (waiting >= cfg.omega_batch) break;
      }
      int store = STORE_FULL;
      int S = admit_batch(mi, lane, std::min(waiting, cfg.omega_batch), store);
      // nothing runs, so nothing else frees memory: models whose requests wait
      // give up their workspaces too
      if (S == 0 && running == 0) S = admit_batch(mi, lane, std::min(waiting, cfg.omega_batch), store, true);
      if (S == 0) {
        if (running == 0) {  // the model cannot run at all
          set_error("model does not fit the HBM budget");
          fail_queue(mi, ELP_ERR_NOMEM);
          cv_work.notify_all();
        } else {
          cv_work.wait(lk);  // a running batch frees memory when it ends
        }
        continue;
      }
      s.lanes_busy |= 1 << lane;
      ++running;
      struct Item { int64_t rid; int k; double w; };
      std::vector<Item> items;
      while (!s.queue.empty() && (int)items.size() < S) {
        Request& r = reqs.at(s.queue.front());
        while (r.next < (int)r.omegas.size() && (int)items.size() < S) {
          items.push_back({r.id, r.next, r.omegas[r.next]});
          r.next++;
        }
        if (r.next >= (int)r.omegas.size()) s.queue.pop_front();
      }
      Model& m = s.h->m;
      lk.unlock();

      std::vector<elp_solve_info> info(items.size());
      const int64_t n = m.n;
      std::vector<double> oms(items.size());
      for (size_t i = 0; i < items.size(); ++i) oms[i] = items[i].w;
      int rc;
      try {
        rc = numeric_solve_lane(m, cfg.precision, lane, oms.data(), (int)oms.size(), nullptr, nullptr, info.data(),
                                cfg.tol, st, store);
      } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        rc = ELP_ERR_NOMEM;
      } catch (const std::exception& e) {
        set_error(std::string("exception: ") + e.what());
        rc = ELP_ERR_CUDA;
      }
      // a frequency short of the tolerance is reported per request (status and residual)
      if (rc == ELP_ERR_NOCONV || rc == ELP_ERR_SINGULAR) rc = ELP_OK;
      if (!rc) {
        // solutions straight from the lane's workspace into the requests' buffers
        const double2* xw = lane_solution(m, cfg.precision, lane);
        std::vector<double*> dst(items.size(), nullptr);
        {
          std::lock_guard<std::mutex> g(mu);
          for (size_t i = 0; i < items.size(); ++i) {
            auto it = reqs.find(items[i].rid);
            if (it != reqs.end()) dst[i] = it->second.x_out + (size_t)items[i].k * 2 * n;
          }
        }
        for (size_t i = 0; i < items.size() && !rc; ++i)
          if (dst[i] && cudaMemcpyAsync(dst[i], xw + i * n, sizeof(double2) * n, cudaMemcpyDeviceToHost, st) !=
                            cudaSuccess)
            rc = ELP_ERR_CUDA;
        if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = ELP_ERR_CUDA;
      }
      if (rc)  // the per-thread error text does not reach the caller's thread
        fprintf(stderr, "[elp server] batch of %zu frequencies on model %d failed (%d): %s\n", items.size(), mi, rc,
                get_error().c_str());
      lk.lock();
      for (size_t i = 0; i < items.size(); ++i) {
        auto it = reqs.find(items[i].rid);
        if (it == reqs.end()) continue;
        Request& r = it->second;
        if (rc) r.status = rc;
        else {
          r.max_res = std::max(r.max_res, info[i].rel_residual);
          if (!(info[i].rel_residual <= cfg.tol) && r.status != ELP_ERR_SINGULAR)
            r.status = info[i].static_pivots > 0 ? ELP_ERR_SINGULAR : ELP_ERR_NOCONV;
        }
        r.done++;
        if (r.done == (int)r.omegas.size()) finish_request(r);
      }
      s.lanes_busy &= ~(1 << lane);
      --running;
      cv_work.notify_all();
    }
    lk.unlock();
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
    if (ms->h == m) { set_error("model already registered"); return ELP_ERR_ARG; }
  std::unique_ptr<ModelSlot> ms(new ModelSlot());
  ms->h = m;  // prepared (and charged) by the first worker that picks it up
  s->models.push_back(std::move(ms));
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
  s->models[model_id]->queue.push_back(r.id);
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
