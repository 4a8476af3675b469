// extern "C" entry points of libelpaso_gb300.so (declared in
// include/elpaso_gb300.h). Every call returns an int status and never
// aborts; the text of the last error is per thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>

#include "device.cuh"
#include "numeric.cuh"
#include "symbolic.hpp"

using namespace elp;


namespace elp {
Model::Model() = default;
Model::~Model() = default;

int model_symbolic_host(Model& m) {
  if (m.sym) return ELP_OK;
  fault_host_alloc_point();
  std::unique_ptr<Symbolic> s(new Symbolic());
  // leaves of the nested dissection: subsets of at most this many DOFs (the
  // model's tuning; ELP_LEAF, default 128)
  int rc = symbolic_analyse(m, *s, resolved_tuning(m).leaf);
  if (rc) return rc;
  if (getenv("ELP_PROF_LEVELS")) {  // per-level work, beside the per-level device times of the profiler
    const Symbolic& S = *s;
    for (int l = 0; l < S.n_levels; ++l) {
      double crout = 0.0, schur = 0.0, m2 = 0.0, fac = 0.0;
      int maxp = 0, maxb = 0;
      for (int t : S.level_fronts[l]) {
        const int p = S.fronts[t].p, b = S.fronts[t].b;
        const double pp = p, bb = b, mm = pp + bb;
        maxp = std::max(maxp, p);
        maxb = std::max(maxb, b);
        schur += 8.0 * bb * bb * pp;
        for (int k0 = 0; k0 < p; k0 += 32) {
          const double w = std::min(32, p - k0), tt = mm - k0 - w;
          crout += 8.0 * (tt * tt - bb * bb) * w;  // trailing updates of the pivot rows and columns
        }
        m2 += mm * mm;
        fac += pp * pp + 2.0 * pp * bb;
      }
      fprintf(stderr, "[elp levels] level %2d fronts %5zu max p %5d max b %5d: crout %8.2f GF, schur %8.2f GF, "
              "sum m^2 %8.1f M, factor %8.1f M entries\n", l, S.level_fronts[l].size(), maxp, maxb, crout / 1e9,
              schur / 1e9, m2 / 1e6, fac / 1e6);
    }
  }
  m.sym = std::move(s);
  return ELP_OK;
}
}  // namespace elp

#define GUARD_BEGIN try {
#define GUARD_END                                   \
  }                                                 \
  catch (const std::bad_alloc&) {                   \
    set_error("host allocation failed");            \
    return ELP_ERR_NOMEM;                           \
  }                                                 \
  catch (const std::exception& ex) {                \
    set_error(std::string("exception: ") + ex.what()); \
    return ELP_ERR_ARG;                             \
  }

static int check_cuda_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device: this library has no CPU path");
    return ELP_ERR_CUDA;
  }
  return ELP_OK;
}

extern "C" {

const char* elp_last_error(void) { return get_error().c_str(); }

int elp_model_create(const elp_model_desc* desc, elp_model** out) {
  GUARD_BEGIN
  if (!out) { set_error("null output handle"); return ELP_ERR_ARG; }
  *out = nullptr;
  elp_model* h = new elp_model();
  std::string err;
  int rc = build_model(desc, h->m, err);
  if (rc) {
    set_error(err);
    delete h;
    return rc;
  }
  *out = h;
  return ELP_OK;
  GUARD_END
}

int elp_model_destroy(elp_model* m) {
  GUARD_BEGIN
  delete m;
  return ELP_OK;
  GUARD_END
}

int elp_model_assemble(elp_model* h) {
  GUARD_BEGIN
  if (!h) { set_error("null model"); return ELP_ERR_ARG; }
  int rc = check_cuda_device();
  if (rc) return rc;
  Model& m = h->m;
  if (!m.dev) {
    rc = device_upload_model(m);
    if (rc) {
      m.dev.reset();  // partly uploaded: the next call starts over
      return rc;
    }
  }
  float ms = 0.f;
  rc = device_assemble(m, 0, &ms);
  if (rc) return rc;
  m.assembled = true;
  return ELP_OK;
  GUARD_END
}

int elp_model_set_assembly(elp_model* h, int arithmetic) {
  GUARD_BEGIN
  if (!h) { set_error("null model"); return ELP_ERR_ARG; }
  if (arithmetic != ELP_ASSEMBLY_FP64 && arithmetic != ELP_ASSEMBLY_DOUBLE_FLOAT) {
    set_error("assembly arithmetic must be ELP_ASSEMBLY_FP64 or ELP_ASSEMBLY_DOUBLE_FLOAT");
    return ELP_ERR_ARG;
  }
  Model& m = h->m;
  if (m.n_members > 1) { set_error("groups assemble in FP64"); return ELP_ERR_ARG; }
  const bool again = m.assembled && m.assembly != arithmetic;
  m.assembly = arithmetic;
  if (again) {
    float ms = 0.f;
    m.assembled = false;
    int rc = device_assemble(m, 0, &ms);
    if (rc) return rc;
    m.assembled = true;
  }
  return ELP_OK;
  GUARD_END
}

int elp_model_time_assembly(elp_model* h, int repeats, double* ms_per_assembly, double* ms_kernel_only) {
  GUARD_BEGIN
  if (!h || !h->m.assembled) { set_error("assemble the model first"); return ELP_ERR_STATE; }
  if (repeats < 1) repeats = 1;
  double tot = 0.0, best = 1e300;
  for (int r = 0; r < repeats; ++r) {
    float ms = 0.f;
    int rc = device_assemble(h->m, 0, &ms);
    if (rc) return rc;
    tot += ms;
    best = std::min(best, (double)ms);
  }
  if (ms_per_assembly) *ms_per_assembly = tot / repeats;
  if (ms_kernel_only) *ms_kernel_only = best;
  return ELP_OK;
  GUARD_END
}

int elp_model_analyse(elp_model* h) {
  GUARD_BEGIN
  if (!h) { set_error("null model"); return ELP_ERR_ARG; }
  Model& m = h->m;
  if (m.analysed) return ELP_OK;
  int rc = model_symbolic_host(m);  // kept when the device step below fails
  if (rc) return rc;
  rc = check_cuda_device();
  if (rc) return rc;
  rc = device_upload_symbolic(m);
  if (rc) return rc;
  m.analysed = true;
  return ELP_OK;
  GUARD_END
}

int elp_model_get_info(const elp_model* h, elp_model_info* info) {
  GUARD_BEGIN
  if (!h || !info) { set_error("null argument"); return ELP_ERR_ARG; }
  const Model& m = h->m;
  memset(info, 0, sizeof(*info));
  info->n_dofs = m.n;
  info->nnz = m.nnz;
  info->n_elements = m.n_elements_total;
  info->n_struct_groups = (int)m.groups.size();
  if (m.sym) {
    info->n_fronts = (int64_t)m.sym->fronts.size();
    info->factor_entries = m.sym->arena;
    info->factor_flops = m.sym->flops;
    info->gemm_flops = m.sym->gemm_flops;
    info->factor_bytes = m.sym->factor_bytes;
    info->n_levels = m.sym->n_levels;
    info->max_front = m.sym->max_front;
    info->factor_stored = m.sym->factor_stored;
    info->front_pool_peak = m.sym->pool_peak;
    info->front_pool = m.sym->pool;
    for (int prec = 0; prec < 2; ++prec)
      for (int st = 0; st < 2; ++st)
        info->workspace_bytes_per_frequency[prec][st] =
            workspace_bytes(m, prec, 1, st == 0 ? STORE_FULL : STORE_COMPACT);
  }
  info->device_array_bytes = model_array_bytes(m);
  if (m.dev) info->n_nonpositive_jacobians = m.dev->bad_jacobians_3d;
  return ELP_OK;
  GUARD_END
}

int elp_model_pattern(const elp_model* h, int32_t* row_ptr, int32_t* col_idx, int64_t* nnz) {
  GUARD_BEGIN
  if (!h) { set_error("null model"); return ELP_ERR_ARG; }
  const Model& m = h->m;
  if (nnz) *nnz = m.nnz;
  if (row_ptr) memcpy(row_ptr, m.row_ptr.data(), sizeof(int32_t) * (m.n + 1));
  if (col_idx) memcpy(col_idx, m.col_idx.data(), sizeof(int32_t) * m.nnz);
  return ELP_OK;
  GUARD_END
}

int elp_model_global_rows(const elp_model* h, int32_t* rows_out) {
  GUARD_BEGIN
  if (!h || !rows_out) { set_error("null argument"); return ELP_ERR_ARG; }
  memcpy(rows_out, h->m.global_rows.data(), sizeof(int32_t) * h->m.global_rows.size());
  return ELP_OK;
  GUARD_END
}

int elp_model_rhs(const elp_model* h, double* f_out) {
  GUARD_BEGIN
  if (!h || !f_out) { set_error("null argument"); return ELP_ERR_ARG; }
  const Model& m = h->m;
  for (int64_t i = 0; i < m.n; ++i) { f_out[2 * i] = m.rhs[i].real(); f_out[2 * i + 1] = m.rhs[i].imag(); }
  return ELP_OK;
  GUARD_END
}

int elp_cell_stresses(const elp_model* h, double omega, const double* x, double* sigma, double* sigma_lower) {
  GUARD_BEGIN
  if (!h || !x || !sigma) { set_error("null argument"); return ELP_ERR_ARG; }
  if (!(omega > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  std::string err;
  // the model is logically unchanged; its device copy is made on first use
  Model& m = const_cast<Model&>(h->m);
  const int rc = cell_stresses(m, omega, reinterpret_cast<const cplx*>(x), reinterpret_cast<cplx*>(sigma),
                               reinterpret_cast<cplx*>(sigma_lower), err);
  if (rc) set_error(err);
  return rc;
  GUARD_END
}

int elp_node_stresses(const elp_model* h, double omega, const double* x, double* sigma_nodes) {
  GUARD_BEGIN
  if (!h || !x || !sigma_nodes) { set_error("null argument"); return ELP_ERR_ARG; }
  if (!(omega > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  std::string err;
  Model& m = const_cast<Model&>(h->m);
  const int rc = node_stresses(m, omega, reinterpret_cast<const cplx*>(x), reinterpret_cast<cplx*>(sigma_nodes), err);
  if (rc) set_error(err);
  return rc;
  GUARD_END
}

int elp_model_rhs_omega(const elp_model* h, double omega, double* f_out) {
  GUARD_BEGIN
  if (!h || !f_out) { set_error("null argument"); return ELP_ERR_ARG; }
  if (!(omega > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  const Model& m = h->m;
  const double iw = 1.0 / omega;
  for (int64_t i = 0; i < m.n; ++i) {
    cplx v = m.rhs[i];
    if (m.has_vn && m.rhs_vn[i] != 0.0) v += m.rhs_vn[i] * iw;
    f_out[2 * i] = v.real();
    f_out[2 * i + 1] = v.imag();
  }
  return ELP_OK;
  GUARD_END
}

int elp_model_system_values(elp_model* h, double omega, double* values_out) {
  GUARD_BEGIN
  if (!h || !values_out) { set_error("null argument"); return ELP_ERR_ARG; }
  Model& m = h->m;
  if (!m.assembled) { set_error("assemble the model first"); return ELP_ERR_STATE; }
  if (!(omega > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  DevBuf<double2> out;
  ELP_CUDA(out.alloc(m.nnz));
  int rc = numeric_system_values(m, omega, out.p);
  if (rc) return rc;
  ELP_CUDA(cudaMemcpy(values_out, out.p, sizeof(double2) * m.nnz, cudaMemcpyDeviceToHost));
  return ELP_OK;
  GUARD_END
}

static int prepare(elp_model* h) {
  if (!h) { set_error("null model"); return ELP_ERR_ARG; }
  int rc = ELP_OK;
  if (!h->m.assembled) rc = elp_model_assemble(h);
  if (rc) return rc;
  if (!h->m.analysed) rc = elp_model_analyse(h);
  return rc;
}

int elp_solve_device(elp_model* h, const double* omegas, int n_omega, int precision, const double* f_dev,
                     double* x_dev, elp_solve_info* info, double tol, void* stream) {
  GUARD_BEGIN
  int rc = prepare(h);
  if (rc) return rc;
  if (precision != ELP_FP64_PLAIN && precision != ELP_MIXED) { set_error("unknown precision"); return ELP_ERR_ARG; }
  if (n_omega < 0 || (n_omega > 0 && (!omegas || !x_dev))) { set_error("bad solve arguments"); return ELP_ERR_ARG; }
  if (!(tol > 0.0)) tol = 1e-10;
  Model& m = h->m;
  const int64_t n = m.n;
  // batch size: as many frequencies as fit half of the free memory (with the
  // bytes this precision's workspaces already hold, which the batch reuses),
  // <= kMaxSlots
  size_t freeb = 0, totb = 0;
  ELP_CUDA(cudaMemGetInfo(&freeb, &totb));
  freeb += (size_t)workspace_held(m, precision);
  // whole fronts when the batch fits half the free memory that way (no factor
  // copy); the compact factor store when it does not (about 2/3 of the bytes)
  const int want = std::min(kMaxSlots, std::max(1, n_omega));
  const int store = choose_store(m, precision, want, (int64_t)(freeb / 2));
  const size_t per_slot = (size_t)workspace_bytes(m, precision, 1, store);
  int slots = (int)std::min<size_t>((size_t)kMaxSlots, std::max<size_t>(1, (freeb / 2) / std::max<size_t>(1, per_slot)));
  if (m.ws[precision] && m.ws[precision]->slots > 0 && m.ws[precision]->store == store)
    slots = std::max(slots, std::min(m.ws[precision]->slots, kMaxSlots));
  slots = std::min(slots, std::max(1, n_omega));
  // equal chunks when the batch must be split (48 over 46 slots: 2 x 24, not
  // 46 + 2, whose small remainder would cost nearly a whole factorisation pass)
  if (n_omega > slots) {
    const int chunks = (n_omega + slots - 1) / slots;
    slots = (n_omega + chunks - 1) / chunks;
  }
  int worst = ELP_OK;
  for (int s0 = 0; s0 < n_omega; s0 += slots) {
    int cnt = std::min(slots, n_omega - s0);
    rc = numeric_solve_batch(m, precision, omegas + s0, cnt,
                             f_dev ? reinterpret_cast<const double2*>(f_dev) + (size_t)s0 * n : nullptr,
                             reinterpret_cast<double2*>(x_dev) + (size_t)s0 * n, info ? info + s0 : nullptr, tol,
                             (cudaStream_t)stream, 4, store);
    if (rc == ELP_ERR_SINGULAR || (rc == ELP_ERR_NOCONV && worst != ELP_ERR_SINGULAR)) worst = rc;
    else if (rc && rc != ELP_ERR_NOCONV) return rc;
  }
  if (worst == ELP_ERR_NOCONV) set_error("iterative refinement did not reach the requested relative residual");
  if (worst == ELP_ERR_SINGULAR) set_error("zero pivot at one or more frequencies: singular system");
  return worst;
  GUARD_END
}

int elp_solve(elp_model* h, const double* omegas, int n_omega, int precision, const double* f_or_null,
              double* x_out, elp_solve_info* info, double tol) {
  GUARD_BEGIN
  int rc = prepare(h);
  if (rc) return rc;
  if (n_omega < 0 || (n_omega > 0 && (!omegas || !x_out))) { set_error("bad solve arguments"); return ELP_ERR_ARG; }
  if (n_omega == 0) return ELP_OK;
  Model& m = h->m;
  const int64_t n = m.n;
  DevBuf<double2> fd, xd;
  if (f_or_null) {
    ELP_CUDA(fd.alloc((size_t)n * n_omega));
    ELP_CUDA(cudaMemcpy(fd.p, f_or_null, sizeof(double2) * n * n_omega, cudaMemcpyHostToDevice));
  }
  ELP_CUDA(xd.alloc((size_t)n * n_omega));
  rc = elp_solve_device(h, omegas, n_omega, precision, f_or_null ? reinterpret_cast<double*>(fd.p) : nullptr,
                        reinterpret_cast<double*>(xd.p), info, tol, nullptr);
  if (rc && rc != ELP_ERR_NOCONV && rc != ELP_ERR_SINGULAR) return rc;
  ELP_CUDA(cudaMemcpy(x_out, xd.p, sizeof(double2) * n * n_omega, cudaMemcpyDeviceToHost));
  return rc;
  GUARD_END
}

int elp_front_update_test(int kernel, int p, int b, int step, int slots, float* fronts, int parent_m,
                          const int32_t* pmap, float* parents) {
  GUARD_BEGIN
  int rc = check_cuda_device();
  if (rc) return rc;
  return front_update_test(kernel, p, b, step, slots, fronts, parent_m, pmap, parents);
  GUARD_END
}

}  // extern "C"
