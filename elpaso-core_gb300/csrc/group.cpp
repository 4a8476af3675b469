// Groups of models solved together (elp_group_*): frontal updates grouped
// across models.
//
// The reference solves one model per process, one frequency at a time
// (analysisfrequencybasic.cpp:101-242). Many small models (plates of a few
// thousand DOFs) leave the GPU idle between launches when each is solved on
// its own: every tree level of every model is a launch of its own. A group
// puts its members into ONE system, their disjoint union:
//  - nodes keep each member's own order (renumbered by rank after the
//    previous members'), so a member's rows are contiguous and in the same
//    order as in the member alone;
//  - the symbolic phase splits the node graph into connected components
//    before the nested dissection, so each member keeps its own assembly tree
//    and every tree level is one launch over the fronts of all members
//    (levels are counted from the leaves);
//  - assembly is one pass over the elements of all members;
//  - each member keeps its own frequencies: the kernels that form A(w) look up
//    the coefficients of a row's member (coef[slot * members + member]);
//  - the right-hand side of each member is scaled by a power of two to about
//    unit norm (exact, so it changes no rounding); convergence is per member:
//    the mixed path runs one Krylov process per (member, frequency) pair on
//    the shared launches (numeric.cu run_gmres_group), the plain path's
//    refinement freezes members that reached tol; each member's residual is
//    measured on its own rows and reported per member and frequency.
// The members' loss-factor groups are merged by value, at most 8 in a group.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "device.cuh"
#include "numeric.cuh"
#include "symbolic.hpp"

using namespace elp;

struct elp_group {
  elp_model combined;
  std::vector<int64_t> n_of;  // DOFs of each member
};

namespace {

int build_group(elp_model* const* models, int count, elp_group& g, std::string& err) {
  // concatenated description; every index is shifted past the earlier members
  std::vector<int64_t> ids;
  std::vector<double> coords;
  std::vector<elp_material> mats;
  std::vector<std::vector<int32_t>> conns;
  std::vector<elp_element_block> blocks;
  std::vector<elp_interface_quad> ifs;
  std::vector<elp_fixed_dof> fixed;
  std::vector<elp_nodal_force> forces;
  std::vector<elp_nodal_moment> moments;
  std::vector<elp_fluid_source> sources;
  std::vector<elp_vn_load> vn;
  std::vector<elp_face_traction> tr;
  std::vector<int64_t> node_base(count + 1, 0);
  int64_t nb = 0;
  int mb = 0, bb = 0;
  for (int k = 0; k < count; ++k) {
    const Model& m = models[k]->m;
    node_base[k] = nb;
    // ids: the member's own order (rank by id) after the earlier members
    std::vector<int64_t> rank(m.n_nodes);
    for (int64_t r = 0; r < m.n_nodes; ++r) rank[m.order[r]] = r;
    for (int64_t v = 0; v < m.n_nodes; ++v) ids.push_back(nb + rank[v]);
    coords.insert(coords.end(), m.coords.begin(), m.coords.end());
    for (size_t i = 0; i < m.materials.size(); ++i) {
      elp_material mt = m.materials[i];
      if (!m.E_tables[i].empty()) {
        mt.n_E_table = (int)(m.E_tables[i].size() / 2);
        mt.E_table = m.E_tables[i].data();
      }
      if (!m.eta_tables[i].empty()) {
        mt.n_eta_table = (int)(m.eta_tables[i].size() / 2);
        mt.eta_table = m.eta_tables[i].data();
      }
      mats.push_back(mt);
    }
    for (const Block& B : m.blocks) {
      std::vector<int32_t> c(B.conn);
      for (int32_t& v : c) v += (int32_t)nb;
      conns.push_back(std::move(c));
      elp_element_block e;
      e.type = B.type;
      e.material = B.material + mb;
      e.n_elements = B.n_elements;
      e.connectivity = nullptr;  // set once conns stops growing
      blocks.push_back(e);
    }
    for (elp_interface_quad q : m.interfaces) {
      for (int j = 0; j < 4; ++j) { q.structure_nodes[j] += (int32_t)nb; q.fluid_nodes[j] += (int32_t)nb; }
      q.fluid_material += mb;
      ifs.push_back(q);
    }
    for (elp_fixed_dof f : m.fixed) { f.node += (int32_t)nb; fixed.push_back(f); }
    for (elp_nodal_force f : m.forces) { f.node += (int32_t)nb; forces.push_back(f); }
    for (elp_nodal_moment f : m.moments) { f.node += (int32_t)nb; moments.push_back(f); }
    for (elp_fluid_source f : m.fluid_sources) { f.node += (int32_t)nb; sources.push_back(f); }
    for (elp_vn_load l : m.vn_loads) { l.block += bb; vn.push_back(l); }
    for (elp_face_traction l : m.face_tractions) { l.block += bb; tr.push_back(l); }
    nb += m.n_nodes;
    mb += (int)m.materials.size();
    bb += (int)m.blocks.size();
    g.n_of.push_back(m.n);
  }
  node_base[count] = nb;
  if (nb >= ((int64_t)1 << 30)) { err = "group too large"; return ELP_ERR_ARG; }
  for (size_t i = 0; i < blocks.size(); ++i) blocks[i].connectivity = conns[i].data();
  elp_model_desc d;
  memset(&d, 0, sizeof(d));
  d.n_nodes = nb;
  d.node_ids = ids.data();
  d.coords = coords.data();
  d.n_materials = (int)mats.size();
  d.materials = mats.data();
  d.n_blocks = (int)blocks.size();
  d.blocks = blocks.data();
  d.n_interfaces = (int64_t)ifs.size();
  d.interfaces = ifs.data();
  d.n_fixed = (int64_t)fixed.size();
  d.fixed = fixed.data();
  d.n_forces = (int64_t)forces.size();
  d.forces = forces.data();
  d.n_moments = (int64_t)moments.size();
  d.moments = moments.data();
  d.n_fluid_sources = (int64_t)sources.size();
  d.fluid_sources = sources.data();
  d.n_vn_loads = (int64_t)vn.size();
  d.vn_loads = vn.data();
  d.n_face_tractions = (int64_t)tr.size();
  d.face_tractions = tr.data();
  Model& M = g.combined.m;
  int rc = build_model(&d, M, err);
  if (rc) return rc;
  // each member's rows: contiguous, its own count, in its own order
  M.n_members = count;
  M.row_model.resize(M.n);
  M.member_row_off.assign(count + 1, 0);
  for (int64_t r = 0; r < M.n; ++r) {
    const int k = (int)(std::upper_bound(node_base.begin(), node_base.end(), (int64_t)M.dof_node[r]) -
                        node_base.begin()) - 1;
    M.row_model[r] = k;
    M.member_row_off[k + 1]++;
  }
  for (int k = 0; k < count; ++k) M.member_row_off[k + 1] += M.member_row_off[k];
  for (int k = 0; k < count; ++k) {
    if (M.member_row_off[k + 1] - M.member_row_off[k] != g.n_of[k]) { err = "group member rows"; return ELP_ERR_ARG; }
    for (int64_t r = M.member_row_off[k]; r < M.member_row_off[k + 1]; ++r)
      if (M.row_model[r] != k) { err = "group member rows are not contiguous"; return ELP_ERR_ARG; }
  }
  // ||F||^2, 2 Re <F, G>, ||G||^2 per member, for ||F + G / w|| at any w
  M.member_f.assign(3 * (size_t)count, 0.0);
  for (int64_t r = 0; r < M.n; ++r) {
    double* q = &M.member_f[3 * (size_t)M.row_model[r]];
    const cplx f = M.rhs[r], gv = M.has_vn ? M.rhs_vn[r] : cplx(0.0);
    q[0] += std::norm(f);
    q[1] += 2.0 * (std::conj(f) * gv).real();
    q[2] += std::norm(gv);
  }
  return ELP_OK;
}

}  // namespace

namespace elp {
Model& group_model(elp_group* g) { return g->combined.m; }
}  // namespace elp

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

int elp_group_create(elp_model* const* models, int n_models, elp_group** out) {
  GUARD_BEGIN
  if (!out || !models || n_models < 1) { set_error("bad group arguments"); return ELP_ERR_ARG; }
  *out = nullptr;
  for (int k = 0; k < n_models; ++k)
    if (!models[k]) { set_error("null model in group"); return ELP_ERR_ARG; }
  elp_group* g = new elp_group();
  std::string err;
  int rc = build_group(models, n_models, *g, err);
  if (rc) {
    set_error(err);
    delete g;
    return rc;
  }
  rc = model_symbolic_host(g->combined.m);  // host ordering and tree now; the device steps at the first solve
  if (rc) {
    delete g;
    return rc;
  }
  *out = g;
  return ELP_OK;
  GUARD_END
}

int elp_group_info(const elp_group* g, elp_model_info* info) {
  if (!g) { set_error("null group"); return ELP_ERR_ARG; }
  return elp_model_get_info(&g->combined, info);
}

int elp_group_solve(elp_group* g, const double* omegas, int n_omega, int precision, double* x_out,
                    elp_solve_info* info, double tol) {
  GUARD_BEGIN
  if (!g) { set_error("null group"); return ELP_ERR_ARG; }
  if (precision != ELP_FP64_PLAIN && precision != ELP_MIXED) { set_error("unknown precision"); return ELP_ERR_ARG; }
  if (n_omega < 0 || (n_omega > 0 && (!omegas || !x_out))) { set_error("bad solve arguments"); return ELP_ERR_ARG; }
  if (n_omega == 0) return ELP_OK;
  if (!(tol > 0.0)) tol = 1e-10;
  elp_model* h = &g->combined;
  int rc = ELP_OK;
  if (!h->m.assembled) rc = elp_model_assemble(h);
  if (!rc && !h->m.analysed) rc = elp_model_analyse(h);
  if (rc) return rc;
  Model& m = h->m;
  const int nm = m.n_members;
  const int64_t n = m.n;
  // frequencies per batch: as many as fit half of the free memory (with what
  // this precision's workspaces hold), in equal chunks
  size_t freeb = 0, totb = 0;
  ELP_CUDA(cudaMemGetInfo(&freeb, &totb));
  freeb += (size_t)workspace_held(m, precision);
  const int want = std::min(kMaxSlots, n_omega);
  const int store = choose_store(m, precision, want, (int64_t)(freeb / 2));
  const size_t per_slot = (size_t)workspace_bytes(m, precision, 1, store) + (size_t)n * sizeof(double2);
  int slots = (int)std::min<size_t>((size_t)kMaxSlots, std::max<size_t>(1, (freeb / 2) / std::max<size_t>(1, per_slot)));
  slots = std::min(slots, n_omega);
  if (n_omega > slots) {
    const int chunks = (n_omega + slots - 1) / slots;
    slots = (n_omega + chunks - 1) / chunks;
  }
  DevBuf<double2> xd;
  ELP_CUDA(xd.alloc((size_t)n * slots));
  std::vector<double> oms((size_t)slots * nm);
  std::vector<elp_solve_info> inf((size_t)slots * nm);
  std::vector<double2> xh((size_t)n * slots);
  std::vector<int64_t> out_off(nm, 0);  // member k's block in x_out: n_omega x n_k after the earlier members'
  for (int k = 1; k < nm; ++k) out_off[k] = out_off[k - 1] + (int64_t)n_omega * g->n_of[k - 1];
  int worst = ELP_OK;
  for (int s0 = 0; s0 < n_omega; s0 += slots) {
    const int cnt = std::min(slots, n_omega - s0);
    for (int s = 0; s < cnt; ++s)
      for (int k = 0; k < nm; ++k) oms[(size_t)s * nm + k] = omegas[(size_t)k * n_omega + s0 + s];
    rc = numeric_solve_batch(m, precision, oms.data(), cnt, nullptr, xd.p, inf.data(), tol, 0, 4, store);
    if (rc == ELP_ERR_SINGULAR || (rc == ELP_ERR_NOCONV && worst != ELP_ERR_SINGULAR)) worst = rc;
    else if (rc) return rc;
    ELP_CUDA(cudaMemcpy(xh.data(), xd.p, sizeof(double2) * n * cnt, cudaMemcpyDeviceToHost));
    for (int k = 0; k < nm; ++k) {
      const int64_t nk = g->n_of[k], r0 = m.member_row_off[k];
      for (int s = 0; s < cnt; ++s) {
        memcpy(x_out + 2 * (out_off[k] + (int64_t)(s0 + s) * nk), xh.data() + (size_t)s * n + r0,
               sizeof(double2) * nk);
        if (info) info[(size_t)k * n_omega + s0 + s] = inf[(size_t)s * nm + k];
      }
    }
  }
  if (worst == ELP_ERR_NOCONV) set_error("a group member did not reach the requested relative residual");
  if (worst == ELP_ERR_SINGULAR) set_error("zero pivot in a group member: singular system");
  return worst;
  GUARD_END
}

int elp_group_destroy(elp_group* g) {
  GUARD_BEGIN
  delete g;
  return ELP_OK;
  GUARD_END
}

}  // extern "C"
