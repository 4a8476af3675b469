// Host-side model construction: DOF numbering, CSR pattern, entry classes,
// Dirichlet rows and the nodal-force right-hand side.
//
// Reference behaviour restated (paths inside elpasoCore/source/):
//  - numbering: nodes in ascending id (std::map, fedata/mesh.h:49), per node
//    the active DOFs in enum order 0..20 each take the next row
//    (analysis/analysis.cpp:499-518); inactive DOFs keep row -1
//    (fedata/dof.cpp:24-26);
//  - active DOFs are the union of getDofs() of the elements touching the
//    node (analysis.cpp:480-490); interface elements activate nothing;
//  - pattern: every element's dense DOF block (analysis.cpp:815-823, values
//    inserted with ADD_VALUES incl. explicit zeros, :1238-1246), every
//    interface's C (structure rows x fluid cols) and C^T block
//    (analysis.cpp:826-866), negative indices dropped, diagonal always
//    present (analysis.cpp:791); Dirichlet rows keep their pattern
//    (MAT_KEEP_NONZERO_PATTERN, analysis.cpp:802);
//  - BC rows: nodes in id order, each BC of the node, DOFs 0..20 that are
//    active and fixed (analysis.cpp:366-414); MatZeroRows(diag = 1) and
//    F[row] = value (analysis.cpp:419-454);
//  - nodal forces add F on active x1, x2, x3 rows (analysis.cpp:171-279),
//    fluid point sources 4 pi p on the fluid row, nodal moments on w1..w3
//    (analysis.cpp:243-265, 281-364); normal-velocity loads on Fluid8 faces
//    form the 1/w part of F (elementfluid3d.cpp:241-309); constant tractions
//    on Brick8 faces add to F before the nodal loads
//    (elementstructurebrick.cpp:556-662).
#include "model.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <stdexcept>
#include <unordered_map>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace elp {

static thread_local std::string g_error;
void set_error(const std::string& s) { g_error = s; }
const std::string& get_error() { return g_error; }

int nodes_per_element(int type) {
  switch (type) {
    case ELP_BRICK8: return 8;
    case ELP_DSG4: return 4;
    case ELP_FLUID8: return 8;
  }
  return 0;
}
int dofs_per_node(int type) {
  switch (type) {
    case ELP_BRICK8: return 3;
    case ELP_DSG4: return 3;
    case ELP_FLUID8: return 1;
  }
  return 0;
}
static const int kBrickDofs[3] = {ELP_DOF_X1, ELP_DOF_X2, ELP_DOF_X3};
static const int kPlateDofs[3] = {ELP_DOF_X3, ELP_DOF_W1, ELP_DOF_W2};
static const int kFluidDofs[1] = {ELP_DOF_FLUID};
const int* element_dofs(int type) {
  switch (type) {
    case ELP_BRICK8: return kBrickDofs;
    case ELP_DSG4: return kPlateDofs;
    case ELP_FLUID8: return kFluidDofs;
  }
  return nullptr;
}

// Value of a (w, value) table at w: the first / last value outside the table,
// linear interpolation between the two rows around w inside
// (cMaterialStructureVisco::updateMaterial, materialstructurevisco.cpp:229-281).
static double table_value(const std::vector<double>& om, const std::vector<double>& val, double w) {
  const size_t n = om.size();
  if (w <= om[0]) return val[0];
  if (w >= om[n - 1]) return val[n - 1];
  size_t k = 1;
  while (!(om[k - 1] <= w && om[k] > w)) ++k;  // ascending table: exactly one interval holds w
  return (val[k] - val[k - 1]) * (w - om[k - 1]) / (om[k] - om[k - 1]) + val[k - 1];
}

cplx group_coefficient(const StructGroup& g, double w) {
  const double scale = g.om_e.empty() ? 1.0 : table_value(g.om_e, g.val_e, w) / g.e_ref;
  const double eta = g.om_eta.empty() ? g.eta : table_value(g.om_eta, g.val_eta, w);
  if (g.visco_type == 1) return scale * cplx(1.0, eta);
  if (g.visco_type == 2) return scale * cplx(1.0, w * eta);
  return cplx(scale, 0.0);
}

// Copies a caller's (frequency [Hz], value) table into (w, value) vectors.
static bool copy_table(int n, const double* tab, std::vector<double>& om, std::vector<double>& val,
                       std::string& err, const char* what) {
  om.clear();
  val.clear();
  if (n <= 0) return true;
  if (!tab) { err = std::string(what) + " table pointer is null"; return false; }
  for (int k = 0; k < n; ++k) {
    const double f = tab[2 * k], v = tab[2 * k + 1];
    if (!std::isfinite(f) || !std::isfinite(v) || (k > 0 && !(f > tab[2 * (k - 1)]))) {
      err = std::string(what) + " table needs finite values at strictly increasing frequencies";
      return false;
    }
    om.push_back(2.0 * M_PI * f);
    val.push_back(v);
  }
  return true;
}

static bool is_structure_type(int t) { return t == ELP_BRICK8 || t == ELP_DSG4; }

// The four nodes of face f (0..5) of a hexahedron, cShapeHex8's surfaces with
// outward normals (shapehex8.cpp:119-150).
static void face_nodes_hex8(int f, const int32_t* en, int32_t* out) {
  static const int kFace[6][4] = {{0, 1, 5, 4}, {2, 3, 7, 6}, {0, 3, 2, 1},
                                  {1, 2, 6, 5}, {4, 5, 6, 7}, {0, 4, 7, 3}};
  for (int k = 0; k < 4; ++k) out[k] = en[kFace[f][k]];
}

// int_face N_z dA of the bilinear face shape functions, 2 x 2 Gauss points,
// surface Jacobian |a1 x a2| from the tangents a1 = dx/dxi, a2 = dx/deta
// (evaluateSurfaceIntegral, elementfluid3d.cpp:169-233: the load is
// sum_s C(z, s) vn with C(z, s) = int N_z N_s dA, and sum_s N_s = 1).
// False if the Jacobian is not positive at a Gauss point.
static bool face_shape_integrals(const Model& m, const int32_t* fn, double* nint) {
  const double g = 1.0 / std::sqrt(3.0);
  const double xi[4] = {-1.0, 1.0, 1.0, -1.0}, et[4] = {-1.0, -1.0, 1.0, 1.0};  // quad4 node corners
  for (int z = 0; z < 4; ++z) nint[z] = 0.0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const double u = (a ? g : -g), v = (b ? g : -g);
      double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0}, N[4];
      for (int k = 0; k < 4; ++k) {
        N[k] = 0.25 * (1.0 + xi[k] * u) * (1.0 + et[k] * v);
        const double dxi = 0.25 * xi[k] * (1.0 + et[k] * v), det = 0.25 * et[k] * (1.0 + xi[k] * u);
        for (int d3 = 0; d3 < 3; ++d3) {
          a1[d3] += dxi * m.coords[3 * (size_t)fn[k] + d3];
          a2[d3] += det * m.coords[3 * (size_t)fn[k] + d3];
        }
      }
      const double s11 = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
      const double s22 = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
      const double s12 = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
      const double jac = std::sqrt(s11 * s22 - s12 * s12);
      if (!(jac > 0.0)) return false;
      for (int z = 0; z < 4; ++z) nint[z] += N[z] * jac;  // Gauss weights 1
    }
  return true;
}

int build_model(const elp_model_desc* d, Model& m, std::string& err) {
  fault_host_alloc_point();
  if (!d) { err = "null model description"; return ELP_ERR_ARG; }
  if (d->n_nodes <= 0 || !d->coords || !d->node_ids) { err = "model has no nodes"; return ELP_ERR_ARG; }
  if (d->n_nodes >= (int64_t)1 << 30) { err = "too many nodes"; return ELP_ERR_ARG; }
  m.n_nodes = d->n_nodes;
  m.node_ids.assign(d->node_ids, d->node_ids + d->n_nodes);
  m.coords.assign(d->coords, d->coords + 3 * d->n_nodes);
  if (d->n_materials < 0 || (d->n_materials > 0 && !d->materials)) { err = "bad materials"; return ELP_ERR_ARG; }
  m.materials.assign(d->materials, d->materials + d->n_materials);
  // frequency tables: copied here, the caller's pointers are not kept
  std::vector<StructGroup> tables(m.materials.size());
  m.E_tables.assign(m.materials.size(), {});
  m.eta_tables.assign(m.materials.size(), {});
  for (size_t i = 0; i < m.materials.size(); ++i) {
    const elp_material& mt = m.materials[i];
    if (mt.n_E_table > 0 && mt.E_table) m.E_tables[i].assign(mt.E_table, mt.E_table + 2 * (size_t)mt.n_E_table);
    if (mt.n_eta_table > 0 && mt.eta_table)
      m.eta_tables[i].assign(mt.eta_table, mt.eta_table + 2 * (size_t)mt.n_eta_table);
  }
  for (size_t i = 0; i < m.materials.size(); ++i) {
    elp_material& mt = m.materials[i];
    const bool any = mt.n_E_table > 0 || mt.n_eta_table > 0;
    if (any && mt.kind != ELP_STR_LIN_VIS_ISO_DIR) { err = "frequency tables need a visco material"; return ELP_ERR_ARG; }
    if (!copy_table(mt.n_E_table, mt.E_table, tables[i].om_e, tables[i].val_e, err, "E") ||
        !copy_table(mt.n_eta_table, mt.eta_table, tables[i].om_eta, tables[i].val_eta, err, "eta"))
      return ELP_ERR_ARG;
    if (!tables[i].om_e.empty() && mt.E == 0.0) mt.E = tables[i].val_e[0];
    tables[i].e_ref = mt.E;
    if (!tables[i].om_e.empty() && !(mt.E != 0.0 && std::isfinite(mt.E))) {
      err = "E table needs a nonzero reference modulus";
      return ELP_ERR_ARG;
    }
    mt.n_E_table = mt.n_eta_table = 0;
    mt.E_table = mt.eta_table = nullptr;
  }
  for (auto& mt : m.materials) {
    if (mt.kind != ELP_STR_LIN_ELA_ISO_DIR && mt.kind != ELP_STR_LIN_VIS_ISO_DIR &&
        mt.kind != ELP_AF_LIN_UAF_ISO_DIR) { err = "unknown material kind"; return ELP_ERR_ARG; }
    if (mt.kind == ELP_STR_LIN_VIS_ISO_DIR && mt.visco_type != 1 && mt.visco_type != 2)
      { err = "visco_type must be 1 or 2"; return ELP_ERR_ARG; }
    if (mt.kind == ELP_AF_LIN_UAF_ISO_DIR && (!(mt.c > 0) || !(mt.rho > 0)))
      { err = "fluid material needs c > 0 and rho > 0"; return ELP_ERR_ARG; }
  }
  for (int b = 0; b < d->n_blocks; ++b) {
    const elp_element_block& eb = d->blocks[b];
    int npe = nodes_per_element(eb.type);
    if (!npe) { err = "unknown element type"; return ELP_ERR_ARG; }
    if (eb.material < 0 || eb.material >= d->n_materials) { err = "element block material out of range"; return ELP_ERR_ARG; }
    int mk = m.materials[eb.material].kind;
    if (is_structure_type(eb.type) == (mk == ELP_AF_LIN_UAF_ISO_DIR))
      { err = "element type / material kind mismatch"; return ELP_ERR_ARG; }
    if (eb.n_elements < 0 || (eb.n_elements > 0 && !eb.connectivity)) { err = "bad connectivity"; return ELP_ERR_ARG; }
    Block blk;
    blk.type = eb.type;
    blk.material = eb.material;
    blk.n_elements = eb.n_elements;
    blk.conn.assign(eb.connectivity, eb.connectivity + (size_t)npe * eb.n_elements);
    for (int32_t v : blk.conn)
      if (v < 0 || v >= d->n_nodes) { err = "connectivity node index out of range"; return ELP_ERR_ARG; }
    m.n_elements_total += eb.n_elements;
    m.blocks.push_back(std::move(blk));
  }
  if (d->n_interfaces > 0) {
    if (!d->interfaces) { err = "bad interfaces"; return ELP_ERR_ARG; }
    m.interfaces.assign(d->interfaces, d->interfaces + d->n_interfaces);
    for (auto& q : m.interfaces)
      for (int k = 0; k < 4; ++k)
        if (q.structure_nodes[k] < 0 || q.structure_nodes[k] >= d->n_nodes || q.fluid_nodes[k] < 0 ||
            q.fluid_nodes[k] >= d->n_nodes) { err = "interface node index out of range"; return ELP_ERR_ARG; }
  }
  if (d->n_fixed > 0) {
    if (!d->fixed) { err = "bad fixed dofs"; return ELP_ERR_ARG; }
    m.fixed.assign(d->fixed, d->fixed + d->n_fixed);
    for (auto& f : m.fixed)
      if (f.node < 0 || f.node >= d->n_nodes || f.dof < 0 || f.dof >= ELP_NUM_KNOWN_DOFS)
        { err = "fixed dof out of range"; return ELP_ERR_ARG; }
  }
  if (d->n_forces > 0) {
    if (!d->forces) { err = "bad forces"; return ELP_ERR_ARG; }
    m.forces.assign(d->forces, d->forces + d->n_forces);
    for (auto& f : m.forces)
      if (f.node < 0 || f.node >= d->n_nodes) { err = "force node out of range"; return ELP_ERR_ARG; }
  }
  if (d->n_moments > 0) {
    if (!d->moments) { err = "bad moments"; return ELP_ERR_ARG; }
    m.moments.assign(d->moments, d->moments + d->n_moments);
    for (auto& f : m.moments)
      if (f.node < 0 || f.node >= d->n_nodes) { err = "moment node out of range"; return ELP_ERR_ARG; }
  }
  if (d->n_fluid_sources > 0) {
    if (!d->fluid_sources) { err = "bad fluid sources"; return ELP_ERR_ARG; }
    m.fluid_sources.assign(d->fluid_sources, d->fluid_sources + d->n_fluid_sources);
    for (auto& f : m.fluid_sources)
      if (f.node < 0 || f.node >= d->n_nodes) { err = "fluid source node out of range"; return ELP_ERR_ARG; }
  }
  if (d->n_vn_loads > 0) {
    if (!d->vn_loads) { err = "bad normal-velocity loads"; return ELP_ERR_ARG; }
    m.vn_loads.assign(d->vn_loads, d->vn_loads + d->n_vn_loads);
    for (auto& l : m.vn_loads) {
      if (l.block < 0 || l.block >= (int)m.blocks.size() || m.blocks[l.block].type != ELP_FLUID8 ||
          l.element < 0 || l.element >= m.blocks[l.block].n_elements || l.face < 1 || l.face > 6 ||
          !std::isfinite(l.vn)) {
        err = "normal-velocity load needs a Fluid8 element, a face 1..6 and a finite value";
        return ELP_ERR_ARG;
      }
    }
  }
  if (d->n_face_tractions > 0) {
    if (!d->face_tractions) { err = "bad face tractions"; return ELP_ERR_ARG; }
    m.face_tractions.assign(d->face_tractions, d->face_tractions + d->n_face_tractions);
    for (auto& l : m.face_tractions) {
      bool finite = true;
      for (double t : l.t) finite = finite && std::isfinite(t);
      if (l.block < 0 || l.block >= (int)m.blocks.size() || m.blocks[l.block].type != ELP_BRICK8 ||
          l.element < 0 || l.element >= m.blocks[l.block].n_elements || l.face < 1 || l.face > 6 || !finite) {
        err = "face traction needs a Brick8 element, a face 1..6 and finite values";
        return ELP_ERR_ARG;
      }
    }
  }

  const int64_t N = m.n_nodes;
  // ---- node order by ascending id, duplicate ids rejected
  m.order.resize(N);
  std::iota(m.order.begin(), m.order.end(), 0);
  std::sort(m.order.begin(), m.order.end(),
            [&](int32_t a, int32_t b) { return m.node_ids[a] < m.node_ids[b]; });
  for (int64_t i = 1; i < N; ++i)
    if (m.node_ids[m.order[i]] == m.node_ids[m.order[i - 1]]) { err = "duplicate node id"; return ELP_ERR_ARG; }

  // ---- active DOFs (bitset of 21 per node)
  std::vector<uint32_t> active(N, 0u);
  for (auto& blk : m.blocks) {
    int npe = nodes_per_element(blk.type), ndn = dofs_per_node(blk.type);
    const int* dofs = element_dofs(blk.type);
    uint32_t mask = 0;
    for (int k = 0; k < ndn; ++k) mask |= 1u << dofs[k];
    for (size_t i = 0; i < blk.conn.size(); ++i) active[blk.conn[i]] |= mask;
    (void)npe;
  }
  m.global_rows.assign((size_t)N * ELP_NUM_KNOWN_DOFS, -1);
  int64_t row = 0;
  for (int64_t r = 0; r < N; ++r) {
    int32_t v = m.order[r];
    for (int k = 0; k < ELP_NUM_KNOWN_DOFS; ++k)
      if (active[v] & (1u << k)) m.global_rows[(size_t)v * ELP_NUM_KNOWN_DOFS + k] = (int32_t)row++;
  }
  if (row >= ((int64_t)1 << 31) - 1) { err = "too many dofs"; return ELP_ERR_ARG; }
  m.n = row;
  const int64_t n = m.n;
  if (n == 0) { err = "model has no active degrees of freedom"; return ELP_ERR_ARG; }
  m.dof_node.resize(n);
  m.dof_kind.resize(n);
  for (int64_t v = 0; v < N; ++v)
    for (int k = 0; k < ELP_NUM_KNOWN_DOFS; ++k) {
      int32_t g = m.global_rows[(size_t)v * ELP_NUM_KNOWN_DOFS + k];
      if (g >= 0) {
        m.dof_node[g] = (int32_t)v;
        m.dof_kind[g] = (k == ELP_DOF_FLUID) ? 1 : 0;
      }
    }
  auto grow = [&](int32_t node, int dof) -> int32_t {
    return m.global_rows[(size_t)node * ELP_NUM_KNOWN_DOFS + dof];
  };

  // ---- structure loss-factor groups
  m.material_group.assign(m.materials.size(), -1);
  {
    std::vector<int64_t> count;
    for (size_t i = 0; i < m.materials.size(); ++i) {
      const elp_material& mt = m.materials[i];
      if (mt.kind == ELP_AF_LIN_UAF_ISO_DIR) continue;
      StructGroup g = tables[i];
      g.visco_type = mt.kind == ELP_STR_LIN_VIS_ISO_DIR ? mt.visco_type : 0;
      g.eta = mt.kind == ELP_STR_LIN_VIS_ISO_DIR ? mt.eta : 0.0;
      if (g.visco_type != 0 && g.eta == 0.0 && !g.tabulated()) g.visco_type = 0;
      int found = -1;
      if (!g.tabulated())  // a tabulated material is a group of its own
        for (size_t j = 0; j < m.groups.size(); ++j)
          if (!m.groups[j].tabulated() && m.groups[j].visco_type == g.visco_type && m.groups[j].eta == g.eta)
            found = (int)j;
      if (found < 0) { found = (int)m.groups.size(); m.groups.push_back(g); count.push_back(0); }
      m.material_group[i] = found;
    }
    // elements per group; the most used group becomes group 0 (array VK)
    for (auto& blk : m.blocks)
      if (m.material_group[blk.material] >= 0) count[m.material_group[blk.material]] += blk.n_elements;
    if (m.groups.size() > 1) {
      size_t best = std::max_element(count.begin(), count.end()) - count.begin();
      if (best != 0) {
        std::swap(m.groups[0], m.groups[best]);
        for (auto& g : m.material_group) {
          if (g == 0) g = (int)best;
          else if (g == (int)best) g = 0;
        }
      }
    }
    if (m.groups.empty()) m.groups.push_back(StructGroup());  // elastic, eta 0
    if (m.groups.size() > (size_t)kMaxStructGroups) {
      err = "more than " + std::to_string(kMaxStructGroups) + " distinct structure loss-factor groups";
      return ELP_ERR_ARG;
    }
  }

  // ---- node -> incident elements (per block), CSR
  std::vector<int64_t> ne_ptr(N + 1, 0);
  for (auto& blk : m.blocks)
    for (int32_t v : blk.conn) ne_ptr[v + 1]++;
  for (int64_t v = 0; v < N; ++v) ne_ptr[v + 1] += ne_ptr[v];
  struct ERef { int32_t block; int64_t elem; };
  std::vector<ERef> ne_list(ne_ptr[N]);
  {
    std::vector<int64_t> fill(ne_ptr.begin(), ne_ptr.end() - 1);
    for (int32_t b = 0; b < (int32_t)m.blocks.size(); ++b) {
      auto& blk = m.blocks[b];
      int npe = nodes_per_element(blk.type);
      for (int64_t e = 0; e < blk.n_elements; ++e)
        for (int k = 0; k < npe; ++k) {
          int32_t v = blk.conn[(size_t)e * npe + k];
          // an element lists each node once; repeated nodes would add twice
          ne_list[fill[v]++] = ERef{b, e};
        }
    }
  }
  // ---- interface contributions per row: struct row -> fluid cols, fluid row -> struct cols
  std::vector<std::vector<int32_t>> extra;  // sparse: only rows touched by interfaces
  std::unordered_map<int32_t, int32_t> extra_slot;
  for (auto& q : m.interfaces) {
    int32_t srows[12], fcols[4];
    for (int k = 0; k < 4; ++k) {
      for (int d3 = 0; d3 < 3; ++d3) srows[k * 3 + d3] = grow(q.structure_nodes[k], d3);
      fcols[k] = grow(q.fluid_nodes[k], ELP_DOF_FLUID);
    }
    auto add = [&](int32_t r, int32_t c) {
      if (r < 0 || c < 0) return;
      auto it = extra_slot.find(r);
      int32_t s;
      if (it == extra_slot.end()) { s = (int32_t)extra.size(); extra_slot[r] = s; extra.emplace_back(); }
      else s = it->second;
      extra[s].push_back(c);
    };
    for (int z = 0; z < 12; ++z)
      for (int s = 0; s < 4; ++s) { add(srows[z], fcols[s]); add(fcols[s], srows[z]); }
  }

  // ---- per-row column lists (parallel over nodes)
  // Row (v, k) holds every DOF of every node of each element at v whose
  // family carries DOF k, the diagonal, and the row's interface columns.
  // Which of v's elements count depends on k only through the families that
  // carry k, so the DOFs of v with the same families share one column set.
  // The set is built from v's neighbour nodes taken in node order, each
  // with the DOFs its selected elements give it in enum order: rows are
  // numbered node by node and DOF by DOF in that order, so the set comes
  // out sorted and unique with no per-row sort. Pass 1 counts the row
  // lengths, pass 2 writes the columns straight into col_idx.
  std::vector<int32_t> node_rank(N);
  for (int64_t i = 0; i < N; ++i) node_rank[m.order[i]] = (int32_t)i;
  uint32_t fam_of_dof[ELP_NUM_KNOWN_DOFS] = {0};  // bit (1 << type) per family carrying the DOF
  uint32_t dofs_of_type[8] = {0};                 // DOF bits carried by each family
  for (int t : {ELP_BRICK8, ELP_DSG4, ELP_FLUID8}) {
    const int* dofs = element_dofs(t);
    for (int q = 0; q < dofs_per_node(t); ++q) {
      fam_of_dof[dofs[q]] |= 1u << t;
      dofs_of_type[t] |= 1u << dofs[q];
    }
  }
  for (auto& e : extra) {
    std::sort(e.begin(), e.end());
    e.erase(std::unique(e.begin(), e.end()), e.end());
  }
  m.row_ptr.assign(n + 1, 0);
  m.diag_idx.resize(n);
  // columns of row r = base (sorted, unique) + r + the row's interface columns
  auto row_columns = [&](int32_t r, const std::vector<int32_t>& base, std::vector<int32_t>& out) {
    out.clear();
    auto it = extra_slot.find(r);
    const int32_t one[1] = {r};
    if (it == extra_slot.end()) {
      if (std::binary_search(base.begin(), base.end(), r)) { out = base; return; }
      std::set_union(base.begin(), base.end(), one, one + 1, std::back_inserter(out));
      return;
    }
    std::vector<int32_t> tmp;
    std::set_union(base.begin(), base.end(), one, one + 1, std::back_inserter(tmp));
    const std::vector<int32_t>& ex = extra[it->second];
    std::set_union(tmp.begin(), tmp.end(), ex.begin(), ex.end(), std::back_inserter(out));
  };
  const int64_t nnodes = N;
  for (int pass = 0; pass < 2; ++pass) {
#pragma omp parallel
    {
      std::vector<std::pair<int32_t, uint32_t>> nbr;  // (node rank, DOF bits)
      // one slot per distinct family set among a node's DOFs (at most one per DOF)
      std::vector<int32_t> base[ELP_NUM_KNOWN_DOFS], cols;
      uint32_t base_fam[ELP_NUM_KNOWN_DOFS];
#pragma omp for schedule(dynamic, 256)
      for (int64_t v = 0; v < nnodes; ++v) {
        int nb = 0;
        for (int k = 0; k < ELP_NUM_KNOWN_DOFS; ++k) {
          const int32_t r = grow((int32_t)v, k);
          if (r < 0) continue;
          const uint32_t fam = fam_of_dof[k];
          int b = 0;
          while (b < nb && base_fam[b] != fam) ++b;
          if (b == nb) {  // first DOF of v with this family set: build its columns
            ++nb;
            base_fam[b] = fam;
            nbr.clear();
            for (int64_t p = ne_ptr[v]; p < ne_ptr[v + 1]; ++p) {
              const Block& blk = m.blocks[ne_list[p].block];
              if (!(fam & (1u << blk.type))) continue;
              const int npe = nodes_per_element(blk.type);
              const int32_t* en = &blk.conn[(size_t)ne_list[p].elem * npe];
              for (int a = 0; a < npe; ++a) nbr.emplace_back(node_rank[en[a]], dofs_of_type[blk.type]);
            }
            std::sort(nbr.begin(), nbr.end());
            std::vector<int32_t>& B = base[b];
            B.clear();
            for (size_t i = 0; i < nbr.size();) {
              uint32_t bits = 0;
              size_t j = i;
              for (; j < nbr.size() && nbr[j].first == nbr[i].first; ++j) bits |= nbr[j].second;
              const int32_t a = m.order[nbr[i].first];
              for (int q = 0; q < ELP_NUM_KNOWN_DOFS; ++q)
                if (bits & (1u << q)) {
                  const int32_t c = grow(a, q);
                  if (c >= 0) B.push_back(c);
                }
              i = j;
            }
          }
          row_columns(r, base[b], cols);
          if (pass == 0) {
            m.row_ptr[r + 1] = (int32_t)cols.size();
          } else {
            std::copy(cols.begin(), cols.end(), m.col_idx.begin() + m.row_ptr[r]);
            m.diag_idx[r] = m.row_ptr[r] + (int32_t)(std::lower_bound(cols.begin(), cols.end(), r) - cols.begin());
          }
        }
      }
    }
    if (pass == 0) {
      int64_t nnz = 0;
      for (int64_t r = 0; r < n; ++r) {
        nnz += m.row_ptr[r + 1];
        if (nnz >= ((int64_t)1 << 31) - 1) { err = "nnz exceeds int32 CSR range"; return ELP_ERR_ARG; }
        m.row_ptr[r + 1] = (int32_t)nnz;
      }
      m.nnz = nnz;
      m.col_idx.resize(nnz);
    }
  }
  const int64_t nnz = m.nnz;

  // ---- BC rows in reference order (analysis.cpp:376-413)
  std::vector<std::vector<int32_t>> node_bcs(N);
  for (size_t i = 0; i < m.fixed.size(); ++i) node_bcs[m.fixed[i].node].push_back((int32_t)i);
  m.is_bc_row.assign(n, 0);
  for (int64_t r = 0; r < N; ++r) {
    int32_t v = m.order[r];
    for (int32_t bi : node_bcs[v]) {
      const elp_fixed_dof& f = m.fixed[bi];
      int32_t g = grow(v, f.dof);
      if (g < 0) continue;  // the dof does not exist at the node
      m.bc_rows.push_back(g);
      m.bc_values.push_back(cplx(f.value_re, f.value_im));
      m.is_bc_row[g] = 1;
    }
  }

  // ---- entry classes
  m.cls.resize(nnz);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    for (int32_t p = m.row_ptr[r]; p < m.row_ptr[r + 1]; ++p) {
      int32_t c = m.col_idx[p];
      uint8_t k;
      if (m.is_bc_row[r]) k = (c == r) ? CLS_BC_DIAG : CLS_BC_OFF;
      else if (m.dof_kind[r] == 0 && m.dof_kind[c] == 0) k = CLS_STRUCT;
      else if (m.dof_kind[r] == 1 && m.dof_kind[c] == 1) k = CLS_FLUID;
      else k = CLS_COUPLE;
      if (!m.is_bc_row[r] && m.is_bc_row[c]) k |= CLS_BC_COLUMN;
      m.cls[p] = k;
    }
  }

  // ---- right-hand side: nodal forces (ADD) then BC values (set)
  m.rhs.assign(n, cplx(0.0, 0.0));
  {
    // element load vectors first (assembleGlobalTensors adds them before the
    // nodal loads): Brick8 face tractions, t_d int_face N_z dA on u_d of each
    // face node (sum_s C(z, s) t_d with sum_s N_s = 1)
    for (const auto& l : m.face_tractions) {
      const int32_t* en = &m.blocks[l.block].conn[(size_t)l.element * 8];
      int32_t fn[4];
      face_nodes_hex8(l.face - 1, en, fn);
      double nint[4];
      if (!face_shape_integrals(m, fn, nint)) { err = "face traction on a degenerate face"; return ELP_ERR_ARG; }
      for (int z = 0; z < 4; ++z)
        for (int d3 = 0; d3 < 3; ++d3) {
          const int32_t g = grow(fn[z], d3);
          if (g >= 0) m.rhs[g] += cplx(l.t[2 * d3], l.t[2 * d3 + 1]) * nint[z];
        }
    }
    // forces are applied per node in id order (analysis.cpp:187-276)
    std::vector<std::vector<int32_t>> node_forces(N);
    for (size_t i = 0; i < m.forces.size(); ++i) node_forces[m.forces[i].node].push_back((int32_t)i);
    for (int64_t r = 0; r < N; ++r) {
      int32_t v = m.order[r];
      for (int32_t fi : node_forces[v])
        for (int d3 = 0; d3 < 3; ++d3) {
          int32_t g = grow(v, d3);
          if (g >= 0) m.rhs[g] += cplx(m.forces[fi].f[d3], 0.0);
        }
    }
    // nodal moments on the active rotations w1 w2 w3 (analysis.cpp:281-364),
    // fluid point sources 4 pi p on the fluid row (analysis.cpp:243-265)
    std::vector<std::vector<int32_t>> node_moments(N), node_sources(N);
    for (size_t i = 0; i < m.moments.size(); ++i) node_moments[m.moments[i].node].push_back((int32_t)i);
    for (size_t i = 0; i < m.fluid_sources.size(); ++i) node_sources[m.fluid_sources[i].node].push_back((int32_t)i);
    for (int64_t r = 0; r < N; ++r) {
      const int32_t v = m.order[r];
      for (int32_t si : node_sources[v]) {
        const int32_t g = grow(v, ELP_DOF_FLUID);
        if (g >= 0) m.rhs[g] += cplx(4.0 * M_PI * m.fluid_sources[si].p, 0.0);
      }
    }
    for (int64_t r = 0; r < N; ++r) {
      const int32_t v = m.order[r];
      for (int32_t mi : node_moments[v])
        for (int d3 = 0; d3 < 3; ++d3) {
          const int32_t g = grow(v, ELP_DOF_W1 + d3);
          if (g >= 0) m.rhs[g] += cplx(m.moments[mi].m[d3], 0.0);
        }
    }
    // normal-velocity loads: G of F(w) = rhs + G / w
    m.rhs_vn.assign(n, cplx(0.0, 0.0));
    for (const auto& l : m.vn_loads) {
      const int32_t* en = &m.blocks[l.block].conn[(size_t)l.element * 8];
      int32_t fn[4];
      face_nodes_hex8(l.face - 1, en, fn);
      double nint[4];
      if (!face_shape_integrals(m, fn, nint)) { err = "normal-velocity load on a degenerate face"; return ELP_ERR_ARG; }
      for (int z = 0; z < 4; ++z) {
        const int32_t g = grow(fn[z], ELP_DOF_FLUID);
        if (g >= 0) m.rhs_vn[g] += cplx(0.0, -l.vn * nint[z]);
      }
      m.has_vn = true;
    }
    for (size_t i = 0; i < m.bc_rows.size(); ++i) {
      m.rhs[m.bc_rows[i]] = m.bc_values[i];
      m.rhs_vn[m.bc_rows[i]] = 0.0;
    }
  }
  return ELP_OK;
}

}  // namespace elp
