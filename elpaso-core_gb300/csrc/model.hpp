// Internal model state of the GB300 frequency-response path.
//
// A model owns (host) the copied description, the DOF numbering, the CSR
// pattern and per-entry physics class, and (device) the w-independent value
// arrays produced by the assembly kernel plus the symbolic factorisation.
#pragma once
#include <complex>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/elpaso_gb300.h"

namespace elp {

using cplx = std::complex<double>;

// Physics class of a CSR entry. The per-w coefficient of each value array
// depends only on this class (and on the structure loss-factor group):
//   A(w) = a_cls(w) * VK + b_cls(w) * VM + sum_g c_g(w) * VKg
enum EntryClass : uint8_t {
  CLS_STRUCT = 0,   // structure-structure: a = c_0(w) (1, 1+i eta, 1+i w eta), b = -w^2
  CLS_FLUID = 1,    // fluid-fluid, VK = K_f/rho, VM = M_f/rho: a = 1/w^2, b = -1
  CLS_COUPLE = 2,   // structure-fluid coupling (-ori)(C + C^T): a = 1, b = 0
  CLS_BC_OFF = 3,   // off-diagonal of a Dirichlet row: 0
  CLS_BC_DIAG = 4,  // diagonal of a Dirichlet row: 1 (MatZeroRows diag = 1)
};
// Flag bit on entries of non-Dirichlet rows whose COLUMN is a Dirichlet dof.
// A(w) keeps them (the reference zeroes rows only); the factorisation drops
// them and the solve lifts them to the right-hand side instead
// (x_bc = f_bc, f_r -= a_r,bc x_bc), which is exact block elimination.
constexpr uint8_t CLS_BC_COLUMN = 0x80;
constexpr uint8_t CLS_MASK = 0x7f;

// Loss-factor group of the structure stiffness: coefficient c_g(w).
// Materials with frequency tables form groups of their own:
// c_g(w) = E(w) / e_ref * (1 + i eta(w)) or (1 + i w eta(w)).
struct StructGroup {
  int visco_type = 0;  // 0 elastic, 1: 1 + i eta, 2: 1 + i w eta
  double eta = 0.0;
  double e_ref = 0.0;                 // modulus the stiffness was assembled with (tables only)
  std::vector<double> om_e, val_e;    // E(w) table (w = 2 pi f), ascending
  std::vector<double> om_eta, val_eta;
  bool tabulated() const { return !om_e.empty() || !om_eta.empty(); }
};
constexpr int kMaxStructGroups = 8;  // groups a model may have (value arrays VK + 7 VKg)

int nodes_per_element(int type);
int dofs_per_node(int type);
// reference getDofs(): Brick8 {x1,x2,x3}, DSG4 {x3,w1,w2}, Fluid8 {fluid}
const int* element_dofs(int type);

// Tuning of a model's factorisation (elp_model_set_tuning, elp_model_autotune).
// A negative value (0 for the tile) takes the process default: the ELP_*
// environment variable if set, else the built-in value measured best on the
// coupled plate-cavity sweep.
struct Tuning {
  int leaf = -1;        // nested-dissection leaf size in DOFs (ELP_LEAF, 128)
  int schur_tile = 0;   // columns of a converter-kernel Schur tile, 32 or 64 (64)
  int pack_count = -1;  // packed Schur kernel on levels of at most this many fronts (ELP_PACK_COUNT, 300)
  int pack_minb = -1;   // ... whose largest border has at least this many rows (ELP_PACK_MINB, 300)
  int lanes = -1;       // workspace lanes a batch of 16+ frequencies is split over (ELP_LANES, 4)
};

struct Block {
  int type = 0;
  int material = 0;
  int64_t n_elements = 0;
  std::vector<int32_t> conn;
};

struct DeviceModel;   // device arrays, defined in device.cuh
struct Symbolic;      // host symbolic factorisation, symbolic.hpp
struct DeviceSymbolic;
struct Workspace;

struct Model {
  // ---- copied description
  int64_t n_nodes = 0;
  std::vector<int64_t> node_ids;
  std::vector<double> coords;
  std::vector<elp_material> materials;
  std::vector<std::vector<double>> E_tables, eta_tables;  // per material: the rows as given (f, value)
  std::vector<Block> blocks;
  std::vector<elp_interface_quad> interfaces;
  std::vector<elp_fixed_dof> fixed;
  std::vector<elp_nodal_force> forces;
  std::vector<elp_nodal_moment> moments;
  std::vector<elp_fluid_source> fluid_sources;
  std::vector<elp_vn_load> vn_loads;
  std::vector<elp_face_traction> face_tractions;

  // ---- numbering (analysis.cpp:475-520)
  std::vector<int32_t> order;        // node indices by ascending id
  std::vector<int32_t> global_rows;  // n_nodes x 21, -1 inactive
  int64_t n = 0;
  std::vector<int32_t> dof_node;     // node index of each dof
  std::vector<uint8_t> dof_kind;     // 0 structure, 1 fluid

  // ---- pattern (analysis.cpp:806-867)
  std::vector<int32_t> row_ptr;      // n + 1   (nnz < 2^31 checked)
  std::vector<int32_t> col_idx;      // nnz
  std::vector<uint8_t> cls;          // nnz
  std::vector<int32_t> diag_idx;     // n: CSR index of (i, i)
  int64_t nnz = 0;

  // ---- BC rows and right-hand side (analysis.cpp:171-279, 366-454)
  std::vector<int32_t> bc_rows;
  std::vector<cplx> bc_values;
  std::vector<uint8_t> is_bc_row;    // n
  std::vector<cplx> rhs;             // n: w-independent part
  std::vector<cplx> rhs_vn;          // n: G of F(w) = rhs + G / w (normal-velocity loads), 0 on BC rows
  bool has_vn = false;

  // ---- structure loss-factor groups
  std::vector<StructGroup> groups;   // groups[0] -> VK, groups[g>0] -> VKg[g-1]
  std::vector<int> material_group;   // per material, -1 for fluid

  // ---- a group of models solved together (elp_group): the member of each
  // row and the first row of each member (a member's rows are contiguous and
  // in its own order); empty for a single model
  std::vector<int32_t> row_model;
  std::vector<int64_t> member_row_off;  // n_members + 1
  std::vector<double> member_f;         // per member: ||F||^2, 2 Re<F, G>, ||G||^2 of F(w) = F + G / w
  int n_members = 1;

  Tuning tune;
  int assembly = 0;  // ELP_ASSEMBLY_FP64 or ELP_ASSEMBLY_DOUBLE_FLOAT

  int64_t n_elements_total = 0;
  bool assembled = false;
  bool analysed = false;

  std::unique_ptr<DeviceModel> dev;
  std::unique_ptr<Symbolic> sym;
  std::unique_ptr<DeviceSymbolic> dsym;
  std::unique_ptr<Workspace> ws[2];      // per precision
  std::unique_ptr<Workspace> ws_b[2][3];  // per precision: lanes 1..3 of a batch solved in parts at once

  Model();
  ~Model();
};

// host-side construction (model.cpp)
int build_model(const elp_model_desc* d, Model& m, std::string& err);

// coefficient of group g at angular frequency w
cplx group_coefficient(const StructGroup& g, double w);

// cell stresses of the solution x at w (stress.cu, on the device): 9 complex per element,
// elements in descriptor order; out2 (may be null) the lower plate surface
int cell_stresses(Model& m, double w, const cplx* x, cplx* out, cplx* out2, std::string& err);
// nodal stresses (stress.cu, on the device): 9 complex per node, nodes in ascending id
int node_stresses(Model& m, double w, const cplx* x, cplx* out, std::string& err);

// thread-local error text
void set_error(const std::string& s);
const std::string& get_error();

// Host-side fault injection (fault.cpp, elp_fault_inject): each returns true
// (or throws std::bad_alloc) exactly once, when its countdown runs out.
bool fault_device_alloc();
void fault_host_alloc_point();
bool fault_tc_wait();

}  // namespace elp

// the opaque handle of the C ABI
struct elp_model {
  elp::Model m;
};
