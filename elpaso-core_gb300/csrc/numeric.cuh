// Numeric multifrontal factorisation and solve: device structures.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "device.cuh"
#include "symbolic.hpp"

namespace elp {

constexpr int kMaxGroups = kMaxStructGroups;  // structure loss-factor groups supported per model
constexpr int kMaxSlots = 64;    // frequencies factorised together

// per-slot coefficients of the value arrays
struct Coef {
  double2 a[3];                  // CLS_STRUCT, CLS_FLUID, CLS_COUPLE coefficient of VK
  double b[3];                   // coefficient of VM
  double2 g[kMaxGroups];         // coefficient of VKg[g - 1] (g >= 1) on structure entries
  double inv_w;                  // 1 / w: weight of the normal-velocity loads in F(w)
  double fscale;                 // a group member's right-hand side is scaled by this (1 / ||F(w)||); 1 otherwise
};

// the w-independent value arrays of a model and the per-w combine
struct CombineArgs {
  const double* VK;
  const double* VM;
  const double* VKg;
  const uint8_t* cls;
  int64_t nnz;
  int ngroups;
  // a group of models (elp_group): each row's member; the coefficient table of
  // slot s and member k is coef[s * n_members + k]. Null for a single model.
  const int32_t* row_model;
  int n_members;
  // a group's GMRES steps: the (slot, member) pairs still iterating; rows of
  // the others are skipped by k_spmv and k_rhs (null: every row)
  const int* pact = nullptr;
};

CombineArgs combine_args(const Model& m);

#ifdef __CUDACC__
// the coefficients of slot s that apply to row i
__device__ __forceinline__ const Coef& row_coef(const CombineArgs& A, const Coef* __restrict__ coef, int s,
                                                int64_t i) {
  return A.row_model ? coef[(int64_t)s * A.n_members + A.row_model[i]] : coef[s];
}
__device__ __forceinline__ bool row_on(const CombineArgs& A, int s, int64_t i) {
  return !A.pact || A.pact[(int64_t)s * A.n_members + A.row_model[i]];
}

// A(w) at CSR entry q, Dirichlet rows included (MatZeroRows, diag = 1)
__device__ __forceinline__ double2 combine(const CombineArgs& A, const Coef& c, int64_t q) {
  const uint8_t k = A.cls[q] & CLS_MASK;
  if (k == CLS_BC_DIAG) return make_double2(1.0, 0.0);
  if (k == CLS_BC_OFF) return make_double2(0.0, 0.0);
  const double vk = A.VK[q], vm = A.VM[q];
  double2 v;
  v.x = c.a[k].x * vk + c.b[k] * vm;
  v.y = c.a[k].y * vk;
  if (k == CLS_STRUCT)
    for (int g = 1; g < A.ngroups; ++g) {
      double e = A.VKg[(int64_t)(g - 1) * A.nnz + q];
      v.x += c.g[g].x * e;
      v.y += c.g[g].y * e;
    }
  return v;
}

// Double-double accumulation for the FP64 residual r = f - A x. Near a
// resonance |A| |x| >> |f|, and a plain FP64 sum leaves ||f - A x|| / ||f||
// at a rounding floor near 1e-10; error-free transformations (products by
// FMA, sums by TwoSum) make the computed residual accurate to the last bits
// of the stored A and x instead.
struct DD {
  double hi, lo;
};
__device__ __forceinline__ void dd_add(DD& s, double b) {
  double t = s.hi + b;
  double bb = t - s.hi;
  double e = (s.hi - (t - bb)) + (b - bb);
  s.hi = t;
  s.lo += e;
}
__device__ __forceinline__ void dd_fma(DD& s, double a, double b) {  // s += a * b exactly (to dd)
  double p = a * b;
  double e = fma(a, b, -p);
  dd_add(s, p);
  s.lo += e;
}
__device__ __forceinline__ void dd_merge(DD& s, const DD& o) {
  dd_add(s, o.hi);
  s.lo += o.lo;
}
// warp-wide sum of a DD held per lane
__device__ __forceinline__ DD dd_warp_sum(DD v) {
  for (int o = 16; o; o >>= 1) {
    DD w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    dd_merge(v, w);
  }
  return v;
}
// FP64 row kernels give each CSR row kRowLanes lanes (rows hold ~10-40
// entries); FP64 instructions are scarce on this part, so a full warp and a
// five-level reduction per row would waste most of them.
constexpr int kRowLanes = 8;

// the kRowLanes-lane group of a row: sum over the group (xor shuffles stay inside it)
__device__ __forceinline__ double row_sum(double v) {
  for (int o = kRowLanes / 2; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ DD row_sum(DD v) {
  for (int o = kRowLanes / 2; o; o >>= 1) {
    DD w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    dd_merge(v, w);
  }
  return v;
}

// f - (a.hi + a.lo), rounded once
__device__ __forceinline__ double dd_residual(double f, const DD& a) {
  DD s{f, 0.0};
  dd_add(s, -a.hi);
  s.lo -= a.lo;
  return s.hi + s.lo;
}
#endif  // __CUDACC__

// How a workspace stores the fronts of a factorisation:
//  STORE_FULL    every front whole (sum of m^2 entries per frequency); the
//                solves read the factors in place;
//  STORE_COMPACT full fronts only while they are assembled and factorised, in
//                a pool whose regions later fronts reuse; each level's factors
//                (the m x p panel and U12) are then copied into a factor store
//                that the solves read (about 2/3 of the memory on the
//                plate-cavity model, at the price of that copy).
enum FrontStore { STORE_FULL = 0, STORE_COMPACT = 1 };

struct DeviceSymbolic {
  DevBuf<int32_t> f_p, f_b, f_parent, f_idx_off, f_map_off, f_cb_off, f_piv_off;
  DevBuf<int64_t> f_off;          // per front: offset of its full m x m front in the front pool
  DevBuf<int64_t> f_off_full;     // per front: offset when every front is kept whole
  DevBuf<int64_t> f_fac;          // per front: offset of its factors in the factor store
  DevBuf<int32_t> new_list;       // per level: fronts whose full front starts there (zeroed, scattered)
  DevBuf<int32_t> scatter_order;  // CSR entries by the start level of their owner front
  DevBuf<int32_t> entry_row;      // per CSR entry: its row
  DevBuf<int32_t> front_dofs, parent_map, child_ptr, child_list;
  DevBuf<int32_t> f_member;  // groups: the member each front belongs to (empty for one model)
  DevBuf<int64_t> entry_local;    // per CSR entry: offset inside its owner front
  DevBuf<int32_t> entry_owner;    // per CSR entry: its owner front
  DevBuf<int32_t> level_list;     // fronts grouped by level
  DevBuf<int32_t> ea_list;        // per (level, child slot): fronts to extend-add
  struct Level {
    int start = 0, count = 0;
    int max_p = 0, max_m = 0, max_b = 0;
    std::vector<int> ea_start, ea_count;   // per child slot
    int ea_max_b = 0;
    int64_t pack_bytes = 0;   // packed Schur operands of the level, per frequency slot
    int pack_blocks = 0;      // most packed blocks of one front of the level
    int schur_tiles = 0;      // most 128 x 128 Schur tiles of one front of the level
    int new_start = 0, new_count = 0;   // fronts starting at this level (in new_list)
    int64_t new_max_m2 = 0;             // their largest m^2
    int64_t ent_start = 0, ent_count = 0;  // their CSR entries (in scatter_order)
    int64_t fac_max = 0;                // largest p^2 + 2 p b of the level's fronts
  };
  std::vector<Level> levels;
  int n_fronts = 0;
  int64_t arena = 0, cb_total = 0;  // arena: entries of the front pool per frequency
  int64_t arena_full = 0;           // entries of every front whole (sum of m^2) per frequency
  int64_t fac = 0;                  // entries of the factor store per frequency
  int max_front = 0;
  DevBuf<int64_t> pack_base;      // per front: byte offset of its packed Schur operands within its level
  int64_t pack_max = 0;           // largest pack_bytes of a level that uses the packed Schur update
};

// Levels whose Schur update runs from packed operands (k_pack_schur + k_schur_tc);
// the others keep the converter kernel. pack_max_count(): fronts per level up
// to which a level is packed (ELP_PACK_COUNT, default 300); pack_min_border():
// the largest border of the level must reach this many rows (ELP_PACK_MINB,
// default 300).
int pack_max_count();
int pack_min_border();
// the model's tuning with its defaults resolved
Tuning resolved_tuning(const Model& m);
inline bool packed_schur_level(const DeviceSymbolic::Level& L, const Tuning& t) {
  return L.count <= t.pack_count && L.max_b >= t.pack_minb;
}

struct Workspace {
  int precision = 0;              // ELP_FP64_PLAIN / ELP_MIXED
  int store = STORE_FULL;         // FrontStore of the arena (and of fac)
  int64_t arena_stride = 0;       // complex entries of the arena per frequency slot
  const int64_t* foff = nullptr;  // device front offsets into the arena (f_off_full or f_off)
  int slots = 0;                  // capacity in frequencies
  size_t elem = 0;                // bytes of one complex front entry
  DevBuf<char> arena;             // slots x fronts: all whole (STORE_FULL) or the pool (STORE_COMPACT)
  DevBuf<char> fac;               // STORE_COMPACT: slots x factor store (L and U of every front)
  DevBuf<char> cb;                // slots x cb_total complex (solve contributions)
  DevBuf<char> z;                 // slots x n complex (solve vector, front precision)
  DevBuf<char> tb;                // slots x n complex (backward pivot-row buffer)
  DevBuf<char> gvec;              // slots x WorkspacePlan::gvec complex (global solve vectors), or empty
  DevBuf<int32_t> perm;           // slots x n local pivot rows
  DevBuf<double> dscale;          // slots x n symmetric diagonal scaling
  DevBuf<double2> x, r, f;        // slots x n FP64 solution, residual, rhs
  DevBuf<Coef> coef;              // slots
  DevBuf<double> norms;           // slots x 2 (||r||^2, ||f||^2)
  DevBuf<double> partial;         // reduction partials
  DevBuf<int> active;             // slots
  DevBuf<unsigned long long> stats;  // slots x 4: static pivots, max|u_jj| bits, min|u_jj| bits, max|a|
  DevBuf<int> tc_err;                // set when a tensor-core wait ran out
  DevBuf<int32_t> swapmap;           // per (front of a level, slot): a panel's row interchanges
  DevBuf<char> pack;                 // mixed path: packed TF32 split Schur operands of one level
  Coef* h_coef = nullptr;         // pinned host staging
  double* h_norms = nullptr;
  int* h_active = nullptr;
  unsigned long long* h_stats = nullptr;
  int* h_flag = nullptr;          // pinned: tc_err read back after the factorisation
  DevBuf<double> mnorms;          // a group: slots x members x (||r||^2, ||f||^2)
  double* h_mnorms = nullptr;     // pinned copy
  DevBuf<int> mdone;              // a group: slots x members, 1 when the member reached the tolerance
  // a group's GMRES, one process per (slot, member) pair: Hessenberg columns,
  // least-squares coefficients, scales, pair activity
  DevBuf<double2> ph1, ph2, phn, py;
  DevBuf<double> pscal;
  DevBuf<int> pact;
  double2* h_ph = nullptr;        // pinned: 3 x pairs x 32
  double2* h_py = nullptr;        // pinned: pairs x 32
  double* h_pscal = nullptr;      // pinned: pairs
  int* h_pact = nullptr;          // pinned: pairs
  int* h_mdone = nullptr;         // pinned copy
  double tol_member = 0.0;        // a group: the members' own tolerance (the group runs to a smaller one)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  int nparts = 0;
  // GMRES: basis (slots x (rst + 1) x n), work vectors, Hessenberg columns
  int rst = 0;
  DevBuf<double2> Vb, Zb, wv, hd1, hd2, hnd, ydev, dpart;
  DevBuf<double> scal;
  DevBuf<int> inner;
  double2* h_h = nullptr;         // pinned: 3 x slots x 32 (h1, h2, |w|^2)
  double2* h_y = nullptr;         // pinned: slots x 32
  double* h_scal = nullptr;       // pinned: slots
  int* h_inner = nullptr;         // pinned: slots
  int iters[kMaxSlots];           // preconditioner applications per slot
  ~Workspace();
};

// Sizes a workspace depends on, from the host symbolic phase alone.
struct WorkspacePlan {
  int64_t arena = 0, arena_full = 0, fac = 0, cb_total = 0, max_count = 1, pack_max = 0;  // arena: the pool
  // complex entries per frequency slot of the solve sweeps' global front
  // vectors, [0] FP64 plain, [1] FP32 mixed: levels whose front vector does
  // not fit shared memory keep it in global memory (solve_level_global)
  int64_t gvec[2] = {0, 0};
};
// Dynamic shared memory the solve sweeps may take per CTA (227 KB opt-in less
// 2,048 complex entries for the kernels' static buffers, which hold at most
// 1,152; solve_smem checks it against the compiled kernels), and whether a
// level with these largest front / pivot counts runs them on global buffers.
// ELP_SOLVE_GLOBAL=1 puts every level on global buffers (same arithmetic).
constexpr int64_t kSolveSmemOptin = 227 * 1024;
inline int64_t solve_smem_cap(int64_t elem) { return kSolveSmemOptin - 2048 * elem; }
bool solve_global_forced();
inline bool solve_level_global(int64_t max_m, int64_t max_p, int64_t elem) {
  return solve_global_forced() || (max_m + max_p) * elem > solve_smem_cap(elem);
}
WorkspacePlan workspace_plan(const Model& m);

int device_upload_symbolic(Model& m);
int workspace_ensure(Model& m, int precision, int slots, int lane, int store);
int64_t workspace_bytes(const Model& m, int precision, int slots, int store);
// The store a batch of `slots` frequencies uses when `budget` bytes are
// available for it: STORE_FULL when the whole batch fits that way (or
// ELP_FACTOR_STORE=full), else STORE_COMPACT (or ELP_FACTOR_STORE=compact).
int choose_store(const Model& m, int precision, int slots, int64_t budget);
int forced_store();  // ELP_FACTOR_STORE: STORE_FULL / STORE_COMPACT, or -1 (choose by memory)
// Device bytes of a model's resident arrays (pattern, value arrays, per-row
// data, element lists, symbolic maps), from host data alone.
int64_t model_array_bytes(const Model& m);
// Host part of the symbolic phase (ordering, tree, maps); no device work.
int model_symbolic_host(Model& m);
// One batch on workspace lane `lane` (0..3) of the model, on `stream` (the
// lane's own when null). Distinct lanes of one model may run on different
// host threads at the same time.
int numeric_solve_lane(Model& m, int precision, int lane, const double* omegas, int n_omega, const double2* f_dev,
                       double2* x_dev, elp_solve_info* info, double tol, cudaStream_t stream, int store);
// The FP64 solution vectors of a lane's last batch (slot s at + s * n).
const double2* lane_solution(const Model& m, int precision, int lane);
// A changed tuning drops what it invalidates (tune.cpp).
void apply_tuning(Model& m, const Tuning& t);
// The combined model of a group (group.cpp).
Model& group_model(elp_group* g);
// One front update kernel on caller-given FP32 complex fronts (elp_front_update_test).
int front_update_test(int kernel, int p, int b, int step, int slots, float* fronts, int parent_m,
                      const int32_t* pmap, float* parents);
// Device bytes held by the model's workspaces of one precision (all lanes):
// reusable by the next batch of that precision.
int64_t workspace_held(const Model& m, int precision);
// max_lanes: upper bound on the workspace lanes a batch is split over (1: one
// lane; callers that overlap several batches themselves, like the serving
// loop, pass 1).
int numeric_solve_batch(Model& m, int precision, const double* omegas, int n_omega,
                        const double2* f_dev, double2* x_dev, elp_solve_info* info, double tol,
                        cudaStream_t user_stream, int max_lanes, int store);
int numeric_system_values(Model& m, double omega, double2* out_dev);
void make_coef(const Model& m, double w, Coef& c);

}  // namespace elp
