// Device-resident arrays of a model and shared CUDA helpers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "model.hpp"

namespace elp {

// An allocation failure maps to ELP_ERR_NOMEM (and clears the runtime's
// last error); every other runtime error to ELP_ERR_CUDA.
#define ELP_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      set_error(std::string("CUDA: ") + cudaGetErrorString(e_) + " at " __FILE__ ":" + std::to_string(__LINE__)); \
      if (e_ == cudaErrorMemoryAllocation) {                                      \
        cudaGetLastError();                                                       \
        return ELP_ERR_NOMEM;                                                     \
      }                                                                           \
      return ELP_ERR_CUDA;                                                        \
    }                                                                             \
  } while (0)


// Per-element material constants for the assembly kernel (real E: the
// loss factor is a per-w coefficient of the group's stiffness array).
struct ElemMaterial {
  double lam, mu;      // Brick8: Lame constants from E, nu (setupC)
  double rho;          // structure density / fluid density
  double Db, nu;       // DSG4: E t^3 / (12 (1 - nu^2)), nu
  double Gt, t;        // DSG4: E / (2 (1 + nu)) * t * 5/6 (setupCs), thickness
  double inv_c2;       // Fluid8: 1 / c^2
  double Es, nus;      // structure: E and nu (the stresses' C(w) and Cm(w))
  int group;           // structure loss-factor group
  int pad;
};

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) return cudaSuccess;
    if (fault_device_alloc()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  cudaError_t upload(const T* h, size_t count) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice);
  }
  cudaError_t upload(const std::vector<T>& v) { return upload(v.data(), v.size()); }
};

struct DeviceModel {
  int device = 0;
  DevBuf<double> coords;           // 3 N
  DevBuf<int32_t> row_ptr, col_idx, diag_idx;
  DevBuf<uint8_t> cls;
  DevBuf<double> VK, VM;           // nnz each
  DevBuf<double> VKg;              // (G - 1) x nnz extra structure groups
  DevBuf<double> rhs;              // 2 n
  DevBuf<double> rhs_vn;           // 2 n: G of F(w) = rhs + G / w (allocated when the model has such loads)
  DevBuf<int32_t> bc_rows;
  // element work lists
  DevBuf<int32_t> brick_conn, plate_conn, fluid_conn;   // 8 / 4 / 8 node indices
  DevBuf<int16_t> brick_mat, plate_mat, fluid_mat;      // index into materials
  DevBuf<int32_t> node_row_brick, node_row_plate, node_row_fluid;  // first row of the type's dofs
  DevBuf<ElemMaterial> materials;
  DevBuf<int32_t> iface_rows;      // per quad: 12 structure rows + 4 fluid rows
  DevBuf<double> iface_scale;      // per quad: -ori
  DevBuf<int32_t> iface_geom;      // per quad: 4 fluid node indices (geometry)
  DevBuf<int32_t> row_model;       // a group: each row's member
  DevBuf<int64_t> member_off;      // a group: first row of each member (n_members + 1)
  DevBuf<int> flags;               // [0] 3D non-positive detJ count, [1] 2D count
  int64_t bad_jacobians_3d = 0;    // flags[0] of the last assembly
  int64_t n_brick = 0, n_plate = 0, n_fluid = 0, n_iface = 0;
  double assembly_ms = 0.0;
  // the element lists are in locality order (lowest node first): per element
  // its position in descriptor order (blocks, then elements), and the host
  // copies of the Brick8 / Fluid8 connectivity the node lists are built from
  std::vector<int32_t> h_brick_eid, h_plate_eid, h_brick_conn, h_fluid_conn;
  // stresses (stress.cu), built on first use: descriptor positions, per node
  // its (element, kind * 8 + corner) entries, element count and output row
  bool stress_ready = false;
  DevBuf<int32_t> brick_eid, plate_eid, node_adj_el, node_count, node_seq;
  DevBuf<int64_t> node_adj_ptr;
  DevBuf<int8_t> node_adj_kc;
};

// assemble.cu
int device_upload_model(Model& m);
int device_assemble(Model& m, cudaStream_t stream, float* kernel_ms);

}  // namespace elp
