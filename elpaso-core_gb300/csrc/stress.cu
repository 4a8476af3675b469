// Stresses after a solve, on the device: per cell (elp_cell_stresses) and per
// node (elp_node_stresses).
//
// Cell stresses (cAnalysis::computeStressesCells,
// analysis/analysis.cpp:869-905): every structure element evaluates its
// stress at the element centre from the solution of one frequency, nine
// complex slots per element (sigma 0..5; slots 6..8 are the fluid pressure
// gradients, zero here). Paths inside elpasoCore/source/:
//  - Brick8 (element/structure/linear/brick/elementstructurebrick.cpp:48-159):
//    B(6 x 24) from the shape-function derivatives at xi = eta = zeta = 0,
//    rows xx, yy, zz, (Ny, Nx), (Nz on u2, Ny on u3), (Nz on u1, Nx on u3);
//    stress = C(w) B u with the 3D constitutive matrix of the material at w;
//  - DSG4 / Mindlin (element/structure/linear/plate/elementstructuremindlin.cpp:51-175):
//    per node the values (w2, w1, w2) of the DOFs (x3, w1, w2), B rows
//    (Nx, 0, 0), (0, Ny, 0), (0, 0, Ny) at the centre, strains scaled to the
//    upper surface (t/2, -t/2, t) and to the lower one (-t/2, t/2, -t) (the
//    second vector), stress = Cm(w) strain in slots 0, 1, 3.
// C and Cm are linear in E_vis(w) (materialstructurevisco.cpp:284-372), so
// they are the real matrices of the material's modulus times its loss-factor
// group coefficient at w.
//
// Nodal stresses (cAnalysis::computeStressesNodes, analysis.cpp:907-935): 9
// complex per node, nodes in ascending id (the reference's GlobalSeqId,
// analysis.cpp:516). A Brick8 element adds its centre stress divided by the
// number of mesh elements of any type at the node (countElementsPerNode,
// analysis.cpp:455-469) to slots 0..5 of its nodes
// (elementstructurebrick.cpp:161-270); a Fluid8 element adds grad p,
// evaluated at each of its corners, to slots 6..8 of that node without
// averaging (elementfluid3d.cpp:380-557); plates add nothing (not
// implemented there). One thread per node gathers over the node's elements in
// a fixed order (no atomics), so the result does not change from run to run.
#include <algorithm>
#include <complex>
#include <string>
#include <vector>

#include "device.cuh"

namespace elp {

namespace {

// corner signs of the trilinear shape functions (cShapeHex8's node order) and
// of the bilinear quad
__constant__ double c_hs[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
__constant__ double c_qs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};

struct StressArgs {
  const double* coords;
  const double2* x;
  const int32_t *brick_conn, *plate_conn, *fluid_conn;
  const int16_t *brick_mat, *plate_mat;
  const int32_t *nr_brick, *nr_plate, *nr_fluid;
  const int32_t *brick_eid, *plate_eid;  // descriptor position of each (locality-ordered) element
  const ElemMaterial* mats;
  const double2* cw;  // per material: its loss-factor group coefficient at w
  int64_t n_brick, n_plate, n_nodes;
  int* flag;          // an element with a singular Jacobian
};

__device__ __forceinline__ double2 cx(double re, double im) { return make_double2(re, im); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cx(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return cx(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return cx(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cdivr(double2 a, double s) { return cx(a.x / s, a.y / s); }

__device__ __forceinline__ bool invert3(const double J[3][3], double I[3][3]) {
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  if (!(det != 0.0) || !isfinite(det)) return false;
  I[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  I[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  I[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  I[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  I[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  I[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  I[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  I[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  I[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  return true;
}

// Brick8 stress at the centre of element e (6 complex); false for a singular Jacobian
__device__ bool brick_centre_stress(const StressArgs& S, int64_t e, double2 sig[6]) {
  int v[8];
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, I[3][3];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = S.brick_conn[e * 8 + k];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) J[a][d] += 0.125 * c_hs[k][a] * S.coords[3 * (int64_t)v[k] + d];
  }
  if (!invert3(J, I)) return false;
  double2 eps[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) eps[i] = cx(0.0, 0.0);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    double dN[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      dN[d] = I[d][0] * 0.125 * c_hs[k][0] + I[d][1] * 0.125 * c_hs[k][1] + I[d][2] * 0.125 * c_hs[k][2];
    const int32_t r = S.nr_brick[v[k]];  // rows of u1, u2, u3 (consecutive) or -1
    const double2 u1 = r >= 0 ? S.x[r] : cx(0.0, 0.0), u2 = r >= 0 ? S.x[r + 1] : cx(0.0, 0.0),
                  u3 = r >= 0 ? S.x[r + 2] : cx(0.0, 0.0);
    eps[0] = cadd(eps[0], cscale(dN[0], u1));
    eps[1] = cadd(eps[1], cscale(dN[1], u2));
    eps[2] = cadd(eps[2], cscale(dN[2], u3));
    eps[3] = cadd(eps[3], cadd(cscale(dN[1], u1), cscale(dN[0], u2)));
    eps[4] = cadd(eps[4], cadd(cscale(dN[2], u2), cscale(dN[1], u3)));
    eps[5] = cadd(eps[5], cadd(cscale(dN[2], u1), cscale(dN[0], u3)));
  }
  const int mi = S.brick_mat[e];
  const ElemMaterial& mt = S.mats[mi];
  const double nu = mt.nus;
  const double2 Ew = cscale(mt.Es, S.cw[mi]);
  const double2 f = cdivr(Ew, (1.0 + nu) * (1.0 - 2.0 * nu));
  sig[0] = cmul(f, cadd(cadd(cscale(1.0 - nu, eps[0]), cscale(nu, eps[1])), cscale(nu, eps[2])));
  sig[1] = cmul(f, cadd(cadd(cscale(nu, eps[0]), cscale(1.0 - nu, eps[1])), cscale(nu, eps[2])));
  sig[2] = cmul(f, cadd(cadd(cscale(nu, eps[0]), cscale(nu, eps[1])), cscale(1.0 - nu, eps[2])));
  const double2 fs = cscale(0.5 * (1.0 - 2.0 * nu), f);
#pragma unroll
  for (int k = 3; k < 6; ++k) sig[k] = cmul(fs, eps[k]);
  return true;
}

// cell stresses of the Brick8 elements (out: descriptor order, 9 slots each)
__global__ void k_cell_brick(StressArgs S, double2* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < S.n_brick; e += (int64_t)gridDim.x * blockDim.x) {
    double2 sig[6];
    if (!brick_centre_stress(S, e, sig)) { atomicAdd(S.flag, 1); continue; }
    double2* o = out + (int64_t)S.brick_eid[e] * 9;
#pragma unroll
    for (int i = 0; i < 6; ++i) o[i] = sig[i];
  }
}

// the same centre stresses in element order, for the nodal averages
__global__ void k_brick_centre(StressArgs S, double2* __restrict__ tb) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < S.n_brick; e += (int64_t)gridDim.x * blockDim.x) {
    double2 sig[6];
    if (!brick_centre_stress(S, e, sig)) { atomicAdd(S.flag, 1); continue; }
#pragma unroll
    for (int i = 0; i < 6; ++i) tb[e * 6 + i] = sig[i];
  }
}

// DSG4 / Mindlin surface stresses (upper surface in out, lower in out2)
__global__ void k_cell_plate(StressArgs S, double2* __restrict__ out, double2* __restrict__ out2) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < S.n_plate; e += (int64_t)gridDim.x * blockDim.x) {
    int v[4];
    double J[2][2] = {{0, 0}, {0, 0}};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = S.plate_conn[e * 4 + k];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int d = 0; d < 2; ++d) J[a][d] += 0.25 * c_qs[k][a] * S.coords[3 * (int64_t)v[k] + d];
    }
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    if (!(det != 0.0) || !isfinite(det)) { atomicAdd(S.flag, 1); continue; }
    const double I00 = J[1][1] / det, I01 = -J[0][1] / det, I10 = -J[1][0] / det, I11 = J[0][0] / det;
    double2 st[3] = {cx(0.0, 0.0), cx(0.0, 0.0), cx(0.0, 0.0)};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double nx = I00 * 0.25 * c_qs[k][0] + I01 * 0.25 * c_qs[k][1];
      const double ny = I10 * 0.25 * c_qs[k][0] + I11 * 0.25 * c_qs[k][1];
      const int32_t r = S.nr_plate[v[k]];  // rows of x3, w1, w2 (consecutive) or -1
      const double2 w1 = r >= 0 ? S.x[r + 1] : cx(0.0, 0.0), w2 = r >= 0 ? S.x[r + 2] : cx(0.0, 0.0);
      st[0] = cadd(st[0], cscale(nx, w2));
      st[1] = cadd(st[1], cscale(ny, w1));
      st[2] = cadd(st[2], cscale(ny, w2));
    }
    const int mi = S.plate_mat[e];
    const ElemMaterial& mt = S.mats[mi];
    const double nu = mt.nus, t = mt.t;
    const double2 f = cdivr(cscale(mt.Es, S.cw[mi]), 1.0 - nu * nu);
    const double2 fs = cscale(0.5 * (1.0 - nu), f);
    double2* o = out + (int64_t)S.plate_eid[e] * 9;
    {
      const double2 e0 = cscale(0.5 * t, st[0]), e1 = cscale(-0.5 * t, st[1]), e2 = cscale(t, st[2]);
      o[0] = cmul(f, cadd(e0, cscale(nu, e1)));
      o[1] = cmul(f, cadd(cscale(nu, e0), e1));
      o[3] = cmul(fs, e2);
    }
    if (out2) {
      double2* o2 = out2 + (int64_t)S.plate_eid[e] * 9;
      const double2 e0 = cscale(-0.5 * t, st[0]), e1 = cscale(0.5 * t, st[1]), e2 = cscale(-t, st[2]);
      o2[0] = cmul(f, cadd(e0, cscale(nu, e1)));
      o2[1] = cmul(f, cadd(cscale(nu, e0), e1));
      o2[3] = cmul(fs, e2);
    }
  }
}

// Nodal stresses: node v (output row seq[v]) sums over its entries adj[ptr[v]
// .. ptr[v + 1]): entry = (element index, kind * 8 + corner), kind 0 Brick8
// (centre stress / count[v] into slots 0..5), kind 1 Fluid8 (grad p at the
// corner into slots 6..8).
__global__ void k_node_stress(StressArgs S, const int64_t* __restrict__ ptr, const int32_t* __restrict__ adj_el,
                              const int8_t* __restrict__ adj_kc, const int32_t* __restrict__ count,
                              const int32_t* __restrict__ seq, const double2* __restrict__ tb,
                              double2* __restrict__ out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < S.n_nodes; v += (int64_t)gridDim.x * blockDim.x) {
    double2 acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = cx(0.0, 0.0);
    const double inv_count = count[v] > 0 ? 1.0 / count[v] : 0.0;
    for (int64_t q = ptr[v]; q < ptr[v + 1]; ++q) {
      const int64_t e = adj_el[q];
      const int kc = adj_kc[q];
      if (kc < 8) {  // Brick8
#pragma unroll
        for (int i = 0; i < 6; ++i) acc[i] = cadd(acc[i], cscale(inv_count, tb[e * 6 + i]));
      } else {  // Fluid8, grad p at corner k
        const int k = kc - 8;
        double dN[8][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, I[3][3];
        double2 pv[8];
#pragma unroll
        for (int f = 0; f < 8; ++f) {
          const int32_t nf = S.fluid_conn[e * 8 + f];
          const int32_t r = S.nr_fluid[nf];
          pv[f] = r >= 0 ? S.x[r] : cx(0.0, 0.0);
          const double a = 1.0 + c_hs[f][0] * c_hs[k][0], b = 1.0 + c_hs[f][1] * c_hs[k][1],
                       c = 1.0 + c_hs[f][2] * c_hs[k][2];
          dN[f][0] = 0.125 * c_hs[f][0] * b * c;
          dN[f][1] = 0.125 * c_hs[f][1] * a * c;
          dN[f][2] = 0.125 * c_hs[f][2] * a * b;
#pragma unroll
          for (int qd = 0; qd < 3; ++qd)
#pragma unroll
            for (int d = 0; d < 3; ++d) J[qd][d] += dN[f][qd] * S.coords[3 * (int64_t)nf + d];
        }
        if (!invert3(J, I)) { atomicAdd(S.flag, 1); continue; }
        double2 g[3] = {cx(0.0, 0.0), cx(0.0, 0.0), cx(0.0, 0.0)};
#pragma unroll
        for (int f = 0; f < 8; ++f)
#pragma unroll
          for (int d = 0; d < 3; ++d)
            g[d] = cadd(g[d], cscale(I[d][0] * dN[f][0] + I[d][1] * dN[f][1] + I[d][2] * dN[f][2], pv[f]));
#pragma unroll
        for (int d = 0; d < 3; ++d) acc[6 + d] = cadd(acc[6 + d], g[d]);
      }
    }
    double2* o = out + (int64_t)seq[v] * 9;
#pragma unroll
    for (int i = 0; i < 9; ++i) o[i] = acc[i];
  }
}

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8192)); }

// per material: the coefficient of its loss-factor group at w (1 without one)
std::vector<double2> material_coefficients(const Model& m, double w) {
  std::vector<double2> cw(m.materials.size());
  for (size_t i = 0; i < m.materials.size(); ++i) {
    const int g = m.material_group[i];
    const cplx c = g >= 0 ? group_coefficient(m.groups[g], w) : cplx(1.0, 0.0);
    cw[i] = make_double2(c.real(), c.imag());
  }
  return cw;
}

// the device model (uploaded on first use) and the stress index arrays: the
// descriptor position of each element, the node-to-element lists, the element
// count per node and each node's output row
int stress_prepare(Model& m) {
  int rc = ELP_OK;
  if (!m.dev) {
    rc = device_upload_model(m);
    if (rc) {
      m.dev.reset();
      return rc;
    }
  }
  DeviceModel& D = *m.dev;
  if (D.stress_ready) return ELP_OK;
  const int64_t N = m.n_nodes;
  std::vector<int64_t> ptr(N + 1, 0);
  std::vector<int32_t> count(N, 0), seq(N);
  for (int64_t r = 0; r < N; ++r) seq[m.order[r]] = (int32_t)r;
  for (const Block& blk : m.blocks) {
    const int npe = nodes_per_element(blk.type);
    for (int64_t e = 0; e < blk.n_elements; ++e)
      for (int k = 0; k < npe; ++k) count[blk.conn[(size_t)e * npe + k]]++;
  }
  for (int64_t e = 0; e < D.n_brick; ++e)
    for (int k = 0; k < 8; ++k) ptr[D.h_brick_conn[e * 8 + k] + 1]++;
  for (int64_t e = 0; e < D.n_fluid; ++e)
    for (int k = 0; k < 8; ++k) ptr[D.h_fluid_conn[e * 8 + k] + 1]++;
  for (int64_t v = 0; v < N; ++v) ptr[v + 1] += ptr[v];
  std::vector<int32_t> adj_el(ptr[N]);
  std::vector<int8_t> adj_kc(ptr[N]);
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (int64_t e = 0; e < D.n_brick; ++e)  // per node: its Brick8 elements, then its Fluid8 elements
    for (int k = 0; k < 8; ++k) {
      const int64_t q = fill[D.h_brick_conn[e * 8 + k]]++;
      adj_el[q] = (int32_t)e;
      adj_kc[q] = (int8_t)k;
    }
  for (int64_t e = 0; e < D.n_fluid; ++e)
    for (int k = 0; k < 8; ++k) {
      const int64_t q = fill[D.h_fluid_conn[e * 8 + k]]++;
      adj_el[q] = (int32_t)e;
      adj_kc[q] = (int8_t)(8 + k);
    }
  ELP_CUDA(D.brick_eid.upload(D.h_brick_eid));
  ELP_CUDA(D.plate_eid.upload(D.h_plate_eid));
  ELP_CUDA(D.node_adj_ptr.upload(ptr));
  ELP_CUDA(D.node_adj_el.upload(adj_el));
  ELP_CUDA(D.node_adj_kc.upload(adj_kc));
  ELP_CUDA(D.node_count.upload(count));
  ELP_CUDA(D.node_seq.upload(seq));
  D.stress_ready = true;
  return ELP_OK;
}

StressArgs stress_args(const Model& m, const double2* x, const double2* cw, int* flag) {
  const DeviceModel& D = *m.dev;
  StressArgs S;
  S.coords = D.coords.p;
  S.x = x;
  S.brick_conn = D.brick_conn.p;
  S.plate_conn = D.plate_conn.p;
  S.fluid_conn = D.fluid_conn.p;
  S.brick_mat = D.brick_mat.p;
  S.plate_mat = D.plate_mat.p;
  S.nr_brick = D.node_row_brick.p;
  S.nr_plate = D.node_row_plate.p;
  S.nr_fluid = D.node_row_fluid.p;
  S.brick_eid = D.brick_eid.p;
  S.plate_eid = D.plate_eid.p;
  S.mats = D.materials.p;
  S.cw = cw;
  S.n_brick = D.n_brick;
  S.n_plate = D.n_plate;
  S.n_nodes = m.n_nodes;
  S.flag = flag;
  return S;
}

}  // namespace

int cell_stresses(Model& m, double w, const cplx* x, cplx* out, cplx* out2, std::string& err) {
  int rc = stress_prepare(m);
  if (rc) {
    err = get_error();
    return rc;
  }
  const DeviceModel& D = *m.dev;
  const int64_t ne = m.n_elements_total;
  const std::vector<double2> cwh = material_coefficients(m, w);
  DevBuf<double2> xd, cw, o1, o2;
  DevBuf<int> flag;
  ELP_CUDA(xd.alloc((size_t)std::max<int64_t>(1, m.n)));
  ELP_CUDA(cw.upload(cwh));
  ELP_CUDA(o1.alloc((size_t)std::max<int64_t>(1, ne) * 9));
  if (out2) ELP_CUDA(o2.alloc((size_t)std::max<int64_t>(1, ne) * 9));
  ELP_CUDA(flag.alloc(1));
  ELP_CUDA(cudaMemcpy(xd.p, x, sizeof(double2) * m.n, cudaMemcpyHostToDevice));
  ELP_CUDA(cudaMemset(o1.p, 0, sizeof(double2) * ne * 9));
  if (out2) ELP_CUDA(cudaMemset(o2.p, 0, sizeof(double2) * ne * 9));
  ELP_CUDA(cudaMemset(flag.p, 0, sizeof(int)));
  const StressArgs S = stress_args(m, xd.p, cw.p, flag.p);
  if (D.n_brick > 0) k_cell_brick<<<grid_for(D.n_brick), 256>>>(S, o1.p);
  if (D.n_plate > 0) k_cell_plate<<<grid_for(D.n_plate), 256>>>(S, o1.p, out2 ? o2.p : nullptr);
  ELP_CUDA(cudaGetLastError());
  int h_flag = 0;
  ELP_CUDA(cudaMemcpy(&h_flag, flag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h_flag) {
    err = "element with a singular Jacobian at its centre";
    return ELP_ERR_ARG;
  }
  ELP_CUDA(cudaMemcpy(out, o1.p, sizeof(double2) * ne * 9, cudaMemcpyDeviceToHost));
  if (out2) ELP_CUDA(cudaMemcpy(out2, o2.p, sizeof(double2) * ne * 9, cudaMemcpyDeviceToHost));
  return ELP_OK;
}

int node_stresses(Model& m, double w, const cplx* x, cplx* out, std::string& err) {
  int rc = stress_prepare(m);
  if (rc) {
    err = get_error();
    return rc;
  }
  const DeviceModel& D = *m.dev;
  const int64_t N = m.n_nodes;
  const std::vector<double2> cwh = material_coefficients(m, w);
  DevBuf<double2> xd, cw, tb, o;
  DevBuf<int> flag;
  ELP_CUDA(xd.alloc((size_t)std::max<int64_t>(1, m.n)));
  ELP_CUDA(cw.upload(cwh));
  ELP_CUDA(tb.alloc((size_t)std::max<int64_t>(1, D.n_brick) * 6));
  ELP_CUDA(o.alloc((size_t)std::max<int64_t>(1, N) * 9));
  ELP_CUDA(flag.alloc(1));
  ELP_CUDA(cudaMemcpy(xd.p, x, sizeof(double2) * m.n, cudaMemcpyHostToDevice));
  ELP_CUDA(cudaMemset(flag.p, 0, sizeof(int)));
  const StressArgs S = stress_args(m, xd.p, cw.p, flag.p);
  if (D.n_brick > 0) k_brick_centre<<<grid_for(D.n_brick), 256>>>(S, tb.p);
  if (N > 0)
    k_node_stress<<<grid_for(N), 256>>>(S, D.node_adj_ptr.p, D.node_adj_el.p, D.node_adj_kc.p, D.node_count.p,
                                       D.node_seq.p, tb.p, o.p);
  ELP_CUDA(cudaGetLastError());
  int h_flag = 0;
  ELP_CUDA(cudaMemcpy(&h_flag, flag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h_flag) {
    err = "element with a singular Jacobian";
    return ELP_ERR_ARG;
  }
  ELP_CUDA(cudaMemcpy(out, o.p, sizeof(double2) * N * 9, cudaMemcpyDeviceToHost));
  return ELP_OK;
}

}  // namespace elp
