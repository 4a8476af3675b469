// K1: one persistent launch that integrates every element of every type and
// scatters K, M (structure), K_f / rho, M_f / rho (fluid) and the coupling
// (-ori)(C + C^T) into w-independent CSR value arrays.
//
// The reference integrates K - w^2 M per element at every frequency
// (analysis/frequency/analysisfrequencybasic.cpp:281-304). Every term of
// A(w) is a fixed w-dependent multiple of one of these arrays, so the
// integration runs once per model and the per-w work becomes an HBM-bound
// combine (numeric.cu).
//
// Element arithmetic follows (paths inside elpasoCore/source/):
//  Brick8  element/structure/linear/brick/elementstructurebrick.cpp:281-554
//          (B(6x24) with engineering shear rows xy, yz, xz; C from
//          material/.../materialstructureisotrop.cpp:130-148), written in the
//          closed form K_ab = lam P + mu P^T + mu tr(P) I,
//          P = sum_gp wdJ grad N_a grad N_b^T (same quantity, fewer flops);
//  DSG4    element/structure/linear/plate/elementstructuremindlindsg4.cpp:37-211
//          (bending Bb, DSG shear Bs, tau = 1/(1 + 0.12 hk^2 / t^2) with hk
//          the longest of edges 0-1, 1-2, 2-3 -- edge 3-0 is not measured),
//          mass elementstructuremindlin.cpp:299-366;
//  Fluid8  element/fluid/elementfluid3d.cpp:54-167 (M carries 1/c^2),
//          divided by rho as in element/fluid/elementfluid.cpp:58-77;
//  InterfaceMindlin element/interface/elementinterfacemindlin.cpp:80-181,
//          scaled by -ori into C and C^T (elementinterfacestructural.cpp:209-237).
// Shape tables and the 15-digit Gauss constants follow shape/shapefunctions.cpp,
// shape/shapehex8.cpp:49-90, shape/shapequad4.cpp:48-73, misc/gausspoints.h:27-43;
// 3D Gauss points are numbered x fastest, 2D points y fastest
// (misc/gausspoints.cpp:76-87, 165-195).
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "device.cuh"
#include "prof.cuh"

namespace elp {

// ---------------------------------------------------------------- tables
__constant__ double c_hex[4][8][8];    // [fun, xi, eta, zeta][node][gp]
__constant__ double c_quad[3][4][4];   // [fun, xi, eta][node][gp]
__constant__ unsigned char c_pair_a[36], c_pair_b[36];
// the same tables split into FP32 pairs (hi + lo = the FP64 value to ~2^-48):
// shape derivatives [xi, eta, zeta][node][gp] and node-pair products
// N_a N_b [pair][gp], for the double-float contractions below
__constant__ float2 c_hexd[3][8][8];
__constant__ float2 c_mass[36][8];
__constant__ double c_massd[36][8];  // N_a N_b [pair][gp] in FP64

// ---------------------------------------------------------------- double-float
// Opt-in (ELP_ASSEMBLY_DOUBLE_FLOAT): the Brick8 / Fluid8 contractions
// (gradients J^-T grad N and the node-pair sums P_ab = sum_gp w g_a g_b^T) in
// FP32 pairs. FP64 executes at about 1/64 of the FP32 rate on this part, and
// these sums are most of the assembly's FP64 work. A value is hi + lo (two
// floats); a product keeps the FMA error of hi * hi plus the two cross terms
// (relative error ~2^-46), a sum adds the high parts error-free (two-sum) and
// collects every error in lo. Results are formed in FP64 as hi + lo; against
// the FP64 sums they differ by ~1e-14 of the sum of the magnitudes of their
// terms. J, det J and J^-1 stay FP64.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_split(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ void df_acc(DF& s, DF x) {
  const float t = s.h + x.h;
  const float bb = t - s.h;
  const float err = (s.h - (t - bb)) + (x.h - bb);
  s.h = t;
  s.l += err + x.l;
}
__device__ __forceinline__ double df_value(DF s) { return (double)s.h + (double)s.l; }
__device__ __forceinline__ DF df_of(float2 v) { return {v.x, v.y}; }

static const double kGp2 = 0.577350269189626;  // misc/gausspoints.h gp4[1]

static double lagrange_hex8(int k, int deriv, const double g[3]) {
  static const int sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
  static const int sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
  static const int sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  double fx = 1. + sx[k] * g[0], fy = 1. + sy[k] * g[1], fz = 1. + sz[k] * g[2];
  switch (deriv) {
    case 0: return fx * fy * fz * 0.125;
    case 1: return sx[k] * fy * fz * 0.125;
    case 2: return sy[k] * fx * fz * 0.125;
    default: return sz[k] * fx * fy * 0.125;
  }
}
static double lagrange_quad4(int k, int deriv, const double g[2]) {
  static const int sx[4] = {-1, 1, 1, -1};
  static const int sy[4] = {-1, -1, 1, 1};
  double fx = 1. + sx[k] * g[0], fy = 1. + sy[k] * g[1];
  switch (deriv) {
    case 0: return 0.25 * fx * fy;
    case 1: return 0.25 * sx[k] * fy;
    default: return 0.25 * sy[k] * fx;
  }
}

void shape_tables(double hex[4][8][8], double quad[3][4][4]) {
  const double pts[2] = {kGp2, -kGp2};
  for (int n = 0; n < 8; ++n) {
    // gausspoints.cpp:76-87: x fastest
    int x = n % 2, y = (n / 2) % 2, z = n / 4;
    double g[3] = {pts[x], pts[y], pts[z]};
    for (int k = 0; k < 8; ++k)
      for (int dv = 0; dv < 4; ++dv) hex[dv][k][n] = lagrange_hex8(k, dv, g);
  }
  for (int n = 0; n < 4; ++n) {
    // gausspoints.cpp:165-195: y fastest
    int y = n % 2, x = n / 2;
    double g[2] = {pts[x], pts[y]};
    for (int k = 0; k < 4; ++k)
      for (int dv = 0; dv < 3; ++dv) quad[dv][k][n] = lagrange_quad4(k, dv, g);
  }
}

// ---------------------------------------------------------------- helpers
// CSR index of (row, col); the pattern guarantees presence.
__device__ __forceinline__ int find_col(const int32_t* __restrict__ row_ptr,
                                        const int32_t* __restrict__ col_idx, int row, int col) {
  int lo = row_ptr[row], hi = row_ptr[row + 1];
  while (hi - lo > 8) {
    int mid = (lo + hi) >> 1;
    if (__ldg(col_idx + mid) <= col) lo = mid; else hi = mid;
  }
  for (int p = lo; p < hi; ++p)
    if (__ldg(col_idx + p) == col) return p;
  return -1;
}

// CSR index of (row0 + i, col) given p0 = index of (row0, col): the rows of one
// node usually share their column list, so the same offset is tried first
// (one load) before a search.
__device__ __forceinline__ int sibling_col(const int32_t* __restrict__ row_ptr,
                                           const int32_t* __restrict__ col_idx, int row0, int p0, int i, int col) {
  if (p0 < 0) return find_col(row_ptr, col_idx, row0 + i, col);
  const int lo = __ldg(row_ptr + row0 + i), hi = __ldg(row_ptr + row0 + i + 1);
  const int p = lo + (p0 - __ldg(row_ptr + row0));
  if (p < hi && __ldg(col_idx + p) == col) return p;
  return find_col(row_ptr, col_idx, row0 + i, col);
}

__device__ __forceinline__ void add_at(double* v, int p, double x) {
  if (p >= 0 && x != 0.0) atomicAdd(v + p, x);
}

struct AsmArgs {
  const double* coords;
  const int32_t *row_ptr, *col_idx;
  double *VK, *VM, *VKg;
  int64_t nnz;
  const int32_t *brick_conn, *plate_conn, *fluid_conn;
  const int16_t *brick_mat, *plate_mat, *fluid_mat;
  const int32_t *nr_brick, *nr_plate, *nr_fluid;
  const ElemMaterial* mats;
  const int32_t* iface_rows;
  const double* iface_scale;
  const int32_t* iface_geom;
  int64_t n_brick, n_plate, n_fluid, n_iface;
  int64_t items_brick, items_fluid, items_plate, items_iface;
  int* flags;
};

constexpr int kThreads = 288;   // 8 hexes x 36 node pairs
constexpr int kHexPerItem = 8;

// 3D Jacobian, determinant and inverse exactly as elementfem.cpp:158-210.
__device__ __forceinline__ double jac3(const double* x, int gp, double inv[3][3]) {
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double d = c_hex[i + 1][k][gp];
      J[i][0] += d * x[3 * k + 0];
      J[i][1] += d * x[3 * k + 1];
      J[i][2] += d * x[3 * k + 2];
    }
  }
  double det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
               J[0][2] * J[1][0] * J[2][1] - J[0][2] * J[1][1] * J[2][0] -
               J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2];
  const double id = 1.0 / det;  // one FP64 division instead of nine
  inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  inv[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * id;
  inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  inv[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
  inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  inv[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * id;
  inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  inv[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * id;
  inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

// ---------------------------------------------------------------- hex items
// Arithmetic of the Brick8 / Fluid8 contractions: FP64 (the default, the
// drop-in) or double-float (elp_model_set_assembly). Shared-memory values are
// 8 bytes in both: a double, or a float pair hi + lo.
template <bool kDF>
struct HexArith;
template <>
struct HexArith<false> {
  using V = double;
  __device__ static V zero() { return 0.0; }
  __device__ static V of(double s) { return s; }
  __device__ static double store(V v) { return v; }
  __device__ static V split(double x) { return x; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static void fma(V& s, V a, V b) { s = ::fma(a, b, s); }
  __device__ static double value(V v) { return v; }
  __device__ static V dshape(int dv, int k, int gp) { return c_hex[dv + 1][k][gp]; }
  __device__ static V mass(int pr, int gp) { return c_massd[pr][gp]; }
};
template <>
struct HexArith<true> {
  using V = DF;
  __device__ static V zero() { return {0.f, 0.f}; }
  __device__ static V of(double s) { return {__int_as_float(__double2loint(s)), __int_as_float(__double2hiint(s))}; }
  __device__ static double store(V v) { return __hiloint2double(__float_as_int(v.l), __float_as_int(v.h)); }
  __device__ static V split(double x) { return df_split(x); }
  __device__ static V mul(V a, V b) { return df_mul(a, b); }
  __device__ static void fma(V& s, V a, V b) { df_acc(s, df_mul(a, b)); }
  __device__ static double value(V v) { return df_value(v); }
  __device__ static V dshape(int dv, int k, int gp) { return df_of(c_hexd[dv][k][gp]); }
  __device__ static V mass(int pr, int gp) { return df_of(c_mass[pr][gp]); }
};

// kind 0 = Brick8, 1 = Fluid8. Per item of 8 elements: 64 threads form
// J, det J and J^-1 (FP64) at one Gauss point each and store g_k = J^-T grad N_k
// and w g_k for the 8 nodes; then one thread per node pair (a <= b) sums
// P_ab = sum_gp (w g_a) g_b^T (and the mass term) and adds the 3 x 3 block
// (and its transpose) into the CSR value arrays.
template <int kKind, bool kDF>
__device__ void hex_item(const AsmArgs& A, int64_t item, double (*sg)[8][8][3], double (*swg)[8][8][3],
                         double (*sw)[8], int (*srow)[8], int* smat) {
  using H = HexArith<kDF>;
  using V = typename H::V;
  const int t = threadIdx.x;
  const int64_t e0 = item * kHexPerItem;
  const int64_t ne = kKind == 0 ? A.n_brick : A.n_fluid;
  const int32_t* conn = kKind == 0 ? A.brick_conn : A.fluid_conn;
  if (t < 64) {
    int el = t >> 3, gp = t & 7;
    int64_t e = e0 + el;
    if (e < ne) {
      double x[24];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        int v = __ldg(conn + e * 8 + k);
        x[3 * k + 0] = __ldg(A.coords + 3 * (int64_t)v + 0);
        x[3 * k + 1] = __ldg(A.coords + 3 * (int64_t)v + 1);
        x[3 * k + 2] = __ldg(A.coords + 3 * (int64_t)v + 2);
      }
      double inv[3][3];
      double det = jac3(x, gp, inv);
      if (det <= 0.0) atomicAdd(A.flags + 0, 1);
      V iv[3][3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int j = 0; j < 3; ++j) iv[d][j] = H::split(inv[d][j]);
      const V w = H::split(det);  // level-2 weights are 1 x 1 x 1
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const V a = H::dshape(0, k, gp), b = H::dshape(1, k, gp), c = H::dshape(2, k, gp);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          V g = H::mul(iv[d][0], a);
          H::fma(g, iv[d][1], b);
          H::fma(g, iv[d][2], c);
          sg[el][gp][k][d] = H::store(g);
          swg[el][gp][k][d] = H::store(H::mul(w, g));
        }
      }
      sw[el][gp] = H::store(w);
    }
  } else if (t < 128) {
    int el = (t - 64) >> 3, k = (t - 64) & 7;
    int64_t e = e0 + el;
    if (e < ne) {
      int v = __ldg(conn + e * 8 + k);
      srow[el][k] = kKind == 0 ? __ldg(A.nr_brick + v) : __ldg(A.nr_fluid + v);
      if (k == 0) smat[el] = kKind == 0 ? A.brick_mat[e] : A.fluid_mat[e];
    }
  }
  __syncthreads();
  if (t < kHexPerItem * 36) {
    int el = t / 36, pr = t % 36;
    int64_t e = e0 + el;
    if (e < ne) {
      const int a = c_pair_a[pr], b = c_pair_b[pr];
      const ElemMaterial& mt = A.mats[smat[el]];
      const int ra = srow[el][a], rb = srow[el][b];
      if (kKind == 0) {
        V Pv[3][3], mv_ = H::zero();
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) Pv[i][j] = H::zero();
#pragma unroll
        for (int gp = 0; gp < 8; ++gp) {
          V wa[3], gb[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            wa[d] = H::of(swg[el][gp][a][d]);
            gb[d] = H::of(sg[el][gp][b][d]);
          }
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) H::fma(Pv[i][j], wa[i], gb[j]);
          H::fma(mv_, H::of(sw[el][gp]), H::mass(pr, gp));
        }
        double P[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) P[i][j] = H::value(Pv[i][j]);
        const double mm = H::value(mv_);
        const double tr = P[0][0] + P[1][1] + P[2][2];
        double Kb[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) Kb[i][j] = mt.lam * P[i][j] + mt.mu * P[j][i] + (i == j ? mt.mu * tr : 0.0);
        const double mv = mt.rho * mm;
        double* VKt = mt.group == 0 ? A.VK : A.VKg + (int64_t)(mt.group - 1) * A.nnz;
        const int pa0 = find_col(A.row_ptr, A.col_idx, ra, rb);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          int p = i == 0 ? pa0 : sibling_col(A.row_ptr, A.col_idx, ra, pa0, i, rb);
#pragma unroll
          for (int j = 0; j < 3; ++j) add_at(VKt, p + j, Kb[i][j]);
          add_at(A.VM, p + i, mv);
        }
        if (a != b) {
          const int pb0 = find_col(A.row_ptr, A.col_idx, rb, ra);
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            int p = j == 0 ? pb0 : sibling_col(A.row_ptr, A.col_idx, rb, pb0, j, ra);
#pragma unroll
            for (int i = 0; i < 3; ++i) add_at(VKt, p + i, Kb[i][j]);
            add_at(A.VM, p + j, mv);
          }
        }
      } else {
        V kv = H::zero(), mv_ = H::zero();
#pragma unroll
        for (int gp = 0; gp < 8; ++gp) {
#pragma unroll
          for (int d = 0; d < 3; ++d) H::fma(kv, H::of(swg[el][gp][a][d]), H::of(sg[el][gp][b][d]));
          H::fma(mv_, H::of(sw[el][gp]), H::mass(pr, gp));
        }
        const double kk = H::value(kv), mm = mt.inv_c2 * H::value(mv_);
        const double ir = 1.0 / mt.rho;
        int p = find_col(A.row_ptr, A.col_idx, ra, rb);
        add_at(A.VK, p, kk * ir);
        add_at(A.VM, p, mm * ir);
        if (a != b) {
          p = find_col(A.row_ptr, A.col_idx, rb, ra);
          add_at(A.VK, p, kk * ir);
          add_at(A.VM, p, mm * ir);
        }
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- DSG4 plate
// 28 plates per CTA item: 112 threads form one Gauss point each (J, det J,
// dN/dx, dN/dy and the DSG shear rows Bs), then one thread per node pair
// (a <= b, 10 per plate) sums its 3 x 3 block of K = sum_gp (Bb^T Cb Bb +
// tau Cs Bs^T Bs) w det J and the mass term, and adds the block (and its
// transpose) into the CSR value arrays.
constexpr int kPlatesPerItem = 28;  // x 10 node pairs = 280 of the 288 threads
__constant__ unsigned char c_qpair_a[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
__constant__ unsigned char c_qpair_b[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};

struct PlateShared {
  double dx[kPlatesPerItem][4][4], dy[kPlatesPerItem][4][4];  // [plate][gp][node] dN/dx, dN/dy
  double bs[kPlatesPerItem][4][2][12];                          // [plate][gp] DSG shear rows, / det J
  double wd[kPlatesPerItem][4];                                 // w det J (weights 1 x 1)
  double cst[kPlatesPerItem][6];                                // Cb00, Cb01, Cb22, tau Cs, m1, m2
  int row[kPlatesPerItem][4];
  int grp[kPlatesPerItem];
};

__device__ void plate_item(const AsmArgs& A, int64_t item, PlateShared& ps) {
  const int t = threadIdx.x;
  const int64_t e0 = item * kPlatesPerItem;
  if (t < kPlatesPerItem * 4) {
    const int el = t >> 2, n = t & 3;
    const int64_t e = e0 + el;
    if (e < A.n_plate) {
      double x[4], y[4], z[4];
      int vv[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int v = __ldg(A.plate_conn + e * 4 + k);
        vv[k] = v;
        x[k] = A.coords[3 * (int64_t)v + 0];
        y[k] = A.coords[3 * (int64_t)v + 1];
        z[k] = A.coords[3 * (int64_t)v + 2];
      }
      double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        J00 += c_quad[1][k][n] * x[k];
        J01 += c_quad[1][k][n] * y[k];
        J10 += c_quad[2][k][n] * x[k];
        J11 += c_quad[2][k][n] * y[k];
      }
      const double det = J00 * J11 - J01 * J10;
      if (det <= 0.0) atomicAdd(A.flags + 1, 1);
      const double a = J00, b = J01, d = J10, c = J11;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ps.dx[el][n][k] = (c * c_quad[1][k][n] - b * c_quad[2][k][n]) / det;
        ps.dy[el][n][k] = (-d * c_quad[1][k][n] + a * c_quad[2][k][n]) / det;
      }
      // DSG shear strains of the edge-based interpolation (elementstructuremindlindsg4.cpp),
      // each row entry / det J stored as it is formed
      const double Nx1 = c_quad[1][1][n], Nx2 = c_quad[1][2][n];
      const double Ne2 = c_quad[2][2][n], Ne3 = c_quad[2][3][n];
      const double idet = 1. / det;
      double (*bs)[12] = ps.bs[el][n];
      bs[0][0] = (-c * Nx1 + b * Ne3) * idet;
      bs[0][1] = (-b * c * Nx1 + b * c * Ne3) * idet;
      bs[0][2] = (a * c * Nx1 - b * d * Ne3) * idet;
      bs[1][0] = (d * Nx1 - a * Ne3) * idet;
      bs[1][1] = (-a * c * Ne3 + b * d * Nx1) * idet;
      bs[1][2] = (a * d * Ne3 - a * d * Nx1) * idet;
      bs[0][3] = (c * Nx1 + b * Ne2) * idet;
      bs[0][4] = (-b * c * Nx1 + b * c * Ne2) * idet;
      bs[0][5] = (a * c * Nx1 - b * d * Ne2) * idet;
      bs[1][3] = (-a * Ne2 - d * Nx1) * idet;
      bs[1][4] = (-a * c * Ne2 + b * d * Nx1) * idet;
      bs[1][5] = (a * d * Ne2 - a * d * Nx1) * idet;
      bs[0][6] = (c * Nx2 - b * Ne2) * idet;
      bs[0][7] = (-b * c * Nx2 + b * c * Ne2) * idet;
      bs[0][8] = (a * c * Nx2 - b * d * Ne2) * idet;
      bs[1][6] = (a * Ne2 - d * Nx2) * idet;
      bs[1][7] = (-a * c * Ne2 + b * d * Nx2) * idet;
      bs[1][8] = (a * d * Ne2 - a * d * Nx2) * idet;
      bs[0][9] = (-c * Nx2 - b * Ne3) * idet;
      bs[0][10] = (-b * c * Nx2 + b * c * Ne3) * idet;
      bs[0][11] = (a * c * Nx2 - b * d * Ne3) * idet;
      bs[1][9] = (a * Ne3 + d * Nx2) * idet;
      bs[1][10] = (-a * c * Ne3 + b * d * Nx2) * idet;
      bs[1][11] = (a * d * Ne3 - a * d * Nx2) * idet;
      ps.wd[el][n] = 1.0 * det;
      if (n == 0) {
        const ElemMaterial& mt = A.mats[A.plate_mat[e]];
        const double thick = mt.t;
        // Lyly-Stenberg: hk = max edge over the pairs (1,0), (2,1), (3,2)
        double hk = 0.0;
        const int seq[5] = {0, 1, 2, 3, 0};
#pragma unroll
        for (int i = 1; i < 4; ++i) {
          const int p = seq[i], q = seq[i - 1];
          const double ex = x[p] - x[q], ey = y[p] - y[q], ez = z[p] - z[q];
          const double dd = sqrt(ex * ex + ey * ey + ez * ez);
          hk = hk > dd ? hk : dd;
        }
        const double tau = 1.0 / (1.0 + 0.12 * hk * hk / (thick * thick));
        ps.cst[el][0] = mt.Db;           // E t^3 / (12 (1 - nu^2))
        ps.cst[el][1] = mt.Db * mt.nu;
        ps.cst[el][2] = mt.Gt;           // G t^3 / 12
        ps.cst[el][3] = mt.lam * tau;    // lam holds G t Ks for plates
        ps.cst[el][4] = mt.rho * thick;
        ps.cst[el][5] = mt.rho * (thick * thick * thick / 12.0);
        ps.grp[el] = mt.group;
#pragma unroll
        for (int k = 0; k < 4; ++k) ps.row[el][k] = A.nr_plate[vv[k]];
      }
    }
  }
  __syncthreads();
  if (t < kPlatesPerItem * 10) {
    const int el = t / 10, pr = t % 10;
    const int64_t e = e0 + el;
    if (e < A.n_plate) {
      const int a = c_qpair_a[pr], b = c_qpair_b[pr];
      const double Cb00 = ps.cst[el][0], Cb01 = ps.cst[el][1], Cb22 = ps.cst[el][2], Cs = ps.cst[el][3];
      double Kb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, mab = 0.0;
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const double wdJ = ps.wd[el][n];
        // bending rows of the nodes' columns (w, theta_x, theta_y): Bb[r][3k + i]
        const double xa = ps.dx[el][n][a], ya = ps.dy[el][n][a], xb = ps.dx[el][n][b], yb = ps.dy[el][n][b];
        const double Ba[3][3] = {{0.0, 0.0, xa}, {0.0, -ya, 0.0}, {0.0, -xa, ya}};
        const double Bn[3][3] = {{0.0, 0.0, xb}, {0.0, -yb, 0.0}, {0.0, -xb, yb}};
        double CB[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          CB[0][j] = Cb00 * Bn[0][j] + Cb01 * Bn[1][j];
          CB[1][j] = Cb01 * Bn[0][j] + Cb00 * Bn[1][j];
          CB[2][j] = Cb22 * Bn[2][j];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            if (a == b && j < i) continue;  // diagonal block: upper triangle, mirrored below
            double s = Ba[0][i] * CB[0][j] + Ba[1][i] * CB[1][j] + Ba[2][i] * CB[2][j];
            s += Cs * (ps.bs[el][n][0][3 * a + i] * ps.bs[el][n][0][3 * b + j] +
                       ps.bs[el][n][1][3 * a + i] * ps.bs[el][n][1][3 * b + j]);
            Kb[i][j] += s * wdJ;
          }
        mab += c_quad[0][a][n] * c_quad[0][b][n] * wdJ;
      }
      if (a == b) {
        Kb[1][0] = Kb[0][1];
        Kb[2][0] = Kb[0][2];
        Kb[2][1] = Kb[1][2];
      }
      const double m1 = ps.cst[el][4], m2 = ps.cst[el][5];
      const int g = ps.grp[el];
      double* VKt = g == 0 ? A.VK : A.VKg + (int64_t)(g - 1) * A.nnz;
      const int ra = ps.row[el][a], rb = ps.row[el][b];
      // rows (node a, dof i), columns (node b, dof j); the mass couples equal dofs
      const int pa0 = find_col(A.row_ptr, A.col_idx, ra, rb);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int p = i == 0 ? pa0 : sibling_col(A.row_ptr, A.col_idx, ra, pa0, i, rb);
#pragma unroll
        for (int j = 0; j < 3; ++j) add_at(VKt, p + j, Kb[i][j]);
        add_at(A.VM, p + i, mab * (i == 0 ? m1 : m2));
      }
      if (a != b) {
        const int pb0 = find_col(A.row_ptr, A.col_idx, rb, ra);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int p = j == 0 ? pb0 : sibling_col(A.row_ptr, A.col_idx, rb, pb0, j, ra);
#pragma unroll
          for (int i = 0; i < 3; ++i) add_at(VKt, p + i, Kb[i][j]);
          add_at(A.VM, p + j, mab * (j == 0 ? m1 : m2));
        }
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- interface
__device__ void interface_quad(const AsmArgs& A, int64_t q) {
  double x[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int v = A.iface_geom[q * 4 + k];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) x[k][dd] = A.coords[3 * (int64_t)v + dd];
  }
  double C[4][4];  // C(3z+2, s)
#pragma unroll
  for (int zz = 0; zz < 4; ++zz)
#pragma unroll
    for (int ss = 0; ss < 4; ++ss) C[zz][ss] = 0.0;
  for (int n = 0; n < 4; ++n) {
    double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        a1[dd] += c_quad[1][k][n] * x[k][dd];
        a2[dd] += c_quad[2][k][n] * x[k][dd];
      }
    double n1 = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
    double n2 = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
    double d12 = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
    double det = sqrt(n1 * n2 - d12 * d12);
#pragma unroll
    for (int zz = 0; zz < 4; ++zz)
#pragma unroll
      for (int ss = 0; ss < 4; ++ss) C[zz][ss] += c_quad[0][zz][n] * c_quad[0][ss][n] * 1.0 * det;
  }
  const int32_t* rows = A.iface_rows + q * 16;  // 12 structure rows then 4 fluid rows
  const double sc = A.iface_scale[q];
  // shell transformation (elementinterfacemindlin.cpp:131-181) when the
  // structure node carries x1: rows 3n, 3n+1 get normal components.
  double Cf[12][4];
  const bool transform = rows[0] >= 0;
#pragma unroll
  for (int zz = 0; zz < 4; ++zz)
#pragma unroll
    for (int ss = 0; ss < 4; ++ss) { Cf[3 * zz][ss] = 0.0; Cf[3 * zz + 1][ss] = 0.0; Cf[3 * zz + 2][ss] = C[zz][ss]; }
  if (transform) {
    const double xi[4] = {-1., 1., 1., -1.}, et[4] = {-1., -1., 1., 1.};
    for (int nn = 0; nn < 4; ++nn) {
      double g[2] = {xi[nn], et[nn]};
      double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
      const int sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
      for (int k = 0; k < 4; ++k) {
        double nxi = 0.25 * sx[k] * (1. + sy[k] * g[1]);
        double net = 0.25 * sy[k] * (1. + sx[k] * g[0]);
        for (int dd = 0; dd < 3; ++dd) { a1[dd] += nxi * x[k][dd]; a2[dd] += net * x[k][dd]; }
      }
      double nv[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
      double nrm = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
      for (int dd = 0; dd < 3; ++dd) nv[dd] *= 1. / nrm;
      for (int ss = 0; ss < 4; ++ss) {
        double cz = Cf[3 * nn + 2][ss];
        Cf[3 * nn][ss] = nv[0] * cz;
        Cf[3 * nn + 1][ss] = nv[1] * cz;
        Cf[3 * nn + 2][ss] = nv[2] * cz;
      }
    }
  }
  for (int zi = 0; zi < 12; ++zi) {
    const int r = rows[zi];
    if (r < 0) continue;
    for (int ss = 0; ss < 4; ++ss) {
      const int f = rows[12 + ss];
      if (f < 0) continue;
      const double v = sc * Cf[zi][ss];
      add_at(A.VK, find_col(A.row_ptr, A.col_idx, r, f), v);
      add_at(A.VK, find_col(A.row_ptr, A.col_idx, f, r), v);
    }
  }
}

// ---------------------------------------------------------------- kernel
// Brick8 / Fluid8 items (8 elements per CTA); register-light, so three CTAs
// share an SM.
// The element integration of every element type in ONE persistent launch:
// items are Brick8 groups, Fluid8 groups (8 elements each, hex_item), DSG4
// groups (28 plates each, plate_item) and interface quads (one per thread),
// in that order; a CTA takes items blockIdx.x, blockIdx.x + gridDim.x, ...,
// so its items of one kind come before those of the next and the shared
// memory of the hex and plate items (a union) is never live in both at once
// (each item ends with a barrier).
struct HexShared {
  double sg[kHexPerItem][8][8][3];
  double swg[kHexPerItem][8][8][3];
  double sw[kHexPerItem][8];
  int srow[kHexPerItem][8];
  int smat[kHexPerItem];
};
union AsmShared {
  HexShared hex;
  PlateShared plate;
};

template <bool kDF>
__global__ void __launch_bounds__(kThreads, 3) assemble_kernel(AsmArgs A) {
  __shared__ AsmShared sh;
  const int64_t i_fluid = A.items_brick, i_plate = i_fluid + A.items_fluid, i_iface = i_plate + A.items_plate;
  const int64_t total = i_iface + A.items_iface;
  for (int64_t it = blockIdx.x; it < total; it += gridDim.x) {
    if (it < i_fluid) {
      hex_item<0, kDF>(A, it, sh.hex.sg, sh.hex.swg, sh.hex.sw, sh.hex.srow, sh.hex.smat);
    } else if (it < i_plate) {
      hex_item<1, kDF>(A, it - i_fluid, sh.hex.sg, sh.hex.swg, sh.hex.sw, sh.hex.srow, sh.hex.smat);
    } else if (it < i_iface) {
      plate_item(A, it - i_plate, sh.plate);
    } else {
      const int64_t q = (it - i_iface) * kThreads + threadIdx.x;
      if (q < A.n_iface) interface_quad(A, q);
    }
  }
}

// ---------------------------------------------------------------- host
static bool g_tables_done[64] = {false};

static int upload_tables(int dev) {
  if (dev < 0 || dev >= 64) return ELP_OK;
  if (g_tables_done[dev]) return ELP_OK;
  double hex[4][8][8], quad[3][4][4];
  shape_tables(hex, quad);
  unsigned char pa[36], pb[36];
  int k = 0;
  for (int a = 0; a < 8; ++a)
    for (int b = a; b < 8; ++b) { pa[k] = (unsigned char)a; pb[k] = (unsigned char)b; ++k; }
  ELP_CUDA(cudaMemcpyToSymbol(c_hex, hex, sizeof(hex)));
  ELP_CUDA(cudaMemcpyToSymbol(c_quad, quad, sizeof(quad)));
  ELP_CUDA(cudaMemcpyToSymbol(c_pair_a, pa, sizeof(pa)));
  ELP_CUDA(cudaMemcpyToSymbol(c_pair_b, pb, sizeof(pb)));
  auto split = [](double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
  };
  float2 hd[3][8][8], ms[36][8];
  for (int dv = 0; dv < 3; ++dv)
    for (int n = 0; n < 8; ++n)
      for (int g = 0; g < 8; ++g) hd[dv][n][g] = split(hex[dv + 1][n][g]);
  for (int q = 0; q < 36; ++q)
    for (int g = 0; g < 8; ++g) ms[q][g] = split(hex[0][pa[q]][g] * hex[0][pb[q]][g]);
  ELP_CUDA(cudaMemcpyToSymbol(c_hexd, hd, sizeof(hd)));
  ELP_CUDA(cudaMemcpyToSymbol(c_mass, ms, sizeof(ms)));
  double md[36][8];
  for (int q = 0; q < 36; ++q)
    for (int g = 0; g < 8; ++g) md[q][g] = hex[0][pa[q]][g] * hex[0][pb[q]][g];
  ELP_CUDA(cudaMemcpyToSymbol(c_massd, md, sizeof(md)));
  g_tables_done[dev] = true;
  return ELP_OK;
}

int device_upload_model(Model& m) {
  if (!m.dev) m.dev.reset(new DeviceModel());
  DeviceModel& D = *m.dev;
  ELP_CUDA(cudaGetDevice(&D.device));
  int rc = upload_tables(D.device);
  if (rc) return rc;
  ELP_CUDA(D.coords.upload(m.coords));
  ELP_CUDA(D.row_ptr.upload(m.row_ptr));
  ELP_CUDA(D.col_idx.upload(m.col_idx));
  ELP_CUDA(D.diag_idx.upload(m.diag_idx));
  ELP_CUDA(D.cls.upload(m.cls));
  if (m.n_members > 1) {
    ELP_CUDA(D.row_model.upload(m.row_model));
    ELP_CUDA(D.member_off.upload(m.member_row_off));
  }
  std::vector<double> rhs(2 * m.n);
  for (int64_t i = 0; i < m.n; ++i) { rhs[2 * i] = m.rhs[i].real(); rhs[2 * i + 1] = m.rhs[i].imag(); }
  ELP_CUDA(D.rhs.upload(rhs));
  if (m.has_vn) {
    for (int64_t i = 0; i < m.n; ++i) { rhs[2 * i] = m.rhs_vn[i].real(); rhs[2 * i + 1] = m.rhs_vn[i].imag(); }
    ELP_CUDA(D.rhs_vn.upload(rhs));
  }
  ELP_CUDA(D.bc_rows.upload(m.bc_rows));
  // element lists per type
  std::vector<int32_t> bc, pc, fc, be, pe, fe;  // connectivity, descriptor positions
  std::vector<int16_t> bm, pm, fm;
  int64_t eid = 0;
  for (auto& blk : m.blocks) {
    std::vector<int32_t>* c = blk.type == ELP_BRICK8 ? &bc : blk.type == ELP_DSG4 ? &pc : &fc;
    std::vector<int16_t>* mm = blk.type == ELP_BRICK8 ? &bm : blk.type == ELP_DSG4 ? &pm : &fm;
    std::vector<int32_t>* ee = blk.type == ELP_BRICK8 ? &be : blk.type == ELP_DSG4 ? &pe : &fe;
    c->insert(c->end(), blk.conn.begin(), blk.conn.end());
    mm->insert(mm->end(), blk.n_elements, (int16_t)blk.material);
    for (int64_t e = 0; e < blk.n_elements; ++e) ee->push_back((int32_t)(eid + e));
    eid += blk.n_elements;
  }
  if (m.materials.size() > 32767) { set_error("too many materials"); return ELP_ERR_ARG; }
  // Each element kind is launched in order of its lowest node (a stable
  // counting sort): the CTAs in flight then add into a narrow band of CSR
  // rows that stays in L2 until its last element. Block by block order
  // sweeps the whole matrix once per material block (four times over on a
  // cube with four randomly assigned materials).
  auto locality_sort = [&](std::vector<int32_t>& conn, std::vector<int16_t>& mat, std::vector<int32_t>& pos,
                           int per) {
    const size_t ne = mat.size();
    if (ne < 2) return;
    std::vector<int64_t> start((size_t)m.n_nodes + 1, 0);
    std::vector<int32_t> key(ne);
    for (size_t e = 0; e < ne; ++e) {
      int32_t k = conn[e * per];
      for (int a = 1; a < per; ++a) k = std::min(k, conn[e * per + a]);
      key[e] = k;
      ++start[(size_t)k + 1];
    }
    for (int64_t v = 0; v < m.n_nodes; ++v) start[v + 1] += start[v];
    std::vector<int32_t> c2(conn.size()), p2(ne);
    std::vector<int16_t> m2(ne);
    for (size_t e = 0; e < ne; ++e) {
      const int64_t d = start[key[e]]++;
      std::copy(conn.begin() + e * per, conn.begin() + (e + 1) * per, c2.begin() + d * per);
      m2[d] = mat[e];
      p2[d] = pos[e];
    }
    conn.swap(c2);
    mat.swap(m2);
    pos.swap(p2);
  };
  locality_sort(bc, bm, be, 8);
  locality_sort(pc, pm, pe, 4);
  locality_sort(fc, fm, fe, 8);
  D.h_brick_eid = be;
  D.h_plate_eid = pe;
  D.h_brick_conn = bc;
  D.h_fluid_conn = fc;
  D.stress_ready = false;
  D.n_brick = (int64_t)bm.size();
  D.n_plate = (int64_t)pm.size();
  D.n_fluid = (int64_t)fm.size();
  ELP_CUDA(D.brick_conn.upload(bc));
  ELP_CUDA(D.plate_conn.upload(pc));
  ELP_CUDA(D.fluid_conn.upload(fc));
  ELP_CUDA(D.brick_mat.upload(bm));
  ELP_CUDA(D.plate_mat.upload(pm));
  ELP_CUDA(D.fluid_mat.upload(fm));
  std::vector<int32_t> nb(m.n_nodes, -1), np(m.n_nodes, -1), nf(m.n_nodes, -1);
  for (int64_t v = 0; v < m.n_nodes; ++v) {
    const int32_t* g = &m.global_rows[(size_t)v * ELP_NUM_KNOWN_DOFS];
    nb[v] = g[ELP_DOF_X1];
    np[v] = g[ELP_DOF_X3];
    nf[v] = g[ELP_DOF_FLUID];
  }
  ELP_CUDA(D.node_row_brick.upload(nb));
  ELP_CUDA(D.node_row_plate.upload(np));
  ELP_CUDA(D.node_row_fluid.upload(nf));
  std::vector<ElemMaterial> em(m.materials.size());
  for (size_t i = 0; i < m.materials.size(); ++i) {
    const elp_material& mt = m.materials[i];
    ElemMaterial& e = em[i];
    memset(&e, 0, sizeof(e));
    e.rho = mt.rho;
    e.Es = mt.E;
    e.nus = mt.nu;
    e.group = m.material_group[i] < 0 ? 0 : m.material_group[i];
    if (mt.kind == ELP_AF_LIN_UAF_ISO_DIR) {
      e.inv_c2 = 1.0 / (mt.c * mt.c);
    } else {
      // Lame constants of setupC with real E (the group coefficient carries eta)
      double f = mt.E / (1.0 + mt.nu) / (1.0 - 2.0 * mt.nu);
      e.mu = f * (1.0 - 2.0 * mt.nu) / 2.0;
      double diag = f * (1. - mt.nu);
      e.lam = diag - 2.0 * e.mu;
      // plate constants (setupCb / setupCs): lam slot reused for G t Ks
      bool plate_material = false;
      for (auto& blk : m.blocks)
        if (blk.material == (int)i && blk.type == ELP_DSG4) plate_material = true;
      if (plate_material) {
        double h = mt.t;
        e.Db = mt.E * h * h * h / (12. * (1. - mt.nu * mt.nu));
        double G = mt.E / (2. * (1. + mt.nu));
        e.Gt = G * h * h * h / 12.;
        e.lam = mt.E / (2. * (1. + mt.nu)) * h * (5. / 6.);
        e.nu = mt.nu;
        e.t = h;
        for (auto& blk : m.blocks)
          if (blk.material == (int)i && blk.type == ELP_BRICK8) {
            set_error("a material used by both Brick8 and DSG4 blocks is not supported");
            return ELP_ERR_ARG;
          }
      }
    }
  }
  ELP_CUDA(D.materials.upload(em));
  // interfaces
  D.n_iface = (int64_t)m.interfaces.size();
  std::vector<int32_t> ir(16 * D.n_iface), ig(4 * D.n_iface);
  std::vector<double> isc(D.n_iface);
  for (int64_t q = 0; q < D.n_iface; ++q) {
    const elp_interface_quad& Q = m.interfaces[q];
    for (int k = 0; k < 4; ++k) {
      for (int d3 = 0; d3 < 3; ++d3)
        ir[16 * q + 3 * k + d3] = m.global_rows[(size_t)Q.structure_nodes[k] * ELP_NUM_KNOWN_DOFS + d3];
      ir[16 * q + 12 + k] = m.global_rows[(size_t)Q.fluid_nodes[k] * ELP_NUM_KNOWN_DOFS + ELP_DOF_FLUID];
      ig[4 * q + k] = Q.fluid_nodes[k];
    }
    // transformC is applied when the first structure node has x1 active
    if (m.global_rows[(size_t)Q.structure_nodes[0] * ELP_NUM_KNOWN_DOFS + ELP_DOF_X1] < 0)
      for (int k = 0; k < 4; ++k) { ir[16 * q + 3 * k] = -1; ir[16 * q + 3 * k + 1] = -1; }
    isc[q] = -1.0 * Q.ori;
  }
  ELP_CUDA(D.iface_rows.upload(ir));
  ELP_CUDA(D.iface_geom.upload(ig));
  ELP_CUDA(D.iface_scale.upload(isc));
  ELP_CUDA(D.VK.alloc(m.nnz));
  ELP_CUDA(D.VM.alloc(m.nnz));
  if (m.groups.size() > 1) ELP_CUDA(D.VKg.alloc((m.groups.size() - 1) * (size_t)m.nnz));
  ELP_CUDA(D.flags.alloc(4));
  return ELP_OK;
}

int device_assemble(Model& m, cudaStream_t stream, float* kernel_ms) {
  DeviceModel& D = *m.dev;
  ELP_CUDA(cudaMemsetAsync(D.VK.p, 0, sizeof(double) * m.nnz, stream));
  ELP_CUDA(cudaMemsetAsync(D.VM.p, 0, sizeof(double) * m.nnz, stream));
  if (D.VKg.p) ELP_CUDA(cudaMemsetAsync(D.VKg.p, 0, sizeof(double) * D.VKg.n, stream));
  ELP_CUDA(cudaMemsetAsync(D.flags.p, 0, sizeof(int) * 4, stream));
  AsmArgs A;
  A.coords = D.coords.p;
  A.row_ptr = D.row_ptr.p;
  A.col_idx = D.col_idx.p;
  A.VK = D.VK.p;
  A.VM = D.VM.p;
  A.VKg = D.VKg.p;
  A.nnz = m.nnz;
  A.brick_conn = D.brick_conn.p;
  A.plate_conn = D.plate_conn.p;
  A.fluid_conn = D.fluid_conn.p;
  A.brick_mat = D.brick_mat.p;
  A.plate_mat = D.plate_mat.p;
  A.fluid_mat = D.fluid_mat.p;
  A.nr_brick = D.node_row_brick.p;
  A.nr_plate = D.node_row_plate.p;
  A.nr_fluid = D.node_row_fluid.p;
  A.mats = D.materials.p;
  A.iface_rows = D.iface_rows.p;
  A.iface_scale = D.iface_scale.p;
  A.iface_geom = D.iface_geom.p;
  A.n_brick = D.n_brick;
  A.n_plate = D.n_plate;
  A.n_fluid = D.n_fluid;
  A.n_iface = D.n_iface;
  A.items_brick = (D.n_brick + kHexPerItem - 1) / kHexPerItem;
  A.items_fluid = (D.n_fluid + kHexPerItem - 1) / kHexPerItem;
  A.items_plate = (D.n_plate + kPlatesPerItem - 1) / kPlatesPerItem;
  A.items_iface = (D.n_iface + kThreads - 1) / kThreads;
  A.flags = D.flags.p;
  int sms = 0, per_sm = 0;
  ELP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D.device));
  const bool df = m.assembly == ELP_ASSEMBLY_DOUBLE_FLOAT;
  auto kernel = df ? assemble_kernel<true> : assemble_kernel<false>;
  ELP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0));
  // one persistent launch: one resident wave over the items of every element type
  const int64_t items = A.items_brick + A.items_fluid + A.items_plate + A.items_iface;
  const int64_t grid = std::min<int64_t>((int64_t)sms * std::max(1, per_sm), items);
  cudaEvent_t e0, e1;
  ELP_CUDA(cudaEventCreate(&e0));
  ELP_CUDA(cudaEventCreate(&e1));
  ELP_CUDA(cudaEventRecord(e0, stream));
  if (grid > 0) PROF_LAUNCH(KC_ASSEMBLE, stream, kernel<<<(unsigned)grid, kThreads, 0, stream>>>(A));
  ELP_CUDA(cudaGetLastError());
  ELP_CUDA(cudaEventRecord(e1, stream));
  ELP_CUDA(cudaEventSynchronize(e1));
  prof_resolve();
  float ms = 0.f;
  ELP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (kernel_ms) *kernel_ms = ms;
  D.assembly_ms = ms;
  int flags[4];
  ELP_CUDA(cudaMemcpy(flags, D.flags.p, sizeof(flags), cudaMemcpyDeviceToHost));
  // Brick8 / Fluid8: the reference reports det J <= 0 and goes on
  // (elementfem.cpp:183-188, its throw commented out); DSG4: it throws (:97-100)
  D.bad_jacobians_3d = flags[0];
  if (flags[1] > 0) {
    set_error("detJac <= 0 in a DSG4 element: check orientation of the elements");
    return ELP_ERR_GEOMETRY;
  }
  return ELP_OK;
}

}  // namespace elp
