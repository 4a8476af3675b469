// Stresses after a solve: per cell (below) and per node (node_stresses, at
// the end of the file).
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
// they are the real matrices of the assembly modulus times the material's
// loss-factor group coefficient at w.
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "model.hpp"

namespace elp {

namespace {

// derivatives of the trilinear shape functions at the centre: +-1/8 by corner
// (node k at (xi, eta, zeta) = (sx, sy, sz) of cShapeHex8's node order)
const double kHexS[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                            {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
const double kQuadS[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};

bool invert3(const double J[3][3], double I[3][3]) {
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  if (!(det != 0.0) || !std::isfinite(det)) return false;
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

}  // namespace

// Brick8 stress at the element centre (6 complex), false for a singular Jacobian
static bool brick_centre_stress(const Model& m, const int32_t* en, cplx Ew, double nu, const cplx* x, cplx* sig) {
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, I[3][3];
  for (int k = 0; k < 8; ++k)
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) J[a][d] += 0.125 * kHexS[k][a] * m.coords[3 * (size_t)en[k] + d];
  if (!invert3(J, I)) return false;
  auto u = [&](int32_t node, int dof) -> cplx {
    const int32_t r = m.global_rows[(size_t)node * ELP_NUM_KNOWN_DOFS + dof];
    return r >= 0 ? x[r] : cplx(0.0, 0.0);
  };
  cplx eps[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < 8; ++k) {
    double dN[3];
    for (int d = 0; d < 3; ++d)
      dN[d] = I[d][0] * 0.125 * kHexS[k][0] + I[d][1] * 0.125 * kHexS[k][1] + I[d][2] * 0.125 * kHexS[k][2];
    const cplx u1 = u(en[k], ELP_DOF_X1), u2 = u(en[k], ELP_DOF_X2), u3 = u(en[k], ELP_DOF_X3);
    eps[0] += dN[0] * u1;
    eps[1] += dN[1] * u2;
    eps[2] += dN[2] * u3;
    eps[3] += dN[1] * u1 + dN[0] * u2;
    eps[4] += dN[2] * u2 + dN[1] * u3;
    eps[5] += dN[2] * u1 + dN[0] * u3;
  }
  const cplx f = Ew / ((1.0 + nu) * (1.0 - 2.0 * nu));
  sig[0] = f * ((1.0 - nu) * eps[0] + nu * eps[1] + nu * eps[2]);
  sig[1] = f * (nu * eps[0] + (1.0 - nu) * eps[1] + nu * eps[2]);
  sig[2] = f * (nu * eps[0] + nu * eps[1] + (1.0 - nu) * eps[2]);
  for (int k = 3; k < 6; ++k) sig[k] = f * (0.5 * (1.0 - 2.0 * nu)) * eps[k];
  return true;
}

static cplx material_modulus(const Model& m, int material, double w) {
  const int g = m.material_group[material];
  return m.materials[material].E * (g >= 0 ? group_coefficient(m.groups[g], w) : cplx(1.0, 0.0));
}

int cell_stresses(const Model& m, double w, const cplx* x, cplx* out, cplx* out2, std::string& err) {
  int64_t base = 0;
  for (const Block& blk : m.blocks) {
    const int64_t ne = blk.n_elements;
    const elp_material& mt = m.materials[blk.material];
    const cplx Ew = material_modulus(m, blk.material, w);
    const double nu = mt.nu;
    bool bad = false;
#pragma omp parallel for schedule(static) reduction(|| : bad)
    for (int64_t e = 0; e < ne; ++e) {
      cplx* s1 = out + (base + e) * 9;
      cplx* s2 = out2 ? out2 + (base + e) * 9 : nullptr;
      for (int k = 0; k < 9; ++k) {
        s1[k] = 0.0;
        if (s2) s2[k] = 0.0;
      }
      const int32_t* en = &blk.conn[(size_t)e * nodes_per_element(blk.type)];
      auto u = [&](int32_t node, int dof) -> cplx {
        const int32_t r = m.global_rows[(size_t)node * ELP_NUM_KNOWN_DOFS + dof];
        return r >= 0 ? x[r] : cplx(0.0, 0.0);
      };
      if (blk.type == ELP_BRICK8) {
        if (!brick_centre_stress(m, en, Ew, nu, x, s1)) { bad = true; continue; }
      } else if (blk.type == ELP_DSG4) {
        double J[2][2] = {{0, 0}, {0, 0}};
        for (int k = 0; k < 4; ++k)
          for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 2; ++d) J[a][d] += 0.25 * kQuadS[k][a] * m.coords[3 * (size_t)en[k] + d];
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        if (!(det != 0.0) || !std::isfinite(det)) { bad = true; continue; }
        const double I[2][2] = {{J[1][1] / det, -J[0][1] / det}, {-J[1][0] / det, J[0][0] / det}};
        cplx st[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k) {
          const double nx = I[0][0] * 0.25 * kQuadS[k][0] + I[0][1] * 0.25 * kQuadS[k][1];
          const double ny = I[1][0] * 0.25 * kQuadS[k][0] + I[1][1] * 0.25 * kQuadS[k][1];
          const cplx w1 = u(en[k], ELP_DOF_W1), w2 = u(en[k], ELP_DOF_W2);
          st[0] += nx * w2;
          st[1] += ny * w1;
          st[2] += ny * w2;
        }
        const double t = mt.t;
        const cplx f = Ew / (1.0 - nu * nu);
        auto plane = [&](cplx e0, cplx e1, cplx e2, cplx* s) {
          s[0] = f * (e0 + nu * e1);
          s[1] = f * (nu * e0 + e1);
          s[3] = f * (0.5 * (1.0 - nu)) * e2;
        };
        plane(0.5 * t * st[0], -0.5 * t * st[1], t * st[2], s1);
        if (s2) plane(-0.5 * t * st[0], 0.5 * t * st[1], -t * st[2], s2);
      }
    }
    if (bad) { err = "element with a singular Jacobian at its centre"; return ELP_ERR_ARG; }
    base += ne;
  }
  return ELP_OK;
}

// Nodal stresses (cAnalysis::computeStressesNodes, analysis.cpp:907-935): 9
// complex per node, nodes in ascending id (the reference's GlobalSeqId,
// analysis.cpp:516). A Brick8 element adds its centre stress divided by the
// number of mesh elements of any type at the node (countElementsPerNode,
// analysis.cpp:455-469) to slots 0..5 of its nodes
// (elementstructurebrick.cpp:161-270); a Fluid8 element adds grad p, evaluated
// at each of its corners, to slots 6..8 of that node without averaging
// (elementfluid3d.cpp:380-557); plates add nothing (not implemented there).
int node_stresses(const Model& m, double w, const cplx* x, cplx* out, std::string& err) {
  const int64_t N = m.n_nodes;
  std::vector<int32_t> seq(N), count(N, 0);
  for (int64_t r = 0; r < N; ++r) seq[m.order[r]] = (int32_t)r;
  for (const Block& blk : m.blocks) {
    const int npe = nodes_per_element(blk.type);
    for (int64_t e = 0; e < blk.n_elements; ++e)
      for (int k = 0; k < npe; ++k) count[blk.conn[(size_t)e * npe + k]]++;
  }
  std::fill(out, out + N * 9, cplx(0.0, 0.0));
  for (const Block& blk : m.blocks) {
    if (blk.type == ELP_BRICK8) {
      const cplx Ew = material_modulus(m, blk.material, w);
      const double nu = m.materials[blk.material].nu;
      for (int64_t e = 0; e < blk.n_elements; ++e) {
        const int32_t* en = &blk.conn[(size_t)e * 8];
        cplx sig[6];
        if (!brick_centre_stress(m, en, Ew, nu, x, sig)) { err = "element with a singular Jacobian"; return ELP_ERR_ARG; }
        for (int k = 0; k < 8; ++k)
          for (int i = 0; i < 6; ++i) out[(size_t)seq[en[k]] * 9 + i] += sig[i] * (1.0 / count[en[k]]);
      }
    } else if (blk.type == ELP_FLUID8) {
      for (int64_t e = 0; e < blk.n_elements; ++e) {
        const int32_t* en = &blk.conn[(size_t)e * 8];
        cplx pv[8];
        for (int f = 0; f < 8; ++f) {
          const int32_t r = m.global_rows[(size_t)en[f] * ELP_NUM_KNOWN_DOFS + ELP_DOF_FLUID];
          pv[f] = r >= 0 ? x[r] : cplx(0.0, 0.0);
        }
        for (int k = 0; k < 8; ++k) {  // corner k at (xi, eta, zeta) = kHexS[k]
          double dN[8][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, I[3][3];
          for (int f = 0; f < 8; ++f) {
            const double a = 1.0 + kHexS[f][0] * kHexS[k][0], b = 1.0 + kHexS[f][1] * kHexS[k][1],
                         c = 1.0 + kHexS[f][2] * kHexS[k][2];
            dN[f][0] = 0.125 * kHexS[f][0] * b * c;
            dN[f][1] = 0.125 * kHexS[f][1] * a * c;
            dN[f][2] = 0.125 * kHexS[f][2] * a * b;
            for (int q = 0; q < 3; ++q)
              for (int d = 0; d < 3; ++d) J[q][d] += dN[f][q] * m.coords[3 * (size_t)en[f] + d];
          }
          if (!invert3(J, I)) { err = "element with a singular Jacobian"; return ELP_ERR_ARG; }
          cplx g[3] = {0, 0, 0};
          for (int f = 0; f < 8; ++f)
            for (int d = 0; d < 3; ++d) g[d] += (I[d][0] * dN[f][0] + I[d][1] * dN[f][1] + I[d][2] * dN[f][2]) * pv[f];
          for (int d = 0; d < 3; ++d) out[(size_t)seq[en[k]] * 9 + 6 + d] += g[d];
        }
      }
    }
  }
  return ELP_OK;
}

}  // namespace elp
