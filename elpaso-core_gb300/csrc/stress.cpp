// Cell stresses after a solve (cAnalysis::computeStressesCells,
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

int cell_stresses(const Model& m, double w, const cplx* x, cplx* out, cplx* out2, std::string& err) {
  int64_t base = 0;
  for (const Block& blk : m.blocks) {
    const int64_t ne = blk.n_elements;
    const elp_material& mt = m.materials[blk.material];
    const int g = m.material_group[blk.material];
    const cplx Ew = mt.E * (g >= 0 ? group_coefficient(m.groups[g], w) : cplx(1.0, 0.0));
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
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, I[3][3];
        for (int k = 0; k < 8; ++k)
          for (int a = 0; a < 3; ++a)
            for (int d = 0; d < 3; ++d) J[a][d] += 0.125 * kHexS[k][a] * m.coords[3 * (size_t)en[k] + d];
        if (!invert3(J, I)) { bad = true; continue; }
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
        s1[0] = f * ((1.0 - nu) * eps[0] + nu * eps[1] + nu * eps[2]);
        s1[1] = f * (nu * eps[0] + (1.0 - nu) * eps[1] + nu * eps[2]);
        s1[2] = f * (nu * eps[0] + nu * eps[1] + (1.0 - nu) * eps[2]);
        for (int k = 3; k < 6; ++k) s1[k] = f * (0.5 * (1.0 - 2.0 * nu)) * eps[k];
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

}  // namespace elp
