/* Test infrastructure (CPU oracle), not product code.
 *
 * A small extern "C" driver around the reference's OWN element, material,
 * shape and Gauss-point classes, compiled unchanged from the reference tree
 * against the PETSc type stand-in in this folder (recipe: oracle/Makefile,
 * target `ref`, output oracle/_ref/libelpref.so). It lets the tests and the
 * golden-vector generator ask the reference code itself for element
 * matrices, so that the C restatement in oracle/elp_oracle.c and the CUDA
 * kernels are pinned against the reference and not against a re-reading.
 *
 * Calls into (reference paths, elpasoCore/source/...):
 *   element/structure/linear/brick/elementstructurebrick.cpp:281-554 (Brick8 K, M)
 *   element/structure/linear/plate/elementstructuremindlindsg4.cpp:37-211 (DSG4 K)
 *   element/structure/linear/plate/elementstructuremindlin.cpp:299-366 (Mindlin M)
 *   element/structure/elementstructure.cpp:43-61 (K - w^2 M)
 *   element/fluid/elementfluid3d.cpp:54-167, element/fluid/elementfluid.cpp:58-77 (Fluid8)
 *   element/interface/elementinterfacemindlin.cpp:80-129 (coupling matrix C)
 *   shape/shapehex8.cpp:49-90, shape/shapequad4.cpp:48-73 (shape tables)
 *
 * The reference element code keeps its Jacobian in static members
 * (element/elementfem.cpp:48-50): call this library from one thread only.
 */
#include <algorithm>
#include <bitset>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <list>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <valarray>
#include <vector>
#include <memory>
#include <stdexcept>
#include "petsc.h"

/* The material classes keep E, nu, eta in private members that only the
 * HDF5 parser fills. The driver opens them up for itself; object layout is
 * unchanged by access specifiers under GCC. */
#define private public
#define protected public
#include "element/structure/linear/brick/elementstructurebrick8.h"
#include "element/structure/linear/plate/elementstructuremindlindsg4.h"
#include "element/fluid/elementfluid8.h"
#include "element/interface/elementinterfacemindlin.h"
#include "material/structure/isotrop/linear/elastic/materialstructureisotrop.h"
#include "material/structure/isotrop/linear/viscoelastic/materialstructurevisco.h"
#include "material/fluid/linear/elastic/materialfluidideal.h"
#include "shape/shapehex8.h"
#include "shape/shapequad4.h"
#undef private
#undef protected

namespace {

/* mat_kind: 0 = STR_LIN_ELA_ISO_DIR (real E), 1 = STR_LIN_VIS_ISO_DIR */
cMaterialStructure* make_structure_material(int mat_kind, double E, double nu, double rho,
                                            double t, double eta, int visco_type,
                                            double omega) {
  if (mat_kind == 0) {
    auto* m = new cMaterialStructureIsotrop();
    m->m_E = E;
    m->m_Nu = nu;
    m->setRho(rho);
    m->setT(t);
    m->setOmega(omega);
    m->updateMaterial();
    return m;
  }
  auto* m = new cMaterialStructureVisco();
  m->m_E = E;
  m->m_Nu = nu;
  m->m_Eta = eta;
  m->m_ViscoType = (short)visco_type;
  m->setRho(rho);
  m->setT(t);
  m->setOmega(omega);
  m->updateMaterial();
  return m;
}

void put_complex(const cElementMatrix& A, int n, int m, double* out) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      out[2 * (i * m + j) + 0] = A(i, j).real();
      out[2 * (i * m + j) + 1] = A(i, j).imag();
    }
}

std::vector<std::unique_ptr<cNode>> make_nodes(const double* xyz, int n) {
  std::vector<std::unique_ptr<cNode>> nodes;
  for (int k = 0; k < n; ++k) {
    nodes.emplace_back(new cNode());
    nodes[k]->setId(k + 1);
    (*nodes[k])[0] = xyz[3 * k + 0];
    (*nodes[k])[1] = xyz[3 * k + 1];
    (*nodes[k])[2] = xyz[3 * k + 2];
  }
  return nodes;
}

template <class Elem>
int structure_element(int nnod, const double* xyz, int mat_kind, double E, double nu,
                      double rho, double t, double eta, int visco_type, double omega,
                      double* K, double* M, double* EM) {
  try {
    const int n = nnod * (nnod == 8 ? 3 : 3);
    auto nodes = make_nodes(xyz, nnod);
    std::unique_ptr<cMaterialStructure> mat(
        make_structure_material(mat_kind, E, nu, rho, t, eta, visco_type, omega));
    Elem el;
    el.setId(1);
    for (int k = 0; k < nnod; ++k) el.setNode(k, nodes[k].get());
    el.setMaterial(mat.get());
    if (K) {
      cElementMatrix KM(n, n);
      el.assembleStiffnessMatrix(KM, NULL, NULL);
      put_complex(KM, n, n, K);
    }
    if (M) {
      cElementMatrix MM(n, n);
      el.assembleMassMatrix(MM);
      put_complex(MM, n, n, M);
    }
    if (EM) {
      cElementMatrix DM(n, n);
      el.assembleDynamicStiffnessMatrix(omega, DM);
      put_complex(DM, n, n, EM);
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // namespace

extern "C" {

/* Brick8: K (24x24 complex), M (24x24 complex, real-valued), EM = K - w^2 M.
 * Outputs are row-major, interleaved (re, im). Any output may be NULL. */
int ref_brick8(const double* xyz, int mat_kind, double E, double nu, double rho, double eta,
               int visco_type, double omega, double* K, double* M, double* EM) {
  return structure_element<cElementStructureBrick8>(8, xyz, mat_kind, E, nu, rho, 0.0, eta,
                                                    visco_type, omega, K, M, EM);
}

/* DSG4 plate (x3, w1, w2 per node): 12x12 complex outputs. */
int ref_dsg4(const double* xyz, int mat_kind, double E, double nu, double rho, double t,
             double eta, int visco_type, double omega, double* K, double* M, double* EM) {
  return structure_element<cElementStructureMindlinDSG4>(4, xyz, mat_kind, E, nu, rho, t, eta,
                                                         visco_type, omega, K, M, EM);
}

/* Fluid8: K (8x8), M (8x8, carries 1/c^2), EM = (K - w^2 M) / (rho w^2). */
int ref_fluid8(const double* xyz, double c, double rho, double omega, double* K, double* M,
               double* EM) {
  try {
    auto nodes = make_nodes(xyz, 8);
    cMaterialFluidIdeal mat;
    mat.setCf(c);
    mat.setRho(rho);
    mat.setOmega(omega);
    mat.updateMaterial();
    cElementFluid8 el;
    el.setId(1);
    for (int k = 0; k < 8; ++k) el.setNode(k, nodes[k].get());
    el.setMaterial(&mat);
    if (K) {
      cElementMatrix KM(8, 8);
      el.assembleStiffnessMatrix(KM, NULL, NULL);
      put_complex(KM, 8, 8, K);
    }
    if (M) {
      cElementMatrix MM(8, 8);
      el.assembleMassMatrix(MM);
      put_complex(MM, 8, 8, M);
    }
    if (EM) {
      cElementMatrix DM(8, 8);
      el.assembleDynamicStiffnessMatrix(omega, DM);
      put_complex(DM, 8, 8, EM);
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

/* InterfaceMindlin coupling matrix C (12x4 complex, rows 3z+{0,1,2} per
 * structural node, columns per fluid node), integrated over the FLUID nodes'
 * geometry as the reference does. Structural nodes carry no active x1/x2, so
 * the shell transformation is not applied (the DSG4 case). */
int ref_interface_mindlin(const double* xyz_fluid, const double* xyz_struct, double c,
                          double rho, double* C) {
  try {
    auto fnodes = make_nodes(xyz_fluid, 4);
    auto snodes = make_nodes(xyz_struct, 4);
    cMaterialFluidIdeal mat;
    mat.setCf(c);
    mat.setRho(rho);
    cElementInterfaceMindlin el(4);
    el.setId(1);
    for (int k = 0; k < 4; ++k) {
      el.setNode(k, fnodes[k].get());
      el.setMatchingNode(k, snodes[k].get());
    }
    el.setMaterial(&mat, 0);
    cElementMatrix CM(12, 4);
    el.computeCouplingMatrix(CM);
    put_complex(CM, 12, 4, C);
    return 0;
  } catch (...) {
    return 1;
  }
}

/* Shape tables as the reference evaluates them at its Gauss points:
 * hex8: N(4, 8, 8) = [fun, xi, eta, zeta] x node x gp  -> 256 doubles
 * quad4: N(3, 4, 4) = [fun, xi, eta] x node x gp       -> 48 doubles */
int ref_shape_hex8(double* out) {
  cShapeHex8 s;
  cArray3d N(s.getShapeFunctions());
  for (int a = 0; a < 4; ++a)
    for (int k = 0; k < 8; ++k)
      for (int g = 0; g < 8; ++g) out[(a * 8 + k) * 8 + g] = N(a, k, g);
  return 0;
}

int ref_shape_quad4(double* out) {
  cShapeQuad4 s;
  cArray3d N(s.getShapeFunctions());
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 4; ++k)
      for (int g = 0; g < 4; ++g) out[(a * 4 + k) * 4 + g] = N(a, k, g);
  return 0;
}

}  // extern "C"
