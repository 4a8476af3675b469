/*
 * A C11 host of the C ABI (include/elpaso_gb300.h), the way elpasoC's
 * FullRun would drive it through a shim: it fills an elp_model_desc from
 * plain arrays, creates the model and reads back what the host-side calls
 * return, printed at full precision for tests/test_c_host.py to compare with
 * the Python binding and the oracle. It runs with or without a GPU:
 * elp_model_analyse runs the symbolic phase on the host and then reports a
 * missing device, and the stresses (computed on the device) are printed
 * only when a device answered.
 *
 * Model: a 3 x 2 x 2 Brick8 box (0.3 x 0.2 x 0.02 m, tabulated visco
 * material) with a DSG4 plate (elastic aluminium) on its top face, node ids
 * descending in array order; x1 x2 x3 fixed on x = 0 and a prescribed
 * complex w1 at one top corner; a nodal force, a nodal moment and three
 * constant face tractions.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "elpaso_gb300.h"

enum { NX = 3, NY = 2, NZ = 2, NNX = NX + 1, NNY = NY + 1, NNZ_ = NZ + 1 };
#define N_NODES (NNX * NNY * NNZ_)
#define N_BRICKS (NX * NY * NZ)
#define N_QUADS (NX * NY)

static int32_t node_index(int i, int j, int k) { return (int32_t)(i + NNX * (j + NNY * k)); }

static void print_ints(const char* tag, const int32_t* a, int64_t n) {
  printf("%s", tag);
  for (int64_t i = 0; i < n; ++i) printf(" %d", (int)a[i]);
  printf("\n");
}

static void print_doubles(const char* tag, const double* a, int64_t n) {
  printf("%s", tag);
  for (int64_t i = 0; i < n; ++i) printf(" %.17g", a[i]);
  printf("\n");
}

static int fail(const char* what, int rc) {
  fprintf(stderr, "%s failed (%d): %s\n", what, rc, elp_last_error());
  return 1;
}

int main(void) {
  static int64_t ids[N_NODES];
  static double xyz[3 * N_NODES];
  for (int k = 0; k < NNZ_; ++k)
    for (int j = 0; j < NNY; ++j)
      for (int i = 0; i < NNX; ++i) {
        const int32_t v = node_index(i, j, k);
        ids[v] = 5000 - 7 * (int64_t)v;
        xyz[3 * v] = 0.1 * i;
        xyz[3 * v + 1] = 0.1 * j;
        xyz[3 * v + 2] = 0.01 * k;
      }

  static int32_t hex[8 * N_BRICKS], quad[4 * N_QUADS];
  int e = 0;
  for (int k = 0; k < NZ; ++k)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i, ++e) {
        const int32_t c[8] = {node_index(i, j, k),         node_index(i + 1, j, k),
                              node_index(i + 1, j + 1, k), node_index(i, j + 1, k),
                              node_index(i, j, k + 1),     node_index(i + 1, j, k + 1),
                              node_index(i + 1, j + 1, k + 1), node_index(i, j + 1, k + 1)};
        memcpy(&hex[8 * e], c, sizeof c);
      }
  e = 0;
  for (int j = 0; j < NY; ++j)
    for (int i = 0; i < NX; ++i, ++e) {
      const int32_t c[4] = {node_index(i, j, NZ), node_index(i + 1, j, NZ), node_index(i + 1, j + 1, NZ),
                            node_index(i, j + 1, NZ)};
      memcpy(&quad[4 * e], c, sizeof c);
    }

  static const double e_table[4] = {50.0, 2.0e11, 300.0, 1.8e11};
  static const double eta_table[4] = {10.0, 0.01, 400.0, 0.04};
  elp_material mats[2];
  memset(mats, 0, sizeof mats);
  mats[0].kind = ELP_STR_LIN_VIS_ISO_DIR;
  mats[0].nu = 0.3;
  mats[0].rho = 7850.0;
  mats[0].visco_type = 1;
  mats[0].n_E_table = 2;
  mats[0].E_table = e_table;
  mats[0].n_eta_table = 2;
  mats[0].eta_table = eta_table;
  mats[1].kind = ELP_STR_LIN_ELA_ISO_DIR;
  mats[1].E = 70e9;
  mats[1].nu = 0.33;
  mats[1].rho = 2700.0;
  mats[1].t = 0.002;

  elp_element_block blocks[2];
  blocks[0].type = ELP_BRICK8;
  blocks[0].material = 0;
  blocks[0].n_elements = N_BRICKS;
  blocks[0].connectivity = hex;
  blocks[1].type = ELP_DSG4;
  blocks[1].material = 1;
  blocks[1].n_elements = N_QUADS;
  blocks[1].connectivity = quad;

  static elp_fixed_dof fixed[3 * NNY * NNZ_ + 1];
  int nf = 0;
  for (int k = 0; k < NNZ_; ++k)
    for (int j = 0; j < NNY; ++j)
      for (int d = 0; d < 3; ++d) {
        fixed[nf].node = node_index(0, j, k);
        fixed[nf].dof = ELP_DOF_X1 + d;
        fixed[nf].value_re = fixed[nf].value_im = 0.0;
        ++nf;
      }
  fixed[nf].node = node_index(NX, NY, NZ);
  fixed[nf].dof = ELP_DOF_W1;
  fixed[nf].value_re = 1e-6;
  fixed[nf].value_im = 2e-6;
  ++nf;

  elp_nodal_force force = {node_index(2, 1, NZ), {0.25, 0.0, 1.0}};
  elp_nodal_moment moment = {node_index(1, 1, NZ), {0.3, -0.5, 0.7}};
  elp_face_traction tractions[3] = {
      {0, 3, 0, {120.0, 40.0, -30.0, 0.0, 0.0, 15.0}},
      {0, 4, 7, {5.0, 0.0, 6.0, -2.0, -7.0, 0.0}},
      {0, 2, 11, {-100.0, 0.0, 0.0, 0.0, 30.0, 10.0}},
  };

  elp_model_desc d;
  memset(&d, 0, sizeof d);
  d.n_nodes = N_NODES;
  d.node_ids = ids;
  d.coords = xyz;
  d.n_materials = 2;
  d.materials = mats;
  d.n_blocks = 2;
  d.blocks = blocks;
  d.n_fixed = nf;
  d.fixed = fixed;
  d.n_forces = 1;
  d.forces = &force;
  d.n_moments = 1;
  d.moments = &moment;
  d.n_face_tractions = 3;
  d.face_tractions = tractions;

  elp_model* m = NULL;
  int rc = elp_model_create(&d, &m);
  if (rc) return fail("elp_model_create", rc);

  elp_model_info info;
  rc = elp_model_get_info(m, &info);
  if (rc) return fail("elp_model_get_info", rc);
  const int64_t n = info.n_dofs;
  int64_t nnz = 0;
  rc = elp_model_pattern(m, NULL, NULL, &nnz);
  if (rc) return fail("elp_model_pattern", rc);
  printf("sizes %lld %lld %d %lld\n", (long long)n, (long long)nnz, N_NODES, (long long)info.n_elements);

  int32_t* row_ptr = malloc(sizeof(int32_t) * (size_t)(n + 1));
  int32_t* col_idx = malloc(sizeof(int32_t) * (size_t)nnz);
  int32_t* rows = malloc(sizeof(int32_t) * N_NODES * ELP_NUM_KNOWN_DOFS);
  double* f = malloc(sizeof(double) * 2 * (size_t)n);
  double* x = malloc(sizeof(double) * 2 * (size_t)n);
  double* sig = malloc(sizeof(double) * 18 * (size_t)info.n_elements);
  double* sig_lower = malloc(sizeof(double) * 18 * (size_t)info.n_elements);
  double* sig_nodes = malloc(sizeof(double) * 18 * N_NODES);
  if (!row_ptr || !col_idx || !rows || !f || !x || !sig || !sig_lower || !sig_nodes) return fail("malloc", -1);

  if ((rc = elp_model_pattern(m, row_ptr, col_idx, NULL))) return fail("elp_model_pattern", rc);
  print_ints("row_ptr", row_ptr, n + 1);
  print_ints("col_idx", col_idx, nnz);
  if ((rc = elp_model_global_rows(m, rows))) return fail("elp_model_global_rows", rc);
  print_ints("rows", rows, (int64_t)N_NODES * ELP_NUM_KNOWN_DOFS);
  if ((rc = elp_model_rhs(m, f))) return fail("elp_model_rhs", rc);
  print_doubles("f", f, 2 * n);
  const double omega = 2.0 * 3.14159265358979323846 * 120.0;
  if ((rc = elp_model_rhs_omega(m, omega, f))) return fail("elp_model_rhs_omega", rc);
  print_doubles("f_omega", f, 2 * n);

  for (int64_t i = 0; i < n; ++i) {
    x[2 * i] = 1e-6 * sin(0.37 * (double)i);
    x[2 * i + 1] = 1e-6 * cos(0.11 * (double)i);
  }
  print_doubles("x", x, 2 * n);
  /* stresses run on the device: without one they report ELP_ERR_CUDA */
  rc = elp_cell_stresses(m, omega, x, sig, sig_lower);
  if (rc == ELP_OK) {
    print_doubles("sigma", sig, 18 * info.n_elements);
    print_doubles("sigma_lower", sig_lower, 18 * info.n_elements);
    if ((rc = elp_node_stresses(m, omega, x, sig_nodes))) return fail("elp_node_stresses", rc);
    print_doubles("sigma_nodes", sig_nodes, 18 * N_NODES);
  } else if (rc != ELP_ERR_CUDA) {
    return fail("elp_cell_stresses", rc);
  }

  /* argument errors come back as status codes, never an abort */
  if (elp_model_rhs_omega(m, -1.0, f) != ELP_ERR_ARG) return fail("negative omega not rejected", -1);
  if (elp_model_rhs(NULL, f) != ELP_ERR_ARG) return fail("null model not rejected", -1);

  /* the symbolic phase runs on the host; without a device the call then
   * fails with ELP_ERR_CUDA and the front statistics are still there */
  rc = elp_model_analyse(m);
  elp_model_get_info(m, &info);
  printf("analyse %d %lld %d %d\n", rc, (long long)info.n_fronts, info.n_levels, info.max_front);
  if (rc != ELP_OK && rc != ELP_ERR_CUDA) return fail("elp_model_analyse", rc);

  if ((rc = elp_model_destroy(m))) return fail("elp_model_destroy", rc);
  free(row_ptr);
  free(col_idx);
  free(rows);
  free(f);
  free(x);
  free(sig);
  free(sig_lower);
  free(sig_nodes);
  return 0;
}
