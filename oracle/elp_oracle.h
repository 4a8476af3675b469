/* Test infrastructure (CPU oracle), not product code.
 * Plain C restatement of the reference's per-element arithmetic and of its
 * per-frequency global assembly, used only by tests/, the smoke check and
 * the CPU baseline of bench.py. */
#ifndef ELP_ORACLE_H
#define ELP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Element matrices, row-major, complex interleaved (re, im).
 * E is complex (E_vis of the visco material, or real E). */
int orc_brick8(const double* xyz, double E_re, double E_im, double nu, double rho, double omega,
               double* K, double* M, double* EM);
int orc_dsg4(const double* xyz, double E_re, double E_im, double nu, double rho, double t, double omega,
             double* K, double* M, double* EM);
int orc_fluid8(const double* xyz, double c, double rho, double omega, double* K, double* M, double* EM);
int orc_interface_mindlin(const double* xyz_fluid, int transform, double* C);
void orc_shape_tables(double* hex /* 4x8x8 */, double* quad /* 3x4x4 */);
void orc_material(double E_re, double E_im, double nu, double t, double* C6, double* Cb, double* Cs);

/* Per-frequency global assembly into a given CSR pattern (0-based, sorted
 * columns), following analysisfrequencybasic.cpp:101-157: element EM(w)
 * inserted with ADD, interface (-ori) C and C^T, then BC rows zeroed with
 * diagonal 1. Element DOF rows are passed per element (node-major). */
typedef struct {
  int64_t n;
  const int32_t* row_ptr;
  const int32_t* col_idx;
  int64_t n_brick, n_plate, n_fluid, n_iface;
  const double* brick_xyz;   /* 24 per element */
  const double* brick_mat;   /* E_re, E_im, nu, rho per element */
  const int32_t* brick_rows; /* 24 per element */
  const double* plate_xyz;   /* 12 per element */
  const double* plate_mat;   /* E_re, E_im, nu, rho, t per element */
  const int32_t* plate_rows; /* 12 per element */
  const double* fluid_xyz;   /* 24 per element */
  const double* fluid_mat;   /* c, rho per element */
  const int32_t* fluid_rows; /* 8 per element */
  const double* iface_xyz;   /* 12 per quad (fluid nodes) */
  const double* iface_ori;   /* per quad */
  const int32_t* iface_rows; /* 12 structure rows (x1 x2 x3 per node, -1 inactive) + 4 fluid rows */
  const int32_t* iface_transform; /* per quad: 1 if the shell transform applies */
  int64_t n_bc;
  const int32_t* bc_rows;
} orc_system;

int orc_assemble(const orc_system* s, double omega, double* values /* 2*nnz */);
/* The same for the rows with keep[r] != 0 only (the pattern may leave the
 * other rows empty; the elements passed are those touching kept rows):
 * A(w) on a sample of rows of a model too large for the full pattern. */
int orc_assemble_rows(const orc_system* s, const uint8_t* keep, double omega, double* values);

#ifdef __cplusplus
}
#endif
#endif
