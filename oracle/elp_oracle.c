/* Test infrastructure (CPU oracle), not product code.
 *
 * Restatement, in plain C, of the reference's element arithmetic as the
 * reference writes it (dense B^T C B per Gauss point with a complex C,
 * infam::BT_C_B_wdJ in math/matrix.h:760-790), and of the per-frequency
 * assembly loop. Only tests/, the smoke check and bench.py's CPU baseline
 * call it. Paths below are inside elpasoCore/source/ of the reference.
 *
 *   Gauss rule + shape tables : misc/gausspoints.h:27-43 (15-digit constants),
 *                               misc/gausspoints.cpp:76-87 (3D: x fastest),
 *                               misc/gausspoints.cpp:165-195 (2D: y fastest),
 *                               shape/shapefunctions.cpp:110- (quad4), :957- (hex8)
 *   Jacobians                 : element/elementfem.cpp:77-210
 *   Brick8 K, M               : element/structure/linear/brick/elementstructurebrick.cpp:281-554
 *   isotropic C (complex E)   : material/.../materialstructurevisco.cpp:351-372
 *   DSG4 K                    : element/structure/linear/plate/elementstructuremindlindsg4.cpp:37-211
 *   Cb, Cs                    : material/.../materialstructurevisco.cpp:296-327, Ks = 5/6
 *                               (material/structure/materialstructure.cpp:30)
 *   Mindlin M                 : element/structure/linear/plate/elementstructuremindlin.cpp:299-366
 *   K - w^2 M                 : element/structure/elementstructure.cpp:43-61
 *   Fluid8 K, M, EM           : element/fluid/elementfluid3d.cpp:54-167, element/fluid/elementfluid.cpp:58-77
 *   InterfaceMindlin C        : element/interface/elementinterfacemindlin.cpp:80-181
 *   C, C^T into K with -ori   : element/interface/elementinterfacestructural.cpp:46-69,152-179,209-237
 *   per-w loop, BC rows       : analysis/frequency/analysisfrequencybasic.cpp:101-157,
 *                               analysis/analysis.cpp:419-454, 1238-1246
 */
#include "elp_oracle.h"

#include <complex.h>
#include <math.h>
#include <string.h>

typedef double complex cx;

static const double GP2 = 0.577350269189626;

static double hex_fn(int k, int d, const double g[3]) {
  static const int sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
  static const int sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
  static const int sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  double fx = 1. + sx[k] * g[0], fy = 1. + sy[k] * g[1], fz = 1. + sz[k] * g[2];
  if (d == 0) return fx * fy * fz * 0.125;
  if (d == 1) return sx[k] * fy * fz * 0.125;
  if (d == 2) return sy[k] * fx * fz * 0.125;
  return sz[k] * fx * fy * 0.125;
}
static double quad_fn(int k, int d, const double g[2]) {
  static const int sx[4] = {-1, 1, 1, -1};
  static const int sy[4] = {-1, -1, 1, 1};
  double fx = 1. + sx[k] * g[0], fy = 1. + sy[k] * g[1];
  if (d == 0) return 0.25 * fx * fy;
  if (d == 1) return 0.25 * sx[k] * fy;
  return 0.25 * sy[k] * fx;
}

static double HEX[4][8][8], QUAD[3][4][4];
static int tables_ready = 0;

void orc_shape_tables(double* hex, double* quad) {
  if (!tables_ready) {
    const double p[2] = {GP2, -GP2};
    for (int n = 0; n < 8; ++n) {
      int x = n % 2, y = (n / 2) % 2, z = n / 4;  /* Start(2)=1: gp4[1+x] */
      double g[3] = {p[x], p[y], p[z]};
      for (int k = 0; k < 8; ++k)
        for (int d = 0; d < 4; ++d) HEX[d][k][n] = hex_fn(k, d, g);
    }
    for (int n = 0; n < 4; ++n) {
      int y = n % 2, x = n / 2;
      double g[2] = {p[x], p[y]};
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) QUAD[d][k][n] = quad_fn(k, d, g);
    }
    tables_ready = 1;
  }
  if (hex) memcpy(hex, HEX, sizeof(HEX));
  if (quad) memcpy(quad, QUAD, sizeof(QUAD));
}

/* KK (n x n) += B^T C B * wdJ, B (r x n), C (r x r), as BT_C_B_wdJ */
static void btcb(cx* KK, int n, const double* B, int r, const cx* C, double wdJ) {
  cx CB[6 * 24];
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < n; ++j) {
      cx s = 0;
      for (int k = 0; k < r; ++k) s += C[i * r + k] * B[k * n + j];
      CB[i * n + j] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      cx s = 0;
      for (int k = 0; k < r; ++k) s += B[k * n + i] * CB[k * n + j];
      KK[i * n + j] += s * wdJ;
    }
}

static void out_cx(const cx* A, int n, double* o) {
  if (!o) return;
  for (int i = 0; i < n * n; ++i) { o[2 * i] = creal(A[i]); o[2 * i + 1] = cimag(A[i]); }
}

static double jac3(const double* x, int gp, double inv[3][3]) {
  double J[3][3] = {{0}};
  for (int k = 0; k < 8; ++k)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J[i][j] += HEX[i + 1][k][gp] * x[3 * k + j];
  double det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1] -
               J[0][2] * J[1][1] * J[2][0] - J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2];
  inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  inv[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
  inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  inv[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
  inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  inv[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
  inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  inv[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
  inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  return det;
}

int orc_brick8(const double* xyz, double E_re, double E_im, double nu, double rho, double omega, double* Ko,
               double* Mo, double* EMo) {
  orc_shape_tables(0, 0);
  cx K[576], M[576];
  memset(K, 0, sizeof(K));
  memset(M, 0, sizeof(M));
  cx E = E_re + I * E_im;
  cx f = E / (1.0 + nu) / (1.0 - 2.0 * nu);
  cx C[36];
  memset(C, 0, sizeof(C));
  C[0] = C[7] = C[14] = f * (1. - nu);
  C[21] = C[28] = C[35] = f * (1.0 - 2.0 * nu) / 2.0;
  C[1] = C[6] = C[2] = C[12] = C[8] = C[13] = f * nu;
  double B[6 * 24];
  for (int n = 0; n < 8; ++n) {
    double inv[3][3];
    double det = jac3(xyz, n, inv);
    memset(B, 0, sizeof(B));
    for (int k = 0; k < 8; ++k) {
      double Nx = inv[0][0] * HEX[1][k][n] + inv[0][1] * HEX[2][k][n] + inv[0][2] * HEX[3][k][n];
      double Ny = inv[1][0] * HEX[1][k][n] + inv[1][1] * HEX[2][k][n] + inv[1][2] * HEX[3][k][n];
      double Nz = inv[2][0] * HEX[1][k][n] + inv[2][1] * HEX[2][k][n] + inv[2][2] * HEX[3][k][n];
      B[0 * 24 + 3 * k + 0] = Nx;
      B[1 * 24 + 3 * k + 1] = Ny;
      B[2 * 24 + 3 * k + 2] = Nz;
      B[3 * 24 + 3 * k + 0] = Ny;
      B[3 * 24 + 3 * k + 1] = Nx;
      B[4 * 24 + 3 * k + 1] = Nz;
      B[4 * 24 + 3 * k + 2] = Ny;
      B[5 * 24 + 3 * k + 0] = Nz;
      B[5 * 24 + 3 * k + 2] = Nx;
    }
    btcb(K, 24, B, 6, C, 1.0 * det);
    double Bm[3 * 24];
    cx Cm[9] = {rho, 0, 0, 0, rho, 0, 0, 0, rho};
    memset(Bm, 0, sizeof(Bm));
    for (int k = 0; k < 8; ++k) Bm[0 * 24 + 3 * k] = Bm[1 * 24 + 3 * k + 1] = Bm[2 * 24 + 3 * k + 2] = HEX[0][k][n];
    btcb(M, 24, Bm, 3, Cm, 1.0 * det);
  }
  out_cx(K, 24, Ko);
  out_cx(M, 24, Mo);
  if (EMo) {
    cx EM[576];
    for (int i = 0; i < 576; ++i) EM[i] = M[i] * (-omega * omega) + K[i];
    out_cx(EM, 24, EMo);
  }
  for (int n = 0; n < 8; ++n) {
    double inv[3][3];
    if (jac3(xyz, n, inv) <= 0.0) return 2; /* the reference only prints here */
  }
  return 0;
}

int orc_dsg4(const double* xyz, double E_re, double E_im, double nu, double rho, double t, double omega, double* Ko,
             double* Mo, double* EMo) {
  orc_shape_tables(0, 0);
  cx K[144], M[144];
  memset(K, 0, sizeof(K));
  memset(M, 0, sizeof(M));
  cx E = E_re + I * E_im;
  double x[4], y[4];
  for (int k = 0; k < 4; ++k) { x[k] = xyz[3 * k]; y[k] = xyz[3 * k + 1]; }
  double hk = 0.0;
  int seq[5] = {0, 1, 2, 3, 0};
  for (int i = 1; i < 4; ++i) {
    const double* a = xyz + 3 * seq[i];
    const double* b = xyz + 3 * seq[i - 1];
    double r = 0.;
    for (int k = 0; k < 3; ++k) r += (a[k] - b[k]) * (a[k] - b[k]);
    double d = sqrt(r);
    if (d > hk) hk = d;
  }
  double tau = 1.0 / (1.0 + 0.12 * hk * hk / (t * t));
  cx Bd = E * t * t * t / (12. * (1. - nu * nu));
  cx G = E / (2. * (1. + nu));
  cx Cb[9] = {Bd, Bd * nu, 0, Bd * nu, Bd, 0, 0, 0, G * t * t * t / 12.};
  cx Ghk = E / (2. * (1. + nu)) * t * (5. / 6.);
  cx Cs[4] = {Ghk * tau, 0, 0, Ghk * tau};
  double Bb[3 * 12], Bs[2 * 12];
  memset(Bb, 0, sizeof(Bb));
  int bad = 0;
  for (int n = 0; n < 4; ++n) {
    double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
    for (int k = 0; k < 4; ++k) {
      J00 += QUAD[1][k][n] * x[k];
      J01 += QUAD[1][k][n] * y[k];
      J10 += QUAD[2][k][n] * x[k];
      J11 += QUAD[2][k][n] * y[k];
    }
    double det = J00 * J11 - J01 * J10;
    if (det <= 0.0) bad = 1;
    double a = J00, b = J01, d = J10, c = J11;
    double wdJ = 1.0 * det;
    for (int k = 0; k < 4; ++k) {
      double dNdx = (c * QUAD[1][k][n] - b * QUAD[2][k][n]) / det;
      double dNdy = (-d * QUAD[1][k][n] + a * QUAD[2][k][n]) / det;
      Bb[0 * 12 + k * 3 + 2] = dNdx;
      Bb[1 * 12 + k * 3 + 1] = -dNdy;
      Bb[2 * 12 + k * 3 + 2] = dNdy;
      Bb[2 * 12 + k * 3 + 1] = -dNdx;
    }
    double N11 = QUAD[1][1][n], N12 = QUAD[1][2][n], N22 = QUAD[2][2][n], N23 = QUAD[2][3][n];
    memset(Bs, 0, sizeof(Bs));
    Bs[0] = -c * N11 + b * N23;
    Bs[1] = -b * c * N11 + b * c * N23;
    Bs[2] = a * c * N11 - b * d * N23;
    Bs[12 + 0] = d * N11 - a * N23;
    Bs[12 + 1] = -a * c * N23 + b * d * N11;
    Bs[12 + 2] = a * d * N23 - a * d * N11;
    Bs[3] = c * N11 + b * N22;
    Bs[4] = -b * c * N11 + b * c * N22;
    Bs[5] = a * c * N11 - b * d * N22;
    Bs[12 + 3] = -a * N22 - d * N11;
    Bs[12 + 4] = -a * c * N22 + b * d * N11;
    Bs[12 + 5] = a * d * N22 - a * d * N11;
    Bs[6] = c * N12 - b * N22;
    Bs[7] = -b * c * N12 + b * c * N22;
    Bs[8] = a * c * N12 - b * d * N22;
    Bs[12 + 6] = a * N22 - d * N12;
    Bs[12 + 7] = -a * c * N22 + b * d * N12;
    Bs[12 + 8] = a * d * N22 - a * d * N12;
    Bs[9] = -c * N12 - b * N23;
    Bs[10] = -b * c * N12 + b * c * N23;
    Bs[11] = a * c * N12 - b * d * N23;
    Bs[12 + 9] = a * N23 + d * N12;
    Bs[12 + 10] = -a * c * N23 + b * d * N12;
    Bs[12 + 11] = a * d * N23 - a * d * N12;
    for (int i = 0; i < 24; ++i) Bs[i] *= 1. / det;
    btcb(K, 12, Bb, 3, Cb, wdJ);
    btcb(K, 12, Bs, 2, Cs, wdJ);
    double m1 = rho * t, m2 = rho * (t * t * t / 12.0);
    for (int z = 0; z < 4; ++z)
      for (int s = 0; s < 4; ++s) {
        double nn = QUAD[0][z][n] * QUAD[0][s][n];
        M[(z * 3) * 12 + s * 3] += nn * m1 * wdJ;
        M[(z * 3 + 1) * 12 + s * 3 + 1] += nn * m2 * wdJ;
        M[(z * 3 + 2) * 12 + s * 3 + 2] += nn * m2 * wdJ;
      }
  }
  out_cx(K, 12, Ko);
  out_cx(M, 12, Mo);
  if (EMo) {
    cx EM[144];
    for (int i = 0; i < 144; ++i) EM[i] = M[i] * (-omega * omega) + K[i];
    out_cx(EM, 12, EMo);
  }
  return bad ? 2 : 0;
}

int orc_fluid8(const double* xyz, double c, double rho, double omega, double* Ko, double* Mo, double* EMo) {
  orc_shape_tables(0, 0);
  cx K[64], M[64];
  memset(K, 0, sizeof(K));
  memset(M, 0, sizeof(M));
  const double cf2 = 1.0 / (c * c);
  for (int n = 0; n < 8; ++n) {
    double inv[3][3];
    double det = jac3(xyz, n, inv);
    double wdJ = 1.0 * det;
    for (int z = 0; z < 8; ++z)
      for (int s = 0; s < 8; ++s) M[z * 8 + s] += cf2 * HEX[0][z][n] * HEX[0][s][n] * wdJ;
    double JH[3][8];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 8; ++k)
        JH[i][k] = inv[i][0] * HEX[1][k][n] + inv[i][1] * HEX[2][k][n] + inv[i][2] * HEX[3][k][n];
    for (int z = 0; z < 8; ++z)
      for (int s = 0; s < 8; ++s) {
        double v = JH[0][z] * JH[0][s] + JH[1][z] * JH[1][s] + JH[2][z] * JH[2][s];
        K[z * 8 + s] += v * wdJ;
      }
  }
  out_cx(K, 8, Ko);
  out_cx(M, 8, Mo);
  if (EMo) {
    cx EM[64];
    double factor = 1. / (rho * omega * omega);
    for (int i = 0; i < 64; ++i) EM[i] = (M[i] * (-omega * omega) + K[i]) * factor;
    out_cx(EM, 8, EMo);
  }
  return 0;
}

int orc_interface_mindlin(const double* xf, int transform, double* Co) {
  orc_shape_tables(0, 0);
  double C[12][4];
  memset(C, 0, sizeof(C));
  for (int n = 0; n < 4; ++n) {
    double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) {
        a1[d] += QUAD[1][k][n] * xf[3 * k + d];
        a2[d] += QUAD[2][k][n] * xf[3 * k + d];
      }
    double A1 = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
    double A2 = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
    double D = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
    double det = sqrt(A1 * A2 - D * D);
    for (int z = 0; z < 4; ++z)
      for (int s = 0; s < 4; ++s) C[3 * z + 2][s] += QUAD[0][z][n] * QUAD[0][s][n] * 1.0 * det;
  }
  if (transform) {
    const double xi[4] = {-1., 1., 1., -1.}, et[4] = {-1., -1., 1., 1.};
    for (int n = 0; n < 4; ++n) {
      double g[2] = {xi[n], et[n]};
      double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) {
          a1[d] += quad_fn(k, 1, g) * xf[3 * k + d];
          a2[d] += quad_fn(k, 2, g) * xf[3 * k + d];
        }
      double nv[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
      double nr = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
      for (int d = 0; d < 3; ++d) nv[d] *= 1. / nr;
      for (int s = 0; s < 4; ++s) {
        C[3 * n][s] = nv[0] * C[3 * n + 2][s];
        C[3 * n + 1][s] = nv[1] * C[3 * n + 2][s];
        C[3 * n + 2][s] = nv[2] * C[3 * n + 2][s];
      }
    }
  }
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j < 4; ++j) { Co[2 * (i * 4 + j)] = C[i][j]; Co[2 * (i * 4 + j) + 1] = 0.0; }
  return 0;
}

static int64_t find(const orc_system* s, int32_t r, int32_t c) {
  int32_t lo = s->row_ptr[r], hi = s->row_ptr[r + 1];
  while (lo < hi) {
    int32_t mid = (lo + hi) / 2;
    if (s->col_idx[mid] < c) lo = mid + 1; else hi = mid;
  }
  if (lo < s->row_ptr[r + 1] && s->col_idx[lo] == c) return lo;
  return -1;
}

/* keep (may be NULL): rows whose entries are assembled; the others are
 * skipped (their pattern rows may then be empty) */
static int add_block(const orc_system* s, const uint8_t* keep, double* v, const int32_t* rows, int n,
                     const double* EM) {
  for (int i = 0; i < n; ++i) {
    if (rows[i] < 0 || (keep && !keep[rows[i]])) continue;
    for (int j = 0; j < n; ++j) {
      if (rows[j] < 0) continue;
      int64_t q = find(s, rows[i], rows[j]);
      if (q < 0) return 3;
      v[2 * q] += EM[2 * (i * n + j)];
      v[2 * q + 1] += EM[2 * (i * n + j) + 1];
    }
  }
  return 0;
}

static int assemble_rows(const orc_system* s, const uint8_t* keep, double omega, double* v) {
  int64_t nnz = s->row_ptr[s->n];
  memset(v, 0, sizeof(double) * 2 * nnz);
  double EM[2 * 576];
  int rc;
  for (int64_t e = 0; e < s->n_brick; ++e) {
    const double* mt = s->brick_mat + 4 * e;
    orc_brick8(s->brick_xyz + 24 * e, mt[0], mt[1], mt[2], mt[3], omega, 0, 0, EM);
    if ((rc = add_block(s, keep, v, s->brick_rows + 24 * e, 24, EM))) return rc;
  }
  for (int64_t e = 0; e < s->n_plate; ++e) {
    const double* mt = s->plate_mat + 5 * e;
    if (orc_dsg4(s->plate_xyz + 12 * e, mt[0], mt[1], mt[2], mt[3], mt[4], omega, 0, 0, EM)) return 2;
    if ((rc = add_block(s, keep, v, s->plate_rows + 12 * e, 12, EM))) return rc;
  }
  for (int64_t e = 0; e < s->n_fluid; ++e) {
    const double* mt = s->fluid_mat + 2 * e;
    orc_fluid8(s->fluid_xyz + 24 * e, mt[0], mt[1], omega, 0, 0, EM);
    if ((rc = add_block(s, keep, v, s->fluid_rows + 8 * e, 8, EM))) return rc;
  }
  for (int64_t q = 0; q < s->n_iface; ++q) {
    double C[2 * 48];
    orc_interface_mindlin(s->iface_xyz + 12 * q, s->iface_transform[q], C);
    const int32_t* R = s->iface_rows + 16 * q;
    double f = -1. * s->iface_ori[q];
    for (int z = 0; z < 12; ++z) {
      if (R[z] < 0) continue;
      for (int c = 0; c < 4; ++c) {
        if (R[12 + c] < 0) continue;
        double val = C[2 * (z * 4 + c)] * f;
        if (!keep || keep[R[z]]) {
          int64_t q1 = find(s, R[z], R[12 + c]);
          if (q1 < 0) return 3;
          v[2 * q1] += val;
        }
        if (!keep || keep[R[12 + c]]) {
          int64_t q2 = find(s, R[12 + c], R[z]);
          if (q2 < 0) return 3;
          v[2 * q2] += val;
        }
      }
    }
  }
  for (int64_t i = 0; i < s->n_bc; ++i) {
    int32_t r = s->bc_rows[i];
    for (int32_t q = s->row_ptr[r]; q < s->row_ptr[r + 1]; ++q) {
      v[2 * q] = (s->col_idx[q] == r) ? 1.0 : 0.0;
      v[2 * q + 1] = 0.0;
    }
  }
  return 0;
}

int orc_assemble(const orc_system* s, double omega, double* v) { return assemble_rows(s, NULL, omega, v); }

int orc_assemble_rows(const orc_system* s, const uint8_t* keep, double omega, double* v) {
  return assemble_rows(s, keep, omega, v);
}

/* Constitutive matrices with complex E as the visco material builds them
 * (material/.../materialstructurevisco.cpp:296-372): C (6x6), Cb (3x3),
 * Cs (2x2); complex interleaved, row-major. */
void orc_material(double E_re, double E_im, double nu, double t, double* C6, double* Cb, double* Cs) {
  cx E = E_re + I * E_im;
  cx f = E / (1.0 + nu) / (1.0 - 2.0 * nu);
  cx C[36];
  memset(C, 0, sizeof(C));
  C[0] = C[7] = C[14] = f * (1. - nu);
  C[21] = C[28] = C[35] = f * (1.0 - 2.0 * nu) / 2.0;
  C[1] = C[6] = C[2] = C[12] = C[8] = C[13] = f * nu;
  out_cx(C, 6, C6);
  cx Bd = E * t * t * t / (12. * (1. - nu * nu));
  cx G = E / (2. * (1. + nu));
  cx B[9] = {Bd, Bd * nu, 0, Bd * nu, Bd, 0, 0, 0, G * t * t * t / 12.};
  out_cx(B, 3, Cb);
  cx Ghk = E / (2. * (1. + nu)) * t * (5. / 6.);
  cx S[4] = {Ghk, 0, 0, Ghk};
  out_cx(S, 2, Cs);
}
