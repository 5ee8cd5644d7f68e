/*
 * ufe_oracle.c -- CPU restatement of UFEMISM 2.0's velocity solve (TEST INFRASTRUCTURE ONLY).
 *
 * Used by the tests, the smoke check and the benchmark's CPU-baseline leg as the reference the
 * GPU results are compared with.  The product (the GPU library) never links or calls this code.
 *
 * Paths are relative to the UFEMISM2.0 source tree.  Arithmetic follows the Fortran expressions
 * in their left-to-right evaluation order, so that a build without FMA contraction
 * (-ffp-contract=off) reproduces the reference's roundings wherever the reference's own
 * operation order is known.  Three places differ from the reference at rounding level and are
 * documented where they occur: the 5x5 inverse (Gauss-Jordan here, a cofactor expansion there),
 * the 3x3 inverse (direct transpose here, an add/subtract swap there), and PETSc's internal
 * reductions (sequential sums here).
 */
#include "ufe_oracle.h"

#include <math.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>
#include <string.h>

/* src/UPSY/basic/parameters.f90:20-27 */
#define ICE_DENSITY 910.0
#define GRAV 9.81
#define R_GAS 8.314   /* parameters.f90:27 */
/* src/UPSY/basic/math_utilities/shape_functions.f90:13 */
#define SHAPE_Q 1.5

/* Fortran column-major, 1-based element access */
#define FA(a, i, j, ld) ((a)[(int64_t)((j) - 1) * (ld) + ((i) - 1)])

/* ---------------------------------------------------------------------------------------- */
/* CSR builder: CSR_matrix_basics.f90:31-154 (allocate), :251-277 (add_entry), :508-527 (finalise) */

static int csr_alloc(orc_csr *A, int32_t m, int32_t n, int64_t nnz_est) {
  A->m = m; A->n = n; A->nnz = 0;
  A->nnz_max = nnz_est > 16 ? nnz_est : 16;
  A->ptr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m + 1));
  A->ind = (int32_t *)malloc(sizeof(int32_t) * (size_t)A->nnz_max);
  A->val = (double *)malloc(sizeof(double) * (size_t)A->nnz_max);
  if (!A->ptr || !A->ind || !A->val) return -1;
  for (int32_t i = 0; i <= m; ++i) A->ptr[i] = 1;
  return 0;
}

void orc_csr_free(orc_csr *A) {
  if (!A) return;
  free(A->ptr); free(A->ind); free(A->val);
  A->ptr = NULL; A->ind = NULL; A->val = NULL; A->nnz = A->nnz_max = 0;
}

/* add_entry_CSR_dist: append (i,j,v); rows must be added in order. ptr(i+1) = nnz+1.  Rows
 * skipped between entries keep ptr = previous end (an empty row), as the reference's ptr(i1:)
 * initialisation to 1 plus the later rows' updates produce after finalise. */
static int csr_add(orc_csr *A, int32_t i, int32_t j, double v) {
  if (A->nnz + 1 > A->nnz_max) {
    int64_t nm = A->nnz_max * 2 + 1000;
    int32_t *ni = (int32_t *)realloc(A->ind, sizeof(int32_t) * (size_t)nm);
    double *nv = (double *)realloc(A->val, sizeof(double) * (size_t)nm);
    if (!ni || !nv) return -1;
    A->ind = ni; A->val = nv; A->nnz_max = nm;
  }
  A->nnz += 1;
  A->ind[A->nnz - 1] = j;
  A->val[A->nnz - 1] = v;
  A->ptr[i] = (int32_t)(A->nnz + 1);   /* ptr(i+1) in 1-based terms */
  return 0;
}

/* Called once per row after its entries, so an empty row carries the running end forward. */
static void csr_close_row(orc_csr *A, int32_t i) {
  /* ptr is 1-based: ptr(i) is stored at A->ptr[i-1]; ptr(i+1) at A->ptr[i] */
  if (A->ptr[i] < A->ptr[i - 1]) A->ptr[i] = A->ptr[i - 1];
  if (A->ptr[i] != (int32_t)(A->nnz + 1)) A->ptr[i] = (int32_t)(A->nnz + 1);
}

/* ---------------------------------------------------------------------------------------- */
/* small dense algebra (src/UPSY/basic/math_utilities/matrix_algebra.f90) */

/* gfortran's NORM2: scaled sum of squares with running scale (a published overflow-safe
 * algorithm).  Used for the LSQ distance weights, shape_functions.f90:169,264,395. */
static double norm2_2(double a, double b) {
  double xs[2] = {a, b};
  double scale = 1.0, result = 0.0;
  for (int i = 0; i < 2; ++i) {
    if (xs[i] != 0.0) {
      double absx = fabs(xs[i]);
      if (scale < absx) {
        double val = scale / absx;
        result = 1.0 + result * val * val;
        scale = absx;
      } else {
        double val = absx / scale;
        result += val * val;
      }
    }
  }
  return sqrt(result) * scale;
}

/* calc_determinant_2_by_2 / calc_matrix_inverse_2_by_2 (matrix_algebra.f90:11-19,110-131);
 * M is column-major 2x2: M[r + 2c]. */
static double det2(const double *A) { return A[0] * A[3] - A[2] * A[1]; }
static void inv2(const double *A, double *Ai) {
  double d = det2(A);
  Ai[0] = A[3] / d;  Ai[2] = -A[2] / d;
  Ai[1] = -A[1] / d; Ai[3] = A[0] / d;
}

/* calc_determinant_3_by_3 / calc_matrix_inverse_3_by_3 (matrix_algebra.f90:21-42,133-183):
 * minors, determinant by the first row, cofactor signs, transpose, divide.  The reference
 * transposes with an add/subtract swap; this one moves the values directly. */
#define M3(A, r, c) (A)[((c) - 1) * 3 + ((r) - 1)]
static double det3(const double *A) {
  double m11 = M3(A,2,2) * M3(A,3,3) - M3(A,2,3) * M3(A,3,2);
  double m12 = M3(A,2,1) * M3(A,3,3) - M3(A,2,3) * M3(A,3,1);
  double m13 = M3(A,2,1) * M3(A,3,2) - M3(A,2,2) * M3(A,3,1);
  return M3(A,1,1) * m11 - M3(A,1,2) * m12 + M3(A,1,3) * m13;
}
static void inv3(const double *A, double *Ai) {
  double m[10];
#define MN(r, c) m[((r) - 1) * 3 + (c)]
  MN(1,1) = M3(A,2,2) * M3(A,3,3) - M3(A,2,3) * M3(A,3,2);
  MN(1,2) = M3(A,2,1) * M3(A,3,3) - M3(A,2,3) * M3(A,3,1);
  MN(1,3) = M3(A,2,1) * M3(A,3,2) - M3(A,2,2) * M3(A,3,1);
  MN(2,1) = M3(A,1,2) * M3(A,3,3) - M3(A,1,3) * M3(A,3,2);
  MN(2,2) = M3(A,1,1) * M3(A,3,3) - M3(A,1,3) * M3(A,3,1);
  MN(2,3) = M3(A,1,1) * M3(A,3,2) - M3(A,1,2) * M3(A,3,1);
  MN(3,1) = M3(A,1,2) * M3(A,2,3) - M3(A,1,3) * M3(A,2,2);
  MN(3,2) = M3(A,1,1) * M3(A,2,3) - M3(A,1,3) * M3(A,2,1);
  MN(3,3) = M3(A,1,1) * M3(A,2,2) - M3(A,1,2) * M3(A,2,1);
  double d = M3(A,1,1) * MN(1,1) - M3(A,1,2) * MN(1,2) + M3(A,1,3) * MN(1,3);
  /* cofactors C(r,c) = (-1)^(r+c) minor(r,c); inverse(r,c) = C(c,r) / d */
  for (int r = 1; r <= 3; ++r)
    for (int c = 1; c <= 3; ++c) {
      double cof = MN(c, r);
      if (((r + c) & 1) != 0) cof = -cof;
      M3(Ai, r, c) = cof / d;
    }
#undef MN
}

/* 5x5 inverse and determinant by Gauss-Jordan elimination with partial pivoting.  The reference
 * (matrix_algebra.f90:44-108,185-457) uses a cofactor expansion; both give the same inverse up to
 * rounding, and the determinant only feeds the "singular to working precision" test. */
static double inv5(const double *A, double *Ai) {
  double a[5][10];
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) {
      a[r][c] = A[c * 5 + r];
      a[r][c + 5] = (r == c) ? 1.0 : 0.0;
    }
  double det = 1.0;
  for (int c = 0; c < 5; ++c) {
    int piv = c;
    double best = fabs(a[c][c]);
    for (int r = c + 1; r < 5; ++r)
      if (fabs(a[r][c]) > best) { best = fabs(a[r][c]); piv = r; }
    if (best == 0.0) return 0.0;
    if (piv != c) {
      for (int k = 0; k < 10; ++k) { double t = a[c][k]; a[c][k] = a[piv][k]; a[piv][k] = t; }
      det = -det;
    }
    double p = a[c][c];
    det *= p;
    for (int k = 0; k < 10; ++k) a[c][k] /= p;
    for (int r = 0; r < 5; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      if (f != 0.0)
        for (int k = 0; k < 10; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) Ai[c * 5 + r] = a[r][c + 5];
  return det;
}

/* ---------------------------------------------------------------------------------------- */
/* shape functions (src/UPSY/basic/math_utilities/shape_functions.f90) */

/* calc_shape_functions_2D_reg_1st_order (:140-210) */
static int shape_reg1(double x, double y, int n_c, const double *x_c, const double *y_c,
                      double *Nfx_i, double *Nfy_i, double *Nfx_c, double *Nfy_c) {
  double A[4] = {0, 0, 0, 0};
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    A[0] = A[0] + w2 * dx * dx;
    A[2] = A[2] + w2 * dx * dy;
    A[1] = A[1] + w2 * dy * dx;
    A[3] = A[3] + w2 * dy * dy;
  }
  double d = det2(A);
  if (fabs(d) < DBL_MIN) return 0;
  double M[4];
  inv2(A, M);
  double sx = 0.0, sy = 0.0;
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    Nfx_c[ci] = w2 * ((M[0] * dx) + (M[2] * dy));
    Nfy_c[ci] = w2 * ((M[1] * dx) + (M[3] * dy));
    sx += Nfx_c[ci];
    sy += Nfy_c[ci];
  }
  *Nfx_i = -sx;
  *Nfy_i = -sy;
  return 1;
}

/* calc_shape_functions_2D_stag_1st_order (:361-453) */
static int shape_stag1(double x, double y, int n_c, const double *x_c, const double *y_c,
                       double *Nf_c, double *Nfx_c, double *Nfy_c) {
  double A[9];
  memset(A, 0, sizeof(A));
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    M3(A,1,1) = M3(A,1,1) + (w2 * 1.0 * 1.0);
    M3(A,1,2) = M3(A,1,2) + (w2 * 1.0 * dx);
    M3(A,1,3) = M3(A,1,3) + (w2 * 1.0 * dy);
    M3(A,2,1) = M3(A,2,1) + (w2 * dx * 1.0);
    M3(A,2,2) = M3(A,2,2) + (w2 * dx * dx);
    M3(A,2,3) = M3(A,2,3) + (w2 * dx * dy);
    M3(A,3,1) = M3(A,3,1) + (w2 * dy * 1.0);
    M3(A,3,2) = M3(A,3,2) + (w2 * dy * dx);
    M3(A,3,3) = M3(A,3,3) + (w2 * dy * dy);
  }
  double d = det3(A);
  if (fabs(d) <= DBL_MIN) return 0;
  double M[9];
  inv3(A, M);
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    Nf_c[ci]  = w2 * ((M3(M,1,1) * 1.0) + (M3(M,1,2) * dx) + (M3(M,1,3) * dy));
    Nfx_c[ci] = w2 * ((M3(M,2,1) * 1.0) + (M3(M,2,2) * dx) + (M3(M,2,3) * dy));
    Nfy_c[ci] = w2 * ((M3(M,3,1) * 1.0) + (M3(M,3,2) * dx) + (M3(M,3,3) * dy));
  }
  return 1;
}

/* calc_shape_functions_2D_reg_2nd_order (:212-359); the 1/2 factors of the Fortran
 * expressions are exact scalings and are written as *0.5 at the same place. */
static int shape_reg2(double x, double y, int n_c, const double *x_c, const double *y_c,
                      double *Ni /*5: x,y,xx,xy,yy*/, double *Nc /*5 x n_c*/) {
  double A[25];
  memset(A, 0, sizeof(A));
#define A5(r, c) A[((c) - 1) * 5 + ((r) - 1)]
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    double dx2 = dx * dx, dy2 = dy * dy;
    A5(1,1) = A5(1,1) + w2 * dx * dx;
    A5(1,2) = A5(1,2) + w2 * dx * dy;
    A5(1,3) = A5(1,3) + w2 * dx * 0.5 * dx2;
    A5(1,4) = A5(1,4) + w2 * dx * dx * dy;
    A5(1,5) = A5(1,5) + w2 * dx * 0.5 * dy2;

    A5(2,1) = A5(2,1) + w2 * dy * dx;
    A5(2,2) = A5(2,2) + w2 * dy * dy;
    A5(2,3) = A5(2,3) + w2 * dy * 0.5 * dx2;
    A5(2,4) = A5(2,4) + w2 * dy * dx * dy;
    A5(2,5) = A5(2,5) + w2 * dy * 0.5 * dy2;

    A5(3,1) = A5(3,1) + w2 * 0.5 * dx2 * dx;
    A5(3,2) = A5(3,2) + w2 * 0.5 * dx2 * dy;
    A5(3,3) = A5(3,3) + w2 * 0.5 * dx2 * 0.5 * dx2;
    A5(3,4) = A5(3,4) + w2 * 0.5 * dx2 * dx * dy;
    A5(3,5) = A5(3,5) + w2 * 0.5 * dx2 * 0.5 * dy2;

    A5(4,1) = A5(4,1) + w2 * dx * dy * dx;
    A5(4,2) = A5(4,2) + w2 * dx * dy * dy;
    A5(4,3) = A5(4,3) + w2 * dx * dy * 0.5 * dx2;
    A5(4,4) = A5(4,4) + w2 * dx * dy * dx * dy;
    A5(4,5) = A5(4,5) + w2 * dx * dy * 0.5 * dy2;

    A5(5,1) = A5(5,1) + w2 * 0.5 * dy2 * dx;
    A5(5,2) = A5(5,2) + w2 * 0.5 * dy2 * dy;
    A5(5,3) = A5(5,3) + w2 * 0.5 * dy2 * 0.5 * dx2;
    A5(5,4) = A5(5,4) + w2 * 0.5 * dy2 * dx * dy;
    A5(5,5) = A5(5,5) + w2 * 0.5 * dy2 * 0.5 * dy2;
  }
  double M[25];
  double d = inv5(A, M);
  if (fabs(d) < DBL_MIN) return 0;
#define M5(r, c) M[((c) - 1) * 5 + ((r) - 1)]
  double s[5] = {0, 0, 0, 0, 0};
  for (int ci = 0; ci < n_c; ++ci) {
    double dx = x_c[ci] - x, dy = y_c[ci] - y;
    double w = 1.0 / pow(norm2_2(dx, dy), SHAPE_Q);
    double w2 = w * w;
    double dx2 = dx * dx, dy2 = dy * dy;
    for (int r = 1; r <= 5; ++r) {
      double v = w2 * ((M5(r,1) * dx) + (M5(r,2) * dy) + (M5(r,3) * 0.5 * dx2) +
                       (M5(r,4) * dx * dy) + (M5(r,5) * 0.5 * dy2));
      Nc[(r - 1) * n_c + ci] = v;
      s[r - 1] += v;
    }
  }
  for (int r = 0; r < 5; ++r) Ni[r] = -s[r];
#undef A5
#undef M5
  return 1;
}

/* ---------------------------------------------------------------------------------------- */
/* flood fill (src/UPSY/mesh/mesh_utilities.f90:1856-1935) */

/* extend_group_single_iteration_a: add all unlisted vertex neighbours of the current stack */
static void extend_a(const ufe_mesh_desc *m, int32_t *map, int32_t *stack, int *stackN) {
  int n = *stackN;
  for (int i = 0; i < n; ++i) {
    int vi = stack[i];
    for (int ci = 1; ci <= m->nC[vi - 1]; ++ci) {
      int vj = FA(m->C, vi, ci, m->nV);
      if (map[vj - 1] == 0) { map[vj - 1] = 1; stack[(*stackN)++] = vj; }
    }
  }
}

/* extend_group_single_iteration_b: add all unlisted triangle neighbours (TriC) */
static void extend_b(const ufe_mesh_desc *m, int32_t *map, int32_t *stack, int *stackN) {
  int n = *stackN;
  for (int i = 0; i < n; ++i) {
    int ti = stack[i];
    for (int n2 = 1; n2 <= 3; ++n2) {
      int tj = FA(m->TriC, ti, n2, m->nTri);
      if (tj == 0) continue;
      if (map[tj - 1] == 0) { map[tj - 1] = 1; stack[(*stackN)++] = tj; }
    }
  }
}

/* ---------------------------------------------------------------------------------------- */
/* operator construction (src/UPSY/mesh/discretisation/mesh_disc_calc_matrix_operators_2D.f90) */

int32_t orc_build_operators(const ufe_mesh_desc *m, orc_csr *ops) {
  const int nV = m->nV, nTri = m->nTri;
  const int nmax = m->nC_mem * m->nC_mem;   /* n_neighbours_max */
  int nbig = (nV > nTri ? nV : nTri) + 1;
  int32_t *map = (int32_t *)calloc((size_t)nbig, sizeof(int32_t));
  int32_t *stack = (int32_t *)calloc((size_t)nbig, sizeof(int32_t));
  int32_t *i_c = (int32_t *)malloc(sizeof(int32_t) * (size_t)nmax);
  double *x_c = (double *)malloc(sizeof(double) * (size_t)nmax);
  double *y_c = (double *)malloc(sizeof(double) * (size_t)nmax);
  double *N0 = (double *)malloc(sizeof(double) * (size_t)nmax * 5);
  double *N1 = N0 + nmax, *N2 = N0 + 2 * nmax;
  int stackN = 0;
  int rc = 0;
  memset(ops, 0, sizeof(orc_csr) * UFE_OP_COUNT);

  /* -- a_a: calc_matrix_operators_mesh_a_a (:61-196) -- */
  csr_alloc(&ops[UFE_OP_DDX_A_A], nV, nV, (int64_t)nV * (m->nC_mem + 1));
  csr_alloc(&ops[UFE_OP_DDY_A_A], nV, nV, (int64_t)nV * (m->nC_mem + 1));
  stackN = 0;
  for (int row = 1; row <= nV; ++row) {
    int vi = row;
    double x = FA(m->V, vi, 1, nV), y = FA(m->V, vi, 2, nV);
    for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
    map[vi - 1] = 1; stackN = 1; stack[0] = vi;
    while (stackN - 1 < 2) {
      extend_a(m, map, stack, &stackN);
      if (stackN - 1 > nmax) { rc = UFE_ERR_CAPACITY; goto done; }
    }
    double Nfx_i = 0, Nfy_i = 0;
    int n_c = 0;
    for (;;) {
      n_c = 0;
      for (int i = 0; i < stackN; ++i) {
        if (n_c == nmax) break;
        int vj = stack[i];
        if (vj == vi) continue;
        i_c[n_c] = vj; x_c[n_c] = FA(m->V, vj, 1, nV); y_c[n_c] = FA(m->V, vj, 2, nV); n_c++;
      }
      if (shape_reg1(x, y, n_c, x_c, y_c, &Nfx_i, &Nfy_i, N0, N1)) break;
      int before = stackN;
      extend_a(m, map, stack, &stackN);
      if (stackN == before) { rc = UFE_ERR_INVALID; goto done; }
    }
    csr_add(&ops[UFE_OP_DDX_A_A], row, row, Nfx_i);
    csr_add(&ops[UFE_OP_DDY_A_A], row, row, Nfy_i);
    for (int i = 0; i < n_c; ++i) {
      csr_add(&ops[UFE_OP_DDX_A_A], row, i_c[i], N0[i]);
      csr_add(&ops[UFE_OP_DDY_A_A], row, i_c[i], N1[i]);
    }
    csr_close_row(&ops[UFE_OP_DDX_A_A], row);
    csr_close_row(&ops[UFE_OP_DDY_A_A], row);
  }

  /* -- a_b: calc_matrix_operators_mesh_a_b (:198-335); map is over vertices -- */
  for (int op = UFE_OP_MAP_A_B; op <= UFE_OP_DDY_A_B; ++op) csr_alloc(&ops[op], nTri, nV, (int64_t)nTri * 3);
  for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
  stackN = 0;
  for (int row = 1; row <= nTri; ++row) {
    int ti = row;
    double x = FA(m->TriGC, ti, 1, nTri), y = FA(m->TriGC, ti, 2, nTri);
    for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
    stackN = 0;
    for (int n = 1; n <= 3; ++n) {
      int vi = FA(m->Tri, ti, n, nTri);
      map[vi - 1] = 1; stack[stackN++] = vi;
    }
    while (stackN < 3) {
      extend_a(m, map, stack, &stackN);
      if (stackN - 1 > nmax) { rc = UFE_ERR_CAPACITY; goto done; }
    }
    int n_c = 0;
    for (;;) {
      n_c = 0;
      for (int i = 0; i < stackN; ++i) {
        if (n_c == nmax) break;
        int vi = stack[i];
        i_c[n_c] = vi; x_c[n_c] = FA(m->V, vi, 1, nV); y_c[n_c] = FA(m->V, vi, 2, nV); n_c++;
      }
      if (shape_stag1(x, y, n_c, x_c, y_c, N0, N1, N2)) break;
      int before = stackN;
      extend_a(m, map, stack, &stackN);
      if (stackN == before) { rc = UFE_ERR_INVALID; goto done; }
    }
    for (int i = 0; i < n_c; ++i) {
      csr_add(&ops[UFE_OP_MAP_A_B], row, i_c[i], N0[i]);
      csr_add(&ops[UFE_OP_DDX_A_B], row, i_c[i], N1[i]);
      csr_add(&ops[UFE_OP_DDY_A_B], row, i_c[i], N2[i]);
    }
    for (int op = UFE_OP_MAP_A_B; op <= UFE_OP_DDY_A_B; ++op) csr_close_row(&ops[op], row);
  }
  for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
  stackN = 0;

  /* -- b_a: calc_matrix_operators_mesh_b_a (:337-474); map is over triangles -- */
  for (int op = UFE_OP_MAP_B_A; op <= UFE_OP_DDY_B_A; ++op) csr_alloc(&ops[op], nV, nTri, (int64_t)nV * (m->nC_mem + 1));
  for (int row = 1; row <= nV; ++row) {
    int vi = row;
    double x = FA(m->V, vi, 1, nV), y = FA(m->V, vi, 2, nV);
    for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
    stackN = 0;
    for (int iti = 1; iti <= m->niTri[vi - 1]; ++iti) {
      int ti = FA(m->iTri, vi, iti, nV);
      map[ti - 1] = 1; stack[stackN++] = ti;
    }
    while (stackN < 3) {
      extend_b(m, map, stack, &stackN);
      if (stackN - 1 > nmax) { rc = UFE_ERR_CAPACITY; goto done; }
    }
    int n_c = 0;
    for (;;) {
      n_c = 0;
      for (int i = 0; i < stackN; ++i) {
        if (n_c == nmax) break;
        int ti = stack[i];
        i_c[n_c] = ti; x_c[n_c] = FA(m->TriGC, ti, 1, nTri); y_c[n_c] = FA(m->TriGC, ti, 2, nTri); n_c++;
      }
      if (shape_stag1(x, y, n_c, x_c, y_c, N0, N1, N2)) break;
      int before = stackN;
      extend_b(m, map, stack, &stackN);
      if (stackN == before) { rc = UFE_ERR_INVALID; goto done; }
    }
    for (int i = 0; i < n_c; ++i) {
      csr_add(&ops[UFE_OP_MAP_B_A], row, i_c[i], N0[i]);
      csr_add(&ops[UFE_OP_DDX_B_A], row, i_c[i], N1[i]);
      csr_add(&ops[UFE_OP_DDY_B_A], row, i_c[i], N2[i]);
    }
    for (int op = UFE_OP_MAP_B_A; op <= UFE_OP_DDY_B_A; ++op) csr_close_row(&ops[op], row);
  }
  for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
  stackN = 0;

  /* -- b_b 2nd order: calc_matrix_operators_mesh_b_b_2nd_order (:612-764) -- */
  for (int op = UFE_OP_M2_DDX_B_B; op <= UFE_OP_M2_D2DY2_B_B; ++op)
    csr_alloc(&ops[op], nTri, nTri, (int64_t)nTri * (m->nC_mem + 1));
  for (int row = 1; row <= nTri; ++row) {
    int ti = row;
    double x = FA(m->TriGC, ti, 1, nTri), y = FA(m->TriGC, ti, 2, nTri);
    for (int i = 0; i < stackN; ++i) map[stack[i] - 1] = 0;
    map[ti - 1] = 1; stackN = 1; stack[0] = ti;
    while (stackN - 1 < 5) {
      int before = stackN;
      extend_b(m, map, stack, &stackN);
      if (stackN - 1 > nmax) { rc = UFE_ERR_CAPACITY; goto done; }
      if (stackN == before) { rc = UFE_ERR_INVALID; goto done; }
    }
    double Ni[5];
    int n_c = 0;
    for (;;) {
      n_c = 0;
      for (int i = 0; i < stackN; ++i) {
        if (n_c == nmax) break;
        int tj = stack[i];
        if (tj == ti) continue;
        i_c[n_c] = tj; x_c[n_c] = FA(m->TriGC, tj, 1, nTri); y_c[n_c] = FA(m->TriGC, tj, 2, nTri); n_c++;
      }
      if (shape_reg2(x, y, n_c, x_c, y_c, Ni, N0)) break;
      int before = stackN;
      extend_b(m, map, stack, &stackN);
      if (stackN == before) { rc = UFE_ERR_INVALID; goto done; }
    }
    for (int k = 0; k < 5; ++k) csr_add(&ops[UFE_OP_M2_DDX_B_B + k], row, row, Ni[k]);
    for (int i = 0; i < n_c; ++i)
      for (int k = 0; k < 5; ++k) csr_add(&ops[UFE_OP_M2_DDX_B_B + k], row, i_c[i], N0[k * n_c + i]);
    for (int op = UFE_OP_M2_DDX_B_B; op <= UFE_OP_M2_D2DY2_B_B; ++op) csr_close_row(&ops[op], row);
  }

done:
  free(map); free(stack); free(i_c); free(x_c); free(y_c); free(N0);
  if (rc != 0)
    for (int op = 0; op < UFE_OP_COUNT; ++op) orc_csr_free(&ops[op]);
  return rc;
}

/* ---------------------------------------------------------------------------------------- */
/* SpMV: multiply_CSR_matrix_with_vector_1D (CSR_matrix_vector_multiplication.f90:266-278);
 * the 2-D form loops over columns (:355-359). */
void orc_spmv(const orc_csr *A, const double *x, double *y, int32_t ncols) {
  for (int32_t c = 0; c < ncols; ++c) {
    const double *xc = x + (int64_t)c * A->n;
    double *yc = y + (int64_t)c * A->m;
#pragma omp parallel for schedule(static) if (A->m > 20000)
    for (int32_t i = 1; i <= A->m; ++i) {
      double s = 0.0;
      for (int32_t k = A->ptr[i - 1]; k <= A->ptr[i] - 1; ++k)
        s = s + A->val[k - 1] * xc[A->ind[k - 1] - 1];
      yc[i - 1] = s;
    }
  }
}

/* ---------------------------------------------------------------------------------------- */
/* stiffness matrix: solve_linearised_SSA_DIVA.f90:58-153 with the row routines at :180-641 */

static int bc_choice(const ufe_solver_params *p, int TriBI, int uv) {
  switch (TriBI) {
    case 1: case 2: return uv == 1 ? p->BC_u_north : p->BC_v_north;
    case 3: case 4: return uv == 1 ? p->BC_u_east : p->BC_v_east;
    case 5: case 6: return uv == 1 ? p->BC_u_south : p->BC_v_south;
    case 7: case 8: return uv == 1 ? p->BC_u_west : p->BC_v_west;
    default: return -1;
  }
}

/* find_ti_copy_SSA_icestream_infinite (src/UPSY/mesh/mesh_utilities.f90:2681-2729) for triangle
 * ti (1-based): the point at the triangle's y, one third (x < 0) or two thirds across the domain;
 * the vertex whose Voronoi cell contains it (find_containing_vertex, :1368-1416: a greedy walk over
 * vertex neighbours, which on a Delaunay mesh ends at the nearest vertex -- taken here by a scan);
 * that vertex's triangles with weights 1/dist^2, normalised by their sum.  Returns the count. */
static int icestream_copy(const ufe_mesh_desc *m, int ti, int32_t *tj_out, double *w_out) {
  const int nV = m->nV, nTri = m->nTri;
  double xmin = m->V[0], xmax = m->V[0];
  for (int v = 1; v < nV; ++v) { if (m->V[v] < xmin) xmin = m->V[v]; if (m->V[v] > xmax) xmax = m->V[v]; }
  const double gx = m->TriGC[ti - 1], gy = m->TriGC[nTri + ti - 1];
  const double px = (gx < 0.0) ? xmin + (xmax - xmin) * 1.0 / 3.0 : xmin + (xmax - xmin) * 2.0 / 3.0;
  const double py = gy;
  int vi = 0;
  double best = 0.0;
  for (int v = 0; v < nV; ++v) {
    const double dx = m->V[v] - px, dy = m->V[nV + v] - py, d = dx * dx + dy * dy;
    if (v == 0 || d < best) { best = d; vi = v; }
  }
  const int n = m->niTri[vi];
  double sum = 0.0;
  for (int iti = 0; iti < n; ++iti) {
    const int tj = m->iTri[(int64_t)iti * nV + vi];
    const double dist = norm2_2(px - m->TriGC[tj - 1], py - m->TriGC[nTri + tj - 1]);
    tj_out[iti] = tj;
    w_out[iti] = 1.0 / (dist * dist);
  }
  for (int iti = 0; iti < n; ++iti) sum = sum + w_out[iti];
  for (int iti = 0; iti < n; ++iti) w_out[iti] = w_out[iti] / sum;
  return n;
}

int32_t orc_assemble_linearised(const ufe_mesh_desc *m, const orc_csr *ops, const ufe_solver_params *p,
                                const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                                const double *beta_b, const double *tau_dx_b, const double *tau_dy_b,
                                const double *u_prev, const double *v_prev,
                                const ufe_bc_prescribed *bc, orc_csr *A, double *bb) {
  (void)v_prev;
  const int nTri = m->nTri;
  const orc_csr *Mx = &ops[UFE_OP_M2_DDX_B_B], *My = &ops[UFE_OP_M2_DDY_B_B];
  const orc_csr *Mxx = &ops[UFE_OP_M2_D2DX2_B_B], *Mxy = &ops[UFE_OP_M2_D2DXDY_B_B];
  const orc_csr *Myy = &ops[UFE_OP_M2_D2DY2_B_B];
  if (csr_alloc(A, 2 * nTri, 2 * nTri, Mx->nnz * 4) != 0) return UFE_ERR_CAPACITY;
  for (int row = 1; row <= 2 * nTri; ++row) {
    int ti = (row + 1) / 2;            /* n2tiuv(row,1) */
    int uv = row - 2 * (ti - 1);       /* n2tiuv(row,2) */
    if (bc && bc->mask_b && bc->mask_b[ti - 1] == 1) {
      csr_add(A, row, row, 1.0);
      bb[row - 1] = (uv == 1) ? bc->u_b[ti - 1] : bc->v_b[ti - 1];
    } else if (m->TriBI[ti - 1] > 0) {
      int choice = bc_choice(p, m->TriBI[ti - 1], uv);
      if (choice == UFE_BC_INFINITE) {
        int n_nb = 0;
        for (int n = 1; n <= 3; ++n) {
          int tj = FA(m->TriC, ti, n, nTri);
          if (tj == 0) continue;
          n_nb++;
          csr_add(A, row, 2 * (tj - 1) + uv, 1.0);
        }
        if (n_nb == 0) return UFE_ERR_INVALID;
        csr_add(A, row, row, -1.0 * (double)n_nb);
        bb[row - 1] = 0.0;
      } else if (choice == UFE_BC_ZERO) {
        csr_add(A, row, row, 1.0);
        bb[row - 1] = 0.0;
      } else if (choice == UFE_BC_INFINITE_SSA_ICESTREAM && uv == 1) {
        /* solve_linearised_SSA_DIVA.f90:562-578 */
        int32_t tjs[64];
        double ws[64];
        if (m->nC_mem > 64) return UFE_ERR_CAPACITY;
        const int n = icestream_copy(m, ti, tjs, ws);
        csr_add(A, row, row, 1.0);
        double u_fixed = 0.0;
        for (int k = 0; k < n; ++k) u_fixed = u_fixed + ws[k] * u_prev[tjs[k] - 1];
        u_fixed = (p->visc_it_relax * u_fixed) + ((1.0 - p->visc_it_relax) * u_prev[ti - 1]);
        bb[row - 1] = u_fixed;
      } else {
        return UFE_ERR_INVALID;
      }
    } else {
      double N = N_b[ti - 1], dNx = dN_dx_b[ti - 1], dNy = dN_dy_b[ti - 1];
      double beta = beta_b[ti - 1];
      int k1 = Mx->ptr[ti - 1], k2 = Mx->ptr[ti] - 1;
      for (int k = k1; k <= k2; ++k) {
        int tj = Mx->ind[k - 1];
        double x_ = Mx->val[k - 1], y_ = My->val[k - 1];
        double xx = Mxx->val[k - 1], xy = Mxy->val[k - 1], yy = Myy->val[k - 1];
        double Au, Av;
        if (p->do_include_SSADIVA_crossterms) {
          if (uv == 1) {
            Au = 4.0 * N * xx + 4.0 * dNx * x_ + N * yy + dNy * y_;
            if (tj == ti) Au = Au - beta;
            Av = 3.0 * N * xy + 2.0 * dNx * y_ + dNy * x_;
          } else {
            Av = 4.0 * N * yy + 4.0 * dNy * y_ + N * xx + dNx * x_;
            if (tj == ti) Av = Av - beta;
            Au = 3.0 * N * xy + 2.0 * dNy * x_ + dNx * y_;
          }
        } else {
          if (uv == 1) {
            Au = 4.0 * xx + yy;
            if (tj == ti) Au = Au - beta / N;
            Av = 3.0 * xy;
          } else {
            Av = 4.0 * yy + xx;
            if (tj == ti) Av = Av - beta / N;
            Au = 3.0 * xy;
          }
        }
        csr_add(A, row, 2 * (tj - 1) + 1, Au);
        csr_add(A, row, 2 * (tj - 1) + 2, Av);
      }
      if (p->do_include_SSADIVA_crossterms)
        bb[row - 1] = (uv == 1) ? -tau_dx_b[ti - 1] : -tau_dy_b[ti - 1];
      else
        bb[row - 1] = (uv == 1) ? -tau_dx_b[ti - 1] / N : -tau_dy_b[ti - 1] / N;
    }
    csr_close_row(A, row);
  }
  return UFE_OK;
}

/* ---------------------------------------------------------------------------------------- */
/* Krylov: PETSc KSPSolve with -ksp_type bcgs -pc_type jacobi (left preconditioning, the
 * preconditioned residual norm, KSPConvergedDefault: ||r|| <= max(rtol*||D^-1 b||, abstol),
 * divergence when ||r|| >= 1e4 ||r0|| or NaN).  PETSc is not part of the reference tree; this is
 * the published BiCGStab recurrence in the form of PETSc's src/ksp/ksp/impls/bcgs/bcgs.c. */

/* Dot product summed in fixed chunks of 4096 (each chunk sequentially, then the chunk sums in
 * order), so the result does not depend on the number of OpenMP threads. */
static double dot(const double *a, const double *b, int64_t n) {
  const int64_t CH = 4096;
  const int64_t nch = (n + CH - 1) / CH;
  double part_stack[64];
  double *part = nch <= 64 ? part_stack : (double *)malloc(sizeof(double) * (size_t)nch);
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int64_t c = 0; c < nch; ++c) {
    double s = 0.0;
    int64_t e = (c + 1) * CH < n ? (c + 1) * CH : n;
    for (int64_t i = c * CH; i < e; ++i) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0.0;
  for (int64_t c = 0; c < nch; ++c) s += part[c];
  if (part != part_stack) free(part);
  return s;
}

int32_t orc_bicgstab(const orc_csr *A, const double *b, double *x, double rtol, double abstol,
                     int32_t max_it, int32_t *its_out) {
  const int64_t n = A->m;
  double *dinv = (double *)malloc(sizeof(double) * n * 8);
  double *R = dinv + n, *RP = R + n, *V = RP + n, *T = V + n, *S = T + n, *P = S + n, *W = P + n;
  int32_t status = UFE_OK;
  /* Jacobi: inverse diagonal, 1 where the diagonal is zero (PCJACOBI's default) */
  for (int32_t i = 1; i <= A->m; ++i) {
    double d = 0.0;
    for (int32_t k = A->ptr[i - 1]; k <= A->ptr[i] - 1; ++k)
      if (A->ind[k - 1] == i) d += A->val[k - 1];
    dinv[i - 1] = (d != 0.0) ? 1.0 / d : 1.0;
  }
  /* R = D^-1 (b - A x) */
  orc_spmv(A, x, W, 1);
  for (int64_t i = 0; i < n; ++i) R[i] = dinv[i] * (b[i] - W[i]);
  double bnorm = 0.0;
  for (int64_t i = 0; i < n; ++i) { double t = dinv[i] * b[i]; bnorm += t * t; }
  bnorm = sqrt(bnorm);
  double dp = sqrt(dot(R, R, n));
  double rnorm0 = bnorm != 0.0 ? bnorm : dp;
  double ttol = fmax(rtol * rnorm0, abstol);
  int32_t its = 0;
  if (dp <= ttol) { *its_out = 0; free(dinv); return UFE_OK; }
  memcpy(RP, R, sizeof(double) * n);
  double rhoold = 1.0, alpha = 1.0, omegaold = 1.0;
  memset(P, 0, sizeof(double) * n);
  memset(V, 0, sizeof(double) * n);
  for (;;) {
    double rho = dot(R, RP, n);
    if (rho == 0.0 || isnan(rho)) { status = UFE_ERR_DIVERGED; break; }
    double beta = (rho / rhoold) * (alpha / omegaold);
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) P[i] = R[i] - beta * omegaold * V[i] + beta * P[i];
    orc_spmv(A, P, W, 1);
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) V[i] = dinv[i] * W[i];
    double d1 = dot(V, RP, n);
    if (d1 == 0.0 || isnan(d1)) { status = UFE_ERR_DIVERGED; break; }
    alpha = rho / d1;
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) S[i] = R[i] - alpha * V[i];
    orc_spmv(A, S, W, 1);
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) T[i] = dinv[i] * W[i];
    d1 = dot(S, T, n);
    double d2 = dot(T, T, n);
    if (d2 == 0.0) {
      /* t = 0: if s = 0 as well, x + alpha p is the solution; otherwise a breakdown (bcgs.c) */
      if (dot(S, S, n) != 0.0) { status = UFE_ERR_DIVERGED; break; }
      for (int64_t i = 0; i < n; ++i) x[i] = x[i] + alpha * P[i] + 0.0 * S[i];
      its++;
      break;
    }
    double omega = d1 / d2;
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + alpha * P[i] + omega * S[i];
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int64_t i = 0; i < n; ++i) R[i] = S[i] - omega * T[i];
    dp = sqrt(dot(R, R, n));
    rhoold = rho; omegaold = omega;
    its++;
    if (isnan(dp)) { status = UFE_ERR_NAN; break; }
    if (dp <= ttol) break;
    if (dp >= 1e4 * rnorm0) { status = UFE_ERR_DIVERGED; break; }
    if (its >= max_it) { status = UFE_WARN_KRYLOV_MAXIT; break; }
  }
  *its_out = its;
  free(dinv);
  return status;
}

/* ---------------------------------------------------------------------------------------- */
/* physics */

/* vertical_average (mesh_zeta.f90:257-283) */
static double vertical_average(const double *zeta, int nz, const double *f, int64_t stride) {
  double a = 0.0;
  for (int k = 1; k <= nz - 1; ++k)
    a = a + 0.5 * (f[(int64_t)k * stride] + f[(int64_t)(k - 1) * stride]) * (zeta[k] - zeta[k - 1]);
  return a;
}

/* integrate_from_zeta_is_one_to_zeta_is_zetap (mesh_zeta.f90:163-193) */
static void integrate_one_to_zetap(const double *zeta, int nz, const double *f, double *out) {
  out[nz - 1] = 0.0;
  for (int k = nz - 1; k >= 1; --k)
    out[k - 1] = out[k] - 0.5 * (f[k] + f[k - 1]) * (zeta[k] - zeta[k - 1]);
}

/* calc_effective_viscosity_Glen_2D (constitutive_equation.f90:25-50) */
static double glen_2d(double eps0, double ux, double uy, double vx, double vy, double A, double n) {
  double e = ux * ux + vy * vy + ux * vy + 0.25 * ((uy + vx) * (uy + vx)) + eps0;
  return 0.5 * pow(A, -1.0 / n) * pow(e, (1.0 - n) / (2.0 * n));
}

/* calc_effective_viscosity_Glen_3D_uv_only (constitutive_equation.f90:52-80) */
static double glen_3d(double eps0, double ux, double uy, double uz, double vx, double vy, double vz,
                      double A, double n) {
  double e = ux * ux + vy * vy + ux * vy + 0.25 * ((uy + vx) * (uy + vx)) + 0.25 * (uz * uz + vz * vz) + eps0;
  return 0.5 * pow(A, -1.0 / n) * pow(e, (1.0 - n) / (2.0 * n));
}

/* The velocity-dependent part of calc_basal_friction_coefficient (sliding_laws.f90:25-81) and
 * the law it dispatches to: Weertman :86-130, Coulomb :132-186, Budd :188-242, Tsai2015 :244-297,
 * Schoof2005 :299-351; then min(slid_beta_max, beta) (:76). */
static double sliding_beta(const ufe_solver_params *p, const ufe_ice_state *ice, int vi0,
                           double u, double v) {
  double uabs = sqrt(p->slid_delta_v * p->slid_delta_v + u * u + v * v);
  double m = p->slid_Weertman_m, beta = 0.0;
  switch (p->choice_sliding_law) {
    case UFE_SLIDING_NO_SLIDING: beta = 0.0; break;
    case UFE_SLIDING_WEERTMAN:
      beta = ice->beta_sq[vi0] * pow(uabs, 1.0 / m - 1.0); break;
    case UFE_SLIDING_COULOMB:
      beta = ice->till_yield_stress[vi0] / uabs; break;
    case UFE_SLIDING_BUDD:
      beta = ice->till_yield_stress[vi0] * pow(uabs, p->slid_Budd_q_plastic - 1.0) /
             pow(p->slid_Budd_u_threshold, p->slid_Budd_q_plastic);
      break;
    case UFE_SLIDING_TSAI2015:
      beta = fmin(ice->alpha_sq[vi0] * ice->effective_pressure[vi0],
                  ice->beta_sq[vi0] * pow(uabs, 1.0 / m)) * pow(uabs, -1.0);
      break;
    case UFE_SLIDING_SCHOOF2005: {
      double b = ice->beta_sq[vi0], aN = ice->alpha_sq[vi0] * ice->effective_pressure[vi0];
      beta = ((b * pow(uabs, 1.0 / m) * ice->alpha_sq[vi0] * ice->effective_pressure[vi0]) /
              pow(pow(b, m) * uabs + pow(aN, m), 1.0 / m)) * pow(uabs, -1.0);
      break;
    }
    case UFE_SLIDING_ZOET_IVERSON:   /* calc_sliding_law_ZoetIverson, :399-400 */
      beta = ice->till_yield_stress[vi0] * (pow(uabs, 1.0 / p->slid_ZI_p - 1.0)) *
             (pow(uabs + p->slid_ZI_ut, -1.0 / p->slid_ZI_p));
      break;
    case UFE_SLIDING_IDEALISED_SSA_ICESTREAM:   /* :477; the yield stress from schoof_yield_stress */
      beta = ice->till_yield_stress[vi0] / uabs;
      break;
    default: beta = 0.0;
  }
  return fmin(p->slid_beta_max, beta);
}

/* apply_velocity_limits (SSA_DIVA_utilities.f90:109-136) */
static void velocity_limits(int nTri, double vel_max, double *u, double *v) {
  for (int ti = 0; ti < nTri; ++ti) {
    double uabs = sqrt(u[ti] * u[ti] + v[ti] * v[ti]);
    if (uabs > vel_max) { u[ti] = u[ti] * vel_max / uabs; v[ti] = v[ti] * vel_max / uabs; }
  }
}

/* relax_viscosity_iterations (SSA_DIVA_utilities.f90:84-107) */
static void relax(int nTri, double r, double *u, double *v, const double *up, const double *vp) {
  for (int ti = 0; ti < nTri; ++ti) {
    u[ti] = (r * u[ti]) + ((1.0 - r) * up[ti]);
    v[ti] = (r * v[ti]) + ((1.0 - r) * vp[ti]);
  }
}

/* calc_L2_norm_uv (SSA_DIVA_utilities.f90:138-184) */
static double l2_norm(int nTri, const double *u, const double *v, const double *up, const double *vp) {
  double r1 = 0.0, r2 = 0.0;
  for (int ti = 0; ti < nTri; ++ti) {
    r1 = r1 + (u[ti] - up[ti]) * (u[ti] - up[ti]);
    r1 = r1 + (v[ti] - vp[ti]) * (v[ti] - vp[ti]);
    r2 = r2 + (u[ti] + up[ti]) * (u[ti] + up[ti]);
    r2 = r2 + (v[ti] + vp[ti]) * (v[ti] + vp[ti]);
  }
  return 2.0 * r1 / fmax(r2, 1e-8);
}

/* The linear solve of one Picard iteration: solve_SSA_DIVA_linearised (:23-178). */
static int32_t linear_solve(const ufe_mesh_desc *m, const orc_csr *ops, const ufe_solver_params *p,
                            double *u, double *v, const double *N_b, const double *dNx, const double *dNy,
                            const double *beta_b, const double *tdx, const double *tdy,
                            double *up, double *vp, const ufe_bc_prescribed *bc, int32_t *its) {
  const int nTri = m->nTri;
  memcpy(up, u, sizeof(double) * nTri);
  memcpy(vp, v, sizeof(double) * nTri);
  orc_csr A;
  double *bb = (double *)malloc(sizeof(double) * 2 * nTri);
  double *xx = (double *)malloc(sizeof(double) * 2 * nTri);
  int32_t rc = orc_assemble_linearised(m, ops, p, N_b, dNx, dNy, beta_b, tdx, tdy, up, vp, bc, &A, bb);
  if (rc != UFE_OK) { free(bb); free(xx); orc_csr_free(&A); return rc; }
  for (int ti = 0; ti < nTri; ++ti) {
    xx[2 * ti] = (p->krylov_initial_guess == UFE_X0_CURRENT) ? u[ti] : 0.0;
    xx[2 * ti + 1] = (p->krylov_initial_guess == UFE_X0_CURRENT) ? v[ti] : 0.0;
  }
  rc = orc_bicgstab(&A, bb, xx, p->stress_balance_PETSc_rtol, p->stress_balance_PETSc_abstol,
                    p->krylov_max_it, its);
  for (int ti = 0; ti < nTri; ++ti) { u[ti] = xx[2 * ti]; v[ti] = xx[2 * ti + 1]; }
  free(bb); free(xx); orc_csr_free(&A);
  return rc;
}

static int any_grounded(const ufe_mesh_desc *m, const ufe_ice_state *ice) {
  for (int vi = 0; vi < m->nV; ++vi) if (ice->mask_grounded_ice[vi]) return 1;
  return 0;
}

/* Picard divergence control shared by SSA_main.f90:196-213 and DIVA_main.f90:211-228. */
static int32_t picard_control(double L2, double L2_prev, int *nit_diverg, double *relax_applied,
                              double *eps0_applied) {
  if (L2 > L2_prev) (*nit_diverg)++; else *nit_diverg = 0;
  if (*nit_diverg > 2) {
    *nit_diverg = 0;
    *relax_applied = *relax_applied * 0.9;
    *eps0_applied = *eps0_applied * 1.2;
  }
  if (*relax_applied <= 0.05 || *eps0_applied >= 1e-5) {
    if (*relax_applied < 0.05) return UFE_ERR_DIVERGED;
    else if (*eps0_applied > 1e-5) return UFE_ERR_DIVERGED;
  }
  return UFE_OK;
}

/* calc_ice_rheology_Glen (constitutive_equation.f90:84-163): A per vertex and layer, uniform or
 * the Arrhenius relation of Huybrechts (1992), then the enhancement factors ('separate' or
 * 'interp').  Called once per solve: the reference recomputes the same field every Picard
 * iteration. */
static void flow_factor(const ufe_mesh_desc *m, const ufe_solver_params *p, const ufe_ice_state *ice, double *A) {
  const int nV = m->nV, nz = m->nz;
  const double T_switch = 263.15, A_low_temp = 1.14E-05, A_high_temp = 5.47E+10;
  const double Q_low_temp = 6.0E+04, Q_high_temp = 13.9E+04;
  for (int vi = 0; vi < nV; ++vi)
    for (int k = 0; k < nz; ++k) {
      const int64_t ix = (int64_t)k * nV + vi;
      if (p->choice_ice_rheology_Glen == UFE_RHEOLOGY_UNIFORM) {
        A[ix] = p->uniform_Glens_flow_factor;
      } else if (ice->Ti[ix] < T_switch) {
        A[ix] = A_low_temp * exp(-Q_low_temp / (R_GAS * ice->Ti[ix]));
      } else {
        A[ix] = A_high_temp * exp(-Q_high_temp / (R_GAS * ice->Ti[ix]));
      }
    }
  for (int vi = 0; vi < nV; ++vi) {
    const int gr = ice->mask_grounded_ice[vi] != 0;
    const int fl = ice->mask_floating_ice && ice->mask_floating_ice[vi] != 0;
    double f = 1.0;
    int apply = 0;
    if (p->choice_enhancement_factor_transition == UFE_ENH_INTERP && ice->Hi[vi] > 0.0 && ice->Hib[vi] < ice->SL[vi]) {
      f = ice->fraction_gr[vi] * p->m_enh_sheet + (1.0 - ice->fraction_gr[vi]) * p->m_enh_shelf;
      apply = 1;
    } else if (gr) {
      f = p->m_enh_sheet; apply = 1;
    } else if (fl) {
      f = p->m_enh_shelf; apply = 1;
    }
    if (apply)
      for (int k = 0; k < nz; ++k) A[(int64_t)k * nV + vi] = A[(int64_t)k * nV + vi] * f;
  }
}

/* The till yield stress of Schoof's (2006) ice stream at every vertex (Schoof2006_icestream,
 * src/UPSY/basic/analytical_solutions/Schoof_SSA_solution.f90:15-64, as
 * calc_sliding_law_idealised_SSA_icestream calls it, sliding_laws.f90:469-473). */
static void schoof_yield_stress(const ufe_mesh_desc *m, const ufe_solver_params *p, double *tys) {
  const double f = -ICE_DENSITY * GRAV * p->SSA_icestream_Hi * p->SSA_icestream_dhdx;
  for (int vi = 0; vi < m->nV; ++vi) {
    const double y = m->V[m->nV + vi];
    tys[vi] = f * pow(fabs(y / p->SSA_icestream_L), p->SSA_icestream_m);
  }
}

/* The ice state a solve reads: the flow factor of calc_ice_rheology_Glen and, for the idealised
 * SSA_icestream law, Schoof's yield stress in place of till_yield_stress.  *owned receives the
 * allocation to free. */
static const ufe_ice_state *solve_ice_state(const ufe_mesh_desc *m, const ufe_solver_params *p,
                                            const ufe_ice_state *ice, ufe_ice_state *eff, double **owned) {
  *eff = *ice;
  *owned = NULL;
  const int rheo = p->choice_ice_rheology_Glen != UFE_RHEOLOGY_INPUT;
  const int ideal = p->choice_sliding_law == UFE_SLIDING_IDEALISED_SSA_ICESTREAM;
  if (!rheo && !ideal) return ice;
  double *buf = (double *)malloc(sizeof(double) * ((size_t)m->nV * m->nz + (size_t)m->nV));
  *owned = buf;
  if (rheo) { flow_factor(m, p, ice, buf); eff->A_flow = buf; }
  if (ideal) { schoof_yield_stress(m, p, buf + (size_t)m->nV * m->nz); eff->till_yield_stress = buf + (size_t)m->nV * m->nz; }
  return eff;
}

/* solve_SSA (SSA_main.f90:87-242) with calc_driving_stress (SSA_DIVA_utilities.f90:21-57),
 * calc_horizontal_strain_rates (:59-82), calc_effective_viscosity (SSA_main.f90:339-392),
 * calc_vertically_averaged_flow_parameter (:312-337) and
 * calc_applied_basal_friction_coefficient (:394-430). */
int32_t orc_solve_ssa(const ufe_mesh_desc *m, const orc_csr *ops, const ufe_solver_params *p,
                      const ufe_ice_state *ice, const ufe_bc_prescribed *bc,
                      double *u_b, double *v_b, ufe_solve_stats *st, const double *eta_first) {
  const int nV = m->nV, nTri = m->nTri, nz = m->nz;
  ufe_solve_stats dummy;
  if (!st) st = &dummy;
  memset(st, 0, sizeof(*st));
  if (!any_grounded(m, ice) || p->choice_sliding_law == UFE_SLIDING_NO_SLIDING) {
    memset(u_b, 0, sizeof(double) * nTri);
    memset(v_b, 0, sizeof(double) * nTri);
    return UFE_OK;
  }
  ufe_ice_state ice_eff;
  double *ice_owned;
  ice = solve_ice_state(m, p, ice, &ice_eff, &ice_owned);
  double *w = (double *)calloc((size_t)(16 * nV + 16 * nTri), sizeof(double));
  double *Hi_b = w, *dHs_dx = Hi_b + nTri, *dHs_dy = dHs_dx + nTri, *tdx = dHs_dy + nTri, *tdy = tdx + nTri;
  double *N_b = tdy + nTri, *dN_dx_b = N_b + nTri, *dN_dy_b = dN_dx_b + nTri, *beta_b = dN_dy_b + nTri;
  double *up = beta_b + nTri, *vp = up + nTri;
  double *ux = vp + nTri, *uy = ux + nV, *vx = uy + nV, *vy = vx + nV, *Avav = vy + nV, *eta = Avav + nV;
  double *N_a = eta + nV, *beta_a = N_a + nV, *ua = beta_a + nV, *va = ua + nV, *tmp = va + nV;
  (void)tmp;
  /* calc_driving_stress */
  orc_spmv(&ops[UFE_OP_MAP_A_B], ice->Hi, Hi_b, 1);
  orc_spmv(&ops[UFE_OP_DDX_A_B], ice->Hs, dHs_dx, 1);
  orc_spmv(&ops[UFE_OP_DDY_A_B], ice->Hs, dHs_dy, 1);
  for (int ti = 0; ti < nTri; ++ti) {
    tdx[ti] = -ICE_DENSITY * GRAV * Hi_b[ti] * dHs_dx[ti];
    tdy[ti] = -ICE_DENSITY * GRAV * Hi_b[ti] * dHs_dy[ti];
  }
  for (int vi = 0; vi < nV; ++vi) Avav[vi] = vertical_average(m->zeta, nz, ice->A_flow + vi, nV);

  const double n_glen = p->Glens_flow_law_exponent;
  double L2 = 1e9, L2_prev;
  int nit_diverg = 0;
  double relax_applied = p->visc_it_relax, eps0_applied = p->Glens_flow_law_epsilon_sq_0;
  int it = 0, converged = 0;
  int32_t status = UFE_OK;
  int32_t n_axb = 0;
  while (!converged) {
    it++;
    /* strain rates */
    orc_spmv(&ops[UFE_OP_DDX_B_A], u_b, ux, 1);
    orc_spmv(&ops[UFE_OP_DDY_B_A], u_b, uy, 1);
    orc_spmv(&ops[UFE_OP_DDX_B_A], v_b, vx, 1);
    orc_spmv(&ops[UFE_OP_DDY_B_A], v_b, vy, 1);
    /* effective viscosity */
    double A_min = 1e-18;
    double eta_max = 0.5 * pow(A_min, -1.0 / n_glen) * pow(eps0_applied, (1.0 - n_glen) / (2.0 * n_glen));
    for (int vi = 0; vi < nV; ++vi) {
      /* eta_first (the learned start's predicted viscosity, no reference counterpart) replaces
       * Glen's law in the first iteration only */
      double e = (eta_first && it == 1) ? eta_first[vi]
                                        : glen_2d(eps0_applied, ux[vi], uy[vi], vx[vi], vy[vi], Avav[vi], n_glen);
      e = fmin(fmax(e, p->visc_eff_min), eta_max);
      eta[vi] = e;
      N_a[vi] = e * fmax(0.1, ice->Hi[vi]);
    }
    orc_spmv(&ops[UFE_OP_MAP_A_B], N_a, N_b, 1);
    orc_spmv(&ops[UFE_OP_DDX_A_B], N_a, dN_dx_b, 1);
    orc_spmv(&ops[UFE_OP_DDY_A_B], N_a, dN_dy_b, 1);
    /* basal friction */
    orc_spmv(&ops[UFE_OP_MAP_B_A], u_b, ua, 1);
    orc_spmv(&ops[UFE_OP_MAP_B_A], v_b, va, 1);
    for (int vi = 0; vi < nV; ++vi) beta_a[vi] = sliding_beta(p, ice, vi, ua[vi], va[vi]);
    orc_spmv(&ops[UFE_OP_MAP_A_B], beta_a, beta_b, 1);
    if (p->do_GL_subgrid_friction)
      for (int ti = 0; ti < nTri; ++ti)
        beta_b[ti] = beta_b[ti] * pow(ice->fraction_gr_b[ti], p->subgrid_friction_exponent_on_B_grid);
    /* linearised solve */
    int32_t its = 0;
    int32_t rc = linear_solve(m, ops, p, u_b, v_b, N_b, dN_dx_b, dN_dy_b, beta_b, tdx, tdy, up, vp, bc, &its);
    n_axb += its;
    /* the reference does not act on PETSc's converged reason: only NaN stops the loop */
    if (rc == UFE_ERR_NAN || rc == UFE_ERR_INVALID) { status = rc; break; }
    if (rc != UFE_OK && status == UFE_OK) status = UFE_WARN_KRYLOV_MAXIT;
    velocity_limits(nTri, p->vel_max, u_b, v_b);
    relax(nTri, relax_applied, u_b, v_b, up, vp);
    L2_prev = L2;
    L2 = l2_norm(nTri, u_b, v_b, up, vp);
    rc = picard_control(L2, L2_prev, &nit_diverg, &relax_applied, &eps0_applied);
    if (rc != UFE_OK) { status = rc; break; }
    converged = L2 < p->visc_it_norm_dUV_tol;
    if (it > p->visc_it_nit) { if (status == UFE_OK) status = UFE_WARN_PICARD_MAXIT; break; }
  }
  st->n_visc_its = it;
  st->n_Axb_its = n_axb;
  st->L2_uv = L2;
  st->visc_it_relax_applied = relax_applied;
  st->status = status;
  free(w);
  free(ice_owned);
  return status;
}

/* solve_DIVA (DIVA_main.f90:88-262) with calc_vertical_shear_strain_rates (:375-410),
 * calc_effective_viscosity (:412-479), calc_F_integrals (:481-520),
 * calc_effective_basal_friction_coefficient (:522-574), calc_basal_shear_stress (:576-598),
 * calc_basal_velocities (:600-627) and calc_3D_velocities (:629-676). */
int32_t orc_solve_diva(const ufe_mesh_desc *m, const orc_csr *ops, const ufe_solver_params *p,
                       const ufe_ice_state *ice, const ufe_bc_prescribed *bc,
                       ufe_diva_state *ds, ufe_solve_stats *st, const double *eta_first) {
  const int nV = m->nV, nTri = m->nTri, nz = m->nz;
  const double *zeta = m->zeta;
  ufe_solve_stats dummy;
  if (!st) st = &dummy;
  memset(st, 0, sizeof(*st));
  const int no_sliding = p->choice_sliding_law == UFE_SLIDING_NO_SLIDING;
  if (!any_grounded(m, ice)) {
    memset(ds->u_vav_b, 0, sizeof(double) * nTri); memset(ds->v_vav_b, 0, sizeof(double) * nTri);
    memset(ds->u_base_b, 0, sizeof(double) * nTri); memset(ds->v_base_b, 0, sizeof(double) * nTri);
    if (ds->u_3D_b) memset(ds->u_3D_b, 0, sizeof(double) * nTri * nz);
    if (ds->v_3D_b) memset(ds->v_3D_b, 0, sizeof(double) * nTri * nz);
    return UFE_OK;
  }
  ufe_ice_state ice_eff;
  double *ice_owned;
  ice = solve_ice_state(m, p, ice, &ice_eff, &ice_owned);
  int64_t n2 = 20 * (int64_t)nV + 20 * (int64_t)nTri + 8 * (int64_t)nz * (nV + nTri) + 4 * nz;
  double *w = (double *)calloc((size_t)n2, sizeof(double));
  double *Hi_b = w, *dHs_dx = Hi_b + nTri, *dHs_dy = dHs_dx + nTri, *tdx = dHs_dy + nTri, *tdy = tdx + nTri;
  double *N_b = tdy + nTri, *dN_dx_b = N_b + nTri, *dN_dy_b = dN_dx_b + nTri, *beta_eff_b = dN_dy_b + nTri;
  double *bfc_b = beta_eff_b + nTri, *up = bfc_b + nTri, *vp = up + nTri, *F2b1 = vp + nTri;
  double *ux = F2b1 + nTri, *uy = ux + nV, *vx = uy + nV, *vy = vx + nV, *eta_vav = vy + nV;
  double *N_a = eta_vav + nV, *beta_a = N_a + nV, *beta_eff_a = beta_a + nV, *ua = beta_eff_a + nV, *va = ua + nV;
  double *F2a1 = va + nV;
  double *du_dz_b = F2a1 + nV;                     /* nTri x nz */
  double *dv_dz_b = du_dz_b + (int64_t)nTri * nz;  /* nTri x nz */
  double *du_dz_a = dv_dz_b + (int64_t)nTri * nz;  /* nV x nz */
  double *dv_dz_a = du_dz_a + (int64_t)nV * nz;
  double *eta_3D_a = dv_dz_a + (int64_t)nV * nz;
  double *F1_3D_a = eta_3D_a + (int64_t)nV * nz;
  double *F2_3D_a = F1_3D_a + (int64_t)nV * nz;
  double *F1_3D_b = F2_3D_a + (int64_t)nV * nz;    /* nTri x nz */
  double *prof = F1_3D_b + (int64_t)nTri * nz;     /* nz */
  double *intg = prof + nz;

  orc_spmv(&ops[UFE_OP_MAP_A_B], ice->Hi, Hi_b, 1);
  orc_spmv(&ops[UFE_OP_DDX_A_B], ice->Hs, dHs_dx, 1);
  orc_spmv(&ops[UFE_OP_DDY_A_B], ice->Hs, dHs_dy, 1);
  for (int ti = 0; ti < nTri; ++ti) {
    tdx[ti] = -ICE_DENSITY * GRAV * Hi_b[ti] * dHs_dx[ti];
    tdy[ti] = -ICE_DENSITY * GRAV * Hi_b[ti] * dHs_dy[ti];
  }
  const double n_glen = p->Glens_flow_law_exponent;
  const double h_floor_sp = (double)0.1f;  /* max(0.1, Hi) with a default-real literal, DIVA_main.f90:468 */
  double L2 = 1e9, L2_prev;
  int nit_diverg = 0;
  double relax_applied = p->visc_it_relax, eps0_applied = p->Glens_flow_law_epsilon_sq_0;
  int it = 0, converged = 0;
  int32_t status = UFE_OK, n_axb = 0;
  while (!converged) {
    it++;
    /* calc_horizontal_strain_rates */
    orc_spmv(&ops[UFE_OP_DDX_B_A], ds->u_vav_b, ux, 1);
    orc_spmv(&ops[UFE_OP_DDY_B_A], ds->u_vav_b, uy, 1);
    orc_spmv(&ops[UFE_OP_DDX_B_A], ds->v_vav_b, vx, 1);
    orc_spmv(&ops[UFE_OP_DDY_B_A], ds->v_vav_b, vy, 1);
    /* calc_vertical_shear_strain_rates */
    for (int k = 0; k < nz; ++k)
      for (int ti = 0; ti < nTri; ++ti) {
        double e = fmax(p->visc_eff_min, ds->eta_3D_b[(int64_t)k * nTri + ti]);
        du_dz_b[(int64_t)k * nTri + ti] = ds->tau_bx_b[ti] * zeta[k] / e;
        dv_dz_b[(int64_t)k * nTri + ti] = ds->tau_by_b[ti] * zeta[k] / e;
      }
    orc_spmv(&ops[UFE_OP_MAP_B_A], du_dz_b, du_dz_a, nz);
    orc_spmv(&ops[UFE_OP_MAP_B_A], dv_dz_b, dv_dz_a, nz);
    /* calc_effective_viscosity */
    double A_min = 1e-18;
    double eta_max = 0.5 * pow(A_min, -1.0 / n_glen) * pow(eps0_applied, (1.0 - n_glen) / (2.0 * n_glen));
    for (int vi = 0; vi < nV; ++vi)
      for (int k = 0; k < nz; ++k) {
        int64_t ix = (int64_t)k * nV + vi;
        /* eta_first: a depth-uniform predicted viscosity in the first iteration only (see SSA) */
        double e = (eta_first && it == 1)
                       ? eta_first[vi]
                       : glen_3d(eps0_applied, ux[vi], uy[vi], du_dz_a[ix], vx[vi], vy[vi], dv_dz_a[ix],
                                 ice->A_flow[ix], n_glen);
        eta_3D_a[ix] = fmin(fmax(e, p->visc_eff_min), eta_max);
      }
    orc_spmv(&ops[UFE_OP_MAP_A_B], eta_3D_a, ds->eta_3D_b, nz);
    for (int vi = 0; vi < nV; ++vi) {
      eta_vav[vi] = vertical_average(zeta, nz, eta_3D_a + vi, nV);
      N_a[vi] = eta_vav[vi] * fmax(h_floor_sp, ice->Hi[vi]);
    }
    orc_spmv(&ops[UFE_OP_MAP_A_B], N_a, N_b, 1);
    orc_spmv(&ops[UFE_OP_DDX_A_B], N_a, dN_dx_b, 1);
    orc_spmv(&ops[UFE_OP_DDY_A_B], N_a, dN_dy_b, 1);
    /* calc_F_integrals */
    for (int vi = 0; vi < nV; ++vi) {
      double h = fmax(0.1, ice->Hi[vi]);
      for (int k = 0; k < nz; ++k) prof[k] = zeta[k] / eta_3D_a[(int64_t)k * nV + vi];
      integrate_one_to_zetap(zeta, nz, prof, intg);
      for (int k = 0; k < nz; ++k) F1_3D_a[(int64_t)k * nV + vi] = -h * intg[k];
      for (int k = 0; k < nz; ++k) prof[k] = zeta[k] * zeta[k] / eta_3D_a[(int64_t)k * nV + vi];
      integrate_one_to_zetap(zeta, nz, prof, intg);
      for (int k = 0; k < nz; ++k) F2_3D_a[(int64_t)k * nV + vi] = -h * intg[k];
    }
    orc_spmv(&ops[UFE_OP_MAP_A_B], F1_3D_a, F1_3D_b, nz);
    for (int vi = 0; vi < nV; ++vi) F2a1[vi] = F2_3D_a[vi];
    orc_spmv(&ops[UFE_OP_MAP_A_B], F2a1, F2b1, 1);   /* layer 1 of map_a_b_3D(F2_3D_a) */
    /* calc_effective_basal_friction_coefficient */
    orc_spmv(&ops[UFE_OP_MAP_B_A], ds->u_base_b, ua, 1);
    orc_spmv(&ops[UFE_OP_MAP_B_A], ds->v_base_b, va, 1);
    for (int vi = 0; vi < nV; ++vi) {
      beta_a[vi] = sliding_beta(p, ice, vi, ua[vi], va[vi]);
      if (no_sliding) beta_eff_a[vi] = 1.0 / F2a1[vi];
      else beta_eff_a[vi] = beta_a[vi] / (1.0 + beta_a[vi] * F2a1[vi]);
    }
    orc_spmv(&ops[UFE_OP_MAP_A_B], beta_a, bfc_b, 1);
    orc_spmv(&ops[UFE_OP_MAP_A_B], beta_eff_a, beta_eff_b, 1);
    if (p->do_GL_subgrid_friction)
      for (int ti = 0; ti < nTri; ++ti)
        beta_eff_b[ti] = beta_eff_b[ti] * pow(ice->fraction_gr_b[ti], p->subgrid_friction_exponent_on_B_grid);
    /* solve */
    int32_t its = 0;
    int32_t rc = linear_solve(m, ops, p, ds->u_vav_b, ds->v_vav_b, N_b, dN_dx_b, dN_dy_b, beta_eff_b,
                              tdx, tdy, up, vp, bc, &its);
    n_axb += its;
    /* the reference does not act on PETSc's converged reason: only NaN stops the loop */
    if (rc == UFE_ERR_NAN || rc == UFE_ERR_INVALID) { status = rc; break; }
    if (rc != UFE_OK && status == UFE_OK) status = UFE_WARN_KRYLOV_MAXIT;
    velocity_limits(nTri, p->vel_max, ds->u_vav_b, ds->v_vav_b);
    relax(nTri, relax_applied, ds->u_vav_b, ds->v_vav_b, up, vp);
    /* calc_basal_velocities */
    for (int ti = 0; ti < nTri; ++ti) {
      if (no_sliding) { ds->u_base_b[ti] = 0.0; ds->v_base_b[ti] = 0.0; }
      else {
        ds->u_base_b[ti] = ds->u_vav_b[ti] / (1.0 + bfc_b[ti] * F2b1[ti]);
        ds->v_base_b[ti] = ds->v_vav_b[ti] / (1.0 + bfc_b[ti] * F2b1[ti]);
      }
    }
    /* calc_basal_shear_stress */
    for (int ti = 0; ti < nTri; ++ti) {
      ds->tau_bx_b[ti] = ds->u_vav_b[ti] * beta_eff_b[ti];
      ds->tau_by_b[ti] = ds->v_vav_b[ti] * beta_eff_b[ti];
    }
    L2_prev = L2;
    L2 = l2_norm(nTri, ds->u_vav_b, ds->v_vav_b, up, vp);
    rc = picard_control(L2, L2_prev, &nit_diverg, &relax_applied, &eps0_applied);
    if (rc != UFE_OK) { status = rc; break; }
    converged = L2 < p->visc_it_norm_dUV_tol;
    if (it > p->visc_it_nit) { if (status == UFE_OK) status = UFE_WARN_PICARD_MAXIT; break; }
  }
  /* calc_3D_velocities */
  if (status >= 0 && ds->u_3D_b && ds->v_3D_b) {
    for (int k = 0; k < nz; ++k)
      for (int ti = 0; ti < nTri; ++ti) {
        int64_t ix = (int64_t)k * nTri + ti;
        if (no_sliding) {
          ds->u_3D_b[ix] = ds->tau_bx_b[ti] * F1_3D_b[ix];
          ds->v_3D_b[ix] = ds->tau_by_b[ti] * F1_3D_b[ix];
        } else {
          ds->u_3D_b[ix] = ds->u_base_b[ti] * (1.0 + bfc_b[ti] * F1_3D_b[ix]);
          ds->v_3D_b[ix] = ds->v_base_b[ti] * (1.0 + bfc_b[ti] * F1_3D_b[ix]);
        }
      }
  }
  st->n_visc_its = it;
  st->n_Axb_its = n_axb;
  st->L2_uv = L2;
  st->visc_it_relax_applied = relax_applied;
  st->status = status;
  free(w);
  free(ice_owned);
  return status;
}

/* ---------------------------------------------------------------------------------------- */
/* handle-based convenience layer for ctypes */

struct orc_ops {
  ufe_mesh_desc mesh;
  orc_csr ops[UFE_OP_COUNT];
  double *eta_first;   /* nV: first-iteration viscosity of the next solve (consumed by it), or NULL */
};

orc_ops *orc_ops_create(const ufe_mesh_desc *mesh, int32_t *status) {
  orc_ops *h = (orc_ops *)calloc(1, sizeof(orc_ops));
  h->mesh = *mesh;
  int32_t rc = orc_build_operators(mesh, h->ops);
  if (status) *status = rc;
  if (rc != 0) { free(h); return NULL; }
  return h;
}

const ufe_mesh_desc *orc_ops_mesh(const orc_ops *h) { return &h->mesh; }
const orc_csr *orc_ops_op(const orc_ops *h, int32_t op) { return &h->ops[op]; }

void orc_ops_destroy(orc_ops *h) {
  if (!h) return;
  for (int op = 0; op < UFE_OP_COUNT; ++op) orc_csr_free(&h->ops[op]);
  free(h->eta_first);
  free(h);
}

/* The learned start's predicted viscosity (per vertex) for the first Picard iteration of the next
 * solve on this handle; NULL clears it.  The next solve consumes it. */
int32_t orc_ops_set_first_viscosity(orc_ops *h, const double *eta_a) {
  if (!h) return UFE_ERR_INVALID;
  free(h->eta_first);
  h->eta_first = NULL;
  if (eta_a) {
    h->eta_first = (double *)malloc(sizeof(double) * (size_t)h->mesh.nV);
    memcpy(h->eta_first, eta_a, sizeof(double) * (size_t)h->mesh.nV);
  }
  return UFE_OK;
}

static double *take_first_viscosity(orc_ops *h) {
  double *e = h->eta_first;
  h->eta_first = NULL;
  return e;
}

int32_t orc_ops_info(orc_ops *h, int32_t op, int32_t *m, int32_t *n, int64_t *nnz) {
  if (!h || op < 0 || op >= UFE_OP_COUNT) return UFE_ERR_INVALID;
  *m = h->ops[op].m; *n = h->ops[op].n; *nnz = h->ops[op].nnz;
  return UFE_OK;
}

int32_t orc_ops_export(orc_ops *h, int32_t op, int32_t *ptr, int32_t *ind, double *val) {
  if (!h || op < 0 || op >= UFE_OP_COUNT) return UFE_ERR_INVALID;
  const orc_csr *A = &h->ops[op];
  memcpy(ptr, A->ptr, sizeof(int32_t) * (size_t)(A->m + 1));
  memcpy(ind, A->ind, sizeof(int32_t) * (size_t)A->nnz);
  memcpy(val, A->val, sizeof(double) * (size_t)A->nnz);
  return UFE_OK;
}

int32_t orc_ops_apply(orc_ops *h, int32_t op, const double *x, double *y, int32_t ncols) {
  if (!h || op < 0 || op >= UFE_OP_COUNT) return UFE_ERR_INVALID;
  orc_spmv(&h->ops[op], x, y, ncols);
  return UFE_OK;
}

int32_t orc_ops_solve_ssa(orc_ops *h, const ufe_solver_params *p, const ufe_ice_state *ice,
                          const ufe_bc_prescribed *bc, double *u_b, double *v_b, ufe_solve_stats *st) {
  double *ef = take_first_viscosity(h);
  int32_t rc = orc_solve_ssa(&h->mesh, h->ops, p, ice, bc, u_b, v_b, st, ef);
  free(ef);
  return rc;
}

int32_t orc_ops_solve_diva(orc_ops *h, const ufe_solver_params *p, const ufe_ice_state *ice,
                           const ufe_bc_prescribed *bc, ufe_diva_state *ds, ufe_solve_stats *st) {
  double *ef = take_first_viscosity(h);
  int32_t rc = orc_solve_diva(&h->mesh, h->ops, p, ice, bc, ds, st, ef);
  free(ef);
  return rc;
}

int32_t orc_ops_calc_dHi_dt(orc_ops *h, const double *A_vor, const double *Cw, const ufe_thickness_params *p,
                            ufe_thickness_fields *f, double *dt, ufe_thickness_stats *st) {
  if (!h || !A_vor || !Cw || !p || !f || !dt) return UFE_ERR_INVALID;
  return orc_calc_dHi_dt(&h->mesh, A_vor, Cw, p, f, dt, st);
}

/* the semi-implicit system, exported 0-based like ufe_thickness_assemble */
int32_t orc_ops_thickness_assemble(orc_ops *h, const double *A_vor, const double *Cw,
                                   const ufe_thickness_params *p, const ufe_thickness_fields *f, double dt,
                                   int32_t *ptr, int32_t *ind, double *val, double *bb, double *x0,
                                   int64_t cap, int64_t *nnz_out) {
  if (!h || !A_vor || !Cw || !p || !f) return UFE_ERR_INVALID;
  orc_csr A;
  int32_t rc = orc_thickness_assemble(&h->mesh, A_vor, Cw, p, f, dt, &A, bb, x0);
  if (rc != UFE_OK) return rc;
  *nnz_out = A.nnz;
  if (A.nnz > cap) { orc_csr_free(&A); return UFE_ERR_CAPACITY; }
  for (int i = 0; i <= A.m; ++i) ptr[i] = A.ptr[i] - 1;
  for (int64_t k = 0; k < A.nnz; ++k) { ind[k] = A.ind[k] - 1; val[k] = A.val[k]; }
  orc_csr_free(&A);
  return UFE_OK;
}

int32_t orc_ops_assemble(orc_ops *h, const ufe_solver_params *p,
                         const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                         const double *beta_b, const double *tau_dx_b, const double *tau_dy_b,
                         const double *u_prev, const double *v_prev, const ufe_bc_prescribed *bc,
                         int32_t *ptr, int32_t *ind, double *val, double *bb, int64_t cap,
                         int64_t *nnz_out) {
  orc_csr A;
  int32_t rc = orc_assemble_linearised(&h->mesh, h->ops, p, N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b,
                                       tau_dy_b, u_prev, v_prev, bc, &A, bb);
  if (rc != UFE_OK) { orc_csr_free(&A); return rc; }
  *nnz_out = A.nnz;
  if (A.nnz > cap) { orc_csr_free(&A); return UFE_ERR_CAPACITY; }
  memcpy(ptr, A.ptr, sizeof(int32_t) * (size_t)(A.m + 1));
  memcpy(ind, A.ind, sizeof(int32_t) * (size_t)A.nnz);
  memcpy(val, A.val, sizeof(double) * (size_t)A.nnz);
  orc_csr_free(&A);
  return UFE_OK;
}

static void wrap_csr(orc_csr *A, int32_t m, int32_t n, int64_t nnz, const int32_t *ptr,
                     const int32_t *ind, const double *val) {
  A->m = m; A->n = n; A->nnz = nnz; A->nnz_max = nnz;
  A->ptr = (int32_t *)ptr; A->ind = (int32_t *)ind; A->val = (double *)val;
}

int32_t orc_csr_solve(int32_t m, int64_t nnz, const int32_t *ptr, const int32_t *ind,
                      const double *val, const double *b, double *x, double rtol, double abstol,
                      int32_t max_it, int32_t *its) {
  orc_csr A;
  wrap_csr(&A, m, m, nnz, ptr, ind, val);
  return orc_bicgstab(&A, b, x, rtol, abstol, max_it, its);
}

int32_t orc_csr_spmv(int32_t m, int32_t n, int64_t nnz, const int32_t *ptr, const int32_t *ind,
                     const double *val, const double *x, double *y, int32_t ncols) {
  orc_csr A;
  wrap_csr(&A, m, n, nnz, ptr, ind, val);
  orc_spmv(&A, x, y, ncols);
  return UFE_OK;
}
