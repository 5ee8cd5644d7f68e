// GPU construction of the mesh matrix operators.
//
// Restates calc_matrix_operators_mesh_{a_a,a_b,b_a,b_b_2nd_order}
// (src/UPSY/mesh/discretisation/mesh_disc_calc_matrix_operators_2D.f90:61-764) as one thread
// per matrix row.  Each thread grows its neighbourhood by the same flood fill as
// extend_group_single_iteration_{a,b} (src/UPSY/mesh/mesh_utilities.f90:1856-1935), in the same
// stack order, so the CSR integer structure equals the reference's; the weights are the
// weighted least-squares shape functions of src/UPSY/basic/math_utilities/shape_functions.f90
// (distance weight 1/r^1.5, Syrakos et al. 2017).
//
// Rows are written into a fixed-width staging buffer, then packed into CSR after an exclusive
// scan of the row lengths.  A row that needs more than the staging width sets an error flag and
// the build fails with UFE_ERR_CAPACITY; nothing is written out of bounds.
#include <cub/device/device_scan.cuh>

#include "ufe_internal.cuh"

namespace {

constexpr int kStackMax = 64;   // neighbourhood entries one row may collect
constexpr int kWidth = 64;      // staging width (entries per row, diagonal included)
constexpr double kShapeQ = 1.5; // shape_functions.f90:13

enum BuildError : int { kErrStack = 1, kErrSingular = 2 };

// gfortran's NORM2 for two numbers (running-scale sum of squares).
__device__ double norm2_2(double a, double b) {
  double xs[2] = {a, b};
  double scale = 1.0, result = 0.0;
#pragma unroll
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

__device__ __forceinline__ double weight_sq(double dx, double dy) {
  double w = 1.0 / pow(norm2_2(dx, dy), kShapeQ);
  return w * w;
}

__device__ __forceinline__ bool in_stack(const int *stack, int n, int v) {
  for (int s = 0; s < n; ++s)
    if (stack[s] == v) return true;
  return false;
}

// one flood-fill step over vertex connections C (extend_group_single_iteration_a)
__device__ bool extend_a(const int32_t *nC, const int32_t *C, int nV, int *stack, int &stackN) {
  int n = stackN;
  for (int i = 0; i < n; ++i) {
    int vi = stack[i];
    int nc = nC[vi - 1];
    for (int ci = 1; ci <= nc; ++ci) {
      int vj = C[(int64_t)(ci - 1) * nV + (vi - 1)];
      if (!in_stack(stack, stackN, vj)) {
        if (stackN >= kStackMax) return false;
        stack[stackN++] = vj;
      }
    }
  }
  return true;
}

// one flood-fill step over triangle neighbours TriC (extend_group_single_iteration_b)
__device__ bool extend_b(const int32_t *TriC, int nTri, int *stack, int &stackN) {
  int n = stackN;
  for (int i = 0; i < n; ++i) {
    int ti = stack[i];
    for (int n2 = 0; n2 < 3; ++n2) {
      int tj = TriC[(int64_t)n2 * nTri + (ti - 1)];
      if (tj == 0) continue;
      if (!in_stack(stack, stackN, tj)) {
        if (stackN >= kStackMax) return false;
        stack[stackN++] = tj;
      }
    }
  }
  return true;
}

// 5x5 inverse with partial pivoting; returns the determinant (0 when exactly singular).
__device__ double inverse5(const double (&A)[5][5], double (&Ai)[5][5]) {
  double a[5][10];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      a[r][c] = A[r][c];
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
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) Ai[r][c] = a[r][c + 5];
  return det;
}

// ---- a_a: 1st-order d/dx, d/dy on vertices (calc_matrix_operators_mesh_a_a, :61-196) ------
__global__ void k_build_a_a(int nV, const double *V, const int32_t *nC, const int32_t *C,
                            int32_t *rowlen, int32_t *ell_ind, double *ell_x, double *ell_y,
                            int *err) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nV) return;
  int stack[kStackMax];
  int vi = row + 1;
  double x = V[vi - 1], y = V[nV + vi - 1];
  int stackN = 1;
  stack[0] = vi;
  while (stackN - 1 < 2) {
    int before = stackN;
    if (!extend_a(nC, C, nV, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  double M[2][2];
  for (;;) {
    double A11 = 0, A12 = 0, A21 = 0, A22 = 0;
    for (int i = 0; i < stackN; ++i) {
      int vj = stack[i];
      if (vj == vi) continue;
      double dx = V[vj - 1] - x, dy = V[nV + vj - 1] - y;
      double w2 = weight_sq(dx, dy);
      A11 = A11 + w2 * dx * dx;
      A12 = A12 + w2 * dx * dy;
      A21 = A21 + w2 * dy * dx;
      A22 = A22 + w2 * dy * dy;
    }
    double det = A11 * A22 - A12 * A21;
    if (fabs(det) >= 2.2250738585072014e-308) {
      M[0][0] = A22 / det; M[0][1] = -A12 / det; M[1][0] = -A21 / det; M[1][1] = A11 / det;
      break;
    }
    int before = stackN;
    if (!extend_a(nC, C, nV, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  if (stackN > kWidth) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
  int64_t base = (int64_t)row * kWidth;
  double sx = 0.0, sy = 0.0;
  int k = 1;
  for (int i = 0; i < stackN; ++i) {
    int vj = stack[i];
    if (vj == vi) continue;
    double dx = V[vj - 1] - x, dy = V[nV + vj - 1] - y;
    double w2 = weight_sq(dx, dy);
    double nx = w2 * ((M[0][0] * dx) + (M[0][1] * dy));
    double ny = w2 * ((M[1][0] * dx) + (M[1][1] * dy));
    ell_ind[base + k] = vj - 1;
    ell_x[base + k] = nx;
    ell_y[base + k] = ny;
    sx += nx;
    sy += ny;
    ++k;
  }
  ell_ind[base] = row;
  ell_x[base] = -sx;
  ell_y[base] = -sy;
  rowlen[row] = k;
}

// ---- staggered 1st order (a_b, :198-335; b_a, :337-474): map, d/dx, d/dy -----------------
// shape functions: calc_shape_functions_2D_stag_1st_order (shape_functions.f90:361-453)
__device__ bool stag1_inverse(double x, double y, const int *stack, int stackN,
                              const double *px, const double *py, int64_t ld, double (&M)[3][3]) {
  double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < stackN; ++i) {
    int j = stack[i] - 1;
    double dx = px[j] - x, dy = py[j] - y;
    double w2 = weight_sq(dx, dy);
    A[0][0] = A[0][0] + (w2 * 1.0 * 1.0);
    A[0][1] = A[0][1] + (w2 * 1.0 * dx);
    A[0][2] = A[0][2] + (w2 * 1.0 * dy);
    A[1][0] = A[1][0] + (w2 * dx * 1.0);
    A[1][1] = A[1][1] + (w2 * dx * dx);
    A[1][2] = A[1][2] + (w2 * dx * dy);
    A[2][0] = A[2][0] + (w2 * dy * 1.0);
    A[2][1] = A[2][1] + (w2 * dy * dx);
    A[2][2] = A[2][2] + (w2 * dy * dy);
  }
  (void)ld;
  // minors and determinant by the first row; adjugate / det
  double mn[3][3];
  mn[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  mn[0][1] = A[1][0] * A[2][2] - A[1][2] * A[2][0];
  mn[0][2] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  mn[1][0] = A[0][1] * A[2][2] - A[0][2] * A[2][1];
  mn[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  mn[1][2] = A[0][0] * A[2][1] - A[0][1] * A[2][0];
  mn[2][0] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  mn[2][1] = A[0][0] * A[1][2] - A[0][2] * A[1][0];
  mn[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  double det = A[0][0] * mn[0][0] - A[0][1] * mn[0][1] + A[0][2] * mn[0][2];
  if (fabs(det) <= 2.2250738585072014e-308) return false;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double cof = mn[c][r];
      if (((r + c) & 1) != 0) cof = -cof;
      M[r][c] = cof / det;
    }
  return true;
}

__device__ void stag1_write(double x, double y, const int *stack, int stackN, const double *px,
                            const double *py, const double (&M)[3][3], int64_t base,
                            int32_t *ell_ind, double *e0, double *e1, double *e2) {
  for (int i = 0; i < stackN; ++i) {
    int j = stack[i] - 1;
    double dx = px[j] - x, dy = py[j] - y;
    double w2 = weight_sq(dx, dy);
    ell_ind[base + i] = j;
    e0[base + i] = w2 * ((M[0][0] * 1.0) + (M[0][1] * dx) + (M[0][2] * dy));
    e1[base + i] = w2 * ((M[1][0] * 1.0) + (M[1][1] * dx) + (M[1][2] * dy));
    e2[base + i] = w2 * ((M[2][0] * 1.0) + (M[2][1] * dx) + (M[2][2] * dy));
  }
}

__global__ void k_build_a_b(int nV, int nTri, const double *V, const double *TriGC,
                            const int32_t *Tri, const int32_t *nC, const int32_t *C,
                            int32_t *rowlen, int32_t *ell_ind, double *e0, double *e1, double *e2,
                            int *err) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nTri) return;
  int stack[kStackMax];
  double x = TriGC[row], y = TriGC[nTri + row];
  int stackN = 0;
  for (int n = 0; n < 3; ++n) stack[stackN++] = Tri[(int64_t)n * nTri + row];
  double M[3][3];
  for (;;) {
    if (stackN >= 3 && stag1_inverse(x, y, stack, stackN, V, V + nV, nV, M)) break;
    int before = stackN;
    if (!extend_a(nC, C, nV, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  if (stackN > kWidth) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
  stag1_write(x, y, stack, stackN, V, V + nV, M, (int64_t)row * kWidth, ell_ind, e0, e1, e2);
  rowlen[row] = stackN;
}

__global__ void k_build_b_a(int nV, int nTri, const double *V, const double *TriGC,
                            const int32_t *niTri, const int32_t *iTri, const int32_t *TriC,
                            int32_t *rowlen, int32_t *ell_ind, double *e0, double *e1, double *e2,
                            int *err) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nV) return;
  int stack[kStackMax];
  double x = V[row], y = V[nV + row];
  int stackN = 0;
  int nt = niTri[row];
  if (nt > kStackMax) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
  for (int k = 0; k < nt; ++k) stack[stackN++] = iTri[(int64_t)k * nV + row];
  double M[3][3];
  for (;;) {
    if (stackN >= 3 && stag1_inverse(x, y, stack, stackN, TriGC, TriGC + nTri, nTri, M)) break;
    int before = stackN;
    if (!extend_b(TriC, nTri, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  if (stackN > kWidth) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
  stag1_write(x, y, stack, stackN, TriGC, TriGC + nTri, M, (int64_t)row * kWidth, ell_ind, e0, e1, e2);
  rowlen[row] = stackN;
}

// ---- b_b 2nd order: d/dx, d/dy, d2/dx2, d2/dxdy, d2/dy2 on triangles (:612-764) -----------
// shape functions: calc_shape_functions_2D_reg_2nd_order (shape_functions.f90:212-359)
__global__ void k_build_b_b2(int nTri, const double *TriGC, const int32_t *TriC, int32_t *rowlen,
                             int32_t *ell_ind, double *e0, double *e1, double *e2, double *e3,
                             double *e4, int *err) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nTri) return;
  int stack[kStackMax];
  const double *gx = TriGC, *gy = TriGC + nTri;
  int ti = row + 1;
  double x = gx[row], y = gy[row];
  int stackN = 1;
  stack[0] = ti;
  while (stackN - 1 < 5) {
    int before = stackN;
    if (!extend_b(TriC, nTri, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  double M[5][5];
  for (;;) {
    double A[5][5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) A[r][c] = 0.0;
    for (int i = 0; i < stackN; ++i) {
      int tj = stack[i];
      if (tj == ti) continue;
      double dx = gx[tj - 1] - x, dy = gy[tj - 1] - y;
      double w2 = weight_sq(dx, dy);
      double dx2 = dx * dx, dy2 = dy * dy;
      A[0][0] = A[0][0] + w2 * dx * dx;
      A[0][1] = A[0][1] + w2 * dx * dy;
      A[0][2] = A[0][2] + w2 * dx * 0.5 * dx2;
      A[0][3] = A[0][3] + w2 * dx * dx * dy;
      A[0][4] = A[0][4] + w2 * dx * 0.5 * dy2;
      A[1][0] = A[1][0] + w2 * dy * dx;
      A[1][1] = A[1][1] + w2 * dy * dy;
      A[1][2] = A[1][2] + w2 * dy * 0.5 * dx2;
      A[1][3] = A[1][3] + w2 * dy * dx * dy;
      A[1][4] = A[1][4] + w2 * dy * 0.5 * dy2;
      A[2][0] = A[2][0] + w2 * 0.5 * dx2 * dx;
      A[2][1] = A[2][1] + w2 * 0.5 * dx2 * dy;
      A[2][2] = A[2][2] + w2 * 0.5 * dx2 * 0.5 * dx2;
      A[2][3] = A[2][3] + w2 * 0.5 * dx2 * dx * dy;
      A[2][4] = A[2][4] + w2 * 0.5 * dx2 * 0.5 * dy2;
      A[3][0] = A[3][0] + w2 * dx * dy * dx;
      A[3][1] = A[3][1] + w2 * dx * dy * dy;
      A[3][2] = A[3][2] + w2 * dx * dy * 0.5 * dx2;
      A[3][3] = A[3][3] + w2 * dx * dy * dx * dy;
      A[3][4] = A[3][4] + w2 * dx * dy * 0.5 * dy2;
      A[4][0] = A[4][0] + w2 * 0.5 * dy2 * dx;
      A[4][1] = A[4][1] + w2 * 0.5 * dy2 * dy;
      A[4][2] = A[4][2] + w2 * 0.5 * dy2 * 0.5 * dx2;
      A[4][3] = A[4][3] + w2 * 0.5 * dy2 * dx * dy;
      A[4][4] = A[4][4] + w2 * 0.5 * dy2 * 0.5 * dy2;
    }
    double det = inverse5(A, M);
    if (fabs(det) >= 2.2250738585072014e-308) break;
    int before = stackN;
    if (!extend_b(TriC, nTri, stack, stackN)) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
    if (stackN == before) { atomicOr(err, kErrSingular); rowlen[row] = 0; return; }
  }
  if (stackN > kWidth) { atomicOr(err, kErrStack); rowlen[row] = 0; return; }
  int64_t base = (int64_t)row * kWidth;
  double s[5] = {0, 0, 0, 0, 0};
  double *outs[5] = {e0, e1, e2, e3, e4};
  int k = 1;
  for (int i = 0; i < stackN; ++i) {
    int tj = stack[i];
    if (tj == ti) continue;
    double dx = gx[tj - 1] - x, dy = gy[tj - 1] - y;
    double w2 = weight_sq(dx, dy);
    double dx2 = dx * dx, dy2 = dy * dy;
    ell_ind[base + k] = tj - 1;
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      double v = w2 * ((M[r][0] * dx) + (M[r][1] * dy) + (M[r][2] * 0.5 * dx2) +
                       (M[r][3] * dx * dy) + (M[r][4] * 0.5 * dy2));
      outs[r][base + k] = v;
      s[r] += v;
    }
    ++k;
  }
  ell_ind[base] = row;
#pragma unroll
  for (int r = 0; r < 5; ++r) outs[r][base] = -s[r];
  rowlen[row] = k;
}

// pack staging rows into CSR (ptr from the exclusive scan of rowlen)
__global__ void k_pack(int m, int nval, const int32_t *ptr, const int32_t *rowlen,
                       const int32_t *ell_ind, const double *const *ell_vals, int32_t *ind,
                       double *const *vals) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  int64_t base = (int64_t)row * kWidth;
  int32_t p = ptr[row];
  int len = rowlen[row];
  for (int k = 0; k < len; ++k) {
    ind[p + k] = ell_ind[base + k];
    for (int f = 0; f < nval; ++f) vals[f][p + k] = ell_vals[f][base + k];
  }
}

struct Staging {
  int32_t *rowlen = nullptr, *ell_ind = nullptr;
  double *ell[5] = {};
};

// Turn a staged family into CSR operators ops[first..first+nval-1] sharing one pattern.
void pack_family(ufe_ctx *ctx, int m, int n, int nval, Staging &st, int first_op) {
  cudaStream_t s = ctx->stream;
  int32_t *ptr = (int32_t *)dev_alloc(sizeof(int32_t) * (m + 1));
  // rowlen has m+1 entries, the last one zero, so the scan's last element is the total
  size_t tmp_bytes = 0;
  UFE_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, st.rowlen, ptr, m + 1, s));
  void *tmp = dev_alloc(tmp_bytes);
  UFE_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, st.rowlen, ptr, m + 1, s));
  int32_t nnz = 0;
  UFE_CUDA(cudaMemcpyAsync(&nnz, ptr + m, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(tmp);
  int32_t *ind = (int32_t *)dev_alloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
  double *vals[5] = {};
  for (int f = 0; f < nval; ++f) vals[f] = (double *)dev_alloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  double **d_ell = (double **)dev_alloc(sizeof(double *) * 5);
  double **d_vals = (double **)dev_alloc(sizeof(double *) * 5);
  UFE_CUDA(cudaMemcpyAsync(d_ell, st.ell, sizeof(double *) * 5, cudaMemcpyHostToDevice, s));
  UFE_CUDA(cudaMemcpyAsync(d_vals, vals, sizeof(double *) * 5, cudaMemcpyHostToDevice, s));
  k_pack<<<(m + 255) / 256, 256, 0, s>>>(m, nval, ptr, st.rowlen, st.ell_ind, d_ell, ind, d_vals);
  UFE_CUDA(cudaGetLastError());
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(d_ell);
  dev_free(d_vals);
  ctx->op_allocs.push_back(ptr);
  ctx->op_allocs.push_back(ind);
  for (int f = 0; f < nval; ++f) {
    ctx->op_allocs.push_back(vals[f]);
    DevCSR &A = ctx->ops[first_op + f];
    A.m = m; A.n = n; A.nnz = nnz; A.ptr = ptr; A.ind = ind; A.val = vals[f];
    ctx->op_set[first_op + f] = true;
  }
}

Staging alloc_staging(int m, int nval) {
  Staging st;
  st.rowlen = (int32_t *)dev_alloc(sizeof(int32_t) * (m + 1));
  st.ell_ind = (int32_t *)dev_alloc(sizeof(int32_t) * (size_t)m * kWidth);
  for (int f = 0; f < nval; ++f) st.ell[f] = (double *)dev_alloc(sizeof(double) * (size_t)m * kWidth);
  return st;
}

void free_staging(Staging &st) {
  dev_free(st.rowlen);
  dev_free(st.ell_ind);
  for (int f = 0; f < 5; ++f) dev_free(st.ell[f]);
  st = Staging{};
}

}  // namespace

void build_operators_gpu(ufe_ctx *ctx) {
  UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "no mesh uploaded");
  cudaStream_t s = ctx->stream;
  free_operators(ctx);
  const int nV = ctx->nV, nTri = ctx->nTri;
  int *d_err = (int *)dev_alloc(sizeof(int));
  UFE_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s));
  const int T = 128;

  // a_a
  {
    Staging st = alloc_staging(nV, 2);
    UFE_CUDA(cudaMemsetAsync(st.rowlen, 0, sizeof(int32_t) * (nV + 1), s));
    k_build_a_a<<<(nV + T - 1) / T, T, 0, s>>>(nV, ctx->V, ctx->nC, ctx->C, st.rowlen, st.ell_ind,
                                               st.ell[0], st.ell[1], d_err);
    UFE_CUDA(cudaGetLastError());
    pack_family(ctx, nV, nV, 2, st, UFE_OP_DDX_A_A);
    free_staging(st);
  }
  // a_b
  {
    Staging st = alloc_staging(nTri, 3);
    UFE_CUDA(cudaMemsetAsync(st.rowlen, 0, sizeof(int32_t) * (nTri + 1), s));
    k_build_a_b<<<(nTri + T - 1) / T, T, 0, s>>>(nV, nTri, ctx->V, ctx->TriGC, ctx->Tri, ctx->nC,
                                                 ctx->C, st.rowlen, st.ell_ind, st.ell[0],
                                                 st.ell[1], st.ell[2], d_err);
    UFE_CUDA(cudaGetLastError());
    pack_family(ctx, nTri, nV, 3, st, UFE_OP_MAP_A_B);
    free_staging(st);
  }
  // b_a
  {
    Staging st = alloc_staging(nV, 3);
    UFE_CUDA(cudaMemsetAsync(st.rowlen, 0, sizeof(int32_t) * (nV + 1), s));
    k_build_b_a<<<(nV + T - 1) / T, T, 0, s>>>(nV, nTri, ctx->V, ctx->TriGC, ctx->niTri, ctx->iTri,
                                               ctx->TriC, st.rowlen, st.ell_ind, st.ell[0],
                                               st.ell[1], st.ell[2], d_err);
    UFE_CUDA(cudaGetLastError());
    pack_family(ctx, nV, nTri, 3, st, UFE_OP_MAP_B_A);
    free_staging(st);
  }
  // b_b 2nd order
  {
    Staging st = alloc_staging(nTri, 5);
    UFE_CUDA(cudaMemsetAsync(st.rowlen, 0, sizeof(int32_t) * (nTri + 1), s));
    k_build_b_b2<<<(nTri + T - 1) / T, T, 0, s>>>(nTri, ctx->TriGC, ctx->TriC, st.rowlen,
                                                  st.ell_ind, st.ell[0], st.ell[1], st.ell[2],
                                                  st.ell[3], st.ell[4], d_err);
    UFE_CUDA(cudaGetLastError());
    pack_family(ctx, nTri, nTri, 5, st, UFE_OP_M2_DDX_B_B);
    free_staging(st);
  }
  int err = 0;
  UFE_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(d_err);
  if (err != 0) {
    free_operators(ctx);
    UFE_REQUIRE(!(err & kErrStack), UFE_ERR_CAPACITY,
                "operator construction: a neighbourhood exceeded 64 entries");
    UFE_REQUIRE(false, UFE_ERR_INVALID,
                "operator construction: singular least-squares system that no flood-fill step can fix");
  }
}
