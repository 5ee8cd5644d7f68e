// CSR matrix-vector products for the operator-application and CSR-algebra entry points.
//
// multiply_CSR_matrix_with_vector_1D (src/UPSY/basic/CSR_matrix_algebra/
// CSR_matrix_vector_multiplication.f90:266-278) sums each row in storage order, one rounding
// per multiply and per add.  This kernel keeps that order (one thread per row and column, no
// FMA contraction), so its results are bit-identical to the reference's loop.  The 2-D form
// (:336-364) is the same product for each of `ncols` column-major columns.
#include "ufe_internal.cuh"

namespace {

__global__ void k_csr_spmv(int32_t m, int32_t n, int32_t ncols, const int32_t *__restrict__ ptr,
                           const int32_t *__restrict__ ind, const double *__restrict__ val,
                           const double *__restrict__ x, double *__restrict__ y) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = (int64_t)m * ncols;
  if (t >= total) return;
  int32_t c = (int32_t)(t / m);
  int32_t i = (int32_t)(t - (int64_t)c * m);
  const double *xc = x + (int64_t)c * n;
  double s = 0.0;
  int32_t k2 = __ldg(ptr + i + 1);
  for (int32_t k = __ldg(ptr + i); k < k2; ++k)
    s = s + __ldg(val + k) * __ldg(xc + __ldg(ind + k));   // built with --fmad=false: two roundings
  y[(int64_t)c * m + i] = s;
}

}  // namespace

void launch_csr_spmv(cudaStream_t s, const DevCSR &A, const double *x, double *y, int32_t ncols) {
  int64_t total = (int64_t)A.m * ncols;
  if (total == 0) return;
  const int T = 256;
  int64_t blocks = (total + T - 1) / T;
  k_csr_spmv<<<(unsigned)blocks, T, 0, s>>>(A.m, A.n, ncols, A.ptr, A.ind, A.val, x, y);
  UFE_CUDA(cudaGetLastError());
}
