// A CSR matrix-equation solve that allocates no memory.
//
// ufe_solve_csr copies the caller's host arrays to the GPU and allocates its Krylov work vectors
// for each call.  Some callers cannot let a library allocate device memory: a host model whose
// device memory is handed out by its own pool or caching allocator (a second allocator would
// fragment or exceed the budget that pool was given), or a coupled model that fixes its GPU
// memory footprint at start-up and must not grow it during a run.  This entry point serves them:
// the matrix, right-hand side and solution are the caller's device buffers, and every work
// vector, reduction partial and scalar lives in one file-scope device array of fixed size.
//
// The array belongs to this library's device module.  Under CUDA's lazy module loading (the
// default since CUDA 12.2) the module, and with it the array's ~9.1 MiB, is loaded on a device by
// the first call there (at cudaGetSymbolAddress); with CUDA_MODULE_LOADING=EAGER it is loaded
// when the CUDA context starts.  Later calls take no device memory.
//
// The array is shared by all calls on a device and keeps the last call's contents; each call
// clears what must start at zero (the reduction tickets, the solver scalars and the input-check
// flag).  Calls that overlap on the GPU -- from two host threads, or on two streams without
// ordering between them -- race on the array.  The first call on a device resolves the array's
// device address; make that first call before any stream capture begins.
//
// The caller's matrix is checked on the device before any kernel reads through its column
// indices: ptr[0] and ptr[m] against 0 and nnz, ptr non-decreasing, every column in [0, m).  A
// malformed matrix returns UFE_ERR_INVALID.
#include <mutex>

#include "ufe_krylov.cuh"

namespace {

constexpr int64_t kNoAllocMaxRows = 1 << 17;   // 131,072 unknowns
constexpr int kNoAllocVectors = 9;             // dinv, r, r^, s, t, p(2), v(2)
constexpr int kNoAllocBlocks = 1024;           // grid cap (reduction partials per site)
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocTickets = 64;

// vectors | reduction partials | tickets + scalars + input-check flag: 9 MiB + 64 KiB + 2 KiB
constexpr int kTailDoubles = 256;
constexpr int64_t kScratchDoubles =
    kNoAllocVectors * kNoAllocMaxRows + kReduceSlots * kMaxReduceBlocks + kTailDoubles;
constexpr size_t kTailBytes = sizeof(unsigned int) * kNoAllocTickets + sizeof(KrylovScalars) + sizeof(int);
static_assert(kTailBytes <= kTailDoubles * sizeof(double), "scratch tail too small");
static_assert((sizeof(unsigned int) * kNoAllocTickets) % alignof(KrylovScalars) == 0, "scalar alignment");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// CSR rows whose ptr/ind may be 0- or 1-based
struct CsrMatBased {
  using Vec = double;
  static constexpr int kLanes = 1;
  int32_t items;
  const int32_t *__restrict__ ptr;
  const int32_t *__restrict__ col;
  const double *__restrict__ val;
  int32_t base;
  template <class G>
  __device__ __forceinline__ double row_partial(int i, int lane, G get) const {
    double y = 0.0;
    const int k2 = __ldg(ptr + i + 1) - base;
    for (int k = __ldg(ptr + i) - base; k < k2; ++k) y = fma(__ldg(val + k), get(__ldg(col + k) - base), y);
    return y;
  }
};

// Device-side check of the caller's CSR arrays, before any kernel indexes through them.  A row's
// columns are read only when its own ptr pair lies inside [0, nnz], so every read stays inside
// the caller's ptr (m+1) and ind (nnz) arrays.  Any violation sets *bad.
__global__ void k_noalloc_check(int32_t m, int64_t nnz, const int32_t *__restrict__ ptr,
                                const int32_t *__restrict__ col, int32_t base, int *bad) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const int64_t a = (int64_t)ptr[i] - base, b = (int64_t)ptr[i + 1] - base;
    bool ok = (i > 0 || a == 0) && (i < m - 1 || b == nnz) && a >= 0 && b >= a && b <= nnz;
    if (ok) {
      for (int64_t k = a; k < b; ++k) {
        const int64_t c = (int64_t)col[k] - base;
        if (c < 0 || c >= m) { ok = false; break; }
      }
    }
    if (!ok) atomicOr(bad, 1);
  }
}

// Jacobi: inverse diagonal, 1 where the diagonal is zero (PCJACOBI)
__global__ void k_noalloc_dinv(CsrMatBased A, double *dinv) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.items; i += stride) {
    double d = 0.0;
    const int k2 = A.ptr[i + 1] - A.base;
    for (int k = A.ptr[i] - A.base; k < k2; ++k)
      if (A.col[k] - A.base == (int)i) d += A.val[k];
    dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
  }
}

// Device address of the scratch array, resolved once per device.
std::mutex g_mutex;
double *g_addr[64] = {};

double *scratch_address(int device) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (device < 0 || device >= 64) return nullptr;
  if (!g_addr[device]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
    g_addr[device] = static_cast<double *>(p);
  }
  return g_addr[device];
}

}  // namespace

extern "C" int32_t ufe_solve_csr_noalloc(int32_t m, int64_t nnz, const int32_t *d_ptr, const int32_t *d_ind,
                                         const double *d_val, int32_t index_base, const double *d_bb, double *d_xx,
                                         double rtol, double abstol, int32_t max_it, int32_t *n_Axb_its,
                                         void *cuda_stream) {
  if (m < 1 || nnz < 0 || nnz > INT32_MAX || !d_ptr || !d_ind || !d_val || !d_bb || !d_xx) return UFE_ERR_INVALID;
  if (index_base != 0 && index_base != 1) return UFE_ERR_INVALID;
  if (max_it < 1 || !(rtol >= 0.0) || !(abstol >= 0.0)) return UFE_ERR_INVALID;
  if (m > kNoAllocMaxRows) return UFE_ERR_CAPACITY;   // the scratch holds 131,072 unknowns
  // an error left pending by earlier work of the caller is not this call's: clear it, so the
  // launch checks below see only this call's launches
  cudaGetLastError();
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return UFE_ERR_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (s) {
    // the scratch address below is the current device's; a stream of another device would run
    // the kernels against the wrong device's array
    int sdev = -1;
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) return UFE_ERR_DEVICE;
    if (sdev != device) return UFE_ERR_INVALID;
  }
  double *base = scratch_address(device);
  if (!base) {
    cudaGetLastError();
    return UFE_ERR_DEVICE;
  }
  double *vec = base;
  double *dinv = vec, *R = vec + m, *RP = R + m, *S = RP + m, *T = S + m, *P0 = T + m, *P1 = P0 + m,
         *V0 = P1 + m, *V1 = V0 + m;
  double *partials = base + (int64_t)kNoAllocVectors * kNoAllocMaxRows;
  unsigned int *tickets = reinterpret_cast<unsigned int *>(partials + (int64_t)kReduceSlots * kMaxReduceBlocks);
  KrylovScalars *ks = reinterpret_cast<KrylovScalars *>(tickets + kNoAllocTickets);
  int *bad = reinterpret_cast<int *>(ks + 1);
  // the array keeps the previous call's contents: reset the tickets, scalars and check flag
  if (cudaMemsetAsync(tickets, 0, kTailBytes, s) != cudaSuccess) return UFE_ERR_DEVICE;

  CsrMatBased A{m, d_ptr, d_ind, d_val, index_base};
  const unsigned g = krylov_grid(A, kNoAllocThreads, kNoAllocBlocks);
  k_noalloc_check<<<g, kNoAllocThreads, 0, s>>>(m, nnz, d_ptr, d_ind, index_base, bad);
  if (cudaGetLastError() != cudaSuccess) return UFE_ERR_DEVICE;
  int h_bad = 0;
  if (cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return UFE_ERR_DEVICE;
  if (cudaStreamSynchronize(s) != cudaSuccess) return UFE_ERR_DEVICE;
  if (h_bad) return UFE_ERR_INVALID;

  KV<double> v;
  v.X = d_xx; v.R = R; v.RP = RP; v.S = S; v.T = T; v.B = const_cast<double *>(d_bb); v.dinv = dinv;
  v.P[0] = P0; v.P[1] = P1; v.V[0] = V0; v.V[1] = V1;
  CondArg none{0, 0};
  k_noalloc_dinv<<<g, kNoAllocThreads, 0, s>>>(A, dinv);
  k_krylov_init<CsrMatBased><<<g, kNoAllocThreads, 0, s>>>(A, v, ks, rtol, abstol, max_it, 0, partials, tickets,
                                                            none);
  if (cudaGetLastError() != cudaSuccess) return UFE_ERR_DEVICE;
  KrylovScalars h;
  for (;;) {
    for (int c = 0; c < 8; ++c) {
      k_p_spmv<CsrMatBased><<<g, kNoAllocThreads, 0, s>>>(A, v, ks, partials, tickets);
      k_s_spmv<CsrMatBased><<<g, kNoAllocThreads, 0, s>>>(A, v, ks, partials, tickets);
      k_xr<CsrMatBased><<<g, kNoAllocThreads, 0, s>>>(A, v, ks, partials, tickets, none);
    }
    if (cudaGetLastError() != cudaSuccess) return UFE_ERR_DEVICE;
    if (cudaMemcpyAsync(&h, ks, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return UFE_ERR_DEVICE;
    if (cudaStreamSynchronize(s) != cudaSuccess) return UFE_ERR_DEVICE;
    if (!h.active) break;
  }
  if (n_Axb_its) *n_Axb_its = h.it;
  return h.status;
}
