// Internal declarations of the GB300 velocity-solve library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <exception>

#include "../../include/ufe_gpu.h"

// ------------------------------------------------------------------------------------------
// error handling: every CUDA call is checked; a failure records a message on the context and
// turns into UFE_ERR_DEVICE at the ABI.
struct ufe_error {
  int32_t code;
  std::string msg;
};

#define UFE_CUDA(call)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      throw ufe_error{UFE_ERR_DEVICE, std::string(#call) + ": " + cudaGetErrorString(e_)};    \
  } while (0)

#define UFE_REQUIRE(cond, code, text)                                                         \
  do {                                                                                        \
    if (!(cond)) throw ufe_error{(code), (text)};                                             \
  } while (0)

// ------------------------------------------------------------------------------------------
// device CSR matrix, 0-based.  Families of operators that share one sparsity pattern share the
// ptr/ind arrays (a_b: map/ddx/ddy; b_a: map/ddx/ddy; a_a: ddx/ddy; b_b 2nd order: 5 operators).
struct DevCSR {
  int32_t m = 0, n = 0;
  int64_t nnz = 0;
  int32_t *ptr = nullptr;
  int32_t *ind = nullptr;
  double *val = nullptr;
};

// Krylov / Picard scalars that live on the device for a whole solve.
struct KrylovScalars {
  double rho, rhoold, alpha, omega, omegaold, beta;
  double dp, ttol, rnorm0;
  int32_t it;          // iterations of the current solve
  int32_t active;      // 1 while iterating
  int32_t status;      // UFE_* of the current solve
  int32_t total_its;   // summed over the Picard iterations
  int32_t max_it;
  int32_t refinements; // FP64 refinement steps of the current Picard iteration
  int32_t tbreak;      // t = 0 in the last iteration: x + alpha p is the final update
  int32_t pad;         // failed inner solves of the current refinement loop
  int32_t fallback;    // the FP32 refinement loop gave up: finish in FP64
  int32_t owner;       // [2]: 1 while the double-word solve owns the current linear solve
  int32_t pair_its;    // of total_its: double-word (UFE_PREC_FP32_PAIR) iterations
  int32_t pair_rounds; // double-word solves of the current linear solve (restarts from the FP64 residual)
  int32_t pair_stop;   // the double-word path declined or failed: finish in FP64
  int32_t pair_rounds_total;
  int32_t pad3;
};

constexpr int kHistMax = 128;   // Picard iterations recorded per solve
constexpr int kHistCols = 5;    // L2, Krylov iterations, Krylov status, final residual, refinements

struct PicardScalars {
  double L2, L2_prev, relax, eps0, eta_max;
  int32_t it, nit_diverg, active, status;
  int32_t n_refine;
  int32_t prev_total_its;
  int32_t phase;       // inexact Picard (krylov_forcing > 0): 0 while forced, 1 once exact solves verify
  int32_t nconv0;      // consecutive forced iterations whose change norm met the tolerance
  int32_t use_pred;    // the first iteration takes the learned start's predicted viscosity
  int32_t pad_;
  double hist[kHistMax * kHistCols];
};

// Partial sums of one reduction stage: each block writes `nparts` values at
// partials[slot * max_blocks + blockIdx.x]; the last block to arrive sums them in block order.
constexpr int kMaxReduceBlocks = 4096;
constexpr int kReduceSlots = 8;

struct ReduceArea {
  double *partials = nullptr;     // kReduceSlots * kMaxReduceBlocks
  unsigned int *tickets = nullptr; // one counter per reduction site
};

// ------------------------------------------------------------------------------------------
struct ufe_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // mesh (device, as uploaded: 1-based, column-major)
  bool has_mesh = false;
  int32_t nV = 0, nTri = 0, nC_mem = 0, nz = 0;
  double *V = nullptr, *TriGC = nullptr, *zeta = nullptr;
  int32_t *nC = nullptr, *C = nullptr, *niTri = nullptr, *iTri = nullptr, *VBI = nullptr;
  int32_t *Tri = nullptr, *TriC = nullptr, *TriBI = nullptr;
  std::vector<double> zeta_host;

  // internal order: internal vertex/triangle i is the caller's perm[i] (ufe_layout.cu)
  std::vector<int32_t> perm_v_h, iperm_v_h, perm_t_h, iperm_t_h;
  int32_t *perm_v = nullptr, *iperm_v = nullptr, *perm_t = nullptr, *iperm_t = nullptr;

  DevCSR ops[UFE_OP_COUNT];
  bool op_set[UFE_OP_COUNT] = {};
  std::vector<void *> op_allocs;   // device allocations owned by the operators

  // solver workspace (allocated lazily for the mesh size)
  struct Work *work = nullptr;
  // thermodynamics workspace and resident heat-equation state (ufe_thermo.cu)
  struct ThermoWork *thermo = nullptr;
  // ice-thickness workspace: the mesh's Voronoi geometry and the M_divQ pattern (ufe_mass.cu)
  struct MassWork *mass = nullptr;
  // rows per warp of the block-row Krylov kernels for this mesh (0: the default; ufe_autotune)
  int32_t lanes = 0;
  // the persistent FP32 inner solve needs the whole GPU; ensembles switch it off for the member
  bool allow_persistent = true;

  ReduceArea red;
};

// Run an ABI body, turning exceptions into status codes and messages.
template <class F>
inline int32_t guarded(ufe_ctx *ctx, F &&body) {
  if (!ctx) return UFE_ERR_INVALID;
  try {
    int32_t rc = body();
    if (rc >= 0) ctx->last_error.clear();
    return rc;
  } catch (const ufe_error &e) {
    ctx->last_error = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    ctx->last_error = e.what();
    return UFE_ERR_DEVICE;
  }
}


// helpers implemented in ufe_ctx.cu
void *dev_alloc(size_t bytes);
void dev_free(void *p);
void free_operators(ufe_ctx *ctx);
void ensure_reduce_area(ufe_ctx *ctx);
int32_t pick_blocks(int64_t items, int threads, int max_blocks);

// ufe_operators.cu
void build_operators_gpu(ufe_ctx *ctx);

// ufe_thermo.cu
void free_thermo(ufe_ctx *ctx);

// ufe_mass.cu
void free_mass(ufe_ctx *ctx);

// ufe_velocity.cu: the mesh side of the learned Picard start (internal order, on stream s)
void gnn_mesh_features(ufe_ctx *ctx, cudaStream_t s, int use_prev, float *x, float *mask);
void gnn_mesh_graph(ufe_ctx *ctx, cudaStream_t s, int32_t *nbr);
void gnn_mesh_velocity(ufe_ctx *ctx, cudaStream_t s, float *y, bool to_state, const float *mask);
void gnn_mesh_smooth(ufe_ctx *ctx, cudaStream_t s, int passes, const float *mask);
void gnn_mesh_viscosity(ufe_ctx *ctx, cudaStream_t s, float *y, bool to_state, const float *mask);

// The network's outputs per triangle: u / 1e3, v / 1e3 (m/yr) and the vertically averaged
// effective viscosity as (log10(eta) - kGnnLogEtaOff) / kGnnLogEtaScale (eta in Pa yr).
constexpr int kGnnOut = 3;
constexpr double kGnnLogEtaOff = 7.5;
constexpr double kGnnLogEtaScale = 2.0;

// ufe_layout.cu: internal (Z-order) numbering and the mappings at the ABI boundary
void layout_upload_mesh(ufe_ctx *ctx, const ufe_mesh_desc *m);
void free_layout(ufe_ctx *ctx);
void to_internal(ufe_ctx *ctx, double *d_dst, const double *h_src, bool tri, int ncols);
void to_internal_i32(ufe_ctx *ctx, int32_t *d_dst, const int32_t *h_src, bool tri);
void to_external(ufe_ctx *ctx, double *h_dst, const double *d_src, bool tri, int ncols);
void pair_to_internal(ufe_ctx *ctx, double2 *d_dst, const double *h_a, const double *h_b);
void pair_to_external(ufe_ctx *ctx, double *h_a, double *h_b, const double2 *d_src);
void csr_to_internal(ufe_ctx *ctx, int op, const std::vector<int32_t> &ptr, const std::vector<int32_t> &ind,
                     const double *val, std::vector<int32_t> &iptr, std::vector<int32_t> &iind, std::vector<double> &ival);
void csr_to_external(ufe_ctx *ctx, int op, const std::vector<int32_t> &iptr, const std::vector<int32_t> &iind,
                     const std::vector<double> &ival, int32_t *ptr, int32_t *ind, double *val);

// ufe_spmv.cu
void launch_csr_spmv(cudaStream_t s, const DevCSR &A, const double *x, double *y, int32_t ncols);

// ufe_velocity.cu
void free_work(ufe_ctx *ctx);
// Work vectors of solve_csr_device for callers that solve repeatedly (nothing is allocated
// inside the solve when a scratch with cap >= the rows is passed).
struct CsrSolveScratch {
  double *vec = nullptr;              // 10 x cap
  struct KrylovScalars *ks = nullptr, *hks = nullptr;   // device, pinned host
  int64_t cap = 0;
  cudaGraphExec_t graph = nullptr;    // the whole solve with a device-side loop, for `key`
  uint64_t key = 0;
};
void csr_scratch_alloc(CsrSolveScratch &scr, int64_t m);
void csr_scratch_free(CsrSolveScratch &scr);
int32_t solve_csr_device(ufe_ctx *ctx, const DevCSR &A, const double *b, double *x, double rtol,
                         double abstol, int32_t max_it, int32_t *its, CsrSolveScratch *scratch = nullptr);

