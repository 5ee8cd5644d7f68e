// Solver workspace and device-side building blocks shared by the Krylov and Picard code.
#pragma once

#include "ufe_internal.cuh"
#include "ufe_dword.cuh"

// ------------------------------------------------------------------------------------------
// Deterministic grid reductions without waiting: each block writes its partial sums, and the
// last block to take a ticket adds all partials in block order (threadFenceReduction pattern).
// Nothing spins, so no kernel can hang on a reduction.

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem /* NV * 32 */) {
#pragma unroll
  for (int j = 0; j < NV; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) smem[j * 32 + warp] = v[j];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double t = (lane < nw) ? smem[j * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      v[j] = t;
    }
  }
}

// Reduce NV values over the grid.  Returns true in thread 0 of the last block, with `tot`
// holding the grid totals; false everywhere else.
template <int NV>
__device__ bool grid_sum(double (&v)[NV], double *partials, unsigned int *ticket, double (&tot)[NV]) {
  __shared__ double smem[NV * 32];
  __shared__ bool am_last;
  block_sum<NV>(v, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) partials[j * kMaxReduceBlocks + blockIdx.x] = v[j];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    acc[j] = 0.0;
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
      acc[j] += __ldcg(partials + j * kMaxReduceBlocks + b);
  }
  block_sum<NV>(acc, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) tot[j] = acc[j];
    *ticket = 0u;   // ready for the next launch (stream order separates launches)
    return true;
  }
  return false;
}

// ------------------------------------------------------------------------------------------
// Block-sparse stiffness matrix: the 2x2 blocks (u,v) x (u,v) of every triangle pair in the
// pattern of the 2nd-order b_b operators.  blk[k] = (uu, uv, vu, vv).
struct BsrView {
  int32_t nb;               // block rows = nTri
  const int32_t *ptr;       // nb+1, 0-based
  const int32_t *col;       // nnzb
  const double4 *blk;       // nnzb (FP64)
  const float4 *blk32;      // nnzb (FP32 copy, or null)
};

// Krylov vectors: interleaved (u,v) per triangle, i.e. row 2(ti-1)+uv of the reference.
struct KrylovVecs {
  double2 *X, *R, *RP, *S, *T, *dinv, *B;
  double2 *P[2], *V[2];
  // inner (correction) solve of the mixed path: FP32 vectors
  float2 *x32, *R32, *RP32, *S32, *T32, *dinv32;
  float2 *P32[2], *V32[2];
};

struct Work {
  int32_t nV = 0, nTri = 0, nz = 0;
  int64_t nnzb = 0;
  // stiffness matrix
  double4 *blk = nullptr;
  float4 *blk32 = nullptr;
  float4 *rowsum32 = nullptr;   // FP64 row sums of the blocks, rounded to FP32 (difference form)
  int32_t *diag = nullptr;      // index of the diagonal block per block row
  KrylovVecs kv{};
  // velocity state and per-solve inputs on triangles
  double2 *uv = nullptr;        // SSA u_b,v_b  /  DIVA u_vav,v_vav
  double2 *tau_d = nullptr;     // driving stress
  double *fgr_b = nullptr;
  int32_t *bc_mask = nullptr;
  double2 *bc_uv = nullptr;
  int32_t has_bc = 0;
  // DIVA state on triangles
  double2 *uv_base = nullptr, *tau_b = nullptr;
  double *eta_3D_b = nullptr;   // nz x nTri
  double2 *duz_b = nullptr;     // nz x nTri: (du/dz, dv/dz) on triangles for the next vertex pass
  double *bfc_b = nullptr, *F2b1 = nullptr;
  double *beta_b = nullptr;     // applied friction on triangles (SSA) / beta_eff_b (DIVA)
  // vertex inputs
  double *Hi = nullptr, *Hs = nullptr, *Avav = nullptr, *A_flow = nullptr;
  double *A_pow = nullptr;      // nz x nV: A_flow^(-1/n) of the current DIVA solve
  double *beta_sq = nullptr, *alpha_sq = nullptr, *effp = nullptr, *tys = nullptr;
  int32_t *mask_gr = nullptr;
  int32_t any_grounded = 0;
  // inputs of calc_ice_rheology_Glen (allocated when first given, then kept for the Work's life so
  // captured graphs never see a freed pointer) and the flow factor it computes
  int32_t has_A = 0;              // the caller gave A_flow
  int32_t has_Ti = 0, has_mask_fl = 0, has_fgr_v = 0, has_Hib = 0, has_SL = 0;
  double *Ti = nullptr;           // nz x nV
  int32_t *mask_fl = nullptr;
  double *fgr_v = nullptr, *Hib = nullptr, *SL = nullptr;
  double *A_rheo = nullptr;       // nz x nV
  // the idealised SSA_icestream sliding law: Schoof's till yield stress per vertex
  double *tys_ideal = nullptr;
  // 'infinite_SSA_icestream' border rows: copy triangles and weights per triangle (CSR over
  // triangles, empty rows elsewhere), built on first use
  int32_t *cp_ptr = nullptr, *cp_idx = nullptr;
  double *cp_w = nullptr;
  // vertex work
  double *N_a = nullptr, *beta_a = nullptr, *beta_eff_a = nullptr, *F2a1 = nullptr;
  double *eta_3D_a = nullptr;   // nz x nV
  double *F1_3D_a = nullptr;    // nz x nV (end of solve)
  // the learned start's predicted vertically averaged viscosity per vertex, and the device flag
  // that arms it for the first Picard iteration of the next solve (the solve's prologue clears it)
  double *eta_pred_a = nullptr;
  int32_t *pred_flag = nullptr;
  // linearised-solve inputs given on triangles (ufe_solve_linearised / ufe_assemble_linearised)
  double *N_b_in = nullptr, *dNx_b_in = nullptr, *dNy_b_in = nullptr, *beta_b_in = nullptr;
  // scalars
  KrylovScalars *ks = nullptr;
  PicardScalars *ps = nullptr;
  KrylovScalars *ks_host = nullptr;   // pinned mirrors
  PicardScalars *ps_host = nullptr;
  int *err = nullptr;             // assembly error flags
  // sliced-ELL copy of the stiffness matrix for the Krylov SpMVs (slices of 32 block rows)
  int64_t nslots = 0;
  int32_t *sell_off = nullptr;   // nslices + 1
  int32_t *sell_col = nullptr;   // nslots; padding slots hold the row itself
  int32_t *sell_map = nullptr;   // nnzb: slot of CSR block k
  double4 *sell_blk = nullptr;   // nslots; padding slots stay zero
  float4 *sell_blk32 = nullptr;
  // patches of the persistent FP32 solve: block b owns rows [b*halo_rpb, (b+1)*halo_rpb)
  int32_t halo_G = 0, halo_rpb = 0, halo_maxlocal = 0;
  int32_t *halo_off = nullptr;   // halo_G + 1
  int32_t *halo_idx = nullptr;   // halo rows of every block
  int32_t *halo_lcol = nullptr;  // nslots: local index of each slot's column
  // double-word Krylov solve (UFE_PREC_FP32_PAIR), allocated on first use: its vectors, the
  // sliced-ELL blocks in double-word form, and the flag of values outside the FP32 range
  dw2 *pX = nullptr, *pR = nullptr, *pRP = nullptr, *pS = nullptr, *pT = nullptr, *pdinv = nullptr;
  dw2 *pP[2] = {nullptr, nullptr}, *pV[2] = {nullptr, nullptr};
  dwblk *sell_blkp = nullptr;
  int *pair_bad = nullptr;
  // persistent Krylov kernel: per-block partial sums of its three phases and its grid barrier
  double *ppart = nullptr;
  struct GridSync *gsync = nullptr;
  // graphs, and their kernel nodes: in the prologue and in one Picard iteration ([0] SSA, [1] DIVA;
  // -1 where a Picard iteration holds a data-dependent loop)
  cudaGraphExec_t graph_ssa = nullptr, graph_diva = nullptr;
  uint64_t graph_ssa_key = 0, graph_diva_key = 0;
  // and in one double-word round (UFE_PREC_FP32_PAIR; 0 for the other persistent path)
  int32_t graph_kernels_pro[2] = {-1, -1}, graph_kernels_it[2] = {-1, -1}, graph_kernels_round[2] = {-1, -1};
  int32_t last_kernels_pro = -1, last_kernels_it = -1, last_kernels_round = -1;   // of the solve last launched
};

Work *ensure_work(ufe_ctx *ctx);

// Lanes per block row in the BSR kernels (1, 2 or 4), chosen by the tuner.
int32_t bsr_lanes(ufe_ctx *ctx);
