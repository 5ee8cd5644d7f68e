// Learned Picard start: a mesh-graph network on the triangle b-grid, BF16 on the tcgen05 tensor
// cores with FP32 accumulation in tensor memory.
//
// This file holds the tensor-core GEMM tile and the C entry point that exercises it alone
// (ufe_umma_gemm_bf16); the network's kernels build on the same tile.
#include <algorithm>
#include <vector>

#include "ufe_internal.cuh"
#include "ufe_umma.cuh"

namespace {

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
  return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Y[M x N] = X[M x K] * W[N x K]^T, X and W BF16 row-major, Y FP32; one CTA per 128 rows.
template <int N>
__global__ void __launch_bounds__(128) k_gemm_tile_test(int M, int K, const __nv_bfloat16 *__restrict__ X,
                                                        const __nv_bfloat16 *__restrict__ W, float *__restrict__ Y,
                                                        int *err) {
  extern __shared__ uint8_t smraw[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  uint8_t *sm = align1024(smraw);
  const int kblocks = K / 64;
  uint8_t *sA = sm;
  uint8_t *sB = sm + kblocks * 128 * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * 128;
  // A: thread tid stages row tid, 16-byte chunks into their swizzled positions
  for (int kb = 0; kb < kblocks; ++kb)
    for (int c = 0; c < 8; ++c) {
      const uint4 v = *reinterpret_cast<const uint4 *>(X + (int64_t)(row0 + tid) * K + kb * 64 + c * 8);
      *reinterpret_cast<uint4 *>(sA + kb * 128 * 128 + umma::sw128_chunk(tid, c)) = v;
    }
  for (int idx = tid; idx < N * kblocks * 8; idx += 128) {
    const int r = idx / (kblocks * 8), rem = idx - r * kblocks * 8, kb = rem >> 3, c = rem & 7;
    const uint4 v = *reinterpret_cast<const uint4 *>(W + (int64_t)r * K + kb * 64 + c * 8);
    *reinterpret_cast<uint4 *>(sB + kb * N * 128 + umma::sw128_chunk(r, c)) = v;
  }
  if (warp == 0) umma::tmem_alloc(&tslot, N);
  if (tid == 0) {
    umma::mbar_init(umma::smem_u32(&mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_smem_async();
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    umma::mma_tile<N>(tmem, umma::smem_u32(sA), umma::smem_u32(sB), kblocks, false);
    umma::commit(umma::smem_u32(&mbar));
  }
  bool ok = umma::mbar_wait(umma::smem_u32(&mbar), 0);
  ok = __syncthreads_and(ok);
  umma::fence_after();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + c0, v);
      float *y = Y + (int64_t)(row0 + 32 * warp + lane) * N + c0;
#pragma unroll
      for (int i = 0; i < 16; ++i) y[i] = v[i];
    }
  } else {
    if (tid == 0) atomicExch(err, 1);
    umma::mbar_wait(umma::smem_u32(&mbar), 0);   // bounded: let the MMAs drain before freeing TMEM
  }
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  if (warp == 0) umma::tmem_dealloc(tmem, N);
}

// ================================================================================================
// The network.  Nodes are triangles; each has up to three neighbours (TriC).  Width C = 64.
//   h0      = relu(We x + be)                                  (x: FIN = 16 features, zero-padded)
//   layer l: a = mean_{j in N(i)} h_j;  t = relu(W1 [h, a] + b1);  h <- h + W2 t + b2   (4 layers)
//   y       = Wd h + bd        (kGnnOut = 3 outputs: u, v scaled, and the log-viscosity)
// BF16 operands, FP32 accumulation (TMEM) and FP32 activations in global memory.
constexpr int kC = 64;
constexpr int kFin = 16;
constexpr int kLayers = 4;
constexpr int kNb = 3;

// parameter offsets (floats) in the flat FP32 parameter vector
constexpr int kOffWe = 0;                                   // [64 x 16]
constexpr int kOffBe = kOffWe + kC * kFin;                  // [64]
constexpr int kOffL0 = kOffBe + kC;
constexpr int kLayerSize = kC * 2 * kC + kC + kC * kC + kC; // W1 [64x128], b1, W2 [64x64], b2
constexpr int kOffWd = kOffL0 + kLayers * kLayerSize;       // [kGnnOut x 64]
constexpr int kOffBd = kOffWd + kGnnOut * kC;               // [kGnnOut]
constexpr int kParams = kOffBd + kGnnOut;
__host__ __device__ constexpr int off_W1(int l) { return kOffL0 + l * kLayerSize; }
__host__ __device__ constexpr int off_b1(int l) { return off_W1(l) + kC * 2 * kC; }
__host__ __device__ constexpr int off_W2(int l) { return off_b1(l) + kC; }
__host__ __device__ constexpr int off_b2(int l) { return off_W2(l) + kC * kC; }

// BF16 weight copies in the layouts the tile reads (B operand: [N rows x K], row-major)
constexpr int kBfWe = 0;                                    // [64 x 64]  (We, inputs padded to 64)
constexpr int kBfL0 = kBfWe + kC * kC;
constexpr int kBfLayer = kC * 2 * kC + kC * kC + kC * kC + 2 * kC * kC;   // W1, W2, W2T, W1T
__host__ __device__ constexpr int bf_W1(int l) { return kBfL0 + l * kBfLayer; }       // [64 x 128]
__host__ __device__ constexpr int bf_W2(int l) { return bf_W1(l) + kC * 2 * kC; }     // [64 x 64]
__host__ __device__ constexpr int bf_W2T(int l) { return bf_W2(l) + kC * kC; }        // [64 x 64]
__host__ __device__ constexpr int bf_W1T(int l) { return bf_W2T(l) + kC * kC; }       // [128 x 64]
constexpr int kBfTotal = kBfL0 + kLayers * kBfLayer;

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  return (uint32_t)bf16_bits(a) | ((uint32_t)bf16_bits(b) << 16);
}
// eight floats -> one 16-byte chunk of BF16
__device__ __forceinline__ uint4 pack8(const float *v) {
  return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

// Stage a [rows x 64*kblocks] BF16 matrix (global, row-major) as a B operand.
__device__ __forceinline__ void stage_weights(uint8_t *dst, const uint16_t *__restrict__ W, int rows, int kblocks) {
  for (int idx = threadIdx.x; idx < rows * kblocks * 8; idx += blockDim.x) {
    const int r = idx / (kblocks * 8), rem = idx - r * kblocks * 8, kb = rem >> 3, c = rem & 7;
    const uint4 v = *reinterpret_cast<const uint4 *>(W + (int64_t)r * 64 * kblocks + kb * 64 + c * 8);
    *reinterpret_cast<uint4 *>(dst + kb * rows * 128 + umma::sw128_chunk(r, c)) = v;
  }
}
// Write this thread's row r of 64 floats (BF16) into K block `blk` of a 128-row A tile.
__device__ __forceinline__ void stage_row64(uint8_t *tile, int r, const float *v) {
#pragma unroll
  for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4 *>(tile + umma::sw128_chunk(r, c)) = pack8(v + 8 * c);
}

struct Sync {
  uint64_t mbar;
  uint32_t tslot;
};

// CTA-wide: make staged shared memory visible to the tensor core and order it before the MMA
__device__ __forceinline__ void smem_to_mma() {
  umma::fence_smem_async();
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
}
// thread 0 issued MMAs and committed to the barrier; every thread waits (bounded).  Returns false
// (CTA-uniform) on a timeout and records it.
__device__ __forceinline__ bool mma_done(Sync &sy, uint32_t &phase, int *err) {
  bool ok = umma::mbar_wait(umma::smem_u32(&sy.mbar), phase);
  phase ^= 1;
  ok = __syncthreads_and(ok);
  umma::fence_after();
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  return ok;
}
__device__ __forceinline__ void sync_setup(Sync &sy, uint32_t tmem_cols) {
  if (threadIdx.x < 32) umma::tmem_alloc(&sy.tslot, tmem_cols);
  if (threadIdx.x == 0) {
    umma::mbar_init(umma::smem_u32(&sy.mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
}
__device__ __forceinline__ void sync_teardown(Sync &sy, uint32_t phase, uint32_t tmem_cols, bool ok) {
  if (!ok) umma::mbar_wait(umma::smem_u32(&sy.mbar), phase ^ 1);   // bounded drain of the failed phase
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  if (threadIdx.x < 32) umma::tmem_dealloc(sy.tslot, tmem_cols);
}
// this thread's TMEM lane (row 32*warp + lane), 64 columns from `col`
__device__ __forceinline__ void tmem_row64(uint32_t tmem, int col, float *v) {
  const uint32_t base = tmem + ((uint32_t)(32 * (threadIdx.x >> 5)) << 16) + col;
#pragma unroll
  for (int c = 0; c < 64; c += 16) umma::tmem_ld16(base + c, v + c);
}

struct Graph {
  int64_t n;                     // nodes
  const int32_t *__restrict__ nbr;   // n x 3, -1: none
};

// ---- forward -----------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_gnn_encoder(Graph g, const float *__restrict__ x,
                                                     const uint16_t *__restrict__ wbf, const float *__restrict__ prm,
                                                     float *__restrict__ h0, int *err) {
  extern __shared__ uint8_t smraw[];
  __shared__ Sync sy;
  uint8_t *sm = align1024(smraw);
  uint8_t *sA = sm, *sB = sm + 128 * 128;
  const int r = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 128 + r;
  float v[64];
#pragma unroll
  for (int k = 0; k < 64; ++k) v[k] = 0.f;
  if (i < g.n)
    for (int k = 0; k < kFin; ++k) v[k] = x[i * kFin + k];
  stage_row64(sA, r, v);
  stage_weights(sB, wbf + kBfWe, kC, 1);
  sync_setup(sy, 64);
  uint32_t phase = 0;
  smem_to_mma();
  if (threadIdx.x == 0) {
    umma::mma_tile<64>(sy.tslot, umma::smem_u32(sA), umma::smem_u32(sB), 1, false);
    umma::commit(umma::smem_u32(&sy.mbar));
  }
  const bool ok = mma_done(sy, phase, err);
  if (ok) {
    tmem_row64(sy.tslot, 0, v);
    if (i < g.n)
      for (int k = 0; k < kC; ++k) h0[i * kC + k] = fmaxf(v[k] + prm[kOffBe + k], 0.f);
  }
  sync_teardown(sy, phase, 64, ok);
}

// mean of the neighbours' rows (FP32, neighbour order), and the degree
__device__ __forceinline__ int neighbour_mean(const Graph &g, const float *__restrict__ h, int64_t i, float *a) {
#pragma unroll
  for (int k = 0; k < kC; ++k) a[k] = 0.f;
  int deg = 0;
  for (int q = 0; q < kNb; ++q) {
    const int32_t j = g.nbr[i * kNb + q];
    if (j < 0) continue;
    const float4 *hj = reinterpret_cast<const float4 *>(h + (int64_t)j * kC);
#pragma unroll
    for (int k = 0; k < kC / 4; ++k) {
      const float4 t = hj[k];
      a[4 * k] += t.x;
      a[4 * k + 1] += t.y;
      a[4 * k + 2] += t.z;
      a[4 * k + 3] += t.w;
    }
    ++deg;
  }
  if (deg > 0) {
    const float inv = 1.0f / (float)deg;
#pragma unroll
    for (int k = 0; k < kC; ++k) a[k] *= inv;
  }
  return deg;
}

__global__ void __launch_bounds__(128) k_gnn_layer_fwd(Graph g, int layer, const uint16_t *__restrict__ wbf,
                                                       const float *__restrict__ prm, const float *__restrict__ h_in,
                                                       float *__restrict__ h_out, uint16_t *__restrict__ t_out,
                                                       int *err) {
  extern __shared__ uint8_t smraw[];
  __shared__ Sync sy;
  uint8_t *sm = align1024(smraw);
  uint8_t *sA1 = sm;                       // 128 x 128 (2 K blocks)
  uint8_t *sB1 = sA1 + 2 * 128 * 128;      // 64 x 128
  uint8_t *sA2 = sB1 + 2 * 64 * 128;       // 128 x 64
  uint8_t *sB2 = sA2 + 128 * 128;          // 64 x 64
  const int r = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 128 + r;
  float v[64];
  if (i < g.n) {
    const float4 *hi = reinterpret_cast<const float4 *>(h_in + i * kC);
#pragma unroll
    for (int k = 0; k < kC / 4; ++k) {
      const float4 t = hi[k];
      v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kC; ++k) v[k] = 0.f;
  }
  stage_row64(sA1, r, v);
  if (i < g.n) {
    neighbour_mean(g, h_in, i, v);
  } else {
#pragma unroll
    for (int k = 0; k < kC; ++k) v[k] = 0.f;
  }
  stage_row64(sA1 + 128 * 128, r, v);
  stage_weights(sB1, wbf + bf_W1(layer), kC, 2);
  stage_weights(sB2, wbf + bf_W2(layer), kC, 1);
  sync_setup(sy, 128);
  uint32_t phase = 0;
  smem_to_mma();
  if (threadIdx.x == 0) {
    umma::mma_tile<64>(sy.tslot, umma::smem_u32(sA1), umma::smem_u32(sB1), 2, false);
    umma::commit(umma::smem_u32(&sy.mbar));
  }
  bool ok = mma_done(sy, phase, err);
  if (ok) {
    tmem_row64(sy.tslot, 0, v);
    const float *b1 = prm + off_b1(layer);
#pragma unroll
    for (int k = 0; k < kC; ++k) v[k] = fmaxf(v[k] + b1[k], 0.f);
    if (i < g.n) {
      uint4 *to = reinterpret_cast<uint4 *>(t_out + i * kC);
#pragma unroll
      for (int c = 0; c < 8; ++c) to[c] = pack8(v + 8 * c);
    }
    stage_row64(sA2, r, v);
    smem_to_mma();
    if (threadIdx.x == 0) {
      umma::mma_tile<64>(sy.tslot + 64, umma::smem_u32(sA2), umma::smem_u32(sB2), 1, false);
      umma::commit(umma::smem_u32(&sy.mbar));
    }
    ok = mma_done(sy, phase, err);
    if (ok) {
      tmem_row64(sy.tslot, 64, v);
      if (i < g.n) {
        const float *b2 = prm + off_b2(layer);
        const float *hi = h_in + i * kC;
        float *ho = h_out + i * kC;
        for (int k = 0; k < kC; ++k) ho[k] = hi[k] + (v[k] + b2[k]);
      }
    }
  }
  sync_teardown(sy, phase, 128, ok);
}

// y = Wd h + bd; with targets: loss partials, dy and dh = Wd^T dy.  w: per-node loss weight
// divided by the batch's total weight (0 for nodes outside the loss).
__global__ void k_gnn_decoder(Graph g, const float *__restrict__ prm, const float *__restrict__ h,
                              float *__restrict__ y, const float *__restrict__ target, const float *__restrict__ w,
                              float *__restrict__ dh, double *__restrict__ loss_part) {
  __shared__ double red[256];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < g.n) {
    const float *hi = h + i * kC;
    float yo[kGnnOut];
#pragma unroll
    for (int c = 0; c < kGnnOut; ++c) {
      float sc = 0.f;
      for (int k = 0; k < kC; ++k) sc += prm[kOffWd + c * kC + k] * hi[k];
      yo[c] = prm[kOffBd + c] + sc;
      y[kGnnOut * i + c] = yo[c];
    }
    if (target) {
      const float wi = w[i];
      float d[kGnnOut];
#pragma unroll
      for (int c = 0; c < kGnnOut; ++c) {
        const float e = yo[c] - target[kGnnOut * i + c];
        l += (double)wi * ((double)e * e);
        d[c] = 2.f * wi * e;
      }
      float *dhi = dh + i * kC;
      for (int k = 0; k < kC; ++k) {
        float a = 0.f;
#pragma unroll
        for (int c = 0; c < kGnnOut; ++c) a += prm[kOffWd + c * kC + k] * d[c];
        dhi[k] = a;
      }
#pragma unroll
      for (int c = 0; c < kGnnOut; ++c) y[kGnnOut * i + c] = d[c];   // dy replaces y when training
    }
  }
  if (loss_part) {
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
  }
}

// ---- backward ------------------------------------------------------------------------------------
// dt = dh_out W2 (masked by t > 0) -> ds; dz = ds W1 -> dh_acc = dh_out + dz[:64],
// dA = dz[64:] / deg (what each neighbour of i receives through the mean).
__global__ void __launch_bounds__(128) k_gnn_layer_bwd(Graph g, int layer, const uint16_t *__restrict__ wbf,
                                                       const float *__restrict__ dh_out,
                                                       const uint16_t *__restrict__ t_in, float *__restrict__ ds_out,
                                                       float *__restrict__ dh_acc, float *__restrict__ dA, int *err) {
  extern __shared__ uint8_t smraw[];
  __shared__ Sync sy;
  uint8_t *sm = align1024(smraw);
  uint8_t *sA = sm;                    // 128 x 64: dh_out
  uint8_t *sB = sA + 128 * 128;        // 64 x 64: W2^T
  uint8_t *sA2 = sB + 64 * 128;        // 128 x 64: ds
  uint8_t *sB2 = sA2 + 128 * 128;      // 128 x 64: W1^T
  const int r = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 128 + r;
  float v[64];
  if (i < g.n) {
    for (int k = 0; k < kC; ++k) v[k] = dh_out[i * kC + k];
  } else {
    for (int k = 0; k < kC; ++k) v[k] = 0.f;
  }
  stage_row64(sA, r, v);
  stage_weights(sB, wbf + bf_W2T(layer), kC, 1);
  stage_weights(sB2, wbf + bf_W1T(layer), 2 * kC, 1);
  sync_setup(sy, 256);
  uint32_t phase = 0;
  smem_to_mma();
  if (threadIdx.x == 0) {
    umma::mma_tile<64>(sy.tslot, umma::smem_u32(sA), umma::smem_u32(sB), 1, false);
    umma::commit(umma::smem_u32(&sy.mbar));
  }
  bool ok = mma_done(sy, phase, err);
  if (ok) {
    tmem_row64(sy.tslot, 0, v);
    if (i < g.n) {
      const uint16_t *ti = t_in + i * kC;
      for (int k = 0; k < kC; ++k) {
        const float tv = __bfloat162float(__ushort_as_bfloat16(ti[k]));
        v[k] = tv > 0.f ? v[k] : 0.f;
        ds_out[i * kC + k] = v[k];
      }
    } else {
      for (int k = 0; k < kC; ++k) v[k] = 0.f;
    }
    stage_row64(sA2, r, v);
    smem_to_mma();
    if (threadIdx.x == 0) {
      umma::mma_tile<128>(sy.tslot + 64, umma::smem_u32(sA2), umma::smem_u32(sB2), 1, false);
      umma::commit(umma::smem_u32(&sy.mbar));
    }
    ok = mma_done(sy, phase, err);
    if (ok) {   // tcgen05.ld is warp-collective: every thread loads, only real rows store
      tmem_row64(sy.tslot, 64, v);
      if (i < g.n)
        for (int k = 0; k < kC; ++k) dh_acc[i * kC + k] = dh_out[i * kC + k] + v[k];
      tmem_row64(sy.tslot, 128, v);
      if (i < g.n) {
        int deg = 0;
        for (int q = 0; q < kNb; ++q) deg += g.nbr[i * kNb + q] >= 0;
        const float inv = deg > 0 ? 1.0f / (float)deg : 0.f;
        for (int k = 0; k < kC; ++k) dA[i * kC + k] = v[k] * inv;
      }
    }
  }
  sync_teardown(sy, phase, 256, ok);
}

// dh_in[j] = dh_acc[j] + sum over the neighbours i of j of dA[i] (the adjacency is symmetric)
__global__ void k_gnn_gather_bwd(Graph g, const float *__restrict__ dh_acc, const float *__restrict__ dA,
                                 float *__restrict__ dh_in) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.n * kC) return;
  const int64_t j = t / kC;
  const int k = (int)(t - j * kC);
  float s = dh_acc[t];
  for (int q = 0; q < kNb; ++q) {
    const int32_t i = g.nbr[j * kNb + q];
    if (i >= 0) s += dA[(int64_t)i * kC + k];
  }
  dh_in[t] = s;
}

// encoder backward: ds_e = dh0 * (h0 > 0) in place
__global__ void k_gnn_relu_bwd(int64_t total, const float *__restrict__ h0, float *__restrict__ dh0) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < total && !(h0[t] > 0.f)) dh0[t] = 0.f;
}

// Weight gradients as tensor-core reductions over nodes: D[128 x 64] += A^T B over chunks of 128
// nodes, A = the layer input rows (up to 128 features, zero-padded), B = the output gradient rows
// (64).  Both are transposed while staged (feature rows, node columns).  Per CTA: partial D and
// the column sums of B (bias gradient).
enum WgradMode { kWgEncoder = 0, kWgW1 = 1, kWgW2 = 2 };

template <int MODE>
__global__ void __launch_bounds__(128) k_gnn_wgrad(Graph g, const float *__restrict__ in0,
                                                   const uint16_t *__restrict__ in_bf, const float *__restrict__ gout,
                                                   float *__restrict__ part, float *__restrict__ bpart, int *err) {
  extern __shared__ uint8_t smraw[];
  __shared__ Sync sy;
  uint8_t *sm = align1024(smraw);
  uint8_t *sA = sm;                    // 128 features x 128 nodes (2 K blocks of 64 nodes)
  uint8_t *sB = sA + 2 * 128 * 128;    // 64 outputs x 128 nodes
  const int r = threadIdx.x;
  sync_setup(sy, 64);
  uint32_t phase = 0;
  float bsum[kC];
  for (int k = 0; k < kC; ++k) bsum[k] = 0.f;
  const int64_t nchunks = (g.n + 127) / 128;
  bool ok = true;
  bool first = true;
  for (int64_t ch = blockIdx.x; ch < nchunks && ok; ch += gridDim.x) {
    const int64_t i = ch * 128 + r;
    const int kb = r >> 6, kk = r & 63;
    uint8_t *aBase = sA + kb * 128 * 128;
    uint8_t *bBase = sB + kb * 64 * 128;
    float v[64];
    // A^T column (features of node i)
    if (MODE == kWgW1) {
      if (i < g.n) {
        for (int k = 0; k < kC; ++k) v[k] = in0[i * kC + k];
      } else {
        for (int k = 0; k < kC; ++k) v[k] = 0.f;
      }
      for (int f = 0; f < kC; ++f)
        *reinterpret_cast<uint16_t *>(aBase + umma::sw128_offset(f, kk)) = bf16_bits(v[f]);
      if (i < g.n) {
        neighbour_mean(g, in0, i, v);
      } else {
        for (int k = 0; k < kC; ++k) v[k] = 0.f;
      }
      for (int f = 0; f < kC; ++f)
        *reinterpret_cast<uint16_t *>(aBase + umma::sw128_offset(kC + f, kk)) = bf16_bits(v[f]);
    } else {
      for (int f = 0; f < 128; ++f) {
        float x = 0.f;
        if (i < g.n) {
          if (MODE == kWgEncoder && f < kFin) x = in0[i * kFin + f];
          if (MODE == kWgW2 && f < kC) x = __bfloat162float(__ushort_as_bfloat16(in_bf[i * kC + f]));
        }
        *reinterpret_cast<uint16_t *>(aBase + umma::sw128_offset(f, kk)) = bf16_bits(x);
      }
    }
    // B^T column (output gradient of node i)
    for (int o = 0; o < kC; ++o) {
      const float gv = i < g.n ? gout[i * kC + o] : 0.f;
      bsum[o] += gv;
      *reinterpret_cast<uint16_t *>(bBase + umma::sw128_offset(o, kk)) = bf16_bits(gv);
    }
    smem_to_mma();
    if (threadIdx.x == 0) {
      umma::mma_tile<64>(sy.tslot, umma::smem_u32(sA), umma::smem_u32(sB), 2, !first);
      umma::commit(umma::smem_u32(&sy.mbar));
    }
    ok = mma_done(sy, phase, err);
    first = false;
  }
  // per-CTA partials: D (row f = input feature, column o = output), bias column sums
  float *pd = part + (int64_t)blockIdx.x * 128 * kC;
  if (ok) {
    float v[64];
    if (!first) {
      tmem_row64(sy.tslot, 0, v);
    } else {
      for (int k = 0; k < kC; ++k) v[k] = 0.f;
    }
    for (int o = 0; o < kC; ++o) pd[(int64_t)r * kC + o] = v[o];
  }
  // bias partial: reduce bsum over the CTA's threads in a fixed order through shared memory
  float *red = reinterpret_cast<float *>(sA);   // 128 x 64 floats = 32 KB, free after the MMAs
  __syncthreads();
  for (int o = 0; o < kC; ++o) red[r * kC + o] = bsum[o];
  __syncthreads();
  if (r < kC) {
    float s = 0.f;
    for (int t = 0; t < 128; ++t) s += red[t * kC + r];
    bpart[(int64_t)blockIdx.x * kC + r] = s;
  }
  sync_teardown(sy, phase, 64, ok);
}

// Sum the per-CTA partials in CTA order into the gradient vector.
//   kWgEncoder: dWe[o][f] (f < 16) and dbe;  kWgW1: dW1[o][f] (f < 128) and db1;  kWgW2: dW2[o][f], db2.
__global__ void k_gnn_wgrad_reduce(int mode, int layer, int nparts, const float *__restrict__ part,
                                   const float *__restrict__ bpart, float *__restrict__ grad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int fin = mode == kWgEncoder ? kFin : (mode == kWgW1 ? 2 * kC : kC);
  const int wsize = kC * fin;
  if (t < wsize) {
    const int o = t / fin, f = t - o * fin;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += part[(int64_t)p * 128 * kC + f * kC + o];
    const int off = mode == kWgEncoder ? kOffWe : (mode == kWgW1 ? off_W1(layer) : off_W2(layer));
    grad[off + o * fin + f] = s;
  } else if (t < wsize + kC) {
    const int o = t - wsize;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += bpart[(int64_t)p * kC + o];
    const int off = mode == kWgEncoder ? kOffBe : (mode == kWgW1 ? off_b1(layer) : off_b2(layer));
    grad[off + o] = s;
  }
}

// decoder gradient partials: per block, dWd[c][k] = sum_i dy_i[c] h_i[k] and dbd[c] over a fixed
// node range; one warp per node row (lane k reads h[k], h[k+32]), warps combined in order.
constexpr int kDecParts = kGnnOut * kC + kGnnOut;
static_assert(kDecParts <= 256, "the decoder partials are summed by one 256-thread block");
__global__ void k_gnn_decoder_grad(Graph g, const float *__restrict__ dy, const float *__restrict__ h,
                                   float *__restrict__ part) {
  __shared__ float red[8][kDecParts];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float a0[kGnnOut], a1[kGnnOut], b[kGnnOut];
#pragma unroll
  for (int c = 0; c < kGnnOut; ++c) a0[c] = a1[c] = b[c] = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * nw + warp; i < g.n; i += (int64_t)gridDim.x * nw) {
    const float h0 = h[i * kC + lane], h1 = h[i * kC + lane + 32];
#pragma unroll
    for (int c = 0; c < kGnnOut; ++c) {
      const float d = dy[kGnnOut * i + c];
      a0[c] += d * h0;
      a1[c] += d * h1;
      b[c] += d;
    }
  }
#pragma unroll
  for (int c = 0; c < kGnnOut; ++c) {
    red[warp][c * kC + lane] = a0[c];
    red[warp][c * kC + lane + 32] = a1[c];
    if (lane == 0) red[warp][kGnnOut * kC + c] = b[c];
  }
  __syncthreads();
  if ((int)threadIdx.x < kDecParts) {
    float s = 0.f;
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    part[(int64_t)blockIdx.x * kDecParts + threadIdx.x] = s;
  }
}

__global__ void k_gnn_decoder_reduce(int nparts, const float *__restrict__ part, float *__restrict__ grad) {
  const int t = threadIdx.x;
  if (t >= kDecParts) return;
  float s = 0.f;
  for (int p = 0; p < nparts; ++p) s += part[(int64_t)p * kDecParts + t];
  grad[t < kGnnOut * kC ? kOffWd + t : kOffBd + (t - kGnnOut * kC)] = s;
}

// Adam (FP32) on the flat parameter vector
__global__ void k_gnn_adam(int n, float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                           float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float g = gr[t];
  const float mt = b1 * m[t] + (1.f - b1) * g;
  const float vt = b2 * v[t] + (1.f - b2) * g * g;
  m[t] = mt;
  v[t] = vt;
  p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

// BF16 tile copies of the weights
__global__ void k_gnn_pack(const float *__restrict__ prm, uint16_t *__restrict__ wbf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < kC * kC) {   // We padded to 64 inputs
    const int o = t / kC, f = t % kC;
    wbf[kBfWe + t] = bf16_bits(f < kFin ? prm[kOffWe + o * kFin + f] : 0.f);
  }
  for (int l = 0; l < kLayers; ++l) {
    if (t < kC * 2 * kC) {
      const int o = t / (2 * kC), f = t % (2 * kC);
      const float w1 = prm[off_W1(l) + o * 2 * kC + f];
      wbf[bf_W1(l) + t] = bf16_bits(w1);
      wbf[bf_W1T(l) + f * kC + o] = bf16_bits(w1);
    }
    if (t < kC * kC) {
      const int o = t / kC, f = t % kC;
      const float w2 = prm[off_W2(l) + t];
      wbf[bf_W2(l) + t] = bf16_bits(w2);
      wbf[bf_W2T(l) + f * kC + o] = bf16_bits(w2);
    }
  }
}

template <int N>
void launch_gemm_tile_test(cudaStream_t s, int M, int K, const __nv_bfloat16 *X, const __nv_bfloat16 *W, float *Y,
                           int *err) {
  const int kblocks = K / 64;
  const size_t smem = (size_t)kblocks * (128 + N) * 128 + 1024;
  UFE_CUDA(cudaFuncSetAttribute(k_gemm_tile_test<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_gemm_tile_test<N><<<M / 128, 128, smem, s>>>(M, K, X, W, Y, err);
  UFE_CUDA(cudaGetLastError());
}

}  // namespace

extern "C" int32_t ufe_umma_gemm_bf16(ufe_ctx *ctx, int32_t M, int32_t N, int32_t K, const uint16_t *X,
                                      const uint16_t *W, float *Y) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(M > 0 && M % 128 == 0 && (N == 64 || N == 128) && K > 0 && K % 64 == 0 && K <= 256,
                UFE_ERR_INVALID, "umma gemm: need M % 128 == 0, N in {64, 128}, K % 64 == 0, K <= 256");
    UFE_REQUIRE(X && W && Y, UFE_ERR_INVALID, "umma gemm: NULL argument");
    UFE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t nx = (size_t)M * K, nw = (size_t)N * K, ny = (size_t)M * N;
    uint8_t *buf = (uint8_t *)dev_alloc(nx * 2 + nw * 2 + ny * 4 + 256);
    __nv_bfloat16 *dX = (__nv_bfloat16 *)buf;
    __nv_bfloat16 *dW = dX + nx;
    float *dY = (float *)(buf + ((nx * 2 + nw * 2 + 15) & ~size_t(15)));
    int *err = (int *)(dY + ny);
    int herr = 0;
    try {
      UFE_CUDA(cudaMemcpyAsync(dX, X, nx * 2, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemcpyAsync(dW, W, nw * 2, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
      if (N == 64)
        launch_gemm_tile_test<64>(s, M, K, dX, dW, dY, err);
      else
        launch_gemm_tile_test<128>(s, M, K, dX, dW, dY, err);
      UFE_CUDA(cudaMemcpyAsync(Y, dY, ny * 4, cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      dev_free(buf);
      throw;
    }
    dev_free(buf);
    UFE_REQUIRE(herr == 0, UFE_ERR_DEVICE, "umma gemm: tensor-core completion timed out");
    return UFE_OK;
  });
}

// ================================================================================================
// Host side
struct GnnMember {
  int64_t n = 0;
  int32_t *nbr = nullptr;
  float *x = nullptr, *y = nullptr, *w = nullptr;   // features, targets, loss weights (sum 1)
};

struct ufe_gnn {
  ufe_ctx *ctx = nullptr;            // device, stream and error text (must outlive the network)
  int device = 0;
  float *prm = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  uint16_t *wbf = nullptr;
  int *err = nullptr;
  int64_t adam_t = 0;
  int64_t cap = 0;                   // node capacity of the work buffers
  float *h[kLayers + 1] = {};
  uint16_t *t[kLayers] = {};
  float *ds = nullptr, *dhA = nullptr, *dhB = nullptr, *dacc = nullptr, *dA = nullptr, *ybuf = nullptr;
  float *part = nullptr, *bpart = nullptr, *dpart = nullptr;
  double *loss_part = nullptr;
  double *loss_host = nullptr;       // pinned
  int64_t loss_cap = 0;
  // scratch for explicit graphs and mesh features
  int32_t *gnbr = nullptr;
  float *gx = nullptr, *gy = nullptr, *gw = nullptr, *gmask = nullptr;
  int64_t gcap = 0;
  std::vector<GnnMember> data;
};

namespace {

constexpr int kWgradBlocks = 2 * 152;
constexpr int kDecBlocks = 152;
constexpr size_t kSmemEncoder = 48 * 1024;      // caps residency at 4 CTAs/SM (64 TMEM columns each)
constexpr size_t kSmemLayerFwd = 74 * 1024;     // 3 CTAs/SM x 128 columns
constexpr size_t kSmemLayerBwd = 100 * 1024;    // 2 CTAs/SM x 256 columns
constexpr size_t kSmemWgrad = 50 * 1024;        // 4 CTAs/SM x 64 columns

void gnn_free_buffers(ufe_gnn *g) {
  for (auto &p : g->h) { dev_free(p); p = nullptr; }
  for (auto &p : g->t) { dev_free(p); p = nullptr; }
  void *ptrs[] = {g->ds, g->dhA, g->dhB, g->dacc, g->dA, g->ybuf, g->loss_part};
  for (void *p : ptrs) dev_free(p);
  g->ds = g->dhA = g->dhB = g->dacc = g->dA = g->ybuf = nullptr;
  g->loss_part = nullptr;
  g->cap = 0;
}

void gnn_ensure(ufe_gnn *g, int64_t n) {
  if (g->cap >= n) return;
  gnn_free_buffers(g);
  const size_t rows = (size_t)n * kC;
  for (auto &p : g->h) p = (float *)dev_alloc(rows * 4);
  for (auto &p : g->t) p = (uint16_t *)dev_alloc(rows * 2);
  g->ds = (float *)dev_alloc(rows * 4);
  g->dhA = (float *)dev_alloc(rows * 4);
  g->dhB = (float *)dev_alloc(rows * 4);
  g->dacc = (float *)dev_alloc(rows * 4);
  g->dA = (float *)dev_alloc(rows * 4);
  g->ybuf = (float *)dev_alloc((size_t)n * kGnnOut * 4);
  const int64_t nb = (n + 255) / 256;
  g->loss_part = (double *)dev_alloc(sizeof(double) * nb);
  if (g->loss_cap < nb) {
    if (g->loss_host) cudaFreeHost(g->loss_host);
    UFE_CUDA(cudaMallocHost(&g->loss_host, sizeof(double) * nb));
    g->loss_cap = nb;
  }
  g->cap = n;
}

void gnn_ensure_scratch(ufe_gnn *g, int64_t n) {
  if (g->gcap >= n) return;
  void *ptrs[] = {g->gnbr, g->gx, g->gy, g->gw, g->gmask};
  for (void *p : ptrs) dev_free(p);
  g->gnbr = (int32_t *)dev_alloc(sizeof(int32_t) * 3 * n);
  g->gx = (float *)dev_alloc(sizeof(float) * kFin * n);
  g->gy = (float *)dev_alloc(sizeof(float) * kGnnOut * n);
  g->gw = (float *)dev_alloc(sizeof(float) * n);
  g->gmask = (float *)dev_alloc(sizeof(float) * n);
  g->gcap = n;
}

void set_attrs() {
  static bool done = false;
  if (done) return;
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_encoder, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemEncoder));
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_layer_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLayerFwd));
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_layer_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLayerBwd));
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_wgrad<kWgEncoder>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kSmemWgrad));
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_wgrad<kWgW1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemWgrad));
  UFE_CUDA(cudaFuncSetAttribute(k_gnn_wgrad<kWgW2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemWgrad));
  done = true;
}

// forward over a graph already on the device; y gets the outputs.  With targets: loss partials,
// dy (in ybuf) and dh of the last layer (in dhA).
void gnn_forward(ufe_gnn *g, cudaStream_t s, const Graph &gr, const float *x, const float *target, const float *w) {
  set_attrs();
  gnn_ensure(g, gr.n);
  const unsigned tiles = (unsigned)((gr.n + 127) / 128);
  k_gnn_encoder<<<tiles, 128, kSmemEncoder, s>>>(gr, x, g->wbf, g->prm, g->h[0], g->err);
  UFE_CUDA(cudaGetLastError());
  for (int l = 0; l < kLayers; ++l) {
    k_gnn_layer_fwd<<<tiles, 128, kSmemLayerFwd, s>>>(gr, l, g->wbf, g->prm, g->h[l], g->h[l + 1], g->t[l], g->err);
    UFE_CUDA(cudaGetLastError());
  }
  k_gnn_decoder<<<(unsigned)((gr.n + 255) / 256), 256, 0, s>>>(gr, g->prm, g->h[kLayers], g->ybuf, target, w, g->dhA,
                                                                 target ? g->loss_part : nullptr);
  UFE_CUDA(cudaGetLastError());
}

void wgrad(ufe_gnn *g, cudaStream_t s, const Graph &gr, int mode, int layer, const float *in0, const uint16_t *in_bf,
           const float *gout) {
  const int64_t nchunks = (gr.n + 127) / 128;
  const int G = (int)std::min<int64_t>(nchunks, kWgradBlocks);
  if (mode == kWgEncoder)
    k_gnn_wgrad<kWgEncoder><<<G, 128, kSmemWgrad, s>>>(gr, in0, in_bf, gout, g->part, g->bpart, g->err);
  else if (mode == kWgW1)
    k_gnn_wgrad<kWgW1><<<G, 128, kSmemWgrad, s>>>(gr, in0, in_bf, gout, g->part, g->bpart, g->err);
  else
    k_gnn_wgrad<kWgW2><<<G, 128, kSmemWgrad, s>>>(gr, in0, in_bf, gout, g->part, g->bpart, g->err);
  UFE_CUDA(cudaGetLastError());
  const int fin = mode == kWgEncoder ? kFin : (mode == kWgW1 ? 2 * kC : kC);
  k_gnn_wgrad_reduce<<<(kC * fin + kC + 255) / 256, 256, 0, s>>>(mode, layer, G, g->part, g->bpart, g->grad);
  UFE_CUDA(cudaGetLastError());
}

// backward after gnn_forward with targets: the full gradient in g->grad
void gnn_backward(ufe_gnn *g, cudaStream_t s, const Graph &gr, const float *x) {
  const unsigned tiles = (unsigned)((gr.n + 127) / 128);
  k_gnn_decoder_grad<<<kDecBlocks, 256, 0, s>>>(gr, g->ybuf, g->h[kLayers], g->dpart);
  UFE_CUDA(cudaGetLastError());
  k_gnn_decoder_reduce<<<1, 256, 0, s>>>(kDecBlocks, g->dpart, g->grad);   // kDecParts <= 256
  UFE_CUDA(cudaGetLastError());
  float *cur = g->dhA, *nxt = g->dhB;
  for (int l = kLayers - 1; l >= 0; --l) {
    k_gnn_layer_bwd<<<tiles, 128, kSmemLayerBwd, s>>>(gr, l, g->wbf, cur, g->t[l], g->ds, g->dacc, g->dA, g->err);
    UFE_CUDA(cudaGetLastError());
    wgrad(g, s, gr, kWgW2, l, nullptr, g->t[l], cur);
    wgrad(g, s, gr, kWgW1, l, g->h[l], nullptr, g->ds);
    k_gnn_gather_bwd<<<(unsigned)((gr.n * kC + 255) / 256), 256, 0, s>>>(gr, g->dacc, g->dA, nxt);
    UFE_CUDA(cudaGetLastError());
    std::swap(cur, nxt);
  }
  k_gnn_relu_bwd<<<(unsigned)((gr.n * kC + 255) / 256), 256, 0, s>>>(gr.n * kC, g->h[0], cur);
  UFE_CUDA(cudaGetLastError());
  wgrad(g, s, gr, kWgEncoder, 0, x, nullptr, cur);
}

double gnn_loss(ufe_gnn *g, cudaStream_t s, int64_t n) {
  const int64_t nb = (n + 255) / 256;
  UFE_CUDA(cudaMemcpyAsync(g->loss_host, g->loss_part, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  double l = 0.0;
  for (int64_t b = 0; b < nb; ++b) l += g->loss_host[b];
  return l;
}

void gnn_check(ufe_gnn *g, cudaStream_t s) {
  int h = 0;
  UFE_CUDA(cudaMemcpyAsync(&h, g->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  UFE_REQUIRE(h == 0, UFE_ERR_DEVICE, "learned start: a tensor-core completion timed out");
}

void gnn_adam(ufe_gnn *g, cudaStream_t s, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  g->adam_t += 1;
  const float c1 = 1.f - (float)std::pow((double)b1, (double)g->adam_t);
  const float c2 = 1.f - (float)std::pow((double)b2, (double)g->adam_t);
  k_gnn_adam<<<(kParams + 255) / 256, 256, 0, s>>>(kParams, g->prm, g->grad, g->m, g->v, lr, b1, b2, eps, c1, c2);
  UFE_CUDA(cudaGetLastError());
  k_gnn_pack<<<(kC * 2 * kC + 255) / 256, 256, 0, s>>>(g->prm, g->wbf);
  UFE_CUDA(cudaGetLastError());
}

// weights: He-style uniform initialisation from a 64-bit LCG (host), biases zero
std::vector<float> init_params(uint64_t seed) {
  std::vector<float> p(kParams, 0.f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  auto fill = [&](int off, int out, int in, double gain) {
    const double a = gain * std::sqrt(3.0 / in);
    for (int i = 0; i < out * in; ++i) p[off + i] = (float)(a * uni());
  };
  fill(kOffWe, kC, kFin, std::sqrt(2.0));
  for (int l = 0; l < kLayers; ++l) {
    fill(off_W1(l), kC, 2 * kC, std::sqrt(2.0));
    fill(off_W2(l), kC, kC, 0.5);   // small residual branches at the start
  }
  fill(kOffWd, kGnnOut, kC, 1.0);
  return p;
}

Graph upload_graph(ufe_gnn *g, cudaStream_t s, int64_t n, const int32_t *nbr, const float *x) {
  gnn_ensure_scratch(g, n);
  for (int64_t i = 0; i < 3 * n; ++i)
    UFE_REQUIRE(nbr[i] >= -1 && nbr[i] < n, UFE_ERR_INVALID, "learned start: neighbour index out of range");
  UFE_CUDA(cudaMemcpyAsync(g->gnbr, nbr, sizeof(int32_t) * 3 * n, cudaMemcpyHostToDevice, s));
  UFE_CUDA(cudaMemcpyAsync(g->gx, x, sizeof(float) * kFin * n, cudaMemcpyHostToDevice, s));
  return Graph{n, g->gnbr};
}

}  // namespace

extern "C" int32_t ufe_gnn_param_count(void) { return kParams; }

extern "C" int32_t ufe_gnn_create(ufe_ctx *ctx, uint64_t seed, ufe_gnn **out) {
  if (!out) return UFE_ERR_INVALID;
  *out = nullptr;
  return guarded(ctx, [&]() -> int32_t {
    UFE_CUDA(cudaSetDevice(ctx->device));
    ufe_gnn *g = new ufe_gnn();
    g->ctx = ctx;
    g->device = ctx->device;
    try {
      g->prm = (float *)dev_alloc(sizeof(float) * kParams);
      g->grad = (float *)dev_alloc(sizeof(float) * kParams);
      g->m = (float *)dev_alloc(sizeof(float) * kParams);
      g->v = (float *)dev_alloc(sizeof(float) * kParams);
      g->wbf = (uint16_t *)dev_alloc(sizeof(uint16_t) * kBfTotal);
      g->err = (int *)dev_alloc(sizeof(int));
      g->part = (float *)dev_alloc(sizeof(float) * kWgradBlocks * 128 * kC);
      g->bpart = (float *)dev_alloc(sizeof(float) * kWgradBlocks * kC);
      g->dpart = (float *)dev_alloc(sizeof(float) * kDecBlocks * kDecParts);
      cudaStream_t s = ctx->stream;
      const std::vector<float> p = init_params(seed);
      UFE_CUDA(cudaMemcpyAsync(g->prm, p.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemsetAsync(g->grad, 0, sizeof(float) * kParams, s));
      UFE_CUDA(cudaMemsetAsync(g->m, 0, sizeof(float) * kParams, s));
      UFE_CUDA(cudaMemsetAsync(g->v, 0, sizeof(float) * kParams, s));
      UFE_CUDA(cudaMemsetAsync(g->wbf, 0, sizeof(uint16_t) * kBfTotal, s));
      UFE_CUDA(cudaMemsetAsync(g->err, 0, sizeof(int), s));
      k_gnn_pack<<<(kC * 2 * kC + 255) / 256, 256, 0, s>>>(g->prm, g->wbf);
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      ufe_gnn_destroy(g);
      throw;
    }
    *out = g;
    return UFE_OK;
  });
}

extern "C" void ufe_gnn_destroy(ufe_gnn *g) {
  if (!g) return;
  // the owning context may already be gone: free through the device, not its stream
  cudaSetDevice(g->device);
  cudaDeviceSynchronize();
  for (auto &m : g->data) {
    dev_free(m.nbr);
    dev_free(m.x);
    dev_free(m.y);
    dev_free(m.w);
  }
  gnn_free_buffers(g);
  void *ptrs[] = {g->prm, g->grad, g->m, g->v, g->wbf, g->err, g->part, g->bpart, g->dpart,
                  g->gnbr, g->gx, g->gy, g->gw, g->gmask};
  for (void *p : ptrs) dev_free(p);
  if (g->loss_host) cudaFreeHost(g->loss_host);
  delete g;
}

extern "C" int32_t ufe_gnn_get_params(ufe_gnn *g, float *params) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(params, UFE_ERR_INVALID, "NULL params");
    UFE_CUDA(cudaMemcpyAsync(params, g->prm, sizeof(float) * kParams, cudaMemcpyDeviceToHost, g->ctx->stream));
    UFE_CUDA(cudaStreamSynchronize(g->ctx->stream));
    return UFE_OK;
  });
}

extern "C" int32_t ufe_gnn_set_params(ufe_gnn *g, const float *params) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(params, UFE_ERR_INVALID, "NULL params");
    cudaStream_t s = g->ctx->stream;
    UFE_CUDA(cudaMemcpyAsync(g->prm, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaMemsetAsync(g->m, 0, sizeof(float) * kParams, s));
    UFE_CUDA(cudaMemsetAsync(g->v, 0, sizeof(float) * kParams, s));
    g->adam_t = 0;
    k_gnn_pack<<<(kC * 2 * kC + 255) / 256, 256, 0, s>>>(g->prm, g->wbf);
    UFE_CUDA(cudaGetLastError());
    UFE_CUDA(cudaStreamSynchronize(s));
    return UFE_OK;
  });
}

extern "C" int32_t ufe_gnn_forward(ufe_gnn *g, int64_t n, const int32_t *nbr, const float *x, float *y) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(n >= 1 && nbr && x && y, UFE_ERR_INVALID, "gnn forward: bad arguments");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    cudaStream_t s = g->ctx->stream;
    const Graph gr = upload_graph(g, s, n, nbr, x);
    gnn_forward(g, s, gr, g->gx, nullptr, nullptr);
    UFE_CUDA(cudaMemcpyAsync(y, g->ybuf, sizeof(float) * kGnnOut * n, cudaMemcpyDeviceToHost, s));
    gnn_check(g, s);
    return UFE_OK;
  });
}

extern "C" int32_t ufe_gnn_loss_grad(ufe_gnn *g, int64_t n, const int32_t *nbr, const float *x, const float *target,
                                     const float *w, double *loss, float *grad) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(n >= 1 && nbr && x && target && w, UFE_ERR_INVALID, "gnn loss/grad: bad arguments");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    cudaStream_t s = g->ctx->stream;
    const Graph gr = upload_graph(g, s, n, nbr, x);
    UFE_CUDA(cudaMemcpyAsync(g->gy, target, sizeof(float) * kGnnOut * n, cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaMemcpyAsync(g->gw, w, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    gnn_forward(g, s, gr, g->gx, g->gy, g->gw);
    gnn_backward(g, s, gr, g->gx);
    if (grad) UFE_CUDA(cudaMemcpyAsync(grad, g->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s));
    const double l = gnn_loss(g, s, n);
    if (loss) *loss = l;
    gnn_check(g, s);
    return UFE_OK;
  });
}

// ---- the mesh path: training data from solves, warm start of a solve ---------------------------
extern "C" int32_t ufe_gnn_dataset_add(ufe_gnn *g, ufe_ctx *mesh_ctx, const float *features_before) {
  if (!g || !mesh_ctx) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(mesh_ctx->device == g->ctx->device, UFE_ERR_INVALID, "gnn and mesh contexts on different devices");
    UFE_REQUIRE(mesh_ctx->has_mesh && mesh_ctx->work, UFE_ERR_INVALID, "gnn dataset: no solved ice state");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    UFE_CUDA(cudaStreamSynchronize(g->ctx->stream));
    cudaStream_t s = mesh_ctx->stream;
    const int64_t n = mesh_ctx->nTri;
    GnnMember m;
    m.n = n;
    m.nbr = (int32_t *)dev_alloc(sizeof(int32_t) * 3 * n);
    m.x = (float *)dev_alloc(sizeof(float) * kFin * n);
    m.y = (float *)dev_alloc(sizeof(float) * kGnnOut * n);
    m.w = (float *)dev_alloc(sizeof(float) * n);
    try {
      gnn_mesh_graph(mesh_ctx, s, m.nbr);
      if (features_before) {
        // features the caller took before the solve (ufe_gnn_features), in the caller's triangle order
        std::vector<float> xi((size_t)kFin * n);
        const std::vector<int32_t> &pt = mesh_ctx->perm_t_h;
        for (int64_t t = 0; t < n; ++t)
          for (int k = 0; k < kFin; ++k) xi[(size_t)t * kFin + k] = features_before[(size_t)pt[t] * kFin + k];
        UFE_CUDA(cudaMemcpyAsync(m.x, xi.data(), sizeof(float) * kFin * n, cudaMemcpyHostToDevice, s));
        UFE_CUDA(cudaStreamSynchronize(s));
      } else {
        gnn_mesh_features(mesh_ctx, s, 0, m.x, nullptr);
      }
      gnn_mesh_velocity(mesh_ctx, s, m.y, false, nullptr);
      gnn_mesh_viscosity(mesh_ctx, s, m.y, false, nullptr);
      // loss weights: triangles with ice, equal weights summing to one
      std::vector<float> hx((size_t)kFin * n);
      UFE_CUDA(cudaMemcpyAsync(hx.data(), m.x, sizeof(float) * kFin * n, cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      int64_t cnt = 0;
      for (int64_t t = 0; t < n; ++t) cnt += hx[(size_t)t * kFin + 13] > 0.f;
      std::vector<float> hw(n);
      for (int64_t t = 0; t < n; ++t) hw[t] = (hx[(size_t)t * kFin + 13] > 0.f && cnt > 0) ? 1.f / (float)cnt : 0.f;
      UFE_CUDA(cudaMemcpyAsync(m.w, hw.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      dev_free(m.nbr);
      dev_free(m.x);
      dev_free(m.y);
      dev_free(m.w);
      throw;
    }
    g->data.push_back(m);
    return (int32_t)g->data.size();
  });
}

extern "C" int32_t ufe_gnn_dataset_clear(ufe_gnn *g) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_CUDA(cudaStreamSynchronize(g->ctx->stream));
    for (auto &m : g->data) {
      dev_free(m.nbr);
      dev_free(m.x);
      dev_free(m.y);
      dev_free(m.w);
    }
    g->data.clear();
    return UFE_OK;
  });
}

// Features of the mesh context's resident ice state, in the caller's triangle order (nTri x 16).
extern "C" int32_t ufe_gnn_features(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity, float *x) {
  if (!g || !mesh_ctx) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(mesh_ctx->device == g->ctx->device, UFE_ERR_INVALID, "gnn and mesh contexts on different devices");
    UFE_REQUIRE(mesh_ctx->has_mesh && mesh_ctx->work && x, UFE_ERR_INVALID, "gnn features: no ice state");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    cudaStream_t s = mesh_ctx->stream;
    const int64_t n = mesh_ctx->nTri;
    gnn_ensure_scratch(g, n);
    gnn_mesh_features(mesh_ctx, s, use_prev_velocity, g->gx, nullptr);
    std::vector<float> xi((size_t)kFin * n);
    UFE_CUDA(cudaMemcpyAsync(xi.data(), g->gx, sizeof(float) * kFin * n, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    const std::vector<int32_t> &pt = mesh_ctx->perm_t_h;
    for (int64_t t = 0; t < n; ++t)
      for (int k = 0; k < kFin; ++k) x[(size_t)pt[t] * kFin + k] = xi[(size_t)t * kFin + k];
    return UFE_OK;
  });
}

// Train on the stored members: `epochs` passes, one member per Adam step, member order shuffled
// per epoch with `seed`.  loss_per_epoch (optional, epochs entries): mean training loss.
extern "C" int32_t ufe_gnn_train(ufe_gnn *g, int32_t epochs, float lr, uint64_t seed, float *loss_per_epoch,
                                 double *device_ms) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(epochs >= 0 && lr > 0.f, UFE_ERR_INVALID, "gnn train: bad arguments");
    UFE_REQUIRE(!g->data.empty(), UFE_ERR_INVALID, "gnn train: empty dataset");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    cudaStream_t s = g->ctx->stream;
    std::vector<int> order(g->data.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    uint64_t st = seed * 2862933555777941757ull + 3037000493ull;
    float total_ms = 0.f;
    for (int e = 0; e < epochs; ++e) {
      for (size_t i = order.size(); i > 1; --i) {   // Fisher-Yates
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        std::swap(order[i - 1], order[(size_t)((st >> 33) % i)]);
      }
      double sum = 0.0;
      UFE_CUDA(cudaEventRecord(g->ctx->ev0, s));
      for (int idx : order) {
        const GnnMember &m = g->data[idx];
        const Graph gr{m.n, m.nbr};
        gnn_forward(g, s, gr, m.x, m.y, m.w);
        gnn_backward(g, s, gr, m.x);
        gnn_adam(g, s, lr);
        if (loss_per_epoch) sum += gnn_loss(g, s, m.n);
      }
      UFE_CUDA(cudaEventRecord(g->ctx->ev1, s));
      UFE_CUDA(cudaEventSynchronize(g->ctx->ev1));
      float ms = 0.f;
      UFE_CUDA(cudaEventElapsedTime(&ms, g->ctx->ev0, g->ctx->ev1));
      total_ms += ms;
      if (loss_per_epoch) loss_per_epoch[e] = (float)(sum / (double)order.size());
    }
    gnn_check(g, s);
    if (device_ms) *device_ms = total_ms;
    return UFE_OK;
  });
}

// Mean loss of the stored members (evaluation; no update).
extern "C" int32_t ufe_gnn_evaluate(ufe_gnn *g, double *mean_loss) {
  if (!g) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(!g->data.empty() && mean_loss, UFE_ERR_INVALID, "gnn evaluate: empty dataset");
    cudaStream_t s = g->ctx->stream;
    double sum = 0.0;
    for (const GnnMember &m : g->data) {
      gnn_forward(g, s, Graph{m.n, m.nbr}, m.x, m.y, m.w);
      sum += gnn_loss(g, s, m.n);
    }
    gnn_check(g, s);
    *mean_loss = sum / (double)g->data.size();
    return UFE_OK;
  });
}

// Warm start: predict the velocity of the mesh context's resident ice state and store it as the
// resident velocity, so that ufe_solve_ssa_resident / ufe_solve_diva_resident with cold_start = 0
// start the Picard loop from it; `smooth_passes` averaging passes over each triangle and its
// neighbours take the prediction's small-scale noise out first.  With `with_viscosity` the
// predicted vertically averaged viscosity is stored on the vertices as well and the next solve's
// first Picard iteration uses it in place of Glen's law (SSA: the viscosity; DIVA: every layer).
// Kernels one prediction launches: graph, features, encoder, the layers, decoder, velocity store,
// two per smoothing pass, and the viscosity store.
extern "C" int32_t ufe_gnn_predict_kernels(int32_t smooth_passes) {
  return 1 + 1 + (2 + kLayers) + 1 + 2 * (smooth_passes > 0 ? smooth_passes : 0);
}

extern "C" int32_t ufe_gnn_predict_start(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity,
                                         int32_t smooth_passes, int32_t with_viscosity, double *device_ms) {
  if (!g || !mesh_ctx) return UFE_ERR_INVALID;
  return guarded(g->ctx, [&]() -> int32_t {
    UFE_REQUIRE(mesh_ctx->device == g->ctx->device, UFE_ERR_INVALID, "gnn and mesh contexts on different devices");
    UFE_REQUIRE(mesh_ctx->has_mesh && mesh_ctx->work, UFE_ERR_INVALID, "gnn predict: upload the ice state first");
    UFE_CUDA(cudaSetDevice(g->ctx->device));
    UFE_CUDA(cudaStreamSynchronize(g->ctx->stream));
    cudaStream_t s = mesh_ctx->stream;
    const int64_t n = mesh_ctx->nTri;
    gnn_ensure_scratch(g, n);
    UFE_CUDA(cudaEventRecord(mesh_ctx->ev0, s));
    gnn_mesh_graph(mesh_ctx, s, g->gnbr);
    gnn_mesh_features(mesh_ctx, s, use_prev_velocity, g->gx, g->gmask);
    gnn_forward(g, s, Graph{n, g->gnbr}, g->gx, nullptr, nullptr);
    gnn_mesh_velocity(mesh_ctx, s, g->ybuf, true, g->gmask);
    if (smooth_passes > 0) gnn_mesh_smooth(mesh_ctx, s, smooth_passes, g->gmask);
    if (with_viscosity) gnn_mesh_viscosity(mesh_ctx, s, g->ybuf, true, g->gmask);
    UFE_CUDA(cudaEventRecord(mesh_ctx->ev1, s));
    gnn_check(g, s);
    if (device_ms) {
      float ms = 0.f;
      UFE_CUDA(cudaEventElapsedTime(&ms, mesh_ctx->ev0, mesh_ctx->ev1));
      *device_ms = ms;
    }
    return UFE_OK;
  });
}

extern "C" int32_t ufe_gnn_predict_velocity(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity,
                                            int32_t smooth_passes, double *device_ms) {
  return ufe_gnn_predict_start(g, mesh_ctx, use_prev_velocity, smooth_passes, 0, device_ms);
}
