// Krylov kernels: Jacobi-preconditioned BiCGStab in the form of PETSc's KSPBCGS with left
// preconditioning (the solver UFEMISM's solve_matrix_equation_CSR_PETSc hands its systems to,
// src/UPSY/basic/petsc_basic.f90:32-141, run with -ksp_type bcgs -pc_type jacobi).
//
// One iteration is three kernels:
//   k_p_spmv : p <- r - beta*omega*v + beta*p (also evaluated on the fly for gathered columns),
//              v <- D^-1 A p, partial (v, r^)                       -> alpha
//   k_s_spmv : s <- r - alpha*v (on the fly for gathered columns),
//              t <- D^-1 A s, partials (s,t), (t,t), (s,s)           -> omega
//   k_xr     : x <- x + alpha*p + omega*s,  r <- s - omega*t,
//              partials (r, r^), (r, r)                             -> convergence test, beta
// p and v are double-buffered by iteration parity, so the on-the-fly updates read old values.
// Every reduction is the deterministic last-block sum of ufe_work.cuh; kernels loop over their
// rows with a grid stride so the grid never exceeds the partial-sum capacity.
#pragma once

#include <type_traits>

#include "ufe_dword.cuh"
#include "ufe_work.cuh"

template <class V> struct ScalarOf { using T = double; };
template <> struct ScalarOf<float2> { using T = float; };
template <> struct ScalarOf<double2> { using T = double; };
template <> struct ScalarOf<dw2> { using T = dw; };

// ---- vector element helpers ---------------------------------------------------------------
// The Krylov arithmetic uses explicit fused multiply-adds: FP64 instructions are the scarce
// resource on GB300, and these sums need no bitwise agreement with the reference.
__device__ __forceinline__ double v_dot(double2 a, double2 b) { return fma(a.y, b.y, a.x * b.x); }
__device__ __forceinline__ double v_dot(float2 a, float2 b) { return (double)fmaf(a.y, b.y, a.x * b.x); }
__device__ __forceinline__ double v_dot(double a, double b) { return a * b; }
__device__ __forceinline__ double2 v_mul(double2 d, double2 y) { return make_double2(d.x * y.x, d.y * y.y); }
__device__ __forceinline__ float2 v_mul(float2 d, float2 y) { return make_float2(d.x * y.x, d.y * y.y); }
__device__ __forceinline__ double v_mul(double d, double y) { return d * y; }
template <class V> __device__ __forceinline__ V v_zero();
template <> __device__ __forceinline__ double2 v_zero<double2>() { return make_double2(0.0, 0.0); }
template <> __device__ __forceinline__ float2 v_zero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double v_zero<double>() { return 0.0; }
// p_new = r - (beta*omega)*v + beta*p   (PETSc VecAXPBYPCZ(P, 1, -beta*omega, beta, R, V))
__device__ __forceinline__ double2 v_pupd(double2 r, double bw, double2 v, double beta, double2 p) {
  return make_double2(fma(beta, p.x, fma(-bw, v.x, r.x)), fma(beta, p.y, fma(-bw, v.y, r.y)));
}
__device__ __forceinline__ float2 v_pupd(float2 r, float bw, float2 v, float beta, float2 p) {
  return make_float2(fmaf(beta, p.x, fmaf(-bw, v.x, r.x)), fmaf(beta, p.y, fmaf(-bw, v.y, r.y)));
}
__device__ __forceinline__ double v_pupd(double r, double bw, double v, double beta, double p) {
  return fma(beta, p, fma(-bw, v, r));
}
// r - a*v
__device__ __forceinline__ double2 v_sub_scaled(double2 r, double a, double2 v) {
  return make_double2(fma(-a, v.x, r.x), fma(-a, v.y, r.y));
}
__device__ __forceinline__ float2 v_sub_scaled(float2 r, float a, float2 v) {
  return make_float2(fmaf(-a, v.x, r.x), fmaf(-a, v.y, r.y));
}
__device__ __forceinline__ double v_sub_scaled(double r, double a, double v) { return fma(-a, v, r); }
// x + a*p + w*s
__device__ __forceinline__ double2 v_xupd(double2 x, double a, double2 p, double w, double2 s) {
  return make_double2(fma(w, s.x, fma(a, p.x, x.x)), fma(w, s.y, fma(a, p.y, x.y)));
}
__device__ __forceinline__ float2 v_xupd(float2 x, float a, float2 p, float w, float2 s) {
  return make_float2(fmaf(w, s.x, fmaf(a, p.x, x.x)), fmaf(w, s.y, fmaf(a, p.y, x.y)));
}
__device__ __forceinline__ double v_xupd(double x, double a, double p, double w, double s) {
  return fma(w, s, fma(a, p, x));
}
__device__ __forceinline__ double2 v_shfl_xor(double2 a, int o) {
  return make_double2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
__device__ __forceinline__ float2 v_shfl_xor(float2 a, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
__device__ __forceinline__ double v_shfl_xor(double a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
__device__ __forceinline__ double2 v_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 v_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double v_add(double a, double b) { return a + b; }

// ---- matrix access policies ---------------------------------------------------------------
// 2x2-block rows (one triangle = its u and v rows); blocks stored in MatReal (FP64 or FP32),
// vectors and accumulation in VecReal; L lanes per block row.
// Sliced ELL (one lane per row): block rows in slices of 32 (one warp), the k-th entry of row
// i at slot soff[i/32] + 32 k + i%32, so that a warp's loads of blocks and columns are
// contiguous.  Short rows are padded with zero blocks whose column is the row itself.
template <typename MatReal, typename VecReal, int L>
struct BsrMat {
  using Vec = typename std::conditional<sizeof(VecReal) == 8, double2, float2>::type;
  using Blk = typename std::conditional<sizeof(MatReal) == 8, double4, float4>::type;
  static constexpr int kLanes = L;
  int32_t items;
  const int32_t *__restrict__ ptr;
  const int32_t *__restrict__ col;
  const Blk *__restrict__ blk;
  const int32_t *__restrict__ soff = nullptr;   // sliced-ELL copy (L == 1), or null
  const int32_t *__restrict__ scol = nullptr;
  const Blk *__restrict__ sblk = nullptr;
  template <class G>
  __device__ __forceinline__ Vec row_partial(int i, int lane, G get) const {
    Vec y = v_zero<Vec>();
    if (L == 1 && soff) {
      const int sl = i >> 5;
      const int s0 = __ldg(soff + sl), w = (__ldg(soff + sl + 1) - s0) >> 5;
      const int base = s0 + (i & 31);
      int k = 0;
      for (; k + 4 <= w; k += 4) {   // four slots' loads in flight at once
        int c[4];
        Blk a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int slot = base + ((k + u) << 5);
          c[u] = __ldg(scol + slot);
          a[u] = sblk[slot];
        }
        Vec x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = get(c[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          y.x = fma(a[u].y, x[u].y, fma(a[u].x, x[u].x, y.x));
          y.y = fma(a[u].w, x[u].y, fma(a[u].z, x[u].x, y.y));
        }
      }
      for (; k < w; ++k) {
        const int slot = base + (k << 5);
        const Blk a = sblk[slot];
        const Vec x = get(__ldg(scol + slot));
        y.x = fma(a.y, x.y, fma(a.x, x.x, y.x));
        y.y = fma(a.w, x.y, fma(a.z, x.x, y.y));
      }
      return y;
    }
    int k2 = __ldg(ptr + i + 1);
    for (int k = __ldg(ptr + i) + lane; k < k2; k += L) {
      Blk a = blk[k];
      Vec x = get(__ldg(col + k));
      y.x = fma(a.y, x.y, fma(a.x, x.x, y.x));
      y.y = fma(a.w, x.y, fma(a.z, x.x, y.y));
    }
    return y;
  }
};

// FP32 2x2-block rows in difference form: y_i = sum_j A_ij (x_j - x_i) + S_i x_i with the row
// sums S_i = sum_j A_ij taken in FP64 at assembly.  For the smooth vectors of an elliptic
// operator, x_j - x_i is exact in FP32 (nearby values) and the products keep full relative
// precision, where the plain form loses the digits that cancel between diagonal and neighbours.
template <int L>
struct BsrDiffMat {
  using Vec = float2;
  using Blk = float4;
  static constexpr int kLanes = L;
  int32_t items;
  const int32_t *__restrict__ ptr;
  const int32_t *__restrict__ col;
  const float4 *__restrict__ blk;
  const float4 *__restrict__ rowsum;
  const int32_t *__restrict__ soff = nullptr;   // sliced-ELL copy (L == 1), or null
  const int32_t *__restrict__ scol = nullptr;
  const float4 *__restrict__ sblk = nullptr;
  template <class G>
  __device__ __forceinline__ float2 row_partial(int i, int lane, G get) const {
    const float2 xi = get(i);
    float2 y = make_float2(0.f, 0.f);
    if (lane == 0) {
      const float4 s = rowsum[i];
      y.x = fmaf(s.y, xi.y, s.x * xi.x);
      y.y = fmaf(s.w, xi.y, s.z * xi.x);
    }
    if (L == 1 && soff) {
      const int sl = i >> 5;
      const int s0 = __ldg(soff + sl), w = (__ldg(soff + sl + 1) - s0) >> 5;
      const int base = s0 + (i & 31);
      int k = 0;
      for (; k + 4 <= w; k += 4) {   // four slots' loads in flight at once
        int c[4];
        float4 a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int slot = base + ((k + u) << 5);
          c[u] = __ldg(scol + slot);
          a[u] = sblk[slot];
        }
        float2 xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xj[u] = get(c[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float dx = xj[u].x - xi.x, dy = xj[u].y - xi.y;
          y.x = fmaf(a[u].y, dy, fmaf(a[u].x, dx, y.x));
          y.y = fmaf(a[u].w, dy, fmaf(a[u].z, dx, y.y));
        }
      }
      for (; k < w; ++k) {
        const int slot = base + (k << 5);
        const float4 a = sblk[slot];
        const float2 xj = get(__ldg(scol + slot));
        const float dx = xj.x - xi.x, dy = xj.y - xi.y;
        y.x = fmaf(a.y, dy, fmaf(a.x, dx, y.x));
        y.y = fmaf(a.w, dy, fmaf(a.z, dx, y.y));
      }
      return y;
    }
    int k2 = __ldg(ptr + i + 1);
    for (int k = __ldg(ptr + i) + lane; k < k2; k += L) {
      const float4 a = blk[k];
      const float2 xj = get(__ldg(col + k));
      const float dx = xj.x - xi.x, dy = xj.y - xi.y;
      y.x = fmaf(a.y, dy, fmaf(a.x, dx, y.x));
      y.y = fmaf(a.w, dy, fmaf(a.z, dx, y.y));
    }
    return y;
  }
};

// scalar CSR rows (the general matrix-equation solve), one lane per row
struct CsrMat {
  using Vec = double;
  static constexpr int kLanes = 1;
  int32_t items;
  const int32_t *__restrict__ ptr;
  const int32_t *__restrict__ col;
  const double *__restrict__ val;
  template <class G>
  __device__ __forceinline__ double row_partial(int i, int lane, G get) const {
    double y = 0.0;
    int k2 = __ldg(ptr + i + 1);
    for (int k = __ldg(ptr + i); k < k2; ++k) y = fma(__ldg(val + k), get(__ldg(col + k)), y);
    return y;
  }
};

template <class Vec>
struct KV {
  Vec *X, *R, *RP, *S, *T, *B;
  const Vec *dinv;
  Vec *P[2], *V[2];
};

// reduction sites (one ticket each)
enum : int {
  kSiteInit = 0, kSiteP, kSiteS, kSiteXR, kSiteResid, kSitePicard, kSiteAux, kSiteInner, kSiteCount
};

struct CondArg {
  cudaGraphConditionalHandle handle;
  int use;
};

__device__ __forceinline__ void set_cond(CondArg c, int value) {
  if (c.use) cudaGraphSetConditional(c.handle, value ? 1u : 0u);
}

template <int L, class Vec>
__device__ __forceinline__ Vec lane_reduce(Vec y) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) y = v_add(y, v_shfl_xor(y, o));
  return y;
}

// Lanes of one group must be in one warp: blockDim.x is a multiple of 32 and L divides 32.
#define KRYLOV_ROWS(M, i, lane)                                                                \
  const int lane = threadIdx.x % M::kLanes;                                                    \
  const int64_t gstride_ = ((int64_t)gridDim.x * blockDim.x) / M::kLanes;                      \
  const int64_t nrows_pad_ = ((mat.items + gstride_ - 1) / gstride_) * gstride_;               \
  for (int64_t i##_64 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / M::kLanes;          \
       i##_64 < nrows_pad_; i##_64 += gstride_)

// r = D^-1 (b - A x), r^ = r, p = v = 0; tests the initial residual (KSPConvergedDefault at
// iteration 0) and primes rho = (r, r^).
// With gate = 1 the kernel only runs when the scalars ask for an FP64 fallback solve.  With
// keep_tol = 1 (a restart inside one linear solve) the stopping tolerance set at the solve's start
// is kept.
template <class M>
__global__ void k_krylov_init(M mat, KV<typename M::Vec> v, KrylovScalars *ks, double rtol,
                              double abstol, int max_it, int x_is_zero, double *partials,
                              unsigned int *tickets, CondArg cond, int gate = 0, int keep_tol = 0) {
  using Vec = typename M::Vec;
  if (gate && !ks->fallback) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0);
    return;
  }
  double acc[2] = {0.0, 0.0};
  KRYLOV_ROWS(M, i, lane) {
    const int i = (int)i_64;
    const bool live = i < mat.items;
    Vec ax = v_zero<Vec>();
    if (!x_is_zero) {
      Vec part = live ? mat.row_partial(i, lane, [&](int j) { return v.X[j]; }) : v_zero<Vec>();
      ax = lane_reduce<M::kLanes>(part);
    }
    if (live && lane == 0) {
      Vec b = v.B[i], d = v.dinv[i];
      Vec r = v_mul(d, v_sub_scaled(b, 1.0, ax));
      Vec db = v_mul(d, b);
      v.R[i] = r;
      v.RP[i] = r;
      v.P[0][i] = v_zero<Vec>();
      v.V[0][i] = v_zero<Vec>();
      if (x_is_zero) v.X[i] = v_zero<Vec>();
      acc[0] += v_dot(r, r);
      acc[1] += v_dot(db, db);
    }
  }
  double tot[2];
  if (grid_sum<2>(acc, partials, tickets + kSiteInit, tot)) {
    double dp = sqrt(tot[0]);
    double bnorm = sqrt(tot[1]);
    double rnorm0 = bnorm != 0.0 ? bnorm : dp;
    KrylovScalars s = *ks;
    s.dp = dp;
    if (!gate && !keep_tol) {
      s.rnorm0 = rnorm0;
      s.ttol = fmax(rtol * rnorm0, abstol);   // a fallback or a restart keeps the solve's tolerance
    }
    s.fallback = 0;
    s.it = 0;
    s.max_it = max_it;
    s.rho = tot[0];
    s.rhoold = 1.0;
    s.alpha = 1.0;
    s.omegaold = 1.0;
    s.omega = 1.0;
    s.beta = s.rho;  // (rho/rhoold)*(alpha/omegaold) with rhoold = alpha = omegaold = 1
    s.status = UFE_OK;
    s.tbreak = 0;
    s.active = 1;
    if (isnan(dp)) { s.status = UFE_ERR_NAN; s.active = 0; }
    else if (dp <= s.ttol) s.active = 0;
    else if (s.rho == 0.0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
    *ks = s;
    set_cond(cond, s.active);
  }
}

// pre = 1: p (and, in k_s_spmv, s) were formed row by row beforehand (k_p_update, k_s_update) and
// the SpMV gathers them; pre = 0 forms them on the fly for every gathered column.  Both give the
// same values -- the same expression on the same inputs -- but the on-the-fly form repeats the
// update's FP64 work once per stored entry, which bounds a scalar CSR solve by the FP64 pipe.
template <class M>
__global__ void k_p_spmv(M mat, KV<typename M::Vec> v, KrylovScalars *ks, double *partials,
                         unsigned int *tickets, int pre = 0) {
  using Vec = typename M::Vec;
  using R = typename ScalarOf<Vec>::T;
  const KrylovScalars s = *ks;
  if (!s.active) return;
  const int cur = s.it & 1, nxt = cur ^ 1;
  const R beta = (R)s.beta, bw = (R)(s.beta * s.omegaold);
  const Vec *__restrict__ Po = v.P[cur];
  const Vec *__restrict__ Vo = v.V[cur];
  const Vec *__restrict__ Rr = v.R;
  const Vec *__restrict__ Pn = v.P[nxt];
  double acc[1] = {0.0};
  KRYLOV_ROWS(M, i, lane) {
    const int i = (int)i_64;
    const bool live = i < mat.items;
    Vec part = !live ? v_zero<Vec>()
               : pre ? mat.row_partial(i, lane, [&](int j) { return Pn[j]; })
                     : mat.row_partial(i, lane, [&](int j) { return v_pupd(Rr[j], bw, Vo[j], beta, Po[j]); });
    Vec y = lane_reduce<M::kLanes>(part);
    if (live && lane == 0) {
      if (!pre) v.P[nxt][i] = v_pupd(Rr[i], bw, Vo[i], beta, Po[i]);
      Vec vn = v_mul(v.dinv[i], y);
      v.V[nxt][i] = vn;
      acc[0] += v_dot(vn, v.RP[i]);
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, partials, tickets + kSiteP, tot)) {
    KrylovScalars t = *ks;
    double d1 = tot[0];
    if (d1 == 0.0 || isnan(d1)) { t.status = isnan(d1) ? UFE_ERR_NAN : UFE_ERR_DIVERGED; t.active = 0; }
    else t.alpha = t.rho / d1;
    *ks = t;
  }
}

template <class M>
__global__ void k_s_spmv(M mat, KV<typename M::Vec> v, KrylovScalars *ks, double *partials,
                         unsigned int *tickets, int pre = 0) {
  using Vec = typename M::Vec;
  using R = typename ScalarOf<Vec>::T;
  const KrylovScalars s = *ks;
  if (!s.active) return;
  const int nxt = (s.it & 1) ^ 1;
  const R alpha = (R)s.alpha;
  const Vec *__restrict__ Vn = v.V[nxt];
  const Vec *__restrict__ Rr = v.R;
  const Vec *__restrict__ Sg = v.S;
  double acc[3] = {0.0, 0.0, 0.0};
  KRYLOV_ROWS(M, i, lane) {
    const int i = (int)i_64;
    const bool live = i < mat.items;
    Vec part = !live ? v_zero<Vec>()
               : pre ? mat.row_partial(i, lane, [&](int j) { return Sg[j]; })
                     : mat.row_partial(i, lane, [&](int j) { return v_sub_scaled(Rr[j], alpha, Vn[j]); });
    Vec y = lane_reduce<M::kLanes>(part);
    if (live && lane == 0) {
      Vec si = pre ? Sg[i] : v_sub_scaled(Rr[i], alpha, Vn[i]);
      Vec ti = v_mul(v.dinv[i], y);
      if (!pre) v.S[i] = si;
      v.T[i] = ti;
      acc[0] += v_dot(si, ti);
      acc[1] += v_dot(ti, ti);
      acc[2] += v_dot(si, si);
    }
  }
  double tot[3];
  if (grid_sum<3>(acc, partials, tickets + kSiteS, tot)) {
    KrylovScalars t = *ks;
    if (tot[1] == 0.0) {
      // t = 0: if s = 0 too, x + alpha p solves the system (bcgs.c's breakdown branch)
      if (tot[2] != 0.0) { t.status = UFE_ERR_DIVERGED; t.active = 0; }
      else { t.omega = 0.0; t.tbreak = 1; }
    } else if (isnan(tot[1])) {
      t.status = UFE_ERR_NAN; t.active = 0;
    } else {
      t.omega = tot[0] / tot[1];
    }
    *ks = t;
  }
}

// Row-wise p <- r - beta omega v + beta p and s <- r - alpha v for the pre form above.
template <class Vec>
__global__ void k_p_update(int64_t n, KV<Vec> v, const KrylovScalars *ks) {
  using R = typename ScalarOf<Vec>::T;
  const KrylovScalars s = *ks;
  if (!s.active) return;
  const int cur = s.it & 1, nxt = cur ^ 1;
  const R beta = (R)s.beta, bw = (R)(s.beta * s.omegaold);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    v.P[nxt][i] = v_pupd(v.R[i], bw, v.V[cur][i], beta, v.P[cur][i]);
}

template <class Vec>
__global__ void k_s_update(int64_t n, KV<Vec> v, const KrylovScalars *ks) {
  using R = typename ScalarOf<Vec>::T;
  const KrylovScalars s = *ks;
  if (!s.active) return;
  const int nxt = (s.it & 1) ^ 1;
  const R alpha = (R)s.alpha;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    v.S[i] = v_sub_scaled(v.R[i], alpha, v.V[nxt][i]);
}

template <class M>
__global__ void k_xr(M mat, KV<typename M::Vec> v, KrylovScalars *ks, double *partials,
                     unsigned int *tickets, CondArg cond) {
  using Vec = typename M::Vec;
  using R = typename ScalarOf<Vec>::T;
  const KrylovScalars s = *ks;
  if (!s.active) {
    // an earlier kernel of this iteration stopped the solve: end the loop here as well, so the
    // while-node never repeats an inactive body
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0);
    return;
  }
  const int nxt = (s.it & 1) ^ 1;
  const R alpha = (R)s.alpha, omega = (R)s.omega;
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mat.items; i += stride) {
    Vec pi = v.P[nxt][i], si = v.S[i], ti = v.T[i];
    v.X[i] = v_xupd(v.X[i], alpha, pi, omega, si);
    Vec ri = v_sub_scaled(si, omega, ti);
    v.R[i] = ri;
    acc[0] += v_dot(ri, v.RP[i]);
    acc[1] += v_dot(ri, ri);
  }
  double tot[2];
  if (grid_sum<2>(acc, partials, tickets + kSiteXR, tot)) {
    KrylovScalars t = *ks;
    t.it += 1;
    t.total_its += 1;
    double dp = sqrt(tot[1]);
    t.dp = dp;
    double rho_new = tot[0];
    t.rhoold = t.rho;
    t.omegaold = t.omega;
    t.rho = rho_new;
    if (t.tbreak) { t.active = 0; t.status = UFE_OK; t.dp = 0.0; }
    else if (isnan(dp)) { t.status = UFE_ERR_NAN; t.active = 0; }
    else if (dp <= t.ttol) { t.active = 0; }
    else if (dp >= 1e4 * t.rnorm0) { t.status = UFE_ERR_DIVERGED; t.active = 0; }
    else if (t.it >= t.max_it) { t.status = UFE_WARN_KRYLOV_MAXIT; t.active = 0; }
    else if (rho_new == 0.0) { t.status = UFE_ERR_DIVERGED; t.active = 0; }
    else t.beta = (t.rho / t.rhoold) * (t.alpha / t.omegaold);
    *ks = t;
    set_cond(cond, t.active);
  }
}

// Grid for the Krylov kernels: enough blocks to cover the rows once, capped so that the
// per-block partial sums fit the reduction area.
template <class M>
inline unsigned krylov_grid(const M &mat, int threads, int max_blocks) {
  int64_t lanes = (int64_t)mat.items * M::kLanes;
  int64_t b = (lanes + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// ---- persistent BiCGStab: the whole iteration loop in one (co-resident) launch ----------------
// The same recurrence as k_p_spmv / k_s_spmv / k_xr, with the launches replaced by grid
// barriers.  After each phase every block writes its partial sums; after the barrier every block
// sums all blocks' partials in the same fixed order, so all blocks hold identical scalars and
// take identical decisions without another round trip.  The barrier's spin is bounded: a block
// that waits too long records the failure and every block leaves the loop.
constexpr int kPersistMaxBlocks = 8 * 152;
constexpr int kPersistSlots = 5;     // partial sums per block per phase

// The barrier counts arrivals monotonically within one launch: barrier k of a launch with G
// blocks is passed once the counter reaches k*G.  Each block's thread 0 adds its arrival with a
// release reduction (no round trip) and polls the counter with acquire loads, so the last
// arrival releases everyone after one L2 write and one read.  The counter must be zero when a
// persistent kernel starts: every launch site resets it (k_reset_gsync / k_inner_init) on the
// same stream just before.  `err` ends every later wait of the launch once one wait gave up.
struct __align__(128) GridSync {
  unsigned int count;
  unsigned int pad0[31];
  unsigned int gen;     // unused by the barrier; kept zero
  int err;
  unsigned int pad1[30];
};

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned int *p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// false (block-uniform) when the wait gave up.  `target` is thread 0's running arrival target
// (zero at kernel start).
__device__ __forceinline__ bool grid_barrier(GridSync *gs, unsigned int &target) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    target += gridDim.x;
    __threadfence();
    red_release_add_u32(&gs->count, 1u);
    for (long long spins = 0; ld_acquire_u32(&gs->count) < target; ++spins) {
      if (spins > (1ll << 24) || *((volatile int *)&gs->err)) {
        ok = 0;
        atomicExch(&gs->err, 1);
        break;
      }
      if (spins > 4096) __nanosleep(64);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// block sum of NP values (fixed tree), written by thread 0 to part[blockIdx.x * NP + k]
template <int NP>
__device__ __forceinline__ void block_partials(double *acc, double *part) {
  __shared__ double red[NP][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      double v = lane < nw ? red[k][lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) part[(int64_t)blockIdx.x * NP + k] = v;
    }
  }
}

// every block: the sum over all blocks' partials in one fixed order (warp 0; broadcast)
template <int NP>
__device__ __forceinline__ void all_partials(const double *part, double *tot) {
  __shared__ double res[NP];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      double v = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32) v += __ldcg(part + (int64_t)b * NP + k);
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) res[k] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NP; ++k) tot[k] = res[k];
}

// Starts from the state k_krylov_init / k_inner_init left in *ks (and P[0], V[0]); runs until the
// scalars stop the solve; leaves x, r, the counters and the status as the three-kernel loop does.
constexpr int kPersistThreads = 1024;   // one block per SM

template <class M>
__global__ void __launch_bounds__(kPersistThreads) k_bicgstab_persist(M mat, KV<typename M::Vec> v, KrylovScalars *ks,
                                                          double *part, GridSync *gs) {
  using Vec = typename M::Vec;
  using R = typename ScalarOf<Vec>::T;
  KrylovScalars s = *ks;
  if (!s.active) return;
  double *partP = part, *partS = part + kPersistMaxBlocks * kPersistSlots,
         *partX = part + 2 * kPersistMaxBlocks * kPersistSlots;
  unsigned int gen = 0;   // barrier arrival target (thread 0)
  const int lane0 = threadIdx.x % M::kLanes;
  const int64_t gstride = ((int64_t)gridDim.x * blockDim.x) / M::kLanes;
  const int64_t nrows_pad = ((mat.items + gstride - 1) / gstride) * gstride;
  const int64_t row0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / M::kLanes;
  bool ok = true;
  while (s.active) {
    const int cur = s.it & 1, nxt = cur ^ 1;
    // -- p <- r - beta omega v + beta p;  v <- D^-1 A p;  (v, r^)
    {
      const R beta = (R)s.beta, bw = (R)(s.beta * s.omegaold);
      const Vec *__restrict__ Po = v.P[cur];
      const Vec *__restrict__ Vo = v.V[cur];
      const Vec *__restrict__ Rr = v.R;
      double acc[1] = {0.0};
      for (int64_t i64 = row0; i64 < nrows_pad; i64 += gstride) {
        const int i = (int)i64;
        const bool live = i < mat.items;
        Vec pt = live ? mat.row_partial(i, lane0, [&](int j) { return v_pupd(Rr[j], bw, Vo[j], beta, Po[j]); })
                      : v_zero<Vec>();
        Vec y = lane_reduce<M::kLanes>(pt);
        if (live && lane0 == 0) {
          v.P[nxt][i] = v_pupd(Rr[i], bw, Vo[i], beta, Po[i]);
          const Vec vn = v_mul(v.dinv[i], y);
          v.V[nxt][i] = vn;
          acc[0] += v_dot(vn, v.RP[i]);
        }
      }
      block_partials<1>(acc, partP);
      if (!(ok = grid_barrier(gs, gen))) break;
      double tot[1];
      all_partials<1>(partP, tot);
      const double d1 = tot[0];
      if (d1 == 0.0 || isnan(d1)) {
        s.status = isnan(d1) ? UFE_ERR_NAN : UFE_ERR_DIVERGED;
        s.active = 0;
        break;
      }
      s.alpha = s.rho / d1;
    }
    // -- s <- r - alpha v;  t <- D^-1 A s;  (s,t), (t,t), (s,s)
    {
      const R alpha = (R)s.alpha;
      const Vec *__restrict__ Vn = v.V[nxt];
      const Vec *__restrict__ Rr = v.R;
      double acc[3] = {0.0, 0.0, 0.0};
      for (int64_t i64 = row0; i64 < nrows_pad; i64 += gstride) {
        const int i = (int)i64;
        const bool live = i < mat.items;
        Vec pt = live ? mat.row_partial(i, lane0, [&](int j) { return v_sub_scaled(Rr[j], alpha, Vn[j]); })
                      : v_zero<Vec>();
        Vec y = lane_reduce<M::kLanes>(pt);
        if (live && lane0 == 0) {
          const Vec si = v_sub_scaled(Rr[i], alpha, Vn[i]);
          const Vec ti = v_mul(v.dinv[i], y);
          v.S[i] = si;
          v.T[i] = ti;
          acc[0] += v_dot(si, ti);
          acc[1] += v_dot(ti, ti);
          acc[2] += v_dot(si, si);
        }
      }
      block_partials<3>(acc, partS);
      if (!(ok = grid_barrier(gs, gen))) break;
      double tot[3];
      all_partials<3>(partS, tot);
      if (tot[1] == 0.0) {
        if (tot[2] != 0.0) { s.status = UFE_ERR_DIVERGED; s.active = 0; break; }
        s.omega = 0.0;
        s.tbreak = 1;
      } else if (isnan(tot[1])) {
        s.status = UFE_ERR_NAN;
        s.active = 0;
        break;
      } else {
        s.omega = tot[0] / tot[1];
      }
    }
    // -- x <- x + alpha p + omega s;  r <- s - omega t;  (r, r^), (r, r)
    {
      const R alpha = (R)s.alpha, omega = (R)s.omega;
      double acc[2] = {0.0, 0.0};
      const int64_t stride = (int64_t)gridDim.x * blockDim.x;
      for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mat.items; i += stride) {
        const Vec pi = v.P[nxt][i], si = v.S[i], ti = v.T[i];
        v.X[i] = v_xupd(v.X[i], alpha, pi, omega, si);
        const Vec ri = v_sub_scaled(si, omega, ti);
        v.R[i] = ri;
        acc[0] += v_dot(ri, v.RP[i]);
        acc[1] += v_dot(ri, ri);
      }
      block_partials<2>(acc, partX);
      if (!(ok = grid_barrier(gs, gen))) break;
      double tot[2];
      all_partials<2>(partX, tot);
      s.it += 1;
      s.total_its += 1;
      const double dp = sqrt(tot[1]);
      s.dp = dp;
      const double rho_new = tot[0];
      s.rhoold = s.rho;
      s.omegaold = s.omega;
      s.rho = rho_new;
      if (s.tbreak) { s.active = 0; s.status = UFE_OK; s.dp = 0.0; }
      else if (isnan(dp)) { s.status = UFE_ERR_NAN; s.active = 0; }
      else if (dp <= s.ttol) { s.active = 0; }
      else if (dp >= 1e4 * s.rnorm0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
      else if (s.it >= s.max_it) { s.status = UFE_WARN_KRYLOV_MAXIT; s.active = 0; }
      else if (rho_new == 0.0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
      else s.beta = (s.rho / s.rhoold) * (s.alpha / s.omegaold);
    }
  }
  if (!ok) {
    s.status = UFE_ERR_DEVICE;
    s.active = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *ks = s;
}

// ---- persistent BiCGStab with shared-memory neighbourhoods (FP32 inner and FP64 solves) --------
// Block b owns the contiguous block rows [b*rpb, (b+1)*rpb) (whole sliced-ELL slices; the rows are
// in Z order, so they form a compact patch of the mesh).  Each SpMV phase first stages, into
// shared memory, the vector its rows read: its own rows (coalesced) and the patch's halo rows
// (listed once per mesh), computing the on-the-fly update (p, or s = r - alpha v) once per staged
// entry; the rows then read neighbours from shared memory through per-slot local indices.
template <class Blk>
struct HaloMat {
  int32_t items;
  int32_t rpb;                          // rows per block (a multiple of 32)
  const int32_t *__restrict__ soff;     // sliced-ELL slice offsets
  const int32_t *__restrict__ lcol;     // local index (own rows, then halo) per slot
  const Blk *__restrict__ sblk;         // blocks per slot
  const float4 *__restrict__ rowsum;    // FP32 difference form: FP64 row sums rounded to FP32
  const int32_t *__restrict__ halo_off; // gridDim.x + 1
  const int32_t *__restrict__ halo_idx; // global rows of each block's halo
};
using HaloDiffMat = HaloMat<float4>;

// FP32 difference form: y_i = S_i x_i + sum_j A_ij (x_j - x_i)
__device__ __forceinline__ float2 halo_row(const HaloMat<float4> &m, int i, int il, const float2 *tab) {
  const float2 xi = tab[il];
  const float4 sr = m.rowsum[i];
  float2 y = make_float2(fmaf(sr.y, xi.y, sr.x * xi.x), fmaf(sr.w, xi.y, sr.z * xi.x));
  const int sl = i >> 5;
  const int s0 = __ldg(m.soff + sl), w = (__ldg(m.soff + sl + 1) - s0) >> 5;
  const int base = s0 + (i & 31);
  int k = 0;
  for (; k + 4 <= w; k += 4) {   // four slots' loads in flight at once
    int c[4];
    float4 a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int slot = base + ((k + u) << 5);
      c[u] = __ldg(m.lcol + slot);
      a[u] = __ldg(m.sblk + slot);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float2 xj = tab[c[u]];
      const float dx = xj.x - xi.x, dy = xj.y - xi.y;
      y.x = fmaf(a[u].y, dy, fmaf(a[u].x, dx, y.x));
      y.y = fmaf(a[u].w, dy, fmaf(a[u].z, dx, y.y));
    }
  }
  for (; k < w; ++k) {
    const int slot = base + (k << 5);
    const float4 a = __ldg(m.sblk + slot);
    const float2 xj = tab[__ldg(m.lcol + slot)];
    const float dx = xj.x - xi.x, dy = xj.y - xi.y;
    y.x = fmaf(a.y, dy, fmaf(a.x, dx, y.x));
    y.y = fmaf(a.w, dy, fmaf(a.z, dx, y.y));
  }
  return y;
}

// FP64 plain form, summed in the row's storage order
__device__ __forceinline__ double2 halo_row(const HaloMat<double4> &m, int i, int il, const double2 *tab) {
  double2 y = make_double2(0.0, 0.0);
  const int sl = i >> 5;
  const int s0 = __ldg(m.soff + sl), w = (__ldg(m.soff + sl + 1) - s0) >> 5;
  const int base = s0 + (i & 31);
  int k = 0;
  for (; k + 4 <= w; k += 4) {
    int c[4];
    double4 a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int slot = base + ((k + u) << 5);
      c[u] = __ldg(m.lcol + slot);
      a[u] = m.sblk[slot];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double2 x = tab[c[u]];
      y.x = fma(a[u].y, x.y, fma(a[u].x, x.x, y.x));
      y.y = fma(a[u].w, x.y, fma(a[u].z, x.x, y.y));
    }
  }
  for (; k < w; ++k) {
    const int slot = base + (k << 5);
    const double4 a = m.sblk[slot];
    const double2 x = tab[__ldg(m.lcol + slot)];
    y.x = fma(a.y, x.y, fma(a.x, x.x, y.x));
    y.y = fma(a.w, x.y, fma(a.z, x.x, y.y));
  }
  return y;
}

// Double-word form (UFE_PREC_FP32_PAIR), summed in the row's storage order with Dot2
// accumulators: the FP64 plain form's arithmetic on the FP32 pipe.
__device__ __forceinline__ dw2 halo_row(const HaloMat<dwblk> &m, int i, int il, const dw2 *tab) {
  dw_acc yu, yv;
  const int sl = i >> 5;
  const int s0 = __ldg(m.soff + sl), w = (__ldg(m.soff + sl + 1) - s0) >> 5;
  const int base = s0 + (i & 31);
  int k = 0;
  for (; k + 2 <= w; k += 2) {   // two slots' loads in flight at once (register budget of 64)
    int c[2];
    dwblk a[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int slot = base + ((k + u) << 5);
      c[u] = __ldg(m.lcol + slot);
      a[u] = m.sblk[slot];
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const float4 x = tab[c[u]].q;
      yu.mac(a[u].hi.x, a[u].lo.x, x.x, x.z);
      yu.mac(a[u].hi.y, a[u].lo.y, x.y, x.w);
      yv.mac(a[u].hi.z, a[u].lo.z, x.x, x.z);
      yv.mac(a[u].hi.w, a[u].lo.w, x.y, x.w);
    }
  }
  for (; k < w; ++k) {
    const int slot = base + (k << 5);
    const dwblk a = m.sblk[slot];
    const float4 x = tab[__ldg(m.lcol + slot)].q;
    yu.mac(a.hi.x, a.lo.x, x.x, x.z);
    yu.mac(a.hi.y, a.lo.y, x.y, x.w);
    yv.mac(a.hi.z, a.lo.z, x.x, x.z);
    yv.mac(a.hi.w, a.lo.w, x.y, x.w);
  }
  return make_dw2(yu.result(), yv.result());
}

// Per-thread dot-product accumulators of the persistent solve: FP64 for the FP64 and FP32 forms;
// Dot2 pairs for the double-word form, summed across the block in double-word arithmetic (FP32
// pipe) and rounded to FP64 once per block for the grid sums.
template <class Vec>
struct DotAcc {
  using Part = double;
  double v = 0.0;
  __device__ __forceinline__ void add(Vec a, Vec b) { v += v_dot(a, b); }
  __device__ __forceinline__ Part part() const { return v; }
  static __device__ __forceinline__ Part zero() { return 0.0; }
  static __device__ __forceinline__ Part warp_sum(Part x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
  }
  static __device__ __forceinline__ double finish(Part x) { return x; }
};
template <>
struct DotAcc<dw2> {
  using Part = float2;   // (hi, lo)
  dw_acc a;
  __device__ __forceinline__ void add(dw2 x, dw2 y) {
    a.mac(x.q.x, x.q.z, y.q.x, y.q.z);
    a.mac(x.q.y, x.q.w, y.q.y, y.q.w);
  }
  __device__ __forceinline__ Part part() const {
    const dw t = a.result();
    return make_float2(t.hi, t.lo);
  }
  static __device__ __forceinline__ Part zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ Part warp_sum(Part x) {
    dw t(x.x, x.y);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      t = dw_add(t, dw(__shfl_xor_sync(0xffffffffu, t.hi, o), __shfl_xor_sync(0xffffffffu, t.lo, o)));
    return make_float2(t.hi, t.lo);
  }
  static __device__ __forceinline__ double finish(Part x) { return dw(x.x, x.y).to_double(); }
};

// Scratch of the FP64 block sums (one instance per kernel that uses it).
__device__ __forceinline__ double *fp64_reduce_scratch() {
  __shared__ double buf[kPersistSlots * kPersistThreads];
  return buf;
}

// block sum of NP accumulators (fixed tree), written by thread 0 to part[blockIdx.x * NP + k].
// FP64 sums run as a shared-memory tree down to one warp: a butterfly of shuffles would issue
// 5 FP64 adds per warp per value, and FP64 issue is scarce on GB300.  Double-word sums stay in
// shuffles (FP32 pipe).
template <int NP, class Acc>
__device__ __forceinline__ void block_partials_acc(const Acc (&acc)[NP], double *part) {
  using P = typename Acc::Part;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if constexpr (std::is_same<P, double>::value) {
    double *t = fp64_reduce_scratch();
    const int n = blockDim.x;   // a power of two
#pragma unroll
    for (int k = 0; k < NP; ++k) t[k * n + threadIdx.x] = acc[k].part();
    __syncthreads();
    for (int st = n >> 1; st >= 32; st >>= 1) {
      if ((int)threadIdx.x < st)
#pragma unroll
        for (int k = 0; k < NP; ++k) t[k * n + threadIdx.x] += t[k * n + threadIdx.x + st];
      __syncthreads();
    }
    if (warp == 0) {
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const double v = Acc::warp_sum(t[k * n + lane]);
        if (lane == 0) part[(int64_t)blockIdx.x * NP + k] = v;
      }
    }
  } else {
    __shared__ P red[NP][32];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const P v = Acc::warp_sum(acc[k].part());
      if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const P v = Acc::warp_sum(lane < nw ? red[k][lane] : Acc::zero());
        if (lane == 0) part[(int64_t)blockIdx.x * NP + k] = Acc::finish(v);
      }
    }
  }
}

// After a phase's barrier: the block loads all blocks' partials at once (one L2 round trip,
// one value per thread; the grid holds at most kHaloMaxBlocks blocks), warp k sums value k in
// block order, and thread 0 runs update(tot) on the block's shared scalars.  Every thread sees
// the result after the closing barrier.
constexpr int kHaloMaxBlocks = kPersistThreads / kPersistSlots;
__device__ __forceinline__ double *phase_scratch() {
  __shared__ double buf[kPersistThreads + kPersistSlots];
  return buf;
}
template <int NP, class F>
__device__ __forceinline__ void phase_update(const double *part, F &&update) {
  double *sp = phase_scratch();
  double *tot = sp + kPersistThreads;
  const int n = (int)gridDim.x * NP;
  if ((int)threadIdx.x < n) sp[threadIdx.x] = __ldcg(part + threadIdx.x);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < NP) {
    double v = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) v += sp[b * NP + warp];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) tot[warp] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) update(tot);
  __syncthreads();
}

// The whole BiCGStab solve in one launch (one 1024-thread block per SM): each block owns the
// contiguous rows [blockIdx.x * rpb, ...) and stages its patch (own rows, then halo rows) in
// shared memory for the two SpMVs.  The scalar recurrence (divisions, square root, stopping
// tests) runs once per block, in thread 0, on the block's shared copy of the scalars; the other
// threads read the coefficients of the next phase from shared memory, already in the solve's
// arithmetic (FP64, FP32 or double-word).
//
// Two grid-wide reductions per iteration instead of three.  The s-phase also forms (s, r^) and
// (t, r^), so the scalars of r_{k+1} = s - omega t follow without reducing over r:
//   (r_{k+1}, r^) = (s, r^) - omega (t, r^),   |r_{k+1}|^2 = (s, s) - omega (2 (s, t) - omega (t, t)),
// and the x/r update of iteration k runs inside the p staging of iteration k+1 (r of a halo row
// is formed on the fly from its s and t; each row's owner writes x and r).  The iterates are
// those of PETSc's KSPBCGS; only the rounding of rho and of the residual norm differs.  The
// x/r update of the last iteration runs after the loop.
template <class Vec, class Blk>
__global__ void __launch_bounds__(kPersistThreads) k_bicgstab_halo(HaloMat<Blk> m, KV<Vec> v, KrylovScalars *ks,
                                                                   double *part, GridSync *gs) {
  using R = typename ScalarOf<Vec>::T;
  extern __shared__ __align__(16) unsigned char tab_raw[];
  Vec *tab = reinterpret_cast<Vec *>(tab_raw);
  __shared__ KrylovScalars s;
  __shared__ int finish;   // 1 when the last iteration's x/r update is still to be applied
  // coefficients in the solve's arithmetic: [0] beta, [1] beta * omega_old, [2] alpha, [3] omega
  __shared__ __align__(16) unsigned char rs_raw[4 * sizeof(R)];
  R *rs = reinterpret_cast<R *>(rs_raw);
  if (threadIdx.x == 0) {
    s = *ks;
    rs[0] = (R)s.beta;
    rs[1] = (R)(s.beta * s.omegaold);
    finish = 0;
  }
  __syncthreads();
  if (!s.active) return;
  double *partP = part, *partS = part + kPersistMaxBlocks * kPersistSlots;
  unsigned int gen = 0;   // barrier arrival target (thread 0)
  const int r0 = blockIdx.x * m.rpb;
  const int r1 = min(m.items, r0 + m.rpb);
  const int own = max(r1 - r0, 0);
  const int h0 = __ldg(m.halo_off + blockIdx.x);
  const int nloc = own + (__ldg(m.halo_off + blockIdx.x + 1) - h0);
  bool ok = true, pending = false;   // pending: iteration k-1's x/r update not yet applied
  for (;;) {
    const int cur = s.it & 1, nxt = cur ^ 1;
    // -- [x <- x + alpha p + omega s; r <- s - omega t]  p <- r - beta omega v + beta p (staged);
    //    v <- D^-1 A p;  (v, r^)
    {
      const R beta = rs[0], bw = rs[1], ap = rs[2], wp = rs[3];
      const Vec *__restrict__ Po = v.P[cur];
      const Vec *__restrict__ Vo = v.V[cur];
      for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
        const int g = e < own ? r0 + e : __ldg(m.halo_idx + h0 + e - own);
        const Vec po = Po[g];
        Vec r;
        if (pending) {
          const Vec sg = v.S[g];
          r = v_sub_scaled(sg, wp, v.T[g]);
          if (e < own) {
            v.X[g] = v_xupd(v.X[g], ap, po, wp, sg);
            v.R[g] = r;
          }
        } else {
          r = v.R[g];
        }
        const Vec pn = v_pupd(r, bw, Vo[g], beta, po);
        tab[e] = pn;
        if (e < own) v.P[nxt][g] = pn;
      }
      __syncthreads();
      DotAcc<Vec> acc[1];
      for (int il = threadIdx.x; il < own; il += blockDim.x) {
        const int i = r0 + il;
        const Vec vn = v_mul(v.dinv[i], halo_row(m, i, il, tab));
        v.V[nxt][i] = vn;
        acc[0].add(vn, v.RP[i]);
      }
      block_partials_acc<1>(acc, partP);
      if (!(ok = grid_barrier(gs, gen))) break;
      phase_update<1>(partP, [&](const double *tot) {
        finish = 0;   // the staging above applied the previous iteration's x/r update
        const double d1 = tot[0];
        if (d1 == 0.0 || isnan(d1)) {
          s.status = isnan(d1) ? UFE_ERR_NAN : UFE_ERR_DIVERGED;
          s.active = 0;
        } else {
          s.alpha = s.rho / d1;
          rs[2] = (R)s.alpha;
        }
      });
      if (!s.active) break;
    }
    // -- s <- r - alpha v (staged);  t <- D^-1 A s;  (s,t), (t,t), (s,s), (s,r^), (t,r^)
    {
      const R alpha = rs[2];
      const Vec *__restrict__ Vn = v.V[nxt];
      for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
        const int g = e < own ? r0 + e : __ldg(m.halo_idx + h0 + e - own);
        const Vec sv = v_sub_scaled(v.R[g], alpha, Vn[g]);
        tab[e] = sv;
        if (e < own) v.S[g] = sv;
      }
      __syncthreads();
      DotAcc<Vec> acc[5];
      for (int il = threadIdx.x; il < own; il += blockDim.x) {
        const int i = r0 + il;
        const Vec si = tab[il];
        const Vec ti = v_mul(v.dinv[i], halo_row(m, i, il, tab));
        v.T[i] = ti;
        const Vec rp = v.RP[i];
        acc[0].add(si, ti);
        acc[1].add(ti, ti);
        acc[2].add(si, si);
        acc[3].add(si, rp);
        acc[4].add(ti, rp);
      }
      block_partials_acc<5>(acc, partS);
      if (!(ok = grid_barrier(gs, gen))) break;
      phase_update<5>(partS, [&](const double *tot) {
        if (tot[1] == 0.0) {
          if (tot[2] != 0.0) {
            s.status = UFE_ERR_DIVERGED;
            s.active = 0;
            return;
          }
          s.omega = 0.0;
          s.tbreak = 1;
        } else if (isnan(tot[1])) {
          s.status = UFE_ERR_NAN;
          s.active = 0;
          return;
        } else {
          s.omega = tot[0] / tot[1];
        }
        const double w = s.omega;
        finish = 1;   // this iteration's x/r update is due from here on
        s.it += 1;
        s.total_its += 1;
        const double rho_new = tot[3] - w * tot[4];
        const double dp = sqrt(fmax(tot[2] - w * (2.0 * tot[0] - w * tot[1]), 0.0));
        s.dp = dp;
        s.rhoold = s.rho;
        s.omegaold = w;
        s.rho = rho_new;
        if (s.tbreak) { s.active = 0; s.status = UFE_OK; s.dp = 0.0; }
        else if (isnan(dp)) { s.status = UFE_ERR_NAN; s.active = 0; }
        else if (dp <= s.ttol) { s.active = 0; }
        else if (dp >= 1e4 * s.rnorm0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
        else if (s.it >= s.max_it) { s.status = UFE_WARN_KRYLOV_MAXIT; s.active = 0; }
        else if (rho_new == 0.0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
        else s.beta = (s.rho / s.rhoold) * (s.alpha / s.omegaold);
        rs[0] = (R)s.beta;
        rs[1] = (R)(s.beta * w);
        rs[3] = (R)w;
      });
      if (!s.active) break;
      pending = true;
    }
  }
  // the x/r update of the last iteration
  if (ok && finish) {
    const R alpha = rs[2], omega = rs[3];
    const int nxt = ((s.it - 1) & 1) ^ 1;   // the parity p was written with in that iteration
    for (int il = threadIdx.x; il < own; il += blockDim.x) {
      const int i = r0 + il;
      const Vec si = v.S[i];
      v.X[i] = v_xupd(v.X[i], alpha, v.P[nxt][i], omega, si);
      v.R[i] = v_sub_scaled(si, omega, v.T[i]);
    }
  }
  if (threadIdx.x == 0) {
    if (!ok) {
      s.status = UFE_ERR_DEVICE;
      s.active = 0;
    }
    if (blockIdx.x == 0) *ks = s;
  }
}
