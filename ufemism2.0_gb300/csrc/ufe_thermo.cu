// Thermodynamics: the implicit column temperature solve of solve_3D_heat_equation
// (src/UFEMISM/thermodynamics/thermodynamics_3D_heat_equation.f90:33-479) as batched GPU kernels.
//
// Each column is one tridiagonal system of nz rows per (sub)step.  One thread owns one column:
// the forward sweep of the Thomas algorithm (tridiagonal_solver.f90:38-42) builds each row's
// coefficients as it goes (solve_1D_heat_equation, :395-462), so the row inputs are read once,
// layer by layer, from the column-major (k stride nV) arrays -- consecutive threads read
// consecutive vertices, every load is coalesced.  The eliminated rows (b', c, d') wait in shared
// memory ([k][thread], conflict-free) for the back substitution (:44-48), which writes the
// clamped result.  Three passes per step:
//   k_heat_columns  all columns with the full dt; columns that fail the stability check
//                   (NaN, < 180 K, > T0; :226-232) are appended to a retry list;
//   k_heat_retry    the listed columns with dt/2, dt/4, ... (2^(it-1) substeps, up to 10
//                   levels, :163-239), each restarting from the profile the last level left,
//                   one warp per column; columns still unstable go to a second list;
//   k_heat_finish   the Robin profile (replace_Ti_with_robin_solution,
//                   thermodynamics_utilities.f90:256-337) for the listed columns when they are
//                   fewer than ceil(nV/100), else the step's error flag (:251-290).
// The lists replace the reference's per-vertex is_unstable array and its MPI_ALLREDUCE.
//
// The mesh-level path computes the prelude inside the column kernel: the zeta gradients of
// calc_zeta_gradients (zeta_gradients.f90:19) from four per-vertex gradients, Cp/K/T_pmp
// (thermodynamics_utilities.f90:130-229) from the starting temperature, and the upwind products
// of calc_upwind_heat_flux_derivatives (:339-434) from the upwind triangle's row of the a->b
// d/dx, d/dy operators.  The upwind triangle, the annual-mean surface temperature and the basal
// heat flux are found once per upload.
//
// The build's --fmad=false keeps each product and sum one IEEE rounding, in the reference's
// evaluation order, so the columns reproduce the reference's arithmetic; exp (Ritz conductivity)
// and erf (Robin profile) are CUDA's and can differ from a host libm in the last bit.
#include <algorithm>
#include <cmath>

#include "ufe_internal.cuh"

namespace {

// src/UPSY/basic/parameters.f90:15-23
constexpr double kPi = 3.141592653589793;
constexpr double kSecPerYear = 31556943.36;
constexpr double kT0 = 273.16;
constexpr double kCCGradient = 8.7E-04;
constexpr double kIceDensity = 910.0;
// src/UPSY/basic/math_utilities/shape_functions.f90:13
constexpr double kShapeQ = 1.5;

constexpr int kMaxNz = 256;
constexpr int kSmemBudget = 200 * 1024;

// Zeta operators in tridiagonal form (device): zeta, then d/dzeta l/d/u, then d2/dzeta2 l/d/u.
struct ZOps {
  const double *zeta, *l1, *d1, *u1, *l2, *d2, *u2;
  int nz;
};

struct Consts {
  double dt, Hi_min, cp_u, k_u;
  int cp_uniform, k_uniform, glbc;
};

// Per-vertex fields shared by both paths.
struct VertexFields {
  const double *Hi_eff, *T_surf, *Q, *fr, *geo, *SMB;
  const int32_t *mask;
};

struct Counters {
  int32_t n_retry;      // columns in the retry list
  int32_t n_unstable;   // columns still unstable after the retries
  int32_t total_unstable;
  int32_t err;          // UFE_* error of the first failing step (0: none)
  int32_t err_step;
  int32_t threshold;    // ceil(nV / 100)
  int32_t bad_mask;     // a column with ice but no grounded/floating mask
  int32_t step;
};

struct Lists {
  int32_t *retry;       // nV
  int32_t *unstable;    // nV
  double *scratch;      // nV x nz (list-indexed current profiles of retried columns)
};

__device__ __forceinline__ double heat_capacity(const Consts &c, double T) {
  return c.cp_uniform ? c.cp_u : 2115.3 + 7.79293 * (T - kT0);
}
__device__ __forceinline__ double conductivity(const Consts &c, double T) {
  return c.k_uniform ? c.k_u : 3.101E08 * exp(-(0.0057 * T));
}
__device__ __forceinline__ double melting_point(double Hi_eff, double zeta) {
  return kT0 - kCCGradient * Hi_eff * zeta;
}
__device__ __forceinline__ bool unstable_value(double T) { return T != T || T < 180.0 || T > kT0; }

// ---- row inputs --------------------------------------------------------------------------
struct Layer {
  double Ti0, u, v, w, udx, vdy, dzx, dzy, dzz, dzt, phi;
};

// Column level: every row input is an nV x nz array.
struct ColumnArrays {
  int64_t nV;
  const double *Ti0, *u, *v, *w, *udx, *vdy, *dzx, *dzy, *dzz, *dzt, *phi;
  struct Col {};
  __device__ __forceinline__ Col col(int64_t) const { return Col{}; }
  __device__ __forceinline__ void layer(const Col &, int64_t vi, int k, double, Layer &L) const {
    const int64_t o = (int64_t)k * nV + vi;
    L.Ti0 = __ldg(Ti0 + o);
    L.u = __ldg(u + o);
    L.v = __ldg(v + o);
    L.w = __ldg(w + o);
    L.udx = __ldg(udx + o);
    L.vdy = __ldg(vdy + o);
    L.dzx = __ldg(dzx + o);
    L.dzy = __ldg(dzy + o);
    L.dzz = __ldg(dzz + o);
    L.dzt = __ldg(dzt + o);
    L.phi = __ldg(phi + o);
  }
  // the two inputs the basal row reads
  __device__ __forceinline__ void basal(const Col &, int64_t vi, int k, double, double &Ti0v, double &dzzv) const {
    const int64_t o = (int64_t)k * nV + vi;
    Ti0v = __ldg(Ti0 + o);
    dzzv = __ldg(dzz + o);
  }
};

// Mesh level: the prelude on the fly.
struct HeatMesh {
  int64_t nV;
  const double *Ti0, *u, *v, *w, *phi, *ub, *vb;   // nV x nz (ub, vb: u_3D_b, v_3D_b of the upwind triangle)
  const double *gHs_x, *gHi_x, *gHs_y, *gHi_y, *dHs_dt, *dHi_dt, *Hc;   // nV
  const int32_t *ti_up;                            // nV, -1: no advection term (Hi < 1)
  const int32_t *ab_ptr, *ab_ind;                  // a->b operator pattern (0-based)
  const double *ddx_ab, *ddy_ab;
  struct Col {
    double inv, gsx, gix, gsy, giy, dsdt, didt;
    int32_t e0, e1;   // entries of the upwind triangle's row; e0 == e1: no advection term
  };
  __device__ __forceinline__ Col col(int64_t vi) const {
    Col c;
    // calc_zeta_gradients (zeta_gradients.f90, vertex terms): Hi = max(10, ice%Hi)
    c.inv = 1.0 / __ldg(Hc + vi);
    c.gsx = __ldg(gHs_x + vi);
    c.gix = __ldg(gHi_x + vi);
    c.gsy = __ldg(gHs_y + vi);
    c.giy = __ldg(gHi_y + vi);
    c.dsdt = __ldg(dHs_dt + vi);
    c.didt = __ldg(dHi_dt + vi);
    const int32_t ti = __ldg(ti_up + vi);
    c.e0 = ti < 0 ? 0 : __ldg(ab_ptr + ti);
    c.e1 = ti < 0 ? 0 : __ldg(ab_ptr + ti + 1);
    return c;
  }
  __device__ __forceinline__ void layer(const Col &c, int64_t vi, int k, double zeta, Layer &L) const {
    const int64_t o = (int64_t)k * nV + vi;
    L.Ti0 = __ldg(Ti0 + o);
    L.u = __ldg(u + o);
    L.v = __ldg(v + o);
    L.w = __ldg(w + o);
    L.phi = __ldg(phi + o);
    L.dzt = c.inv * (c.dsdt - zeta * c.didt);
    L.dzx = c.inv * (c.gsx - zeta * c.gix);
    L.dzy = c.inv * (c.gsy - zeta * c.giy);
    L.dzz = -c.inv;
    if (c.e1 > c.e0) {
      // ddx_a_b_3D / ddy_a_b_3D of Ti at the upwind triangle, summed in storage order
      const double *Tk = Ti0 + (int64_t)k * nV;
      double sx = 0.0, sy = 0.0;
      for (int32_t e = c.e0; e < c.e1; ++e) {
        const double t = __ldg(Tk + __ldg(ab_ind + e));
        sx = sx + __ldg(ddx_ab + e) * t;
        sy = sy + __ldg(ddy_ab + e) * t;
      }
      L.udx = __ldg(ub + o) * sx;
      L.vdy = __ldg(vb + o) * sy;
    } else {
      L.udx = 0.0;
      L.vdy = 0.0;
    }
  }
  __device__ __forceinline__ void basal(const Col &c, int64_t vi, int k, double, double &Ti0v, double &dzzv) const {
    Ti0v = __ldg(Ti0 + (int64_t)k * nV + vi);
    dzzv = -c.inv;
  }
};

// ---- one column solve ----------------------------------------------------------------------
// solve_1D_heat_equation for one column and one (sub)step: `cur` is the current profile (stride
// cs), the result goes to `out` (stride os) clamped to T_pmp.  combine: out = fr*x + (1-fr)*out
// (the subgrid grounding-line mix, :185-186, with the floating solution already in out).
// Returns true when every written value passes the stability check.
template <class In>
__device__ bool solve_column(const In &in, const typename In::Col &col, const ZOps &z, const Consts &cs_,
                             int64_t vi, const double *cur, int64_t cs, double *out, int64_t os, double dt,
                             double Hi_eff, double T_surf, bool grounded, double Q, bool combine, double fr,
                             double *Bs, double *Cs, double *Ds, int T) {
  const int nz = z.nz;
  const double inv_dt = 1.0 / dt;
  // row 1: T = MIN(T_surf, T0)
  double bprev = 1.0, cprev = 0.0, dprev = fmin(T_surf, kT0);
  Bs[0] = bprev;
  Cs[0] = cprev;
  Ds[0] = dprev;
  double cur_nzm1 = 0.0;
#pragma unroll 2
  for (int k = 1; k < nz - 1; ++k) {
    const double zk = __ldg(z.zeta + k);
    Layer L;
    in.layer(col, vi, k, zk, L);
    const double Tc = cur[(int64_t)k * cs];
    const double Cpi = heat_capacity(cs_, L.Ti0);
    const double Ki = conductivity(cs_, L.Ti0);
    const double c1 = L.dzt + (L.u * L.dzx) + (L.v * L.dzy) + (L.w * L.dzz);
    const double c2 = -(Ki / (kIceDensity * Cpi) * (L.dzz * L.dzz));
    const double a = (c1 * __ldg(z.l1 + k)) + (c2 * __ldg(z.l2 + k));
    double b = inv_dt + (c1 * __ldg(z.d1 + k)) + (c2 * __ldg(z.d2 + k));
    const double c = (c1 * __ldg(z.u1 + k)) + (c2 * __ldg(z.u2 + k));
    double d = Tc / dt - L.udx - L.vdy + L.phi / (kIceDensity * Cpi);
    // Thomas forward elimination
    const double wgt = a / bprev;
    b = b - wgt * cprev;
    d = d - wgt * dprev;
    Bs[k * T] = b;
    Cs[k * T] = c;
    Ds[k * T] = d;
    bprev = b;
    cprev = c;
    dprev = d;
    cur_nzm1 = Tc;
  }
  // row nz: basal boundary condition
  const int kb = nz - 1;
  const double pmp_b = melting_point(Hi_eff, __ldg(z.zeta + kb));
  double d_b;
  if (grounded) {
    double Ti0b, dzzb;
    in.basal(col, vi, kb, __ldg(z.zeta + kb), Ti0b, dzzb);
    const double Kb = conductivity(cs_, Ti0b);
    d_b = fmin(pmp_b, cur_nzm1 - (__ldg(z.zeta + kb) - __ldg(z.zeta + kb - 1)) * Q / (dzzb * Kb));
  } else {
    d_b = pmp_b;   // MIN(T_base_float, T_pmp) with T_base_float = T_pmp at the base (:103-105)
  }
  {
    const double wgt = 0.0 / bprev;
    const double b = 1.0 - wgt * cprev;
    d_b = d_b - wgt * dprev;
    bprev = b;
  }
  // back substitution, clamp to T_pmp
  bool stable = true;
  double x = d_b / bprev;
  {
    double v = fmin(x, pmp_b);
    if (combine) v = fr * v + (1.0 - fr) * out[(int64_t)kb * os];
    out[(int64_t)kb * os] = v;
    stable &= !unstable_value(v);
  }
  for (int k = nz - 2; k >= 0; --k) {
    x = (Ds[k * T] - Cs[k * T] * x) / Bs[k * T];
    double v = fmin(x, melting_point(Hi_eff, __ldg(z.zeta + k)));
    if (combine) v = fr * v + (1.0 - fr) * out[(int64_t)k * os];
    out[(int64_t)k * os] = v;
    stable &= !unstable_value(v);
  }
  return stable;
}

// One substep of a column with its mask's boundary conditions (:168-214).
template <class In>
__device__ bool column_substep(const In &in, const ZOps &z, const Consts &c, int64_t vi, int32_t mask,
                               const double *cur, int64_t cs, double *out, int64_t os, double dt, double Hi_eff,
                               double T_surf, double Q, double fr, double *Bs, double *Cs, double *Ds, int T) {
  const typename In::Col col = in.col(vi);
  if (mask == UFE_COL_GL_GR) {
    if (c.glbc == UFE_GLBC_SUBGRID) {
      solve_column(in, col, z, c, vi, cur, cs, out, os, dt, Hi_eff, T_surf, false, Q, false, fr, Bs, Cs, Ds, T);
      return solve_column(in, col, z, c, vi, cur, cs, out, os, dt, Hi_eff, T_surf, true, Q, true, fr, Bs, Cs, Ds, T);
    }
    if (c.glbc == UFE_GLBC_PMP)
      return solve_column(in, col, z, c, vi, cur, cs, out, os, dt, Hi_eff, T_surf, false, Q, false, fr, Bs, Cs, Ds, T);
    return solve_column(in, col, z, c, vi, cur, cs, out, os, dt, Hi_eff, T_surf, true, Q, false, fr, Bs, Cs, Ds, T);
  }
  return solve_column(in, col, z, c, vi, cur, cs, out, os, dt, Hi_eff, T_surf, mask == UFE_COL_GROUNDED, Q, false,
                      fr, Bs, Cs, Ds, T);
}

// ---- the three passes ------------------------------------------------------------------------
template <class In>
__global__ void __launch_bounds__(128) k_heat_columns(In in, ZOps z, Consts c, VertexFields vf, int64_t nV,
                                                      const double *__restrict__ Ti_cur, double *__restrict__ Ti_next,
                                                      Lists lists, Counters *cnt) {
  if (cnt->err) return;
  extern __shared__ double sm[];
  const int T = blockDim.x;
  double *Bs = sm + threadIdx.x, *Cs = Bs + z.nz * T, *Ds = Cs + z.nz * T;
  const int64_t vi = (int64_t)blockIdx.x * T + threadIdx.x;
  if (vi >= nV) return;
  const double Hi_eff = __ldg(vf.Hi_eff + vi);
  const double Ts = __ldg(vf.T_surf + vi);
  if (Hi_eff < c.Hi_min) {
    // thin ice: the profile is the surface temperature (:136-140)
    for (int k = 0; k < z.nz; ++k) Ti_next[(int64_t)k * nV + vi] = Ts;
    return;
  }
  const int32_t mask = __ldg(vf.mask + vi);
  if (mask != UFE_COL_GROUNDED && mask != UFE_COL_FLOATING && mask != UFE_COL_GL_GR) {
    atomicAdd(&cnt->bad_mask, 1);
    return;
  }
  const double fr = (c.glbc == UFE_GLBC_SUBGRID) ? __ldg(vf.fr + vi) : 0.0;
  const bool ok = column_substep(in, z, c, vi, mask, Ti_cur + vi, nV, Ti_next + vi, nV, c.dt, Hi_eff, Ts,
                                 __ldg(vf.Q + vi), fr, Bs, Cs, Ds, T);
  if (!ok) {
    const int32_t j = atomicAdd(&cnt->n_retry, 1);
    lists.retry[j] = (int32_t)vi;
  }
}

// The dt-halving retries (:161-239), one warp per listed column.  Per column the row
// coefficients that do not depend on dt or on the current profile (c_ddzeta, c_d2dzeta2, the
// off-diagonals, the advection and heating terms) are computed once, one row per lane.  Per dt
// level the matrix part of the Thomas elimination (w = a / b', b' = b - w c) is done once by lane 0:
// it is the same in every substep, so hoisting it changes no value.  Per substep the two
// recurrences of the solve -- the forward sweep d'_k = d_k - w_k d'_{k-1} and the back substitution
// x_k = (d'_k - c_k x_{k+1}) / b'_k -- are first-order affine recurrences, evaluated across the warp
// as parallel prefix compositions of affine maps y -> a + b y (Kogge-Stone, 5 shuffle steps; rows
// beyond 32 are composed sequentially inside each lane first).  The back substitution is split as
// x_k = A_k + B_k x_base, so both basal conditions of a subgrid grounding-line column come from one
// scan.  Divisions by b'_k and dt become multiplications by reciprocals formed once per dt level
// (FP64 division is a long dependent sequence on GB300).  The scans reassociate the sums and the
// reciprocals round differently, so retried columns differ from the sequential recurrence in the
// last bits (well below 1e-9 K); the lanes then clamp, mix and check the rows in parallel.
constexpr int kRetryArrays = 16;
constexpr int kRetryWarps = 1;
constexpr int kRetryBlocks = 4 * 152;

struct Affine {   // y -> a + b y
  double a, b;
};
// g after f
__device__ __forceinline__ Affine compose(const Affine &g, const Affine &f) {
  return Affine{fma(g.b, f.a, g.a), g.b * f.b};
}
// Inclusive scan over the lanes in increasing (up = true) or decreasing lane order: lane l gets
// M_l o M_{l-1} o ... o M_0 (up) or M_l o M_{l+1} o ... o M_31 (down).
__device__ __forceinline__ Affine warp_scan(Affine m, int lane, bool up) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double qa = up ? __shfl_up_sync(0xffffffffu, m.a, off) : __shfl_down_sync(0xffffffffu, m.a, off);
    const double qb = up ? __shfl_up_sync(0xffffffffu, m.b, off) : __shfl_down_sync(0xffffffffu, m.b, off);
    if (up ? lane >= off : lane + off < 32) m = compose(m, Affine{qa, qb});
  }
  return m;
}

template <class In>
__global__ void __launch_bounds__(32 * kRetryWarps) k_heat_retry(In in, ZOps z, Consts c, VertexFields vf,
                                                                  int64_t nV, double *__restrict__ Ti_next,
                                                                  Lists lists, Counters *cnt) {
  if (cnt->err) return;
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nz = z.nz;
  const int R = (nz + 31) / 32;                      // rows per lane: [lane*R, lane*R + R)
  const int k0 = lane * R, k1 = min(k0 + R, nz);
  double *base = sm + (size_t)warp * kRetryArrays * nz;
  double *C1 = base, *C2 = C1 + nz, *UDX = C2 + nz, *VDY = UDX + nz, *PHI = VDY + nz, *A = PHI + nz,
         *Cc = A + nz, *Bp = Cc + nz, *W = Bp + nz, *D = W + nz, *X = D + nz, *PMP = X + nz, *NB = PMP + nz,
         *XB = NB + nz, *SB = XB + nz, *RB = SB + nz;
  const int32_t n = cnt->n_retry;
  const int warps_total = gridDim.x * kRetryWarps;
  for (int32_t j = blockIdx.x * kRetryWarps + warp; j < n; j += warps_total) {
    const int64_t vi = lists.retry[j];
    const double Hi_eff = __ldg(vf.Hi_eff + vi);
    const double Ts = __ldg(vf.T_surf + vi);
    const int32_t mask = __ldg(vf.mask + vi);
    const double Q = __ldg(vf.Q + vi);
    const double fr = (c.glbc == UFE_GLBC_SUBGRID) ? __ldg(vf.fr + vi) : 0.0;
    const bool two_solves = mask == UFE_COL_GL_GR && c.glbc == UFE_GLBC_SUBGRID;
    const bool grounded = mask == UFE_COL_GROUNDED || (mask == UFE_COL_GL_GR && c.glbc == UFE_GLBC_GROUNDED);
    const typename In::Col col = in.col(vi);
    for (int k = lane; k < nz; k += 32) {
      const double zk = __ldg(z.zeta + k);
      PMP[k] = melting_point(Hi_eff, zk);
      X[k] = Ti_next[(int64_t)k * nV + vi];   // the profile the full-dt solve left (:222)
      if (k >= 1 && k < nz - 1) {
        Layer L;
        in.layer(col, vi, k, zk, L);
        const double Cpi = heat_capacity(c, L.Ti0);
        const double Ki = conductivity(c, L.Ti0);
        const double c1 = L.dzt + (L.u * L.dzx) + (L.v * L.dzy) + (L.w * L.dzz);
        const double c2 = -(Ki / (kIceDensity * Cpi) * (L.dzz * L.dzz));
        C1[k] = c1;
        C2[k] = c2;
        UDX[k] = L.udx;
        VDY[k] = L.vdy;
        PHI[k] = L.phi / (kIceDensity * Cpi);
        A[k] = (c1 * __ldg(z.l1 + k)) + (c2 * __ldg(z.l2 + k));
        Cc[k] = (c1 * __ldg(z.u1 + k)) + (c2 * __ldg(z.u2 + k));
      } else {
        A[k] = 0.0;    // boundary rows: AA_ldiag / AA_udiag stay zero (:389-391)
        Cc[k] = 0.0;
      }
    }
    // basal row inputs (grounded flux condition)
    const int kb = nz - 1;
    const double pmp_b = melting_point(Hi_eff, __ldg(z.zeta + kb));
    double Ti0b, dzzb;
    in.basal(col, vi, kb, __ldg(z.zeta + kb), Ti0b, dzzb);
    const double Kb = conductivity(c, Ti0b);
    const double dzeta_b = __ldg(z.zeta + kb) - __ldg(z.zeta + kb - 1);
    __syncwarp();
    bool found = false;
    for (int it_dt = 2; it_dt <= 10 && !found; ++it_dt) {
      double half = 1.0;
      for (int i = 1; i < it_dt; ++i) half *= 0.5;   // 0.5**(it_dt-1), exact
      const double dt = c.dt * half;
      const double inv_dt = 1.0 / dt;
      if (lane == 0) {
        // matrix part of the forward elimination for this dt
        double bprev = 1.0, cprev = 0.0;
        Bp[0] = 1.0;
        for (int k = 1; k < nz - 1; ++k) {
          double b = inv_dt + (C1[k] * __ldg(z.d1 + k)) + (C2[k] * __ldg(z.d2 + k));
          const double wgt = A[k] / bprev;
          b = b - wgt * cprev;
          W[k] = wgt;
          Bp[k] = b;
          bprev = b;
          cprev = Cc[k];
        }
        const double wgt = 0.0 / bprev;
        W[kb] = wgt;
        Bp[kb] = 1.0 - wgt * cprev;
      }
      __syncwarp();
      // per row for this dt: 1 / b'_k and the back
      // substitution's slope, x_k = d'_k / b'_k - (c_k / b'_k) x_{k+1}
      for (int k = lane; k < nz; k += 32) {
        const double rb = 1.0 / Bp[k];
        RB[k] = rb;
        NB[k] = (k < kb) ? -(Cc[k] * rb) : 0.0;
      }
      __syncwarp();
      const int nsub = 1 << (it_dt - 1);
      bool ok = true;
      for (int sub = 0; sub < nsub; ++sub) {
        // right-hand side (rows 0 .. nz-2) and the basal row's value from the current profile
        for (int k = lane; k < nz - 1; k += 32)
          D[k] = (k == 0) ? fmin(Ts, kT0) : X[k] * inv_dt - UDX[k] - VDY[k] + PHI[k];
        const double d_gr = fmin(pmp_b, X[nz - 2] - dzeta_b * Q / (dzzb * Kb));
        __syncwarp();
        // forward sweep over rows 0 .. nz-2: d'_k = D_k - W_k d'_{k-1} (row 0: the constant D_0)
        Affine mine{0.0, 1.0};
        for (int k = k0; k < min(k1, kb); ++k)
          mine = compose(Affine{D[k], k == 0 ? 0.0 : -W[k]}, mine);
        const Affine pre = warp_scan(mine, lane, true);
        double y = __shfl_up_sync(0xffffffffu, pre.a, 1);   // d' of the row before this lane's first
        if (lane == 0) y = 0.0;
        for (int k = k0; k < min(k1, kb); ++k) {
          y = (k == 0) ? D[0] : fma(-W[k], y, D[k]);
          D[k] = y;
        }
        __syncwarp();
        const double dprev = D[kb - 1];
        // back substitution over rows nz-2 .. 0 as x_k = XB_k + SB_k x_base: each lane composes its
        // rows (m_k: x_{k+1} -> x_k), the suffix scan gives the map from x_base to each lane's rows
        Affine mb{0.0, 1.0};
        for (int k = min(k1, kb) - 1; k >= k0; --k) mb = compose(Affine{D[k] * RB[k], NB[k]}, mb);
        const Affine suf = warp_scan(mb, lane, false);
        double sa = __shfl_down_sync(0xffffffffu, suf.a, 1), sb = __shfl_down_sync(0xffffffffu, suf.b, 1);
        if (lane == 31) { sa = 0.0; sb = 1.0; }
        for (int k = min(k1, kb) - 1; k >= k0; --k) {   // (sa, sb): x_base -> x_{k+1}
          const Affine r = compose(Affine{D[k] * RB[k], NB[k]}, Affine{sa, sb});
          XB[k] = r.a;
          SB[k] = r.b;
          sa = r.a;
          sb = r.b;
        }
        __syncwarp();
        // basal values and the rows' solutions, clamped (and mixed for the subgrid condition)
        const double x_gr = ((grounded ? d_gr : pmp_b) - W[kb] * dprev) * RB[kb];
        const double x_fl = (pmp_b - W[kb] * dprev) * RB[kb];
        const double x_sel = two_solves ? (d_gr - W[kb] * dprev) * RB[kb] : x_gr;
        bool bad = false;
        for (int k = lane; k < nz; k += 32) {
          const double xg = (k == kb) ? x_sel : fma(SB[k], x_sel, XB[k]);
          double v = fmin(xg, PMP[k]);
          if (two_solves) {
            const double xf = (k == kb) ? x_fl : fma(SB[k], x_fl, XB[k]);
            v = fr * v + (1.0 - fr) * fmin(xf, PMP[k]);
          }
          X[k] = v;
          bad |= unstable_value(v);
        }
        ok = !__any_sync(0xffffffffu, bad);
        __syncwarp();
      }
      found = ok;
    }
    for (int k = lane; k < nz; k += 32) Ti_next[(int64_t)k * nV + vi] = X[k];
    if (!found && lane == 0) {
      const int32_t u = atomicAdd(&cnt->n_unstable, 1);
      lists.unstable[u] = (int32_t)vi;
    }
    __syncwarp();
  }
}

// replace_Ti_with_robin_solution for the listed columns, or the step's error.
__global__ void k_heat_finish(ZOps z, Consts c, VertexFields vf, int64_t nV, double *__restrict__ Ti_next,
                              Lists lists, Counters *cnt) {
  if (cnt->err) return;
  const int32_t n = cnt->n_unstable;
  if (cnt->bad_mask > 0 || n >= cnt->threshold) return;   // k_heat_close records the error
  const double K_R = 9.828 * kSecPerYear * exp(-(0.0057 * kT0));
  const double kappa_R = K_R / (kIceDensity * 2127.5);
  for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int64_t vi = lists.unstable[j];
    const double Hi_eff = vf.Hi_eff[vi];
    const int32_t mask = vf.mask[vi];
    const double Ts = fmin(kT0, vf.T_surf[vi]);
    const double grad = -(1.0 * vf.geo[vi] / K_R);
    const double SMB = vf.SMB[vi];
    const double pmp_b = melting_point(Hi_eff, z.zeta[z.nz - 1]);
    for (int k = 0; k < z.nz; ++k) {
      const double zk = z.zeta[k];
      double T = Ti_next[(int64_t)k * nV + vi];
      if (Hi_eff > c.Hi_min) {
        if (mask == UFE_COL_GROUNDED || mask == UFE_COL_GL_GR) {
          if (SMB > 0.0) {
            const double L = sqrt(2.0 * kappa_R * Hi_eff / SMB);
            const double erf1 = erf((1.0 - zk) * Hi_eff / L);
            const double erf2 = erf(Hi_eff / L);
            T = Ts + sqrt(kPi) / 2.0 * L * grad * (erf1 - erf2);
          } else {
            T = Ts + ((kT0 - kCCGradient * Hi_eff) - Ts) * zk;
          }
        } else if (mask == UFE_COL_FLOATING) {
          T = Ts + zk * (pmp_b - Ts);
        }
      } else {
        T = Ts;
      }
      Ti_next[(int64_t)k * nV + vi] = fmin(T, melting_point(Hi_eff, zk));
    }
  }
}

// End of a step: record an error, accumulate the Robin count, reset the lists.
__global__ void k_heat_close(Counters *cnt) {
  if (cnt->err == 0) {
    if (cnt->bad_mask > 0) {
      cnt->err = UFE_ERR_INVALID;
      cnt->err_step = cnt->step;
    } else if (cnt->n_unstable >= cnt->threshold) {
      cnt->err = UFE_ERR_THERMO_UNSTABLE;
      cnt->err_step = cnt->step;
    }
    cnt->total_unstable += cnt->n_unstable;
  }
  cnt->n_retry = 0;
  cnt->n_unstable = 0;
  cnt->step += 1;
}

// ---- mesh prelude kernels --------------------------------------------------------------------
// Upwind triangle of each vertex (calc_upwind_heat_flux_derivatives, :375-413); -1 for Hi < 1.
__global__ void k_upwind_triangle(int64_t nV, int64_t nTri, const double *__restrict__ V,
                                  const int32_t *__restrict__ niTri, const int32_t *__restrict__ iTri,
                                  const int32_t *__restrict__ Tri, const double *__restrict__ Hi,
                                  const double *__restrict__ u_vav, const double *__restrict__ v_vav,
                                  int32_t *__restrict__ ti_up, int32_t *__restrict__ err) {
  const int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  if (Hi[vi] < 1.0) {
    ti_up[vi] = -1;
    return;
  }
  const double ux = -u_vav[vi], uy = -v_vav[vi];
  const double x0 = V[vi], y0 = V[nV + vi];
  int32_t found = -1;
  for (int vti = 0; vti < niTri[vi] && found < 0; ++vti) {
    const int64_t ti = iTri[(int64_t)vti * nV + vi] - 1;
    int64_t vib = -1, vic = -1;
    for (int n1 = 0; n1 < 3; ++n1) {
      const int n2 = n1 == 2 ? 0 : n1 + 1, n3 = n2 == 2 ? 0 : n2 + 1;
      if (Tri[n1 * nTri + ti] - 1 == vi) {
        vib = Tri[n2 * nTri + ti] - 1;
        vic = Tri[n3 * nTri + ti] - 1;
        break;
      }
    }
    if (vib < 0) continue;
    const double abx = V[vib] - x0, aby = V[nV + vib] - y0;
    const double acx = V[vic] - x0, acy = V[nV + vic] - y0;
    if ((abx * uy) - (aby * ux) >= 0.0 && (ux * acy) - (uy * acx) >= 0.0) found = (int32_t)ti;
  }
  ti_up[vi] = found;
  if (found < 0) atomicExch(err, 1);
}

// Upwind triangle's u_3D_b, v_3D_b per vertex and layer.
__global__ void k_gather_upwind(int64_t nV, int64_t nTri, int nz, const int32_t *__restrict__ ti_up,
                                const double *__restrict__ u_b, const double *__restrict__ v_b,
                                double *__restrict__ ub, double *__restrict__ vb) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nV * nz) return;
  const int64_t k = t / nV, vi = t - k * nV;
  const int32_t ti = ti_up[vi];
  ub[t] = ti < 0 ? 0.0 : u_b[k * nTri + ti];
  vb[t] = ti < 0 ? 0.0 : v_b[k * nTri + ti];
}

// Hi for the zeta gradients, the annual-mean surface temperature (:118-120), Q_base_grnd (:131-133).
// calc_strain_heating (thermodynamics_utilities.f90:24-78): Phi = 2 A^(-1/n) D^(1/n + 1) with the
// total strain rate D = sqrt(Dij Dij / 2); no heating where Hi < 0.1 m.  Caller-ordered inputs
// (k * nV + vi), internal-ordered output through perm (internal vi holds caller perm[vi]).
struct StrainRates {
  const double *ux, *uy, *uz, *vx, *vy, *vz, *wx, *wy, *wz;
};
__global__ void k_strain_heating(int64_t nV, int nz, const double *__restrict__ Hi_ext,
                                 const double *__restrict__ A_ext, StrainRates e, double n_glen,
                                 const int32_t *__restrict__ perm, double *__restrict__ phi) {
  const int64_t total = nV * nz, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t ix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ix < total; ix += stride) {
    const int64_t k = ix / nV, vi = ix % nV, o = k * nV + perm[vi];
    if (Hi_ext[perm[vi]] < 0.1) { phi[ix] = 0.0; continue; }
    const double a = e.uy[o] + e.vx[o], b = e.uz[o] + e.wx[o], c = e.vz[o] + e.wy[o];
    const double D = sqrt(0.5 * (e.ux[o] * e.ux[o] + e.vy[o] * e.vy[o] + e.wz[o] * e.wz[o] + 0.5 * (a * a) +
                                 0.5 * (b * b) + 0.5 * (c * c)));
    phi[ix] = 2.0 * pow(A_ext[o], -1.0 / n_glen) * pow(D, 1.0 / n_glen + 1.0);
  }
}

// calc_frictional_heating (:80-128): beta * |u_base| on grounded vertices, zero elsewhere and
// without sliding.  Internal order in and out.
__global__ void k_frictional_heating(int64_t nV, const double *__restrict__ bfc, const double *__restrict__ ub,
                                     const int32_t *__restrict__ mask, int no_sliding, double *__restrict__ fric) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vi < nV; vi += stride) {
    const bool grounded = mask[vi] == UFE_COL_GROUNDED || mask[vi] == UFE_COL_GL_GR;
    fric[vi] = (!no_sliding && grounded) ? bfc[vi] * ub[vi] : 0.0;
  }
}

__global__ void k_vertex_prelude(int64_t nV, int n_months, const double *__restrict__ Hi,
                                 const double *__restrict__ T2m, const double *__restrict__ fric,
                                 const double *__restrict__ geo, double *__restrict__ Hc,
                                 double *__restrict__ T_surf, double *__restrict__ Q) {
  const int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  Hc[vi] = fmax(10.0, Hi[vi]);
  double s = 0.0;
  for (int m = 0; m < n_months; ++m) s = s + T2m[(int64_t)m * nV + vi];
  T_surf[vi] = s / (double)n_months;
  Q[vi] = fric[vi] + geo[vi];
}

// solve_tridiagonal_matrix_equation, one thread per system (system j contiguous at j*n).
__global__ void k_tridiag(int32_t n, int64_t nsys, const double *__restrict__ a, const double *__restrict__ b,
                          const double *__restrict__ c, const double *__restrict__ d, double *__restrict__ bw,
                          double *__restrict__ dw, double *__restrict__ x) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nsys) return;
  const int64_t o = j * n;
  double bp = b[o], dp = d[o];
  bw[o] = bp;
  dw[o] = dp;
  for (int i = 1; i < n; ++i) {
    const double w = a[o + i] / bp;
    bp = b[o + i] - w * c[o + i - 1];
    dp = d[o + i] - w * dp;
    bw[o + i] = bp;
    dw[o + i] = dp;
  }
  double xv = dp / bp;
  x[o + n - 1] = xv;
  for (int i = n - 2; i >= 0; --i) {
    xv = (dw[o + i] - c[o + i] * xv) / bw[o + i];
    x[o + i] = xv;
  }
}

// ---- host: zeta operators (calc_vertical_operators_reg_1D + calc_zeta_operators_tridiagonal) ----
// calc_shape_functions_1D_reg_2nd_order (shape_functions.f90:17-79) for two neighbours, with the
// 2x2 inverse of matrix_algebra.f90:110-131.
bool shape_1d(double x, const double xc[2], double &fi, double &fii, double fc[2], double fcc[2]) {
  double dx[2], w[2];
  for (int i = 0; i < 2; ++i) dx[i] = xc[i] - x;
  for (int i = 0; i < 2; ++i) w[i] = 1.0 / std::pow(std::fabs(dx[i]), kShapeQ);
  double A11 = 0.0, A12 = 0.0, A21 = 0.0, A22 = 0.0;
  for (int i = 0; i < 2; ++i) {
    const double w2 = w[i] * w[i], dx2 = dx[i] * dx[i];
    A11 = A11 + w2 * dx[i] * dx[i];
    A12 = A12 + w2 * dx[i] * 1.0 / 2.0 * dx2;
    A21 = A21 + w2 * 1.0 / 2.0 * dx2 * dx[i];
    A22 = A22 + w2 * 1.0 / 2.0 * dx2 * 1.0 / 2.0 * dx2;
  }
  const double det = A11 * A22 - A12 * A21;
  if (!(std::fabs(det) >= 2.2250738585072014e-308)) return false;
  const double M11 = A22 / det, M12 = -A12 / det, M21 = -A21 / det, M22 = A11 / det;
  for (int i = 0; i < 2; ++i) {
    const double w2 = w[i] * w[i], dx2 = dx[i] * dx[i];
    fc[i] = w2 * ((M11 * dx[i]) + (M12 * 1.0 / 2.0 * dx2));
    fcc[i] = w2 * ((M21 * dx[i]) + (M22 * 1.0 / 2.0 * dx2));
  }
  fi = -(fc[0] + fc[1]);
  fii = -(fcc[0] + fcc[1]);
  return true;
}

bool zeta_operators_host(int nz, const double *zeta, double *l1, double *d1, double *u1, double *l2, double *d2,
                         double *u2) {
  if (nz < 3) return false;
  for (int k = 0; k < nz; ++k) {
    int ic[2];
    if (k == 0) {
      ic[0] = 1;
      ic[1] = 2;
    } else if (k == nz - 1) {
      ic[0] = nz - 3;
      ic[1] = nz - 2;
    } else {
      ic[0] = k - 1;
      ic[1] = k + 1;
    }
    const double zc[2] = {zeta[ic[0]], zeta[ic[1]]};
    double fi, fii, fc[2], fcc[2];
    if (!shape_1d(zeta[k], zc, fi, fii, fc, fcc)) return false;
    l1[k] = u1[k] = l2[k] = u2[k] = 0.0;
    d1[k] = fi;
    d2[k] = fii;
    for (int i = 0; i < 2; ++i) {
      if (ic[i] == k - 1) {
        l1[k] = fc[i];
        l2[k] = fcc[i];
      }
      if (ic[i] == k + 1) {
        u1[k] = fc[i];
        u2[k] = fcc[i];
      }
    }
  }
  return true;
}

Consts make_consts(const ufe_thermo_params *p) {
  Consts c;
  c.dt = p->dt;
  c.Hi_min = p->Hi_min_thermo;
  c.cp_u = p->uniform_ice_heat_capacity;
  c.k_u = p->uniform_ice_thermal_conductivity;
  c.cp_uniform = p->choice_ice_heat_capacity == UFE_CP_UNIFORM;
  c.k_uniform = p->choice_ice_thermal_conductivity == UFE_K_UNIFORM;
  c.glbc = p->choice_GL_temperature_BC;
  return c;
}

void validate_thermo_params(const ufe_thermo_params *p) {
  UFE_REQUIRE(p, UFE_ERR_INVALID, "thermo params are NULL");
  UFE_REQUIRE(p->dt > 0.0 && std::isfinite(p->dt), UFE_ERR_INVALID, "thermo dt must be positive");
  UFE_REQUIRE(p->choice_ice_heat_capacity == UFE_CP_UNIFORM || p->choice_ice_heat_capacity == UFE_CP_POUNDER1965,
              UFE_ERR_INVALID, "unknown choice_ice_heat_capacity");
  UFE_REQUIRE(p->choice_ice_thermal_conductivity == UFE_K_UNIFORM ||
                  p->choice_ice_thermal_conductivity == UFE_K_RITZ1987,
              UFE_ERR_INVALID, "unknown choice_ice_thermal_conductivity");
  UFE_REQUIRE(p->choice_GL_temperature_BC >= UFE_GLBC_GROUNDED && p->choice_GL_temperature_BC <= UFE_GLBC_PMP,
              UFE_ERR_INVALID, "unknown choice_GL_temperature_BC");
}

int threads_for(int nz) {
  int T = 128;
  while (T > 32 && (size_t)3 * nz * T * sizeof(double) > (size_t)kSmemBudget) T /= 2;
  return T;
}

}  // namespace

// ---- work area -------------------------------------------------------------------------------
struct ThermoWork {
  int64_t nV = 0;
  int nz = 0;
  double *zops = nullptr;       // 7 x nz
  Counters *cnt = nullptr;
  Counters *cnt_host = nullptr; // pinned
  Lists lists{};
  int64_t list_nv = 0, list_nl = 0;
  // column-level inputs (uploaded per call)
  double *col_buf = nullptr;    // 12 x nV x nz + 6 x nV
  int32_t *col_mask = nullptr;
  int64_t col_cap = 0, col_mask_cap = 0;
  // mesh-level resident state
  bool mesh_ready = false;
  double *Ti[2] = {nullptr, nullptr};
  int cur = 0;
  double *u = nullptr, *v = nullptr, *w = nullptr, *phi = nullptr, *ub = nullptr, *vb = nullptr;
  double *vert = nullptr;       // 13 x nV per-vertex scalars
  int32_t *mask = nullptr, *ti_up = nullptr;
  bool has_fr = false;
};

void free_thermo(ufe_ctx *ctx) {
  ThermoWork *t = ctx->thermo;
  if (!t) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  void *ptrs[] = {t->zops, t->cnt, t->lists.retry, t->lists.unstable, t->lists.scratch, t->col_buf, t->col_mask,
                  t->Ti[0], t->Ti[1], t->u, t->v, t->w, t->phi, t->ub, t->vb, t->vert, t->mask, t->ti_up};
  for (void *p : ptrs) dev_free(p);
  if (t->cnt_host) cudaFreeHost(t->cnt_host);
  delete t;
  ctx->thermo = nullptr;
}

namespace {

ThermoWork *thermo_work(ufe_ctx *ctx) {
  if (!ctx->thermo) {
    ctx->thermo = new ThermoWork();
    ctx->thermo->cnt = (Counters *)dev_alloc(sizeof(Counters));
    UFE_CUDA(cudaMallocHost(&ctx->thermo->cnt_host, sizeof(Counters)));
  }
  return ctx->thermo;
}

void ensure_lists(ThermoWork *t, int64_t nV, int nz) {
  if (t->list_nv < nV) {
    dev_free(t->lists.retry);
    dev_free(t->lists.unstable);
    t->lists.retry = (int32_t *)dev_alloc(sizeof(int32_t) * nV);
    t->lists.unstable = (int32_t *)dev_alloc(sizeof(int32_t) * nV);
    t->list_nv = nV;
  }
  if (t->list_nl < nV * nz) {
    dev_free(t->lists.scratch);
    t->lists.scratch = (double *)dev_alloc(sizeof(double) * nV * nz);
    t->list_nl = nV * nz;
  }
}

void set_zops(ufe_ctx *ctx, ThermoWork *t, int nz, const double *zeta_host) {
  std::vector<double> h(7 * (size_t)nz);
  std::copy(zeta_host, zeta_host + nz, h.begin());
  UFE_REQUIRE(zeta_operators_host(nz, zeta_host, &h[nz], &h[2 * nz], &h[3 * nz], &h[4 * nz], &h[5 * nz],
                                  &h[6 * nz]),
              UFE_ERR_INVALID, "zeta operators: singular shape-function system (repeated zeta values?)");
  if (t->nz != nz || !t->zops) {
    dev_free(t->zops);
    t->zops = (double *)dev_alloc(sizeof(double) * 7 * nz);
  }
  UFE_CUDA(cudaMemcpyAsync(t->zops, h.data(), sizeof(double) * 7 * nz, cudaMemcpyHostToDevice, ctx->stream));
  t->nz = nz;
}

ZOps zops_of(const ThermoWork *t) {
  const int nz = t->nz;
  const double *b = t->zops;
  return ZOps{b, b + nz, b + 2 * nz, b + 3 * nz, b + 4 * nz, b + 5 * nz, b + 6 * nz, nz};
}

void reset_counters(ufe_ctx *ctx, ThermoWork *t, int64_t nV) {
  Counters h{};
  h.threshold = (int32_t)((nV + 99) / 100);
  *t->cnt_host = h;
  UFE_CUDA(cudaMemcpyAsync(t->cnt, t->cnt_host, sizeof(Counters), cudaMemcpyHostToDevice, ctx->stream));
}

template <class In>
void launch_step(ufe_ctx *ctx, ThermoWork *t, const In &in, const Consts &c, const VertexFields &vf, int64_t nV,
                 const double *Ti_cur, double *Ti_next) {
  const ZOps z = zops_of(t);
  const int T = threads_for(z.nz);
  const size_t smem = (size_t)3 * z.nz * T * sizeof(double);
  const size_t smem_retry = (size_t)kRetryArrays * z.nz * kRetryWarps * sizeof(double);
  UFE_CUDA(cudaFuncSetAttribute(k_heat_columns<In>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  UFE_CUDA(cudaFuncSetAttribute(k_heat_retry<In>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_retry));
  cudaStream_t s = ctx->stream;
  const unsigned blocks = (unsigned)((nV + T - 1) / T);
  k_heat_columns<In><<<blocks, T, smem, s>>>(in, z, c, vf, nV, Ti_cur, Ti_next, t->lists, t->cnt);
  UFE_CUDA(cudaGetLastError());
  // the retry list is short: a fixed grid of warps (4 per SM) strides over it
  k_heat_retry<In><<<kRetryBlocks, 32 * kRetryWarps, smem_retry, s>>>(in, z, c, vf, nV, Ti_next, t->lists, t->cnt);
  UFE_CUDA(cudaGetLastError());
  k_heat_finish<<<152, 128, 0, s>>>(z, c, vf, nV, Ti_next, t->lists, t->cnt);
  UFE_CUDA(cudaGetLastError());
  k_heat_close<<<1, 1, 0, s>>>(t->cnt);
  UFE_CUDA(cudaGetLastError());
}

int32_t finish_counters(ufe_ctx *ctx, ThermoWork *t, int32_t *n_unstable) {
  UFE_CUDA(cudaMemcpyAsync(t->cnt_host, t->cnt, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
  UFE_CUDA(cudaStreamSynchronize(ctx->stream));
  const Counters &h = *t->cnt_host;
  if (n_unstable) *n_unstable = h.total_unstable;
  if (h.err == UFE_ERR_INVALID)
    throw ufe_error{UFE_ERR_INVALID, "heat equation: a column with Hi_eff >= Hi_min_thermo is neither grounded nor "
                                     "floating (step " + std::to_string(h.err_step) + ")"};
  if (h.err == UFE_ERR_THERMO_UNSTABLE)
    throw ufe_error{UFE_ERR_THERMO_UNSTABLE,
                    "heat equation solver unstable for more than 1% of vertices (step " + std::to_string(h.err_step) + ")"};
  return UFE_OK;
}

}  // namespace

// ---- C ABI -------------------------------------------------------------------------------------
extern "C" void ufe_default_thermo_params(ufe_thermo_params *p) {
  if (!p) return;
  *p = ufe_thermo_params{};
  p->dt = 1.0;                                   // dt_thermodynamics
  p->Hi_min_thermo = 10.0;                       // model_configuration.f90:579
  p->choice_ice_heat_capacity = UFE_CP_POUNDER1965;
  p->choice_ice_thermal_conductivity = UFE_K_RITZ1987;
  p->uniform_ice_heat_capacity = 2009.0;
  p->uniform_ice_thermal_conductivity = 6.626958E7;
  p->choice_GL_temperature_BC = UFE_GLBC_GROUNDED;
}

extern "C" int32_t ufe_zeta_operators(int32_t nz, const double *zeta, double *ddz_l, double *ddz_d, double *ddz_u,
                                      double *d2dz2_l, double *d2dz2_d, double *d2dz2_u) {
  if (nz < 3 || nz > kMaxNz || !zeta || !ddz_l || !ddz_d || !ddz_u || !d2dz2_l || !d2dz2_d || !d2dz2_u)
    return UFE_ERR_INVALID;
  return zeta_operators_host(nz, zeta, ddz_l, ddz_d, ddz_u, d2dz2_l, d2dz2_d, d2dz2_u) ? UFE_OK : UFE_ERR_INVALID;
}

extern "C" int32_t ufe_thermo_step(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t nV, int32_t nz,
                                   const double *zeta, const ufe_thermo_columns *cols, double *Ti_next,
                                   int32_t *n_unstable) {
  return guarded(ctx, [&]() -> int32_t {
    validate_thermo_params(p);
    UFE_REQUIRE(nV >= 1 && nz >= 3 && nz <= kMaxNz, UFE_ERR_INVALID, "thermo: need nV >= 1 and 3 <= nz <= 256");
    UFE_REQUIRE(zeta && cols && Ti_next, UFE_ERR_INVALID, "thermo: NULL argument");
    const double *layer_in[11] = {cols->Ti, cols->u_3D, cols->v_3D, cols->w_3D, cols->u_times_dTdxp_upwind,
                                  cols->v_times_dTdyp_upwind, cols->dzeta_dx, cols->dzeta_dy, cols->dzeta_dz,
                                  cols->dzeta_dt, cols->internal_heating};
    for (const double *q : layer_in) UFE_REQUIRE(q, UFE_ERR_INVALID, "thermo: NULL column array");
    UFE_REQUIRE(cols->Hi_eff && cols->T_surf_annual && cols->Q_base_grnd && cols->mask && cols->geothermal_heat_flux &&
                    cols->SMB,
                UFE_ERR_INVALID, "thermo: NULL per-vertex array");
    UFE_REQUIRE(p->choice_GL_temperature_BC != UFE_GLBC_SUBGRID || cols->fraction_gr, UFE_ERR_INVALID,
                "thermo: UFE_GLBC_SUBGRID needs fraction_gr");
    UFE_CUDA(cudaSetDevice(ctx->device));
    ThermoWork *t = thermo_work(ctx);
    set_zops(ctx, t, nz, zeta);
    const int64_t nl = (int64_t)nV * nz;
    const int64_t need = 12 * nl + 6 * (int64_t)nV;
    if (t->col_cap < need) {
      dev_free(t->col_buf);
      t->col_buf = (double *)dev_alloc(sizeof(double) * need);
      t->col_cap = need;
    }
    if (t->col_mask_cap < nV) {
      dev_free(t->col_mask);
      t->col_mask = (int32_t *)dev_alloc(sizeof(int32_t) * nV);
      t->col_mask_cap = nV;
    }
    ensure_lists(t, nV, nz);
    cudaStream_t s = ctx->stream;
    double *d = t->col_buf;
    for (int i = 0; i < 11; ++i)
      UFE_CUDA(cudaMemcpyAsync(d + i * nl, layer_in[i], sizeof(double) * nl, cudaMemcpyHostToDevice, s));
    double *out = d + 11 * nl;
    double *vtx = d + 12 * nl;
    const double *vert_in[6] = {cols->Hi_eff, cols->T_surf_annual, cols->Q_base_grnd, cols->fraction_gr,
                                cols->geothermal_heat_flux, cols->SMB};
    for (int i = 0; i < 6; ++i) {
      if (vert_in[i])
        UFE_CUDA(cudaMemcpyAsync(vtx + i * (int64_t)nV, vert_in[i], sizeof(double) * nV, cudaMemcpyHostToDevice, s));
      else
        UFE_CUDA(cudaMemsetAsync(vtx + i * (int64_t)nV, 0, sizeof(double) * nV, s));
    }
    UFE_CUDA(cudaMemcpyAsync(t->col_mask, cols->mask, sizeof(int32_t) * nV, cudaMemcpyHostToDevice, s));
    ColumnArrays in{nV, d, d + nl, d + 2 * nl, d + 3 * nl, d + 4 * nl, d + 5 * nl, d + 6 * nl, d + 7 * nl, d + 8 * nl,
                    d + 9 * nl, d + 10 * nl};
    VertexFields vf{vtx, vtx + nV, vtx + 2 * (int64_t)nV, vtx + 3 * (int64_t)nV, vtx + 4 * (int64_t)nV,
                    vtx + 5 * (int64_t)nV, t->col_mask};
    reset_counters(ctx, t, nV);
    launch_step(ctx, t, in, make_consts(p), vf, nV, d, out);
    UFE_CUDA(cudaMemcpyAsync(Ti_next, out, sizeof(double) * nl, cudaMemcpyDeviceToHost, s));
    return finish_counters(ctx, t, n_unstable);
  });
}

namespace {

HeatMesh heat_mesh_inputs(ufe_ctx *ctx, ThermoWork *t, const double *Ti_cur) {
  const int64_t nV = t->nV;
  const double *vt = t->vert;
  const DevCSR &Ax = ctx->ops[UFE_OP_DDX_A_B], &Ay = ctx->ops[UFE_OP_DDY_A_B];
  HeatMesh in;
  in.nV = nV;
  in.Ti0 = Ti_cur;
  in.u = t->u;
  in.v = t->v;
  in.w = t->w;
  in.phi = t->phi;
  in.ub = t->ub;
  in.vb = t->vb;
  in.gHs_x = vt;
  in.gHi_x = vt + nV;
  in.gHs_y = vt + 2 * nV;
  in.gHi_y = vt + 3 * nV;
  in.dHs_dt = vt + 4 * nV;
  in.dHi_dt = vt + 5 * nV;
  in.Hc = vt + 6 * nV;
  in.ti_up = t->ti_up;
  in.ab_ptr = Ax.ptr;
  in.ab_ind = Ax.ind;
  in.ddx_ab = Ax.val;
  in.ddy_ab = Ay.val;
  return in;
}

VertexFields heat_vertex_fields(ThermoWork *t) {
  const int64_t nV = t->nV;
  const double *vt = t->vert;
  // Hi_eff, T_surf, Q, fr, geo, SMB at slots 7..12
  return VertexFields{vt + 7 * nV, vt + 8 * nV, vt + 9 * nV, vt + 10 * nV, vt + 11 * nV, vt + 12 * nV, t->mask};
}

}  // namespace

extern "C" int32_t ufe_heat_upload(ufe_ctx *ctx, const ufe_heat_fields *f) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "heat upload: no mesh uploaded");
    UFE_REQUIRE(f, UFE_ERR_INVALID, "heat upload: NULL fields");
    const int ops_needed[4] = {UFE_OP_DDX_A_A, UFE_OP_DDY_A_A, UFE_OP_DDX_A_B, UFE_OP_DDY_A_B};
    for (int op : ops_needed)
      UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "heat upload: the a-a and a-b d/dx, d/dy operators are needed");
    UFE_REQUIRE(ctx->ops[UFE_OP_DDX_A_B].ptr == ctx->ops[UFE_OP_DDY_A_B].ptr &&
                    ctx->ops[UFE_OP_DDX_A_B].ind == ctx->ops[UFE_OP_DDY_A_B].ind,
                UFE_ERR_INVALID, "heat upload: ddx_a_b and ddy_a_b must share one sparsity pattern");
    const double *need[] = {f->Ti, f->Hi, f->Hi_eff, f->Hs, f->dHi_dt, f->dHs_dt, f->u_vav, f->v_vav, f->u_3D,
                            f->v_3D, f->w_3D, f->u_3D_b, f->v_3D_b, f->geothermal_heat_flux, f->T2m, f->SMB};
    for (const double *q : need) UFE_REQUIRE(q, UFE_ERR_INVALID, "heat upload: NULL field");
    // the heating terms: given, or computed here from their inputs
    const bool strain = f->internal_heating == nullptr, friction = f->frictional_heating == nullptr;
    if (strain) {
      const double *sr[] = {f->A_flow, f->du_dx_3D, f->du_dy_3D, f->du_dz_3D, f->dv_dx_3D, f->dv_dy_3D, f->dv_dz_3D,
                            f->dw_dx_3D, f->dw_dy_3D, f->dw_dz_3D};
      for (const double *q : sr)
        UFE_REQUIRE(q, UFE_ERR_INVALID, "heat upload: strain heating needs A_flow and the nine 3-D strain rates");
    }
    if (friction)
      UFE_REQUIRE(f->basal_friction_coefficient && f->uabs_base, UFE_ERR_INVALID,
                  "heat upload: frictional heating needs basal_friction_coefficient and uabs_base");
    UFE_REQUIRE(f->mask && f->n_months >= 1, UFE_ERR_INVALID, "heat upload: need mask and n_months >= 1");
    const int64_t nV = ctx->nV, nTri = ctx->nTri;
    const int nz = ctx->nz;
    UFE_REQUIRE(nz >= 3 && nz <= kMaxNz, UFE_ERR_INVALID, "heat upload: the mesh needs 3 <= nz <= 256");
    UFE_CUDA(cudaSetDevice(ctx->device));
    ThermoWork *t = thermo_work(ctx);
    cudaStream_t s = ctx->stream;
    if (t->nV != nV || t->nz != nz || !t->Ti[0]) {
      void *old[] = {t->Ti[0], t->Ti[1], t->u, t->v, t->w, t->phi, t->ub, t->vb, t->vert, t->mask, t->ti_up};
      for (void *q : old) dev_free(q);
      const size_t nl = sizeof(double) * nV * nz;
      t->Ti[0] = (double *)dev_alloc(nl);
      t->Ti[1] = (double *)dev_alloc(nl);
      t->u = (double *)dev_alloc(nl);
      t->v = (double *)dev_alloc(nl);
      t->w = (double *)dev_alloc(nl);
      t->phi = (double *)dev_alloc(nl);
      t->ub = (double *)dev_alloc(nl);
      t->vb = (double *)dev_alloc(nl);
      t->vert = (double *)dev_alloc(sizeof(double) * 13 * nV);
      t->mask = (int32_t *)dev_alloc(sizeof(int32_t) * nV);
      t->ti_up = (int32_t *)dev_alloc(sizeof(int32_t) * nV);
    }
    t->nV = nV;
    t->mesh_ready = false;
    set_zops(ctx, t, nz, ctx->zeta_host.data());
    ensure_lists(t, nV, nz);
    t->cur = 0;
    to_internal(ctx, t->Ti[0], f->Ti, false, nz);
    to_internal(ctx, t->u, f->u_3D, false, nz);
    to_internal(ctx, t->v, f->v_3D, false, nz);
    to_internal(ctx, t->w, f->w_3D, false, nz);
    to_internal_i32(ctx, t->mask, f->mask, false);
    if (!strain) {
      to_internal(ctx, t->phi, f->internal_heating, false, nz);
    } else {
      // the inputs go up in the caller's order; the kernel gathers them while it computes
      const size_t nl = (size_t)nV * nz;
      double *buf = (double *)dev_alloc(sizeof(double) * (nl * 10 + nV));
      try {
        const double *src[] = {f->A_flow, f->du_dx_3D, f->du_dy_3D, f->du_dz_3D, f->dv_dx_3D, f->dv_dy_3D,
                               f->dv_dz_3D, f->dw_dx_3D, f->dw_dy_3D, f->dw_dz_3D};
        for (int q = 0; q < 10; ++q)
          UFE_CUDA(cudaMemcpyAsync(buf + q * nl, src[q], sizeof(double) * nl, cudaMemcpyHostToDevice, s));
        UFE_CUDA(cudaMemcpyAsync(buf + 10 * nl, f->Hi, sizeof(double) * nV, cudaMemcpyHostToDevice, s));
        StrainRates e{buf + nl, buf + 2 * nl, buf + 3 * nl, buf + 4 * nl, buf + 5 * nl, buf + 6 * nl, buf + 7 * nl,
                      buf + 8 * nl, buf + 9 * nl};
        k_strain_heating<<<(unsigned)std::min<int64_t>((nl + 255) / 256, 65535), 256, 0, s>>>(
            nV, nz, buf + 10 * nl, buf, e, f->Glens_flow_law_exponent > 0.0 ? f->Glens_flow_law_exponent : 3.0, ctx->perm_v,
            t->phi);
        UFE_CUDA(cudaGetLastError());
        UFE_CUDA(cudaStreamSynchronize(s));
      } catch (...) {
        dev_free(buf);
        throw;
      }
      dev_free(buf);
    }
    double *vt = t->vert;
    // slots: 0 gHs_x, 1 gHi_x, 2 gHs_y, 3 gHi_y, 4 dHs_dt, 5 dHi_dt, 6 Hc, 7 Hi_eff, 8 T_surf, 9 Q,
    //        10 fr, 11 geo, 12 SMB
    to_internal(ctx, vt + 4 * nV, f->dHs_dt, false, 1);
    to_internal(ctx, vt + 5 * nV, f->dHi_dt, false, 1);
    to_internal(ctx, vt + 7 * nV, f->Hi_eff, false, 1);
    to_internal(ctx, vt + 11 * nV, f->geothermal_heat_flux, false, 1);
    to_internal(ctx, vt + 12 * nV, f->SMB, false, 1);
    t->has_fr = f->fraction_gr != nullptr;
    if (f->fraction_gr)
      to_internal(ctx, vt + 10 * nV, f->fraction_gr, false, 1);
    else
      UFE_CUDA(cudaMemsetAsync(vt + 10 * nV, 0, sizeof(double) * nV, s));
    // temporaries: Hi, Hs, u_vav, v_vav, frictional heating, T2m, u_3D_b, v_3D_b
    double *Hi = (double *)dev_alloc(sizeof(double) * nV * 5);
    double *Hs = Hi + nV, *uv = Hi + 2 * nV, *vv = Hi + 3 * nV, *fric = Hi + 4 * nV;
    double *T2m = (double *)dev_alloc(sizeof(double) * nV * f->n_months);
    double *ubt = (double *)dev_alloc(sizeof(double) * nTri * nz * 2);
    double *vbt = ubt + nTri * nz;
    int32_t *err = (int32_t *)dev_alloc(sizeof(int32_t));
    int32_t herr = 0;
    try {
      to_internal(ctx, Hi, f->Hi, false, 1);
      to_internal(ctx, Hs, f->Hs, false, 1);
      to_internal(ctx, uv, f->u_vav, false, 1);
      to_internal(ctx, vv, f->v_vav, false, 1);
      if (!friction) {
        to_internal(ctx, fric, f->frictional_heating, false, 1);
      } else {
        double *bfc = ubt, *uab = ubt + nV;   // ubt is filled below; use it as scratch first
        to_internal(ctx, bfc, f->basal_friction_coefficient, false, 1);
        to_internal(ctx, uab, f->uabs_base, false, 1);
        k_frictional_heating<<<(unsigned)((nV + 255) / 256), 256, 0, s>>>(nV, bfc, uab, t->mask, f->no_sliding,
                                                                          fric);
        UFE_CUDA(cudaGetLastError());
      }
      to_internal(ctx, T2m, f->T2m, false, f->n_months);
      to_internal(ctx, ubt, f->u_3D_b, true, nz);
      to_internal(ctx, vbt, f->v_3D_b, true, nz);
      // calc_zeta_gradients: ddx_a_a / ddy_a_a of Hi and Hs
      launch_csr_spmv(s, ctx->ops[UFE_OP_DDX_A_A], Hs, vt + 0 * nV, 1);
      launch_csr_spmv(s, ctx->ops[UFE_OP_DDX_A_A], Hi, vt + 1 * nV, 1);
      launch_csr_spmv(s, ctx->ops[UFE_OP_DDY_A_A], Hs, vt + 2 * nV, 1);
      launch_csr_spmv(s, ctx->ops[UFE_OP_DDY_A_A], Hi, vt + 3 * nV, 1);
      const unsigned bv = (unsigned)((nV + 255) / 256);
      k_vertex_prelude<<<bv, 256, 0, s>>>(nV, f->n_months, Hi, T2m, fric, vt + 11 * nV, vt + 6 * nV, vt + 8 * nV,
                                          vt + 9 * nV);
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
      k_upwind_triangle<<<bv, 256, 0, s>>>(nV, nTri, ctx->V, ctx->niTri, ctx->iTri, ctx->Tri, Hi, uv, vv, t->ti_up,
                                           err);
      UFE_CUDA(cudaGetLastError());
      k_gather_upwind<<<(unsigned)((nV * nz + 255) / 256), 256, 0, s>>>(nV, nTri, nz, t->ti_up, ubt, vbt, t->ub,
                                                                        t->vb);
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      dev_free(Hi);
      dev_free(T2m);
      dev_free(ubt);
      dev_free(err);
      throw;
    }
    dev_free(Hi);
    dev_free(T2m);
    dev_free(ubt);
    dev_free(err);
    UFE_REQUIRE(herr == 0, UFE_ERR_INVALID, "heat upload: could not find upwind triangle for a vertex with ice");
    t->mesh_ready = true;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_heat_step_resident(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t nsteps,
                                          int32_t *n_unstable_total, double *device_ms) {
  return guarded(ctx, [&]() -> int32_t {
    validate_thermo_params(p);
    UFE_REQUIRE(nsteps >= 0, UFE_ERR_INVALID, "heat stepping: nsteps < 0");
    ThermoWork *t = ctx->thermo;
    UFE_REQUIRE(t && t->mesh_ready, UFE_ERR_INVALID, "heat stepping: call ufe_heat_upload first");
    UFE_REQUIRE(p->choice_GL_temperature_BC != UFE_GLBC_SUBGRID || t->has_fr, UFE_ERR_INVALID,
                "heat stepping: UFE_GLBC_SUBGRID needs fraction_gr in the uploaded fields");
    UFE_CUDA(cudaSetDevice(ctx->device));
    const Consts c = make_consts(p);
    const VertexFields vf = heat_vertex_fields(t);
    reset_counters(ctx, t, t->nV);
    const int cur0 = t->cur;
    UFE_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    for (int32_t st = 0; st < nsteps; ++st) {
      const int a = (cur0 + st) & 1;
      const HeatMesh in = heat_mesh_inputs(ctx, t, t->Ti[a]);
      launch_step(ctx, t, in, c, vf, t->nV, t->Ti[a], t->Ti[a ^ 1]);
    }
    UFE_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    int32_t rc;
    try {
      rc = finish_counters(ctx, t, n_unstable_total);
    } catch (...) {
      t->cur = (cur0 + t->cnt_host->err_step) & 1;
      throw;
    }
    t->cur = (cur0 + nsteps) & 1;
    if (device_ms) {
      float ms = 0.f;
      UFE_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      *device_ms = ms;
    }
    return rc;
  });
}

namespace {
__global__ void k_count_active(int64_t nV, const double *__restrict__ Hi_eff, double Hi_min,
                               unsigned long long *count) {
  const int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = vi < nV && !(Hi_eff[vi] < Hi_min);
  const unsigned ballot = __ballot_sync(0xffffffffu, active);
  if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(count, (unsigned long long)__popc(ballot));
}
}  // namespace

extern "C" int32_t ufe_profile_heat_kernels(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t repeats, double *us,
                                            int64_t *counts) {
  return guarded(ctx, [&]() -> int32_t {
    validate_thermo_params(p);
    UFE_REQUIRE(repeats >= 1 && us, UFE_ERR_INVALID, "heat profile: need repeats >= 1 and us[4]");
    ThermoWork *t = ctx->thermo;
    UFE_REQUIRE(t && t->mesh_ready, UFE_ERR_INVALID, "heat profile: call ufe_heat_upload first");
    UFE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const Consts c = make_consts(p);
    const VertexFields vf = heat_vertex_fields(t);
    const HeatMesh in = heat_mesh_inputs(ctx, t, t->Ti[t->cur]);
    double *out = t->Ti[t->cur ^ 1];
    const ZOps z = zops_of(t);
    const int T = threads_for(z.nz);
    const size_t smem = (size_t)3 * z.nz * T * sizeof(double);
    const size_t smem_retry = (size_t)kRetryArrays * z.nz * kRetryWarps * sizeof(double);
    UFE_CUDA(cudaFuncSetAttribute(k_heat_columns<HeatMesh>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    UFE_CUDA(cudaFuncSetAttribute(k_heat_retry<HeatMesh>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_retry));
    const int64_t nV = t->nV;
    const unsigned blocks = (unsigned)((nV + T - 1) / T);
    reset_counters(ctx, t, nV);
    float ms[4] = {0, 0, 0, 0};
    for (int which = 0; which < 4; ++which) {
      UFE_CUDA(cudaEventRecord(ctx->ev0, s));
      for (int r = 0; r < repeats; ++r) {
        if (which == 0) {
          k_heat_columns<HeatMesh><<<blocks, T, smem, s>>>(in, z, c, vf, nV, in.Ti0, out, t->lists, t->cnt);
        } else if (which == 1) {
          k_heat_retry<HeatMesh><<<kRetryBlocks, 32 * kRetryWarps, smem_retry, s>>>(in, z, c, vf, nV, out,
                                                                                      t->lists, t->cnt);
        } else if (which == 2) {
          k_heat_finish<<<152, 128, 0, s>>>(z, c, vf, nV, out, t->lists, t->cnt);
        } else {
          k_heat_close<<<1, 1, 0, s>>>(t->cnt);
        }
        UFE_CUDA(cudaGetLastError());
        // keep the retry list from growing across repeats of the column pass
        if (which == 0) UFE_CUDA(cudaMemsetAsync(&t->cnt->n_retry, 0, sizeof(int32_t), s));
      }
      UFE_CUDA(cudaEventRecord(ctx->ev1, s));
      UFE_CUDA(cudaEventSynchronize(ctx->ev1));
      UFE_CUDA(cudaEventElapsedTime(&ms[which], ctx->ev0, ctx->ev1));
    }
    for (int i = 0; i < 4; ++i) us[i] = 1000.0 * ms[i] / repeats;
    if (counts) {
      unsigned long long *d = (unsigned long long *)dev_alloc(sizeof(unsigned long long));
      unsigned long long h = 0;
      UFE_CUDA(cudaMemsetAsync(d, 0, sizeof(h), s));
      k_count_active<<<(unsigned)((nV + 255) / 256), 256, 0, s>>>(nV, vf.Hi_eff, c.Hi_min, d);
      UFE_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      dev_free(d);
      counts[0] = (int64_t)h;
      counts[1] = nV - (int64_t)h;
    }
    reset_counters(ctx, t, nV);
    UFE_CUDA(cudaStreamSynchronize(s));
    return UFE_OK;
  });
}

extern "C" int32_t ufe_heat_download(ufe_ctx *ctx, double *Ti) {
  return guarded(ctx, [&]() -> int32_t {
    ThermoWork *t = ctx->thermo;
    UFE_REQUIRE(t && t->mesh_ready, UFE_ERR_INVALID, "heat download: nothing uploaded");
    UFE_REQUIRE(Ti, UFE_ERR_INVALID, "heat download: NULL output");
    UFE_CUDA(cudaSetDevice(ctx->device));
    to_external(ctx, Ti, t->Ti[t->cur], false, t->nz);
    return UFE_OK;
  });
}

extern "C" int32_t ufe_solve_3D_heat_equation(ufe_ctx *ctx, const ufe_thermo_params *p, const ufe_heat_fields *f,
                                              double *Ti_next, int32_t *n_unstable) {
  if (!ctx) return UFE_ERR_INVALID;
  if (!Ti_next) {
    ctx->last_error = "solve_3D_heat_equation: NULL output";
    return UFE_ERR_INVALID;
  }
  int32_t rc = ufe_heat_upload(ctx, f);
  if (rc != UFE_OK) return rc;
  rc = ufe_heat_step_resident(ctx, p, 1, n_unstable, nullptr);
  if (rc != UFE_OK) return rc;
  return ufe_heat_download(ctx, Ti_next);
}

extern "C" int32_t ufe_tridiagonal_solve(ufe_ctx *ctx, int32_t n, int32_t nsys, const double *a, const double *b,
                                         const double *c, const double *d, double *x) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(n >= 1 && nsys >= 0, UFE_ERR_INVALID, "tridiagonal: need n >= 1, nsys >= 0");
    UFE_REQUIRE(a && b && c && d && x, UFE_ERR_INVALID, "tridiagonal: NULL argument");
    if (nsys == 0) return UFE_OK;
    UFE_CUDA(cudaSetDevice(ctx->device));
    const int64_t N = (int64_t)n * nsys;
    cudaStream_t s = ctx->stream;
    double *buf = (double *)dev_alloc(sizeof(double) * N * 7);
    try {
      double *da = buf, *db = buf + N, *dc = buf + 2 * N, *dd = buf + 3 * N, *bw = buf + 4 * N, *dw = buf + 5 * N,
             *dx = buf + 6 * N;
      UFE_CUDA(cudaMemcpyAsync(da, a, sizeof(double) * N, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemcpyAsync(db, b, sizeof(double) * N, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemcpyAsync(dc, c, sizeof(double) * N, cudaMemcpyHostToDevice, s));
      UFE_CUDA(cudaMemcpyAsync(dd, d, sizeof(double) * N, cudaMemcpyHostToDevice, s));
      k_tridiag<<<(unsigned)((nsys + 127) / 128), 128, 0, s>>>(n, nsys, da, db, dc, dd, bw, dw, dx);
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      dev_free(buf);
      throw;
    }
    dev_free(buf);
    return UFE_OK;
  });
}
