// The SSA/DIVA velocity solve on the GPU.
//
// One Picard (viscosity) iteration of solve_SSA / solve_DIVA
// (src/UFEMISM/ice_dynamics/conservation_of_momentum/SSA_DIVA/SSA_main.f90:165-234,
//  DIVA_main.f90:170-251) is a handful of fused kernels:
//
//   k_vertex_{ssa,diva}  one thread per vertex: the b->a operator row (strain rates, velocities
//                        on vertices, DIVA vertical shear), Glen viscosity, N = eta H, the
//                        sliding law (and DIVA's F-integral and beta_eff)
//   k_assemble<MODE>     one thread per triangle: the a->b operator row (N_b, dN/dx, dN/dy,
//                        beta_b), the 2x2-block stiffness row on the 2nd-order b_b pattern
//                        (solve_linearised_SSA_DIVA.f90:180-641), the Jacobi diagonal, the FP32
//                        copy, and the Krylov initial residual
//   Krylov               ufe_krylov.cuh, three kernels per BiCGStab iteration
//   k_finalize_{ssa,diva} velocity limits, relaxation, (DIVA basal velocity and stress), the
//                        Picard L2 norm and divergence control (SSA_DIVA_utilities.f90:84-184)
//
// The whole solve is one CUDA graph: a conditional while-node for the Picard loop holds a
// nested while-node for the Krylov loop; the last block of the relevant reduction sets each
// loop condition on the device, so no host round trip happens inside a solve.
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <algorithm>

#include "ufe_krylov.cuh"

namespace {

constexpr double kIceDensity = 910.0;  // src/UPSY/basic/parameters.f90:23
constexpr double kGrav = 9.81;         // parameters.f90:20
constexpr double kRGas = 8.314;        // parameters.f90:27
constexpr int kMaxNz = 64;
constexpr int kThreads = 256;
constexpr int kMaxRefine = 60;

enum ErrFlags : int { kErrNoDiag = 1, kErrBcNeighbour = 2, kErrNoNeighbour = 4 };

int sm_count(ufe_ctx *ctx) {
  static int cached = -1;
  if (cached < 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx->device);
    cached = v > 0 ? v : 148;
  }
  return cached;
}

int max_grid(ufe_ctx *ctx) {
  int g = sm_count(ctx) * 8;
  return g < kMaxReduceBlocks ? g : kMaxReduceBlocks;
}

// ---- physics (device) ---------------------------------------------------------------------
struct PhysParams {
  int sliding_law, crossterms, gl_subgrid, has_bc;
  int bc_u[4], bc_v[4];   // N, E, S, W
  double n_glen, visc_eff_min, vel_max, m_weertman, delta_v, beta_max, fgr_exp;
  double budd_q, budd_u0;
  double zi_p, zi_ut;
  int inexact;        // krylov_forcing > 0: the two-phase inexact Picard iteration
  double relax_cfg;   // visc_it_relax as configured (the 'infinite_SSA_icestream' border rows)
  double picard_tol;
  int visc_it_nit;
};

PhysParams make_phys(const ufe_solver_params &p, int has_bc) {
  PhysParams q;
  q.sliding_law = p.choice_sliding_law;
  q.crossterms = p.do_include_SSADIVA_crossterms;
  q.gl_subgrid = p.do_GL_subgrid_friction;
  q.has_bc = has_bc;
  q.bc_u[0] = p.BC_u_north; q.bc_u[1] = p.BC_u_east; q.bc_u[2] = p.BC_u_south; q.bc_u[3] = p.BC_u_west;
  q.bc_v[0] = p.BC_v_north; q.bc_v[1] = p.BC_v_east; q.bc_v[2] = p.BC_v_south; q.bc_v[3] = p.BC_v_west;
  q.n_glen = p.Glens_flow_law_exponent;
  q.visc_eff_min = p.visc_eff_min;
  q.vel_max = p.vel_max;
  q.m_weertman = p.slid_Weertman_m;
  q.delta_v = p.slid_delta_v;
  q.beta_max = p.slid_beta_max;
  q.fgr_exp = p.subgrid_friction_exponent_on_B_grid;
  q.budd_q = p.slid_Budd_q_plastic;
  q.budd_u0 = p.slid_Budd_u_threshold;
  q.zi_p = p.slid_ZI_p;
  q.zi_ut = p.slid_ZI_ut;
  q.relax_cfg = p.visc_it_relax;
  q.inexact = p.krylov_forcing > 0.0;
  q.picard_tol = p.visc_it_norm_dUV_tol;
  q.visc_it_nit = p.visc_it_nit;
  return q;
}

// e^((1-n)/(2n)), the strain-rate power of Glen's law.  For the usual n = 3 the exponent is -1/3 and
// the reciprocal cube root replaces the general power (several times fewer FP64 instructions, which
// bound the viscosity passes on this GPU); n = 1 gives 1.  Both agree with pow to within an ulp or so.
__device__ __forceinline__ double glen_epow(double e, double n) {
  if (n == 3.0) return rcbrt(e);
  if (n == 1.0) return 1.0;
  return pow(e, (1.0 - n) / (2.0 * n));
}

// calc_effective_viscosity_Glen_2D / _3D_uv_only (constitutive_equation.f90:25-80)
// Glen's flow law, 3-D (constitutive_equation.f90:25-80), with A^(-1/n) evaluated beforehand:
// 0.5 A^(-1/n) (eps^2 + eps0^2)^((1-n)/(2n))
__device__ __forceinline__ double glen_apow(double eps0, double ux, double uy, double vx, double vy,
                                            double uz, double vz, double A_pow, double n) {
  double e = ux * ux + vy * vy + ux * vy + 0.25 * ((uy + vx) * (uy + vx)) + 0.25 * (uz * uz + vz * vz) + eps0;
  return 0.5 * A_pow * glen_epow(e, n);
}
__device__ __forceinline__ double glen2d(double eps0, double ux, double uy, double vx, double vy,
                                         double A, double n) {
  double e = ux * ux + vy * vy + ux * vy + 0.25 * ((uy + vx) * (uy + vx)) + eps0;
  return 0.5 * (n == 3.0 ? rcbrt(A) : pow(A, -1.0 / n)) * glen_epow(e, n);
}

struct SlidingIn {
  const double *beta_sq, *alpha_sq, *effp, *tys;
};

// x^(1/m) and x^m of the sliding exponent; the usual m = 3 (and m = 1) without the general power
__device__ __forceinline__ double pow_inv_m(double x, double m) {
  if (m == 3.0) return cbrt(x);
  if (m == 1.0) return x;
  return pow(x, 1.0 / m);
}
__device__ __forceinline__ double pow_m(double x, double m) {
  if (m == 3.0) return x * x * x;
  if (m == 1.0) return x;
  return pow(x, m);
}

// velocity-dependent part of the sliding laws (sliding_laws.f90:25-351) and the beta_max cap (:76)
__device__ double sliding_beta(const PhysParams &q, const SlidingIn &s, int vi, double u, double v) {
  double uabs = sqrt(q.delta_v * q.delta_v + u * u + v * v);
  double m = q.m_weertman, beta = 0.0;
  switch (q.sliding_law) {
    case UFE_SLIDING_NO_SLIDING: beta = 0.0; break;
    case UFE_SLIDING_WEERTMAN: beta = s.beta_sq[vi] * (pow_inv_m(uabs, m) / uabs); break;
    case UFE_SLIDING_COULOMB: beta = s.tys[vi] / uabs; break;
    case UFE_SLIDING_BUDD:
      beta = s.tys[vi] * pow(uabs, q.budd_q - 1.0) / pow(q.budd_u0, q.budd_q);
      break;
    case UFE_SLIDING_TSAI2015:
      beta = fmin(s.alpha_sq[vi] * s.effp[vi], s.beta_sq[vi] * pow_inv_m(uabs, m)) / uabs;
      break;
    case UFE_SLIDING_SCHOOF2005: {
      double b = s.beta_sq[vi], aN = s.alpha_sq[vi] * s.effp[vi];
      beta = ((b * pow_inv_m(uabs, m) * s.alpha_sq[vi] * s.effp[vi]) / pow_inv_m(pow_m(b, m) * uabs + pow_m(aN, m), m)) /
             uabs;
      break;
    }
    case UFE_SLIDING_ZOET_IVERSON:   // :399-400
      beta = s.tys[vi] * pow(uabs, 1.0 / q.zi_p - 1.0) * pow(uabs + q.zi_ut, -1.0 / q.zi_p);
      break;
    case UFE_SLIDING_IDEALISED_SSA_ICESTREAM:   // :477 (tys: Schoof's yield stress, k_icestream_yield)
      beta = s.tys[vi] / uabs;
      break;
    default: beta = 0.0;
  }
  return fmin(q.beta_max, beta);
}

struct OpRow {  // a CSR family with shared pattern
  const int32_t *ptr, *ind;
  const double *v0, *v1, *v2;
};

// ---- prologue: driving stress (calc_driving_stress, SSA_DIVA_utilities.f90:21-57) and the
// vertically averaged flow factor (calc_vertically_averaged_flow_parameter, SSA_main.f90:312-337)
__global__ void k_prologue(int nV, int nTri, int nz, OpRow ab, const double *Hi, const double *Hs,
                           const double *A_flow, const double *zeta, double2 *tau_d, double *Avav,
                           double *A_pow, PicardScalars *ps, KrylovScalars *ks, double relax0, double eps0,
                           double n_glen, int32_t *pred_flag) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride) {
    double Hib = 0.0, dx = 0.0, dy = 0.0;
    for (int k = ab.ptr[t]; k < ab.ptr[t + 1]; ++k) {
      int v = ab.ind[k];
      Hib = Hib + ab.v0[k] * Hi[v];
      dx = dx + ab.v1[k] * Hs[v];
      dy = dy + ab.v2[k] * Hs[v];
    }
    tau_d[t] = make_double2(-kIceDensity * kGrav * Hib * dx, -kIceDensity * kGrav * Hib * dy);
  }
  if (Avav)
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += stride) {
      double a = 0.0;
      for (int k = 1; k < nz; ++k)
        a = a + 0.5 * (A_flow[(int64_t)k * nV + v] + A_flow[(int64_t)(k - 1) * nV + v]) * (zeta[k] - zeta[k - 1]);
      Avav[v] = a;
    }
  // DIVA: A^(-1/n) per vertex and layer, constant over the Picard iterations of a solve
  if (A_pow)
    for (int64_t ix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ix < (int64_t)nV * nz; ix += stride)
      A_pow[ix] = pow(A_flow[ix], -1.0 / n_glen);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    PicardScalars &p = *ps;
    p.L2 = 1e9;
    p.L2_prev = 1e9;
    p.relax = relax0;
    p.eps0 = eps0;
    p.eta_max = 0.5 * pow(1e-18, -1.0 / n_glen) * pow(eps0, (1.0 - n_glen) / (2.0 * n_glen));
    p.it = 0;
    p.nit_diverg = 0;
    p.status = UFE_OK;
    p.n_refine = 0;
    p.prev_total_its = 0;
    p.phase = 0;
    p.nconv0 = 0;
    p.use_pred = *pred_flag;   // consumed: a later solve starts from its own viscosity again
    *pred_flag = 0;
    p.active = 1;
    KrylovScalars k;
    memset(&k, 0, sizeof(k));
    *ks = k;
  }
}

// ---- calc_ice_rheology_Glen (constitutive_equation.f90:84-163) --------------------------------
// Per vertex and layer: the uniform flow factor or the Arrhenius relation of Huybrechts (1992),
// then the enhancement factor of the vertex.  The reference evaluates it inside every Picard
// iteration; it depends only on the ice state, so one evaluation per solve gives the same field.
struct RheologyIn {
  int choice, enh;
  double A_uniform, m_sheet, m_shelf;
  const double *Ti, *Hi, *Hib, *SL, *fgr;
  const int32_t *mask_gr, *mask_fl;
};
__global__ void k_rheology(int nV, int nz, RheologyIn r, double *A_out) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t ix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ix < (int64_t)nV * nz; ix += stride) {
    const int vi = (int)(ix % nV);
    double A;
    if (r.choice == UFE_RHEOLOGY_UNIFORM) {
      A = r.A_uniform;
    } else {
      const double T = r.Ti[ix];
      // T_switch 263.15 K; a = 1.14e-5 / 5.47e10 Pa^-3 yr^-1; Q = 6.0e4 / 13.9e4 J mol^-1 (:94-98)
      A = (T < 263.15) ? 1.14E-05 * exp(-6.0E+04 / (kRGas * T)) : 5.47E+10 * exp(-13.9E+04 / (kRGas * T));
    }
    const bool gr = r.mask_gr[vi] != 0, fl = r.mask_fl && r.mask_fl[vi] != 0;
    if (r.enh == UFE_ENH_INTERP && r.Hi[vi] > 0.0 && r.Hib[vi] < r.SL[vi])
      A = A * (r.fgr[vi] * r.m_sheet + (1.0 - r.fgr[vi]) * r.m_shelf);
    else if (gr)
      A = A * r.m_sheet;
    else if (fl)
      A = A * r.m_shelf;
    A_out[ix] = A;
  }
}

// The till yield stress of Schoof's (2006) ice stream at each vertex's y coordinate
// (Schoof2006_icestream, src/UPSY/basic/analytical_solutions/Schoof_SSA_solution.f90:15-64, the
// part calc_sliding_law_idealised_SSA_icestream reads, sliding_laws.f90:469-473).
__global__ void k_icestream_yield(int nV, const double *Vy, double H, double tantheta, double L, double m,
                                  double *tys) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double f = -kIceDensity * kGrav * H * tantheta;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += stride)
    tys[v] = f * pow(fabs(Vy[v] / L), m);
}

// The triangle terms of calc_vertical_shear_strain_rates (DIVA_main.f90:375-410):
// du/dz_b = tau_bx_b zeta / max(visc_eff_min, eta_3D_b) (and v), per triangle and layer, from the
// previous iteration's basal stress and 3-D viscosity.  Formed once per triangle (the vertex
// kernel's b->a sums then read them) rather than once per vertex row entry, as tau (zeta / eta):
// one FP64 division per layer instead of two (the reference's (tau zeta) / eta rounds differently
// by an ulp or so).
__device__ __forceinline__ void diva_shear_b(int64_t t, int nTri, int nz, double2 tb, const double *eta_3D_b,
                                             const double *zeta, double visc_eff_min, double2 *duz_b) {
  for (int l = 0; l < nz; ++l) {
    const double f = zeta[l] / fmax(visc_eff_min, eta_3D_b[(int64_t)l * nTri + t]);
    duz_b[(int64_t)l * nTri + t] = make_double2(tb.x * f, tb.y * f);
  }
}
__global__ void k_diva_shear_b(int nTri, int nz, const double2 *tau_b, const double *eta_3D_b, const double *zeta,
                               double visc_eff_min, double2 *duz_b) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride)
    diva_shear_b(t, nTri, nz, tau_b[t], eta_3D_b, zeta, visc_eff_min, duz_b);
}

// ---- SSA vertex kernel ----------------------------------------------------------------------
// calc_horizontal_strain_rates (SSA_DIVA_utilities.f90:59-82), calc_effective_viscosity
// (SSA_main.f90:339-392) up to N_a, and the vertex part of calc_basal_friction_coefficient
// (sliding_laws.f90:25-81): all from one pass over the b->a operator row.
// eta_pred: the learned start's predicted viscosity, which replaces Glen's law in the first
// iteration of a solve that the prediction armed (no reference counterpart).
__global__ void k_vertex_ssa(int nV, OpRow ba, const double2 *uv, const double *Avav, const double *Hi,
                             SlidingIn sl, PhysParams q, const PicardScalars *ps, const double *eta_pred,
                             double *N_a, double *beta_a) {
  const double eps0 = ps->eps0, eta_max = ps->eta_max;
  const bool pred = ps->use_pred != 0 && ps->it == 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vi < nV; vi += stride) {
    double ux = 0, uy = 0, vx = 0, vy = 0, ua = 0, va = 0;
    for (int k = ba.ptr[vi]; k < ba.ptr[vi + 1]; ++k) {
      double2 w = uv[ba.ind[k]];
      double m = ba.v0[k], dx = ba.v1[k], dy = ba.v2[k];
      ux = ux + dx * w.x;
      uy = uy + dy * w.x;
      vx = vx + dx * w.y;
      vy = vy + dy * w.y;
      ua = ua + m * w.x;
      va = va + m * w.y;
    }
    double eta = pred ? eta_pred[vi] : glen2d(eps0, ux, uy, vx, vy, Avav[vi], q.n_glen);
    eta = fmin(fmax(eta, q.visc_eff_min), eta_max);
    N_a[vi] = eta * fmax(0.1, Hi[vi]);
    beta_a[vi] = sliding_beta(q, sl, (int)vi, ua, va);
  }
}

// ---- DIVA vertex kernel ---------------------------------------------------------------------
// calc_horizontal_strain_rates, calc_vertical_shear_strain_rates (DIVA_main.f90:375-410),
// calc_effective_viscosity (:412-479), the surface value of calc_F_integrals' F2 (:481-520) and
// the vertex part of calc_effective_basal_friction_coefficient (:522-574).
// One thread per vertex, the layers in a loop.  The FP64 pipe issues a warp instruction at the
// same cost whatever its active mask, so this pass -- bound by that pipe (the layers' powers, the
// divisions of F2 and the sliding law) -- keeps every lane busy on its own vertex; per-layer loads
// and stores of the [layer][vertex] fields stay coalesced across the warp.  du/dz and dv/dz on the
// triangles come in precomputed (duz_b, formed once per triangle).  The vertical average is summed
// on the fly in the reference's order (zeta increasing); the F2 integral runs from the base up, so
// its per-layer terms wait in shared memory, layer-major with one column per thread.
// In the first iteration of a solve the learned start armed, every layer takes the predicted
// vertically averaged viscosity eta_pred instead (a depth-uniform first viscosity).
// Dynamic shared memory: (kMaxNz + nz * blockDim.x) doubles.
__global__ void __launch_bounds__(128, 4) k_vertex_diva(int nV, int nTri, int nz, OpRow ba, const double2 *uv,
                                                        const double2 *uv_base, const double2 *duz_b,
                                                        const double *A_pow, const double *Hi, const double *zeta_g,
                                                        SlidingIn sl, PhysParams q, const PicardScalars *ps,
                                                        const double *eta_pred, double *eta_3D_a, double *N_a,
                                                        double *F2a1, double *beta_a, double *beta_eff_a) {
  extern __shared__ double vsm[];
  double *zeta = vsm, *f2 = vsm + kMaxNz + threadIdx.x;
  for (int k = threadIdx.x; k < nz; k += blockDim.x) zeta[k] = zeta_g[k];
  __syncthreads();
  const double eps0 = ps->eps0, eta_max = ps->eta_max;
  const bool pred = ps->use_pred != 0 && ps->it == 0;
  const float h_floor_sp = 0.1f;  // max(0.1, Hi) with a default-real literal (DIVA_main.f90:468)
  const int bd = blockDim.x;
  const int64_t stride = (int64_t)gridDim.x * bd;
  for (int64_t vi = (int64_t)blockIdx.x * bd + threadIdx.x; vi < nV; vi += stride) {
    const int k1 = ba.ptr[vi], k2 = ba.ptr[vi + 1];
    double ux = 0, uy = 0, vx = 0, vy = 0, ua = 0, va = 0;
    for (int k = k1; k < k2; ++k) {
      const int t = ba.ind[k];
      const double2 w = uv[t], wb = uv_base[t];
      const double m = ba.v0[k], dx = ba.v1[k], dy = ba.v2[k];
      ux = ux + dx * w.x;
      uy = uy + dy * w.x;
      vx = vx + dx * w.y;
      vy = vy + dy * w.y;
      ua = ua + m * wb.x;
      va = va + m * wb.y;
    }
    double vav = 0.0, e_prev = 0.0;
    const double e_pred = pred ? eta_pred[vi] : 0.0;
    for (int l = 0; l < nz; ++l) {
      const int64_t ix = (int64_t)l * nV + vi;
      double e = e_pred;
      if (!pred) {
        double duz = 0.0, dvz = 0.0;
        const double2 *dl = duz_b + (int64_t)l * nTri;
        for (int k = k1; k < k2; ++k) {
          const double2 d = dl[ba.ind[k]];
          const double m = ba.v0[k];
          duz = duz + m * d.x;
          dvz = dvz + m * d.y;
        }
        e = glen_apow(eps0, ux, uy, vx, vy, duz, dvz, A_pow[ix], q.n_glen);
      }
      e = fmin(fmax(e, q.visc_eff_min), eta_max);
      eta_3D_a[ix] = e;
      f2[l * bd] = zeta[l] * zeta[l] / e;
      if (l > 0) vav = vav + 0.5 * (e + e_prev) * (zeta[l] - zeta[l - 1]);
      e_prev = e;
    }
    N_a[vi] = vav * fmax((double)h_floor_sp, Hi[vi]);
    // F2 at the surface: integrate zeta^2/eta from the base (zeta = 1) up to zeta(1) = 0
    double intg = 0.0;
    for (int l = nz - 1; l >= 1; --l) intg = intg - 0.5 * (f2[l * bd] + f2[(l - 1) * bd]) * (zeta[l] - zeta[l - 1]);
    const double F2 = -fmax(0.1, Hi[vi]) * intg;
    F2a1[vi] = F2;
    const double b = sliding_beta(q, sl, (int)vi, ua, va);
    beta_a[vi] = b;
    beta_eff_a[vi] = (q.sliding_law == UFE_SLIDING_NO_SLIDING) ? 1.0 / F2 : b / (1.0 + b * F2);
  }
}

// ---- assembly -----------------------------------------------------------------------------
enum AssembleMode : int { kFromTriangles = 0, kFromSSA = 1, kFromDIVA = 2 };

struct AssembleArgs {
  int nV, nTri, nz;
  OpRow ab;
  const int32_t *m2_ptr, *m2_ind;
  const double *m2_x, *m2_y, *m2_xx, *m2_xy, *m2_yy;
  const int32_t *TriBI, *TriC;
  // inputs (by mode)
  const double *N_b, *dNx_b, *dNy_b, *beta_b_in;          // kFromTriangles
  const double *N_a, *beta_a, *beta_eff_a, *F2a1, *eta_3D_a; // kFromSSA / kFromDIVA
  const double *fgr_b;
  const double2 *tau_d;
  const int32_t *bc_mask;
  const double2 *bc_uv;
  const double2 *x0;        // Krylov initial guess (or null = zero)
  const double2 *uprev;     // velocity before this linear solve (u_b_prev, v_b_prev)
  const int32_t *cp_ptr, *cp_idx;   // 'infinite_SSA_icestream' copy triangles (null: none built)
  const double *cp_w;
  // outputs
  double4 *blk;
  float4 *blk32, *rowsum32;
  double2 *rhs, *dinv, *X, *R, *RP, *P0, *V0;
  float2 *dinv32;
  double *beta_b_out, *bfc_b, *F2b1, *eta_3D_b;
  int *err;
  // Krylov
  KrylovScalars *ks;
  const PicardScalars *ps;  // the Picard phase (null outside a Picard solve)
  double rtol, abstol, forcing;
  int max_it;
  double *partials;
  unsigned int *tickets;
};

__device__ __forceinline__ int find_col(const int32_t *ind, int k1, int k2, int col) {
  for (int k = k1; k < k2; ++k)
    if (ind[k] == col) return k;
  return -1;
}

template <int MODE>
__global__ void k_assemble(AssembleArgs a, PhysParams q, CondArg cond) {
  double acc[2] = {0.0, 0.0};
  const int nTri = a.nTri;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t64 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t64 < nTri; t64 += stride) {
    const int t = (int)t64;
    // -- coefficients of this triangle
    double N, dNx, dNy, beta;
    if (MODE == kFromTriangles) {
      N = a.N_b[t]; dNx = a.dNx_b[t]; dNy = a.dNy_b[t]; beta = a.beta_b_in[t];
    } else {
      N = 0.0; dNx = 0.0; dNy = 0.0; beta = 0.0;
      double bfc = 0.0, f2 = 0.0;
      const double *bsrc = (MODE == kFromSSA) ? a.beta_a : a.beta_eff_a;
      for (int k = a.ab.ptr[t]; k < a.ab.ptr[t + 1]; ++k) {
        int v = a.ab.ind[k];
        double m = a.ab.v0[k], na = a.N_a[v];
        N = N + m * na;
        dNx = dNx + a.ab.v1[k] * na;
        dNy = dNy + a.ab.v2[k] * na;
        beta = beta + m * bsrc[v];
        if (MODE == kFromDIVA) {
          bfc = bfc + m * a.beta_a[v];
          f2 = f2 + m * a.F2a1[v];
        }
      }
      if (q.gl_subgrid) {   // f_gr^p; the default p = 2 as a product
        const double f = a.fgr_b[t];
        beta = beta * (q.fgr_exp == 2.0 ? f * f : q.fgr_exp == 1.0 ? f : pow(f, q.fgr_exp));
      }
      if (MODE == kFromDIVA) {
        a.bfc_b[t] = bfc;
        a.F2b1[t] = f2;
        for (int l = 0; l < a.nz; ++l) {
          double e = 0.0;
          for (int k = a.ab.ptr[t]; k < a.ab.ptr[t + 1]; ++k)
            e = e + a.ab.v0[k] * a.eta_3D_a[(int64_t)l * a.nV + a.ab.ind[k]];
          a.eta_3D_b[(int64_t)l * nTri + t] = e;
        }
      }
      a.beta_b_out[t] = beta;
    }
    // -- block row on the 2nd-order b_b pattern
    const int k1 = a.m2_ptr[t], k2 = a.m2_ptr[t + 1];
    const int kd = find_col(a.m2_ind, k1, k2, t);
    if (kd < 0) { atomicOr(a.err, kErrNoDiag); continue; }
    double2 rhs;
    const int bcm = q.has_bc ? a.bc_mask[t] : 0;
    const int tbi = a.TriBI[t];
    if (bcm == 1 || tbi > 0) {
      for (int k = k1; k < k2; ++k) a.blk[k] = make_double4(0.0, 0.0, 0.0, 0.0);
      double *bd = reinterpret_cast<double *>(a.blk);
      if (bcm == 1) {
        // prescribed velocity (solve_linearised_SSA_DIVA.f90:94-109)
        bd[4 * (int64_t)kd + 0] = 1.0;
        bd[4 * (int64_t)kd + 3] = 1.0;
        rhs = a.bc_uv[t];
      } else {
        // domain border (:111-143, row routine :481-641)
        const int side = (tbi - 1) / 2;  // 0 N (1,2), 1 E (3,4), 2 S (5,6), 3 W (7,8)
        rhs = make_double2(0.0, 0.0);
        for (int uvc = 0; uvc < 2; ++uvc) {
          const int choice = uvc == 0 ? q.bc_u[side] : q.bc_v[side];
          const int comp = uvc == 0 ? 0 : 3;  // uu or vv entry of the block
          if (choice == UFE_BC_INFINITE_SSA_ICESTREAM) {
            // u = relaxed previous u at the copy point (:562-578); validated to be u only
            bd[4 * (int64_t)kd + comp] = 1.0;
            double u_fixed = 0.0;
            if (a.cp_ptr)
              for (int k = a.cp_ptr[t]; k < a.cp_ptr[t + 1]; ++k) u_fixed = u_fixed + a.cp_w[k] * a.uprev[a.cp_idx[k]].x;
            else
              atomicOr(a.err, kErrBcNeighbour);
            rhs.x = (q.relax_cfg * u_fixed) + ((1.0 - q.relax_cfg) * a.uprev[t].x);
          } else if (choice == UFE_BC_INFINITE) {
            int nnb = 0;
            for (int n = 0; n < 3; ++n) {
              int tj = a.TriC[(int64_t)n * nTri + t];
              if (tj == 0) continue;
              nnb++;
              int kk = find_col(a.m2_ind, k1, k2, tj - 1);
              if (kk < 0) { atomicOr(a.err, kErrBcNeighbour); continue; }
              bd[4 * (int64_t)kk + comp] = 1.0;
            }
            if (nnb == 0) atomicOr(a.err, kErrNoNeighbour);
            bd[4 * (int64_t)kd + comp] = -1.0 * (double)nnb;
          } else {  // UFE_BC_ZERO
            bd[4 * (int64_t)kd + comp] = 1.0;
          }
        }
      }
    } else {
      // free rows (calc_SSA_DIVA_stiffness_matrix_row_free :180-329, sans variant :331-479)
      for (int k = k1; k < k2; ++k) {
        const int tj = a.m2_ind[k];
        const double x_ = a.m2_x[k], y_ = a.m2_y[k], xx = a.m2_xx[k], xy = a.m2_xy[k], yy = a.m2_yy[k];
        double uAu, uAv, vAu, vAv;
        if (q.crossterms) {
          uAu = 4.0 * N * xx + 4.0 * dNx * x_ + N * yy + dNy * y_;
          uAv = 3.0 * N * xy + 2.0 * dNx * y_ + dNy * x_;
          vAv = 4.0 * N * yy + 4.0 * dNy * y_ + N * xx + dNx * x_;
          vAu = 3.0 * N * xy + 2.0 * dNy * x_ + dNx * y_;
          if (tj == t) { uAu = uAu - beta; vAv = vAv - beta; }
        } else {
          uAu = 4.0 * xx + yy;
          uAv = 3.0 * xy;
          vAv = 4.0 * yy + xx;
          vAu = 3.0 * xy;
          if (tj == t) { uAu = uAu - beta / N; vAv = vAv - beta / N; }
        }
        a.blk[k] = make_double4(uAu, uAv, vAu, vAv);
      }
      double2 td = a.tau_d[t];
      rhs = q.crossterms ? make_double2(-td.x, -td.y) : make_double2(-td.x / N, -td.y / N);
    }
    // -- Jacobi diagonal (PCJACOBI; a zero diagonal entry is replaced by one)
    const double4 dg = a.blk[kd];
    const double2 di = make_double2(dg.x != 0.0 ? 1.0 / dg.x : 1.0, dg.w != 0.0 ? 1.0 / dg.w : 1.0);
    a.dinv[t] = di;
    a.rhs[t] = rhs;
    if (a.blk32) {
      double4 rs = make_double4(0.0, 0.0, 0.0, 0.0);
      for (int k = k1; k < k2; ++k) {
        double4 b = a.blk[k];
        a.blk32[k] = make_float4((float)b.x, (float)b.y, (float)b.z, (float)b.w);
        rs.x += b.x; rs.y += b.y; rs.z += b.z; rs.w += b.w;
      }
      a.rowsum32[t] = make_float4((float)rs.x, (float)rs.y, (float)rs.z, (float)rs.w);
      a.dinv32[t] = make_float2((float)di.x, (float)di.y);
    }
    // -- Krylov initial residual r = D^-1 (b - A x0)
    double2 ax = make_double2(0.0, 0.0);
    double2 x0t = make_double2(0.0, 0.0);
    if (a.x0) {
      x0t = a.x0[t];
      for (int k = k1; k < k2; ++k) {
        double4 b = a.blk[k];
        double2 xj = a.x0[a.m2_ind[k]];
        ax.x += b.x * xj.x + b.y * xj.y;
        ax.y += b.z * xj.x + b.w * xj.y;
      }
    }
    a.X[t] = x0t;
    double2 r = make_double2(di.x * (rhs.x - ax.x), di.y * (rhs.y - ax.y));
    double2 db = make_double2(di.x * rhs.x, di.y * rhs.y);
    a.R[t] = r;
    a.RP[t] = r;
    a.P0[t] = make_double2(0.0, 0.0);
    a.V0[t] = make_double2(0.0, 0.0);
    acc[0] += r.x * r.x + r.y * r.y;
    acc[1] += db.x * db.x + db.y * db.y;
  }
  double tot[2];
  if (grid_sum<2>(acc, a.partials, a.tickets + kSiteInit, tot)) {
    double dp = sqrt(tot[0]);
    double bnorm = sqrt(tot[1]);
    double rnorm0 = bnorm != 0.0 ? bnorm : dp;
    KrylovScalars s = *a.ks;
    s.dp = dp;
    s.rnorm0 = rnorm0;
    // the reference's fixed tolerance (KSPSetTolerances, petsc_basic.f90:110), or for an inexact
    // Picard iteration krylov_forcing times this Picard iterate's own residual, if larger
    // the forced solves' reduction also tightens with the last Picard change norm (its square root,
    // the relative step), so forced steps near convergence are close to exact ones
    const double forcing = !a.ps ? a.forcing : (a.ps->phase != 0) ? 0.0 : fmin(a.forcing, sqrt(a.ps->L2));
    s.ttol = fmax(fmax(a.rtol * rnorm0, a.abstol), forcing * dp);
    s.it = 0;
    s.max_it = a.max_it;
    s.rho = tot[0];
    s.rhoold = 1.0;
    s.alpha = 1.0;
    s.omegaold = 1.0;
    s.omega = 1.0;
    s.beta = s.rho;
    s.status = UFE_OK;
    s.tbreak = 0;
    s.refinements = 0;
    s.pad = 0;
    s.fallback = 0;
    s.pair_rounds = 0;
    s.pair_stop = 0;
    s.active = 1;
    if (isnan(dp)) { s.status = UFE_ERR_NAN; s.active = 0; }
    else if (dp <= s.ttol) s.active = 0;
    else if (s.rho == 0.0) { s.status = UFE_ERR_DIVERGED; s.active = 0; }
    *a.ks = s;
    set_cond(cond, s.active);
  }
}

// ---- FP32 inner solve with FP64 refinement ---------------------------------------------------
// The inner BiCGStab runs entirely in FP32 (blocks, vectors, Jacobi scaling; dot products summed
// in FP64) on the correction system (D^-1 A) d = r, r the FP64 residual; the outer loop adds d to
// x and recomputes r in FP64 with the FP64 blocks until the FP64 test passes.  FP64 instructions
// are scarce on GB300, FP32 ones are not.
__global__ void k_inner_init(int nTri, const double2 *R, float2 *R32, float2 *RP32, float2 *x32,
                             float2 *P32, float2 *V32, const KrylovScalars *outer, KrylovScalars *ksi,
                             double inner_rtol, int max_it, double *partials, unsigned int *tickets,
                             CondArg cond, GridSync *gsync) {
  // reset the persistent solve's grid barrier (nothing else uses it now)
  if (gsync && blockIdx.x == 0 && threadIdx.x == 0) *gsync = GridSync{0u, 0u, 0, 0};
  double acc[1] = {0.0};
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride) {
    double2 r = R[t];
    float2 r32 = make_float2((float)r.x, (float)r.y);
    R32[t] = r32;
    RP32[t] = r32;
    x32[t] = make_float2(0.f, 0.f);
    P32[t] = make_float2(0.f, 0.f);
    V32[t] = make_float2(0.f, 0.f);
    acc[0] += (double)r32.x * r32.x + (double)r32.y * r32.y;
  }
  double tot[1];
  if (grid_sum<1>(acc, partials, tickets + kSiteInner, tot)) {
    KrylovScalars s;
    memset(&s, 0, sizeof(s));
    const KrylovScalars o = *outer;
    s.total_its = ksi->total_its;
    double dp = sqrt(tot[0]);
    s.dp = dp;
    s.rnorm0 = dp;
    // reduce the residual by inner_rtol, but never below what the outer test needs
    s.ttol = fmax(inner_rtol * dp, 0.5 * o.ttol);
    s.max_it = max_it;
    s.rho = tot[0];
    s.rhoold = s.alpha = s.omegaold = s.omega = 1.0;
    s.beta = s.rho;
    s.active = (dp > s.ttol && s.rho != 0.0 && isfinite(dp)) ? 1 : 0;
    *ksi = s;
    set_cond(cond, s.active);
  }
}

// x += d in FP64, unless the inner solve failed or its correction is not finite
__global__ void k_xadd(int nTri, double2 *X, const float2 *x32, const KrylovScalars *ksi) {
  if (ksi->status < 0) return;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride) {
    double2 x = X[t];
    float2 d = x32[t];
    if (isfinite(d.x) && isfinite(d.y)) X[t] = make_double2(x.x + (double)d.x, x.y + (double)d.y);
  }
}

// FP64 residual r = D^-1 (b - A x) and the outer (refinement) convergence test
template <int L>
__global__ void k_residual64(BsrMat<double, double, L> mat, const double2 *X, const double2 *B, const double2 *dinv,
                             double2 *R, KrylovScalars *ks, const KrylovScalars *ks32, double *partials,
                             unsigned int *tickets, CondArg cond) {
  using MT = BsrMat<double, double, L>;
  double acc[1] = {0.0};
  KRYLOV_ROWS(MT, i, lane) {
    const int i = (int)i_64;
    const bool live = i < mat.items;
    double2 part = live ? mat.row_partial(i, lane, [&](int j) { return X[j]; }) : make_double2(0.0, 0.0);
    double2 ax = lane_reduce<L>(part);
    if (live && lane == 0) {
      double2 b = B[i], d = dinv[i];
      double2 r = make_double2(d.x * (b.x - ax.x), d.y * (b.y - ax.y));
      R[i] = r;
      acc[0] += r.x * r.x + r.y * r.y;
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, partials, tickets + kSiteResid, tot)) {
    KrylovScalars s = *ks;
    const KrylovScalars in = *ks32;
    double dp = sqrt(tot[0]);
    s.dp = dp;
    s.refinements += 1;
    s.it += in.it;
    if (in.status < 0) s.pad += 1;   // a failed inner solve added nothing; count it
    if (isnan(dp)) { s.status = UFE_ERR_NAN; s.active = 0; }
    else if (dp <= s.ttol) s.active = 0;
    else if (s.pad >= 2 || s.refinements >= kMaxRefine || s.it >= s.max_it) {
      s.active = 0;
      s.fallback = 1;   // finish this linear solve with FP64 BiCGStab from the current x
    }
    *ks = s;
    set_cond(cond, s.active);
  }
}

// ---- Picard bookkeeping ---------------------------------------------------------------------
// Divergence control of SSA_main.f90:196-213 / DIVA_main.f90:211-228, convergence (:222-225),
// iteration limit (:228-232).  Runs in the last block of the finalize reduction.
__device__ void picard_step(PicardScalars *psp, KrylovScalars *ks, double r1, double r2, const PhysParams &q,
                            double n_glen, CondArg cond) {
  PicardScalars &p = *psp;
  const KrylovScalars k = *ks;
  const KrylovScalars kin = ks[1];
  p.it += 1;
  p.n_refine += k.refinements;
  const int total = kin.total_its + k.total_its;
  if (p.it <= kHistMax) {
    double *h = p.hist + (p.it - 1) * kHistCols;
    h[0] = 2.0 * r1 / fmax(r2, 1e-8);
    h[1] = (double)(total - p.prev_total_its);
    h[2] = (double)k.status;
    h[3] = k.dp;
    h[4] = (double)k.refinements;
  }
  p.prev_total_its = total;
  // A Krylov solve that did not reach its tolerance (iteration limit, divergence, breakdown)
  // leaves its last iterate, and the viscosity iteration goes on: solve_matrix_equation_PETSc
  // does not act on PETSc's converged reason (petsc_basic.f90:106-141).  NaN stops the solve.
  if (k.status == UFE_ERR_NAN) {
    p.status = k.status;
    p.active = 0;
    set_cond(cond, 0);
    return;
  }
  if (k.status != UFE_OK && p.status == UFE_OK) p.status = UFE_WARN_KRYLOV_MAXIT;
  p.L2_prev = p.L2;
  p.L2 = 2.0 * r1 / fmax(r2, 1e-8);
  if (p.L2 > p.L2_prev) p.nit_diverg += 1; else p.nit_diverg = 0;
  if (p.nit_diverg > 2) {
    p.nit_diverg = 0;
    p.relax = p.relax * 0.9;
    p.eps0 = p.eps0 * 1.2;
    p.eta_max = 0.5 * pow(1e-18, -1.0 / n_glen) * pow(p.eps0, (1.0 - n_glen) / (2.0 * n_glen));
  }
  int stop = 0;
  if (p.relax <= 0.05 || p.eps0 >= 1e-5) {
    if (p.relax < 0.05 || p.eps0 > 1e-5) { p.status = UFE_ERR_DIVERGED; stop = 1; }
  }
  if (isnan(p.L2)) { p.status = UFE_ERR_NAN; stop = 1; }
  int converged = p.L2 < q.picard_tol;
  // inexact Picard: once the change norm has met the tolerance in two forced iterations in a row
  // (one tiny step from a loosely solved system does not count), the next linear solve runs to
  // the full Krylov tolerance; the iteration stops when the change norm meets the tolerance after
  // such a solve, and otherwise goes back to forced solves (a good start makes forced steps small
  // long before the iterate has converged, so the check is repeated rather than made the rule)
  if (!stop && q.inexact) {
    if (p.phase == 0) {
      p.nconv0 = converged ? p.nconv0 + 1 : 0;
      if (converged && p.nconv0 >= 2) p.phase = 1;
      converged = 0;
    } else if (!converged) {
      p.phase = 0;
      p.nconv0 = 0;
    }
  }
  if (!stop && !converged && p.it > q.visc_it_nit) {
    if (p.status == UFE_OK) p.status = UFE_WARN_PICARD_MAXIT;
    stop = 1;
  }
  if (!stop && converged && p.it > q.visc_it_nit && p.status == UFE_OK) {
    // converged on the last allowed iteration: the reference still warns (SSA_main.f90:229)
    p.status = UFE_WARN_PICARD_MAXIT;
  }
  p.active = (!stop && !converged) ? 1 : 0;
  set_cond(cond, p.active);
}

// apply_velocity_limits + relax_viscosity_iterations + calc_L2_norm_uv (SSA_DIVA_utilities.f90:84-184)
template <bool DIVA>
__global__ void k_finalize(int nTri, const double2 *X, double2 *uv, PhysParams q, PicardScalars *ps,
                           KrylovScalars *ks, const double *beta_eff_b, const double *bfc_b, const double *F2b1,
                           double2 *uv_base, double2 *tau_b, double *partials, unsigned int *tickets,
                           CondArg cond, int nz = 0, const double *eta_3D_b = nullptr,
                           const double *zeta = nullptr, double2 *duz_b = nullptr) {
  const double r = ps->relax;
  double acc[2] = {0.0, 0.0};
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride) {
    double2 x = X[t], o = uv[t];
    double u = x.x, v = x.y;
    double uabs = sqrt(u * u + v * v);
    if (uabs > q.vel_max) { u = u * q.vel_max / uabs; v = v * q.vel_max / uabs; }
    u = (r * u) + ((1.0 - r) * o.x);
    v = (r * v) + ((1.0 - r) * o.y);
    uv[t] = make_double2(u, v);
    if (DIVA) {
      if (q.sliding_law == UFE_SLIDING_NO_SLIDING) uv_base[t] = make_double2(0.0, 0.0);
      else {
        double den = 1.0 + bfc_b[t] * F2b1[t];
        uv_base[t] = make_double2(u / den, v / den);
      }
      double be = beta_eff_b[t];
      const double2 tb = make_double2(u * be, v * be);
      tau_b[t] = tb;
      diva_shear_b(t, nTri, nz, tb, eta_3D_b, zeta, q.visc_eff_min, duz_b);   // for the next iteration
    }
    acc[0] += (u - o.x) * (u - o.x) + (v - o.y) * (v - o.y);
    acc[1] += (u + o.x) * (u + o.x) + (v + o.y) * (v + o.y);
  }
  double tot[2];
  if (grid_sum<2>(acc, partials, tickets + kSitePicard, tot)) picard_step(ps, ks, tot[0], tot[1], q, q.n_glen, cond);
}

// ---- DIVA 3-D velocities (calc_3D_velocities, DIVA_main.f90:629-676) -------------------------
__global__ void k_diva_F1(int nV, int nz, const double *eta_3D_a, const double *Hi, const double *zeta_g,
                          double *F1_3D_a) {
  __shared__ double zeta[kMaxNz];
  for (int k = threadIdx.x; k < nz; k += blockDim.x) zeta[k] = zeta_g[k];
  __syncthreads();
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t vi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vi < nV; vi += stride) {
    double h = fmax(0.1, Hi[vi]);
    double intg = 0.0;
    F1_3D_a[(int64_t)(nz - 1) * nV + vi] = -h * intg;
    for (int l = nz - 1; l >= 1; --l) {
      double f1 = zeta[l] / eta_3D_a[(int64_t)l * nV + vi];
      double f0 = zeta[l - 1] / eta_3D_a[(int64_t)(l - 1) * nV + vi];
      intg = intg - 0.5 * (f1 + f0) * (zeta[l] - zeta[l - 1]);
      F1_3D_a[(int64_t)(l - 1) * nV + vi] = -h * intg;
    }
  }
}

__global__ void k_diva_u3d(int nV, int nTri, int nz, OpRow ab, const double *F1_3D_a, const double2 *uv_base,
                           const double2 *tau_b, const double *bfc_b, int no_sliding, double *u3, double *v3) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t total = (int64_t)nTri * nz;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    int l = (int)(e / nTri), t = (int)(e - (int64_t)l * nTri);
    double f = 0.0;
    for (int k = ab.ptr[t]; k < ab.ptr[t + 1]; ++k) f = f + ab.v0[k] * F1_3D_a[(int64_t)l * nV + ab.ind[k]];
    if (no_sliding) {
      double2 tb = tau_b[t];
      u3[e] = tb.x * f;
      v3[e] = tb.y * f;
    } else {
      double2 ub = uv_base[t];
      double c = 1.0 + bfc_b[t] * f;
      u3[e] = ub.x * c;
      v3[e] = ub.y * c;
    }
  }
}

// ---- small helpers ---------------------------------------------------------------------------
// Sets *flag when any of the n values is NaN or infinite.
__global__ void k_check_finite(const double *a, int64_t n, int *flag) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) bad |= !isfinite(a[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void k_interleave(int n, const double *a, const double *b, double2 *out) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = make_double2(a ? a[i] : 0.0, b ? b[i] : 0.0);
}

__global__ void k_deinterleave(int n, const double2 *in, double *a, double *b) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double2 w = in[i];
    a[i] = w.x;
    b[i] = w.y;
  }
}

// Export of the stiffness matrix in the reference's CSR layout (rows 2(ti-1)+uv, entries in the
// order add_entry_CSR_dist appends them): first the row lengths, then the entries.
__device__ int bc_choice_dev(const PhysParams &q, int tbi, int uvc) {
  int side = (tbi - 1) / 2;
  return uvc == 0 ? q.bc_u[side] : q.bc_v[side];
}

__global__ void k_export_len(int nTri, const int32_t *m2_ptr, const int32_t *TriBI, const int32_t *TriC,
                             const int32_t *bc_mask, PhysParams q, const int32_t *perm_t, int32_t *rowlen) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nTri; t += stride) {
    int len_free = 2 * (m2_ptr[t + 1] - m2_ptr[t]);
    int bcm = q.has_bc ? bc_mask[t] : 0;
    for (int uvc = 0; uvc < 2; ++uvc) {
      int len;
      if (bcm == 1) len = 1;
      else if (TriBI[t] > 0) {
        if (bc_choice_dev(q, TriBI[t], uvc) == UFE_BC_INFINITE) {
          int nnb = 0;
          for (int n = 0; n < 3; ++n) nnb += TriC[(int64_t)n * nTri + t] != 0;
          len = nnb + 1;
        } else len = 1;
      } else len = len_free;
      rowlen[2 * perm_t[t] + uvc] = len;
    }
  }
}

__global__ void k_export_fill(int nTri, const int32_t *m2_ptr, const int32_t *m2_ind, const int32_t *TriBI,
                              const int32_t *TriC, const int32_t *bc_mask, PhysParams q, const double4 *blk,
                              const int32_t *perm_t, const int32_t *ptr, int32_t *ind, double *val) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t64 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t64 < nTri; t64 += stride) {
    const int t = (int)t64;
    const int k1 = m2_ptr[t], k2 = m2_ptr[t + 1];
    const int kd = find_col(m2_ind, k1, k2, t);
    const int bcm = q.has_bc ? bc_mask[t] : 0;
    const double *bd = reinterpret_cast<const double *>(blk);
    for (int uvc = 0; uvc < 2; ++uvc) {
      const int row = 2 * perm_t[t] + uvc;   // 0-based row 2(ti-1)+uv of the caller's triangle
      int p = ptr[row];
      const int comp = uvc == 0 ? 0 : 3;
      if (bcm == 1) {
        ind[p] = row; val[p] = 1.0;
      } else if (TriBI[t] > 0) {
        if (bc_choice_dev(q, TriBI[t], uvc) == UFE_BC_INFINITE) {
          int nnb = 0;
          for (int n = 0; n < 3; ++n) {
            int tj = TriC[(int64_t)n * nTri + t];
            if (tj == 0) continue;
            nnb++;
            ind[p] = 2 * perm_t[tj - 1] + uvc; val[p] = 1.0; ++p;
          }
          ind[p] = row; val[p] = -1.0 * (double)nnb;
        } else {
          ind[p] = row; val[p] = 1.0;
        }
      } else {
        for (int k = k1; k < k2; ++k) {
          int tj = perm_t[m2_ind[k]];
          ind[p] = 2 * tj;     val[p] = bd[4 * (int64_t)k + (uvc == 0 ? 0 : 2)]; ++p;
          ind[p] = 2 * tj + 1; val[p] = bd[4 * (int64_t)k + (uvc == 0 ? 1 : 3)]; ++p;
        }
      }
    }
    (void)kd;
  }
}

}  // namespace

// ============================================================================================
// workspace

template <class T>
static T *alloc_n(size_t n) { return (T *)dev_alloc(sizeof(T) * (n ? n : 1)); }

static void check_operators(ufe_ctx *ctx) {
  UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "no mesh uploaded");
  for (int op = UFE_OP_MAP_A_B; op <= UFE_OP_DDY_B_A; ++op)
    UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "a->b and b->a operators missing");
  for (int op = UFE_OP_M2_DDX_B_B; op <= UFE_OP_M2_D2DY2_B_B; ++op)
    UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "2nd-order b_b operators missing");
  auto same = [&](int a, int b) { return ctx->ops[a].ptr == ctx->ops[b].ptr && ctx->ops[a].ind == ctx->ops[b].ind; };
  UFE_REQUIRE(same(UFE_OP_MAP_A_B, UFE_OP_DDX_A_B) && same(UFE_OP_MAP_A_B, UFE_OP_DDY_A_B), UFE_ERR_INVALID,
              "a->b operators must share one sparsity pattern");
  UFE_REQUIRE(same(UFE_OP_MAP_B_A, UFE_OP_DDX_B_A) && same(UFE_OP_MAP_B_A, UFE_OP_DDY_B_A), UFE_ERR_INVALID,
              "b->a operators must share one sparsity pattern");
  for (int op = UFE_OP_M2_DDY_B_B; op <= UFE_OP_M2_D2DY2_B_B; ++op)
    UFE_REQUIRE(same(UFE_OP_M2_DDX_B_B, op), UFE_ERR_INVALID, "2nd-order b_b operators must share one pattern");
}

// The sliced-ELL layout of the stiffness pattern (the 2nd-order b_b operators' pattern).
// Entries a double-word copy cannot carry: beyond the FP32 range, not finite, or so small
// (below 1e-30) that the low word would leave the normal FP32 range.
__device__ __forceinline__ bool pair_unsafe(double a, bool tiny_matters) {
  const double m = fabs(a);
  return !(m <= 1e36) || (tiny_matters && m != 0.0 && m < 1e-30);
}

__global__ void k_sell_fill(int64_t nnzb, const int32_t *__restrict__ map, const double4 *__restrict__ blk,
                            const float4 *__restrict__ blk32, double4 *__restrict__ sblk, float4 *__restrict__ sblk32,
                            dwblk *__restrict__ sblkp, int *pair_bad) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnzb) return;
  const int32_t slot = map[k];
  const double4 b = blk[k];
  sblk[slot] = b;
  sblk32[slot] = blk32[k];
  if (sblkp) {
    sblkp[slot] = to_dwblk(b);
    if (pair_unsafe(b.x, true) || pair_unsafe(b.y, true) || pair_unsafe(b.z, true) || pair_unsafe(b.w, true))
      atomicOr(pair_bad, 1);
  }
}

// UFE_PREC_FP32_PAIR, around the persistent double-word BiCGStab.  One round:
//   k_pair_enter  the FP64 start (x, r, r^, D^-1; p = v = 0) in double-word form
//   k_pair_decide the double-word solve takes the linear solve ([0] -> [2], [0] inactive) unless a
//                 matrix or vector value is outside what a pair of FP32 numbers carries; then the
//                 FP64 solve keeps it (pair_stop)
//   k_pair_exit   x back to FP64, the scalars back to [0] (iterations counted in pair_its); a
//                 failed double-word solve leaves x alone and sets pair_stop
//   then the FP64 residual of the new x (k_krylov_init from x): converged means done; otherwise
//   k_pair_gate starts another round from that residual (the double-word recurrence residual
//   drifts from the true one about 2^-46 per operation), up to kPairRounds, after which the FP64
//   solve finishes from the current x.
__global__ void k_pair_enter(int n, const double2 *__restrict__ X, const double2 *__restrict__ R,
                             const double2 *__restrict__ RP, const double2 *__restrict__ dinv, dw2 *pX, dw2 *pR,
                             dw2 *pRP, dw2 *pdinv, dw2 *pP0, dw2 *pV0, const KrylovScalars *ks, int *pair_bad) {
  if (!ks->active) return;
  bool bad = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 x = X[i], r = R[i], rp = RP[i], d = dinv[i];
    bad |= pair_unsafe(x.x, false) || pair_unsafe(x.y, false) || pair_unsafe(r.x, false) ||
           pair_unsafe(r.y, false) || pair_unsafe(d.x, false) || pair_unsafe(d.y, false);
    pX[i] = to_dw2(x);
    pR[i] = to_dw2(r);
    pRP[i] = to_dw2(rp);
    pdinv[i] = to_dw2(d);
    pP0[i] = dw2{make_float4(0.f, 0.f, 0.f, 0.f)};
    pV0[i] = dw2{make_float4(0.f, 0.f, 0.f, 0.f)};
  }
  if (bad) atomicOr(pair_bad, 1);
}

constexpr int kPairRounds = 4;

__global__ void k_pair_decide(KrylovScalars *ks, int *pair_bad) {
  KrylovScalars s = ks[0];
  if (*pair_bad == 0 && s.active && !s.pair_stop) {
    s.owner = 1;
    ks[0].active = 0;
  } else {
    if (s.active) ks[0].pair_stop = 1;
    s.owner = 0;
    s.active = 0;
  }
  ks[2] = s;
  *pair_bad = 0;
}

__global__ void k_pair_exit(int n, const dw2 *__restrict__ pX, double2 *X, KrylovScalars *ks) {
  if (!ks[2].owner) return;
  const bool failed = ks[2].status < 0;
  if (!failed)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) X[i] = to_double2(pX[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    KrylovScalars s = ks[2];
    s.pair_its = ks[0].pair_its + s.it;
    s.pair_rounds = ks[0].pair_rounds + 1;
    s.pair_rounds_total = ks[0].pair_rounds_total + 1;
    s.owner = 0;
    if (failed) s.pair_stop = 1;
    ks[0] = s;
  }
}

// after the FP64 residual of a round: another round while not converged, allowed and useful
__global__ void k_pair_gate(KrylovScalars *ks, CondArg cond) {
  const KrylovScalars s = ks[0];
  set_cond(cond, s.active && !s.pair_stop && s.pair_rounds < kPairRounds);
}

void build_sell(ufe_ctx *ctx, Work *w) {
  const DevCSR &m2 = ctx->ops[UFE_OP_M2_DDX_B_B];
  const int32_t n = w->nTri;
  std::vector<int32_t> ptr(n + 1), ind(m2.nnz);
  UFE_CUDA(cudaMemcpy(ptr.data(), m2.ptr, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
  UFE_CUDA(cudaMemcpy(ind.data(), m2.ind, sizeof(int32_t) * m2.nnz, cudaMemcpyDeviceToHost));
  const int32_t nsl = (n + 31) / 32;
  std::vector<int32_t> off(nsl + 1, 0);
  for (int32_t sl = 0; sl < nsl; ++sl) {
    int32_t wmax = 0;
    for (int32_t i = sl * 32; i < std::min(n, sl * 32 + 32); ++i) wmax = std::max(wmax, ptr[i + 1] - ptr[i]);
    off[sl + 1] = off[sl] + 32 * wmax;
  }
  const int64_t nslots = off[nsl];
  std::vector<int32_t> col(nslots), map(m2.nnz);
  for (int32_t sl = 0; sl < nsl; ++sl) {
    const int32_t wsl = (off[sl + 1] - off[sl]) / 32;
    for (int32_t t = 0; t < 32; ++t) {
      const int32_t i = sl * 32 + t;
      for (int32_t k = 0; k < wsl; ++k) {
        const int64_t slot = off[sl] + (int64_t)k * 32 + t;
        const int32_t e = (i < n) ? ptr[i] + k : -1;
        if (i < n && e < ptr[i + 1]) {
          col[slot] = ind[e];
          map[e] = (int32_t)slot;
        } else {
          col[slot] = i < n ? i : 0;   // padding: zero block on the row itself
        }
      }
    }
  }
  w->nslots = nslots;
  auto up = [&](const std::vector<int32_t> &h) {
    int32_t *d = alloc_n<int32_t>(std::max<size_t>(h.size(), 1));
    UFE_CUDA(cudaMemcpy(d, h.data(), sizeof(int32_t) * h.size(), cudaMemcpyHostToDevice));
    return d;
  };
  w->sell_off = up(off);
  w->sell_col = up(col);
  w->sell_map = up(map);
  // patches for the shared-memory persistent solve: one per SM
  int dev = 0, sms = 0;
  UFE_CUDA(cudaGetDevice(&dev));
  UFE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int32_t G = std::max(1, std::min<int32_t>(std::min<int32_t>(sms, nsl), kHaloMaxBlocks));
  const int32_t rpb = ((n + G - 1) / G + 31) / 32 * 32;
  std::vector<int32_t> hoff(G + 1, 0), hidx, lcol(nslots, 0);
  int32_t maxlocal = 0;
  std::vector<int32_t> halo;
  for (int32_t b = 0; b < G; ++b) {
    const int32_t r0 = std::min(n, b * rpb), r1 = std::min(n, r0 + rpb);
    halo.clear();
    // a block without rows owns no slice (r0 = n may sit inside the last, partial slice)
    const int32_t sl0 = r0 / 32, sl1 = r1 > r0 ? (r1 + 31) / 32 : sl0;
    for (int64_t slot = off[sl0]; slot < off[sl1]; ++slot)
      if (col[slot] < r0 || col[slot] >= r1) halo.push_back(col[slot]);
    std::sort(halo.begin(), halo.end());
    halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
    const int32_t own = r1 - r0;
    for (int64_t slot = off[sl0]; slot < off[sl1]; ++slot) {
      const int32_t c = col[slot];
      lcol[slot] = (c >= r0 && c < r1) ? c - r0
                                       : own + (int32_t)(std::lower_bound(halo.begin(), halo.end(), c) - halo.begin());
    }
    hidx.insert(hidx.end(), halo.begin(), halo.end());
    hoff[b + 1] = (int32_t)hidx.size();
    maxlocal = std::max(maxlocal, own + (int32_t)halo.size());
  }
  w->halo_G = G;
  w->halo_rpb = rpb;
  w->halo_maxlocal = maxlocal;
  w->halo_off = up(hoff);
  w->halo_idx = up(hidx);
  w->halo_lcol = up(lcol);
  w->sell_blk = alloc_n<double4>(nslots);
  w->sell_blk32 = alloc_n<float4>(nslots);
  UFE_CUDA(cudaMemsetAsync(w->sell_blk, 0, sizeof(double4) * nslots, ctx->stream));
  UFE_CUDA(cudaMemsetAsync(w->sell_blk32, 0, sizeof(float4) * nslots, ctx->stream));
}

bool use_sell() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("UFE_NO_SELL");
    v = (e && *e && *e != '0') ? 0 : 1;
  }
  return v == 1;
}

Work *ensure_work(ufe_ctx *ctx) {
  check_operators(ctx);
  if (ctx->work) return ctx->work;
  Work *w = new Work();
  ctx->work = w;
  const int nV = ctx->nV, nTri = ctx->nTri, nz = ctx->nz;
  w->nV = nV; w->nTri = nTri; w->nz = nz;
  w->nnzb = ctx->ops[UFE_OP_M2_DDX_B_B].nnz;
  w->blk = alloc_n<double4>(w->nnzb);
  w->blk32 = alloc_n<float4>(w->nnzb);
  w->rowsum32 = alloc_n<float4>(nTri);
  KrylovVecs &k = w->kv;
  double2 **d2[] = {&k.X, &k.R, &k.RP, &k.S, &k.T, &k.dinv, &k.B, &k.P[0], &k.P[1], &k.V[0], &k.V[1]};
  for (auto p : d2) *p = alloc_n<double2>(nTri);
  float2 **f2[] = {&k.x32, &k.R32, &k.RP32, &k.S32, &k.T32, &k.dinv32, &k.P32[0], &k.P32[1], &k.V32[0], &k.V32[1]};
  for (auto p : f2) *p = alloc_n<float2>(nTri);
  w->uv = alloc_n<double2>(nTri);
  w->tau_d = alloc_n<double2>(nTri);
  w->fgr_b = alloc_n<double>(nTri);
  w->bc_mask = alloc_n<int32_t>(nTri);
  w->bc_uv = alloc_n<double2>(nTri);
  w->uv_base = alloc_n<double2>(nTri);
  w->tau_b = alloc_n<double2>(nTri);
  w->eta_3D_b = alloc_n<double>((size_t)nTri * nz);
  w->duz_b = alloc_n<double2>((size_t)nTri * nz);
  w->bfc_b = alloc_n<double>(nTri);
  w->F2b1 = alloc_n<double>(nTri);
  w->beta_b = alloc_n<double>(nTri);
  w->Hi = alloc_n<double>(nV);
  w->Hs = alloc_n<double>(nV);
  w->Avav = alloc_n<double>(nV);
  w->A_flow = alloc_n<double>((size_t)nV * nz);
  w->A_pow = alloc_n<double>((size_t)nV * nz);
  w->beta_sq = alloc_n<double>(nV);
  w->alpha_sq = alloc_n<double>(nV);
  w->effp = alloc_n<double>(nV);
  w->tys = alloc_n<double>(nV);
  w->mask_gr = alloc_n<int32_t>(nV);
  w->N_a = alloc_n<double>(nV);
  w->beta_a = alloc_n<double>(nV);
  w->beta_eff_a = alloc_n<double>(nV);
  w->F2a1 = alloc_n<double>(nV);
  w->eta_3D_a = alloc_n<double>((size_t)nV * nz);
  w->eta_pred_a = alloc_n<double>(nV);
  w->pred_flag = alloc_n<int32_t>(1);
  build_sell(ctx, w);
  w->ppart = alloc_n<double>((size_t)3 * kPersistMaxBlocks * kPersistSlots);
  w->gsync = alloc_n<GridSync>(1);
  w->F1_3D_a = alloc_n<double>((size_t)nV * nz);
  w->N_b_in = alloc_n<double>(nTri);
  w->dNx_b_in = alloc_n<double>(nTri);
  w->dNy_b_in = alloc_n<double>(nTri);
  w->beta_b_in = alloc_n<double>(nTri);
  w->ks = alloc_n<KrylovScalars>(3);   // [0] outer/FP64, [1] FP32 inner, [2] double-word solve
  w->ps = alloc_n<PicardScalars>(1);
  w->err = alloc_n<int>(1);
  UFE_CUDA(cudaMallocHost(&w->ks_host, sizeof(KrylovScalars) * 3));
  UFE_CUDA(cudaMallocHost(&w->ps_host, sizeof(PicardScalars)));
  cudaStream_t s = ctx->stream;
  UFE_CUDA(cudaMemsetAsync(w->uv, 0, sizeof(double2) * nTri, s));
  UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * nTri, s));
  UFE_CUDA(cudaMemsetAsync(w->tau_b, 0, sizeof(double2) * nTri, s));
  UFE_CUDA(cudaMemsetAsync(w->eta_3D_b, 0, sizeof(double) * (size_t)nTri * nz, s));
  UFE_CUDA(cudaMemsetAsync(w->ks, 0, sizeof(KrylovScalars) * 3, s));
  UFE_CUDA(cudaMemsetAsync(w->err, 0, sizeof(int), s));
  UFE_CUDA(cudaMemsetAsync(w->pred_flag, 0, sizeof(int32_t), s));
  UFE_CUDA(cudaStreamSynchronize(s));
  return w;
}

void free_work(ufe_ctx *ctx) {
  free_thermo(ctx);   // the resident heat state depends on the mesh and its operators
  free_mass(ctx);     // so do the Voronoi geometry and the thickness matrix pattern
  Work *w = ctx->work;
  if (!w) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (w->graph_ssa) cudaGraphExecDestroy(w->graph_ssa);
  if (w->graph_diva) cudaGraphExecDestroy(w->graph_diva);
  void *ptrs[] = {w->blk, w->blk32, w->rowsum32, w->kv.X, w->kv.R, w->kv.RP, w->kv.S, w->kv.T, w->kv.dinv, w->kv.B,
                  w->kv.P[0], w->kv.P[1], w->kv.V[0], w->kv.V[1], w->kv.x32, w->kv.R32, w->kv.RP32,
                  w->kv.S32, w->kv.T32, w->kv.dinv32, w->kv.P32[0], w->kv.P32[1], w->kv.V32[0],
                  w->kv.V32[1], w->uv, w->tau_d, w->fgr_b, w->bc_mask, w->bc_uv, w->uv_base, w->tau_b,
                  w->eta_3D_b, w->bfc_b, w->F2b1, w->beta_b, w->Hi, w->Hs, w->Avav, w->A_flow, w->beta_sq, w->A_pow,
                  w->alpha_sq, w->effp, w->tys, w->mask_gr, w->N_a, w->beta_a, w->beta_eff_a, w->F2a1,
                  w->eta_3D_a, w->F1_3D_a, w->N_b_in, w->dNx_b_in, w->dNy_b_in, w->beta_b_in, w->ks,
                  w->ps, w->err, w->ppart, w->gsync, w->sell_off, w->sell_col, w->sell_map, w->sell_blk,
                  w->sell_blk32, w->halo_off, w->halo_idx, w->halo_lcol, w->pX, w->pR, w->pRP, w->pS, w->pT,
                  w->pdinv, w->pP[0], w->pP[1], w->pV[0], w->pV[1], w->sell_blkp, w->pair_bad,
                  w->Ti, w->mask_fl, w->fgr_v, w->Hib, w->SL, w->A_rheo, w->tys_ideal, w->cp_ptr, w->cp_idx,
                  w->cp_w, w->duz_b, w->eta_pred_a, w->pred_flag};
  for (void *p : ptrs) dev_free(p);
  if (w->ks_host) cudaFreeHost(w->ks_host);
  if (w->ps_host) cudaFreeHost(w->ps_host);
  delete w;
  ctx->work = nullptr;
}

int32_t bsr_lanes(ufe_ctx *ctx) {
  if (ctx && ctx->lanes > 0) return ctx->lanes;   // chosen by ufe_autotune for this mesh
  static int lanes = -1;
  if (lanes < 0) {
    const char *e = getenv("UFE_BSR_LANES");
    int v = e ? atoi(e) : 1;
    lanes = (v == 1 || v == 2 || v == 4 || v == 8) ? v : 1;
  }
  return lanes;
}

// gfortran's NORM2 of a 2-vector: the scaled sum of squares with a running scale
static double host_norm2(double a, double b) {
  const double xs[2] = {a, b};
  double scale = 1.0, result = 0.0;
  for (double x : xs) {
    if (x == 0.0) continue;
    const double ax = fabs(x);
    if (scale < ax) {
      const double r = scale / ax;
      result = 1.0 + result * r * r;
      scale = ax;
    } else {
      const double r = ax / scale;
      result += r * r;
    }
  }
  return sqrt(result) * scale;
}

static bool icestream_bc(const ufe_solver_params &p) {
  return p.BC_u_west == UFE_BC_INFINITE_SSA_ICESTREAM || p.BC_u_east == UFE_BC_INFINITE_SSA_ICESTREAM ||
         p.BC_u_south == UFE_BC_INFINITE_SSA_ICESTREAM || p.BC_u_north == UFE_BC_INFINITE_SSA_ICESTREAM;
}

// Copy triangles and weights of every border triangle for the 'infinite_SSA_icestream' rows
// (find_ti_copy_SSA_icestream_infinite, src/UPSY/mesh/mesh_utilities.f90:2681-2729): the point
// at the triangle's y, one third (x < 0) or two thirds (x >= 0) across the domain; the vertex
// whose Voronoi cell holds it (the nearest vertex; find_containing_vertex's walk, :1368-1416,
// ends there on a Delaunay mesh); that vertex's triangles weighted by 1/distance^2, normalised.
// Host computation on the internal numbering, once per mesh.
void build_icestream_copy(ufe_ctx *ctx, Work *w) {
  const int64_t nV = ctx->nV, nTri = ctx->nTri, nCm = ctx->nC_mem;
  cudaStream_t s = ctx->stream;
  std::vector<double> V(2 * nV), GC(2 * nTri);
  std::vector<int32_t> niTri(nV), iTri(nV * nCm), TriBI(nTri);
  UFE_CUDA(cudaMemcpyAsync(V.data(), ctx->V, sizeof(double) * 2 * nV, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaMemcpyAsync(GC.data(), ctx->TriGC, sizeof(double) * 2 * nTri, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaMemcpyAsync(niTri.data(), ctx->niTri, sizeof(int32_t) * nV, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaMemcpyAsync(iTri.data(), ctx->iTri, sizeof(int32_t) * nV * nCm, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaMemcpyAsync(TriBI.data(), ctx->TriBI, sizeof(int32_t) * nTri, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  double xmin = V[0], xmax = V[0];
  for (int64_t v = 1; v < nV; ++v) { xmin = std::min(xmin, V[v]); xmax = std::max(xmax, V[v]); }
  std::vector<int32_t> ptr(nTri + 1, 0), idx;
  std::vector<double> wts;
  for (int64_t t = 0; t < nTri; ++t) {
    if (TriBI[t] > 0) {
      const double py = GC[nTri + t];
      const double px = GC[t] < 0.0 ? xmin + (xmax - xmin) * 1.0 / 3.0 : xmin + (xmax - xmin) * 2.0 / 3.0;
      int64_t vi = 0;
      double best = 0.0;
      for (int64_t v = 0; v < nV; ++v) {
        const double dx = V[v] - px, dy = V[nV + v] - py, d = dx * dx + dy * dy;
        if (v == 0 || d < best) { best = d; vi = v; }
      }
      const size_t k0 = wts.size();
      double sum = 0.0;
      for (int c = 0; c < niTri[vi]; ++c) {
        const int32_t tj = iTri[c * nV + vi] - 1;
        const double dist = host_norm2(px - GC[tj], py - GC[nTri + tj]);
        idx.push_back(tj);
        wts.push_back(1.0 / (dist * dist));
      }
      for (size_t k = k0; k < wts.size(); ++k) sum = sum + wts[k];
      for (size_t k = k0; k < wts.size(); ++k) wts[k] = wts[k] / sum;
    }
    ptr[t + 1] = (int32_t)idx.size();
  }
  w->cp_ptr = alloc_n<int32_t>(nTri + 1);
  w->cp_idx = alloc_n<int32_t>(idx.size());
  w->cp_w = alloc_n<double>(wts.size());
  UFE_CUDA(cudaMemcpyAsync(w->cp_ptr, ptr.data(), sizeof(int32_t) * (nTri + 1), cudaMemcpyHostToDevice, s));
  if (!idx.empty()) {
    UFE_CUDA(cudaMemcpyAsync(w->cp_idx, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaMemcpyAsync(w->cp_w, wts.data(), sizeof(double) * wts.size(), cudaMemcpyHostToDevice, s));
  }
  UFE_CUDA(cudaStreamSynchronize(s));
}

// ============================================================================================
// enqueue helpers

namespace {

__global__ void k_reset_gsync(GridSync *g) {
  g->count = 0u;
  g->gen = 0u;
  g->err = 0;
}

// The FP32 inner BiCGStab runs as one persistent launch unless UFE_NO_PERSIST=1.
bool persistent_krylov() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("UFE_NO_PERSIST");
    v = (e && *e && *e != '0') ? 0 : 1;
  }
  return v == 1;
}

// Blocks of kPersistThreads for a persistent kernel: all co-resident, at most kPersistMaxBlocks,
// no more than the rows need.
unsigned persist_blocks(const void *kernel, int64_t lanes_total) {
  int dev = 0, sms = 0, per_sm = 0;
  UFE_CUDA(cudaGetDevice(&dev));
  UFE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  UFE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistThreads, 0));
  int64_t nb = (int64_t)std::max(per_sm, 1) * sms;
  nb = std::min<int64_t>(nb, kPersistMaxBlocks);
  nb = std::min<int64_t>(nb, (lanes_total + kPersistThreads - 1) / kPersistThreads);
  return (unsigned)std::max<int64_t>(nb, 1);
}

struct Solver {
  ufe_ctx *ctx;
  Work *w;
  ufe_solver_params p;
  PhysParams q;
  int grid, lanes;
  unsigned persist_grid = 1;   // co-resident blocks of the persistent Krylov kernel
  OpRow ab, ba;
  cudaStream_t s;

  Solver(ufe_ctx *c, const ufe_solver_params &pp) : ctx(c), p(pp) {
    w = ensure_work(ctx);
    q = make_phys(p, w->has_bc);
    grid = max_grid(ctx);
    lanes = bsr_lanes(ctx);
    s = ctx->stream;
    switch (lanes) {
      case 1: persist_grid = persist_blocks(reinterpret_cast<const void *>(k_bicgstab_persist<BsrDiffMat<1>>), 1ll << 40); break;
      case 2: persist_grid = persist_blocks(reinterpret_cast<const void *>(k_bicgstab_persist<BsrDiffMat<2>>), 1ll << 40); break;
      case 8: persist_grid = persist_blocks(reinterpret_cast<const void *>(k_bicgstab_persist<BsrDiffMat<8>>), 1ll << 40); break;
      default: persist_grid = persist_blocks(reinterpret_cast<const void *>(k_bicgstab_persist<BsrDiffMat<4>>), 1ll << 40); break;
    }
    const DevCSR &mab = ctx->ops[UFE_OP_MAP_A_B];
    ab = OpRow{mab.ptr, mab.ind, mab.val, ctx->ops[UFE_OP_DDX_A_B].val, ctx->ops[UFE_OP_DDY_A_B].val};
    const DevCSR &mba = ctx->ops[UFE_OP_MAP_B_A];
    ba = OpRow{mba.ptr, mba.ind, mba.val, ctx->ops[UFE_OP_DDX_B_A].val, ctx->ops[UFE_OP_DDY_B_A].val};
    if (pair_ok()) ensure_pair();
    if (icestream_bc(p) && !w->cp_ptr) build_icestream_copy(ctx, w);
  }

  int eblocks(int64_t n) const { return pick_blocks(n, kThreads, grid); }
  // blocks of 256 threads for one G-lane group per vertex

  SlidingIn sliding() const {
    const double *tys = p.choice_sliding_law == UFE_SLIDING_IDEALISED_SSA_ICESTREAM ? w->tys_ideal : w->tys;
    return SlidingIn{w->beta_sq, w->alpha_sq, w->effp, tys};
  }
  // the flow factor the solve reads: the caller's A_flow, or calc_ice_rheology_Glen's
  const double *A_src() const {
    return p.choice_ice_rheology_Glen == UFE_RHEOLOGY_INPUT ? w->A_flow : w->A_rheo;
  }
  // Inputs a resident solve needs beyond the uploaded ice state, checked and allocated before
  // any graph is captured.
  void setup_solve_inputs() {
    const size_t nV = w->nV, nz = w->nz;
    if (p.choice_ice_rheology_Glen == UFE_RHEOLOGY_INPUT) {
      UFE_REQUIRE(w->has_A, UFE_ERR_INVALID, "A_flow missing (choice_ice_rheology_Glen is 'input')");
    } else {
      UFE_REQUIRE(p.choice_ice_rheology_Glen != UFE_RHEOLOGY_HUYBRECHTS1992 || w->has_Ti, UFE_ERR_INVALID,
                  "Huybrechts1992 rheology needs the ice temperature Ti");
      UFE_REQUIRE(p.choice_enhancement_factor_transition != UFE_ENH_INTERP ||
                      (w->has_fgr_v && w->has_Hib && w->has_SL),
                  UFE_ERR_INVALID, "'interp' enhancement factors need fraction_gr, Hib and SL");
      if (!w->A_rheo) w->A_rheo = alloc_n<double>(nV * nz);
    }
    if (p.choice_sliding_law == UFE_SLIDING_IDEALISED_SSA_ICESTREAM && !w->tys_ideal)
      w->tys_ideal = alloc_n<double>(nV);
  }

  AssembleArgs assemble_args(const double2 *x0, int mode) const {
    AssembleArgs a;
    memset(&a, 0, sizeof(a));
    a.nV = w->nV; a.nTri = w->nTri; a.nz = w->nz;
    a.ab = ab;
    const DevCSR &m2 = ctx->ops[UFE_OP_M2_DDX_B_B];
    a.m2_ptr = m2.ptr; a.m2_ind = m2.ind;
    a.m2_x = m2.val; a.m2_y = ctx->ops[UFE_OP_M2_DDY_B_B].val;
    a.m2_xx = ctx->ops[UFE_OP_M2_D2DX2_B_B].val; a.m2_xy = ctx->ops[UFE_OP_M2_D2DXDY_B_B].val;
    a.m2_yy = ctx->ops[UFE_OP_M2_D2DY2_B_B].val;
    a.TriBI = ctx->TriBI; a.TriC = ctx->TriC;
    a.N_b = w->N_b_in; a.dNx_b = w->dNx_b_in; a.dNy_b = w->dNy_b_in; a.beta_b_in = w->beta_b_in;
    a.N_a = w->N_a; a.beta_a = w->beta_a; a.beta_eff_a = w->beta_eff_a; a.F2a1 = w->F2a1; a.eta_3D_a = w->eta_3D_a;
    a.fgr_b = w->fgr_b; a.tau_d = w->tau_d; a.bc_mask = w->bc_mask; a.bc_uv = w->bc_uv;
    a.x0 = x0;
    a.uprev = w->uv;
    a.cp_ptr = w->cp_ptr; a.cp_idx = w->cp_idx; a.cp_w = w->cp_w;
    a.blk = w->blk;
    a.blk32 = (p.precision == UFE_PREC_FP32_REFINE) ? w->blk32 : nullptr;
    a.rowsum32 = w->rowsum32;
    a.rhs = w->kv.B; a.dinv = w->kv.dinv; a.X = w->kv.X; a.R = w->kv.R; a.RP = w->kv.RP;
    a.P0 = w->kv.P[0]; a.V0 = w->kv.V[0]; a.dinv32 = w->kv.dinv32;
    a.beta_b_out = w->beta_b; a.bfc_b = w->bfc_b; a.F2b1 = w->F2b1; a.eta_3D_b = w->eta_3D_b;
    a.err = w->err;
    a.ks = w->ks;
    a.rtol = p.stress_balance_PETSc_rtol;
    a.abstol = p.stress_balance_PETSc_abstol;
    a.forcing = p.krylov_forcing;
    a.ps = (mode == kFromTriangles) ? nullptr : w->ps;
    a.max_it = p.krylov_max_it;
    a.partials = ctx->red.partials;
    a.tickets = ctx->red.tickets;
    return a;
  }

  void enqueue_assemble(int mode, bool x0_current, CondArg c) {
    AssembleArgs a = assemble_args(x0_current ? w->uv : nullptr, mode);
    int g = eblocks(w->nTri);
    if (mode == kFromTriangles) k_assemble<kFromTriangles><<<g, kThreads, 0, s>>>(a, q, c);
    else if (mode == kFromSSA) k_assemble<kFromSSA><<<g, kThreads, 0, s>>>(a, q, c);
    else k_assemble<kFromDIVA><<<g, kThreads, 0, s>>>(a, q, c);
    UFE_CUDA(cudaGetLastError());
    if (use_sell()) {
      k_sell_fill<<<(unsigned)((w->nnzb + 255) / 256), 256, 0, s>>>(
          w->nnzb, w->sell_map, w->blk, w->blk32, w->sell_blk, w->sell_blk32, pair_ok() ? w->sell_blkp : nullptr,
          w->pair_bad);
      UFE_CUDA(cudaGetLastError());
    }
  }

  template <class M>
  void enqueue_krylov_iter(const M &mat, KV<typename M::Vec> v, KrylovScalars *ks, CondArg c) {
    unsigned g = krylov_grid(mat, kThreads, grid);
    k_p_spmv<M><<<g, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets);
    k_s_spmv<M><<<g, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets);
    unsigned g2 = pick_blocks(mat.items, kThreads, grid);
    k_xr<M><<<g2, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, c);
    UFE_CUDA(cudaGetLastError());
  }

  template <int L>
  BsrMat<double, double, L> mat64() const {
    const DevCSR &m2 = ctx->ops[UFE_OP_M2_DDX_B_B];
    BsrMat<double, double, L> m{w->nTri, m2.ptr, m2.ind, w->blk};
    if (L == 1 && use_sell()) {
      m.soff = w->sell_off;
      m.scol = w->sell_col;
      m.sblk = w->sell_blk;
    }
    return m;
  }
  template <int L>
  BsrDiffMat<L> mat32() const {
    const DevCSR &m2 = ctx->ops[UFE_OP_M2_DDX_B_B];
    BsrDiffMat<L> m{w->nTri, m2.ptr, m2.ind, w->blk32, w->rowsum32};
    if (L == 1 && use_sell()) {
      m.soff = w->sell_off;
      m.scol = w->sell_col;
      m.sblk = w->sell_blk32;
    }
    return m;
  }
  KV<double2> kv64() const {
    KV<double2> v;
    v.X = w->kv.X; v.R = w->kv.R; v.RP = w->kv.RP; v.S = w->kv.S; v.T = w->kv.T; v.B = w->kv.B;
    v.dinv = w->kv.dinv;
    v.P[0] = w->kv.P[0]; v.P[1] = w->kv.P[1]; v.V[0] = w->kv.V[0]; v.V[1] = w->kv.V[1];
    return v;
  }
  KV<float2> kv_inner() const {
    KV<float2> v;
    v.X = w->kv.x32; v.R = w->kv.R32; v.RP = w->kv.RP32; v.S = w->kv.S32; v.T = w->kv.T32; v.B = nullptr;
    v.dinv = w->kv.dinv32;
    v.P[0] = w->kv.P32[0]; v.P[1] = w->kv.P32[1]; v.V[0] = w->kv.V32[0]; v.V[1] = w->kv.V32[1];
    return v;
  }
  void krylov_iter64(CondArg c) {
    switch (lanes) {
      case 1: enqueue_krylov_iter(mat64<1>(), kv64(), w->ks, c); break;
      case 2: enqueue_krylov_iter(mat64<2>(), kv64(), w->ks, c); break;
      case 8: enqueue_krylov_iter(mat64<8>(), kv64(), w->ks, c); break;
      default: enqueue_krylov_iter(mat64<4>(), kv64(), w->ks, c); break;
    }
  }
  void krylov_iter32(CondArg c) {
    switch (lanes) {
      case 1: enqueue_krylov_iter(mat32<1>(), kv_inner(), w->ks + 1, c); break;
      case 2: enqueue_krylov_iter(mat32<2>(), kv_inner(), w->ks + 1, c); break;
      case 8: enqueue_krylov_iter(mat32<8>(), kv_inner(), w->ks + 1, c); break;
      default: enqueue_krylov_iter(mat32<4>(), kv_inner(), w->ks + 1, c); break;
    }
  }
  void enqueue_inner_init(CondArg c) {
    k_inner_init<<<eblocks(w->nTri), kThreads, 0, s>>>(
        w->nTri, w->kv.R, w->kv.R32, w->kv.RP32, w->kv.x32, w->kv.P32[0], w->kv.V32[0], w->ks, w->ks + 1,
        p.krylov_inner_rtol, p.krylov_max_it, ctx->red.partials, ctx->red.tickets, c, w->gsync);
    UFE_CUDA(cudaGetLastError());
  }
  // the FP32 inner BiCGStab as one persistent launch (replaces the while(in32) loop)
  // shared-memory patches fit: one 1024-thread block per SM, the table in shared memory
  bool halo_ok() const {
    return use_sell() && lanes == 1 && w->halo_G > 0 &&
           (size_t)w->halo_maxlocal * sizeof(float2) <= 160 * 1024 && !getenv("UFE_NO_HALO");
  }
  void inner_halo() {
    const size_t smem = (size_t)w->halo_maxlocal * sizeof(float2);
    static size_t attr = 0;
    if (smem > attr) {
      UFE_CUDA(cudaFuncSetAttribute(k_bicgstab_halo<float2, float4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
      attr = smem;
    }
    HaloDiffMat m{w->nTri, w->halo_rpb, w->sell_off, w->halo_lcol, w->sell_blk32, w->rowsum32, w->halo_off,
                  w->halo_idx};
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    UFE_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      k_bicgstab_halo<float2, float4><<<w->halo_G, kPersistThreads, smem, s>>>(m, kv_inner(), w->ks + 1, w->ppart,
                                                                              w->gsync);
      UFE_CUDA(cudaGetLastError());
      return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w->halo_G);
    cfg.blockDim = dim3(kPersistThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr1[1];
    attr1[0].id = cudaLaunchAttributeCooperative;
    attr1[0].val.cooperative = 1;
    cfg.attrs = attr1;
    cfg.numAttrs = 1;
    UFE_CUDA(cudaLaunchKernelEx(&cfg, k_bicgstab_halo<float2, float4>, m, kv_inner(), w->ks + 1, w->ppart, w->gsync));
  }
  // the FP64 solve as one persistent launch with shared-memory patches (the plain FP64 path)
  bool halo64_ok() const {
    return persistent_krylov() && ctx->allow_persistent && use_sell() && lanes == 1 && w->halo_G > 0 &&
           (size_t)w->halo_maxlocal * sizeof(double2) <= 160 * 1024 && !getenv("UFE_NO_HALO");
  }
  void enqueue_outer_halo64() {
    const size_t smem = (size_t)w->halo_maxlocal * sizeof(double2);
    static size_t attr = 0;
    if (smem > attr) {
      UFE_CUDA(cudaFuncSetAttribute(k_bicgstab_halo<double2, double4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
      attr = smem;
    }
    HaloMat<double4> m{w->nTri, w->halo_rpb, w->sell_off, w->halo_lcol, w->sell_blk, nullptr, w->halo_off,
                       w->halo_idx};
    k_reset_gsync<<<1, 1, 0, s>>>(w->gsync);
    UFE_CUDA(cudaGetLastError());
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    UFE_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      k_bicgstab_halo<double2, double4><<<w->halo_G, kPersistThreads, smem, s>>>(m, kv64(), w->ks, w->ppart,
                                                                                 w->gsync);
      UFE_CUDA(cudaGetLastError());
      return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w->halo_G);
    cfg.blockDim = dim3(kPersistThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    UFE_CUDA(cudaLaunchKernelEx(&cfg, k_bicgstab_halo<double2, double4>, m, kv64(), w->ks, w->ppart, w->gsync));
  }
  // UFE_PREC_FP32_PAIR: the linear solve in double-word arithmetic, one persistent launch with the
  // FP64 solve's shared-memory patches; the FP64 persistent solve runs after it and does the work
  // only when the double-word solve declined (k_pair_decide)
  bool pair_ok() const { return p.precision == UFE_PREC_FP32_PAIR && halo64_ok(); }
  void ensure_pair() {
    if (w->sell_blkp) return;
    const int n = w->nTri;
    dw2 **v[] = {&w->pX, &w->pR, &w->pRP, &w->pS, &w->pT, &w->pdinv, &w->pP[0], &w->pP[1], &w->pV[0], &w->pV[1]};
    for (auto q : v) *q = static_cast<dw2 *>(dev_alloc(sizeof(dw2) * (size_t)(n ? n : 1)));
    w->sell_blkp = static_cast<dwblk *>(dev_alloc(sizeof(dwblk) * (size_t)(w->nslots ? w->nslots : 1)));
    w->pair_bad = static_cast<int *>(dev_alloc(sizeof(int)));
    UFE_CUDA(cudaMemsetAsync(w->sell_blkp, 0, sizeof(dwblk) * (size_t)(w->nslots ? w->nslots : 1), s));
    UFE_CUDA(cudaMemsetAsync(w->pair_bad, 0, sizeof(int), s));
  }
  KV<dw2> kvpair() const {
    KV<dw2> v;
    v.X = w->pX; v.R = w->pR; v.RP = w->pRP; v.S = w->pS; v.T = w->pT; v.B = nullptr;
    v.dinv = w->pdinv;
    v.P[0] = w->pP[0]; v.P[1] = w->pP[1]; v.V[0] = w->pV[0]; v.V[1] = w->pV[1];
    return v;
  }
  // one double-word solve from the FP64 state in ks[0] (conversions in and out)
  void pair_solve_once() {
    const int g = eblocks(w->nTri);
    k_pair_enter<<<g, kThreads, 0, s>>>(w->nTri, w->kv.X, w->kv.R, w->kv.RP, w->kv.dinv, w->pX, w->pR, w->pRP,
                                        w->pdinv, w->pP[0], w->pV[0], w->ks, w->pair_bad);
    k_pair_decide<<<1, 1, 0, s>>>(w->ks, w->pair_bad);
    UFE_CUDA(cudaGetLastError());
    const size_t smem = (size_t)w->halo_maxlocal * sizeof(dw2);
    static size_t attr = 0;
    if (smem > attr) {
      UFE_CUDA(cudaFuncSetAttribute(k_bicgstab_halo<dw2, dwblk>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
      attr = smem;
    }
    HaloMat<dwblk> m{w->nTri, w->halo_rpb, w->sell_off, w->halo_lcol, w->sell_blkp, nullptr, w->halo_off,
                     w->halo_idx};
    k_reset_gsync<<<1, 1, 0, s>>>(w->gsync);
    UFE_CUDA(cudaGetLastError());
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    UFE_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      k_bicgstab_halo<dw2, dwblk><<<w->halo_G, kPersistThreads, smem, s>>>(m, kvpair(), w->ks + 2, w->ppart, w->gsync);
      UFE_CUDA(cudaGetLastError());
    } else {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(w->halo_G);
      cfg.blockDim = dim3(kPersistThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      UFE_CUDA(cudaLaunchKernelEx(&cfg, k_bicgstab_halo<dw2, dwblk>, m, kvpair(), w->ks + 2, w->ppart, w->gsync));
    }
    k_pair_exit<<<g, kThreads, 0, s>>>(w->nTri, w->pX, w->kv.X, w->ks);
    UFE_CUDA(cudaGetLastError());
  }
  // a round: the double-word solve, the FP64 residual of its x, and the decision on another round
  void pair_round(CondArg c) {
    pair_solve_once();
    BsrMat<double, double, 1> m = mat64<1>();
    CondArg none{0, 0};
    k_krylov_init<BsrMat<double, double, 1>><<<krylov_grid(m, kThreads, grid), kThreads, 0, s>>>(
        m, kv64(), w->ks, p.stress_balance_PETSc_rtol, p.stress_balance_PETSc_abstol, p.krylov_max_it, 0,
        ctx->red.partials, ctx->red.tickets, none, 0, 1);
    k_pair_gate<<<1, 1, 0, s>>>(w->ks, c);
    UFE_CUDA(cudaGetLastError());
  }
  // the linear solve of UFE_PREC_FP32_PAIR with host-side loop control (graphs off, the
  // linearised-solve entry point): rounds while the FP64 residual asks for them, then the FP64
  // solve, which does the work only when the rounds ended unconverged
  void run_pair_host() {
    for (int r = 0; r < kPairRounds; ++r) {
      UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      if (!w->ks_host[0].active || w->ks_host[0].pair_stop) break;
      pair_round(CondArg{0, 0});
    }
    enqueue_outer_halo64();
  }
  template <int L>
  void inner_persist_l() {
    using MT = BsrDiffMat<L>;
    const MT m = mat32<L>();
    auto kern = k_bicgstab_persist<MT>;
    // grid: all blocks co-resident (computed before any capture begins, see Solver())
    const unsigned nb =
        std::max(1u, std::min(persist_grid, (unsigned)(((int64_t)m.items * L + kPersistThreads - 1) / kPersistThreads)));
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    UFE_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      // graph body: plain launch (the solve's kernels run one after another, so the grid is resident)
      kern<<<nb, kPersistThreads, 0, s>>>(m, kv_inner(), w->ks + 1, w->ppart, w->gsync);
      UFE_CUDA(cudaGetLastError());
      return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(kPersistThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UFE_CUDA(cudaLaunchKernelEx(&cfg, kern, m, kv_inner(), w->ks + 1, w->ppart, w->gsync));
  }
  void enqueue_inner_persist() {
    if (halo_ok()) {
      inner_halo();
      return;
    }
    switch (lanes) {
      case 1: inner_persist_l<1>(); break;
      case 2: inner_persist_l<2>(); break;
      case 8: inner_persist_l<8>(); break;
      default: inner_persist_l<4>(); break;
    }
  }
  template <int L>
  void residual64_l(CondArg c) {
    BsrMat<double, double, L> m = mat64<L>();
    k_residual64<L><<<krylov_grid(m, kThreads, grid), kThreads, 0, s>>>(
        m, w->kv.X, w->kv.B, w->kv.dinv, w->kv.R, w->ks, w->ks + 1, ctx->red.partials, ctx->red.tickets, c);
  }
  void enqueue_refine_update(CondArg c) {
    k_xadd<<<eblocks(w->nTri), kThreads, 0, s>>>(w->nTri, w->kv.X, w->kv.x32, w->ks + 1);
    switch (lanes) {
      case 1: residual64_l<1>(c); break;
      case 2: residual64_l<2>(c); break;
      case 8: residual64_l<8>(c); break;
      default: residual64_l<4>(c); break;
    }
    UFE_CUDA(cudaGetLastError());
  }

  template <int L>
  void fallback_init_l(CondArg c) {
    BsrMat<double, double, L> m = mat64<L>();
    k_krylov_init<BsrMat<double, double, L>><<<krylov_grid(m, kThreads, grid), kThreads, 0, s>>>(
        m, kv64(), w->ks, p.stress_balance_PETSc_rtol, p.stress_balance_PETSc_abstol, p.krylov_max_it, 0,
        ctx->red.partials, ctx->red.tickets, c, 1);
  }
  void enqueue_fallback_init(CondArg c) {
    switch (lanes) {
      case 1: fallback_init_l<1>(c); break;
      case 2: fallback_init_l<2>(c); break;
      case 8: fallback_init_l<8>(c); break;
      default: fallback_init_l<4>(c); break;
    }
    UFE_CUDA(cudaGetLastError());
  }

  void enqueue_prologue(bool diva) {
    if (p.choice_ice_rheology_Glen != UFE_RHEOLOGY_INPUT) {
      RheologyIn r{p.choice_ice_rheology_Glen, p.choice_enhancement_factor_transition, p.uniform_Glens_flow_factor,
                   p.m_enh_sheet, p.m_enh_shelf, w->Ti, w->Hi, w->Hib, w->SL, w->fgr_v, w->mask_gr,
                   w->has_mask_fl ? w->mask_fl : nullptr};
      k_rheology<<<eblocks((int64_t)w->nV * w->nz), kThreads, 0, s>>>(w->nV, w->nz, r, w->A_rheo);
    }
    if (p.choice_sliding_law == UFE_SLIDING_IDEALISED_SSA_ICESTREAM)
      k_icestream_yield<<<eblocks(w->nV), kThreads, 0, s>>>(w->nV, ctx->V + w->nV, p.SSA_icestream_Hi,
                                                           p.SSA_icestream_dhdx, p.SSA_icestream_L, p.SSA_icestream_m,
                                                           w->tys_ideal);
    k_prologue<<<eblocks(std::max(w->nV, w->nTri)), kThreads, 0, s>>>(
        w->nV, w->nTri, w->nz, ab, w->Hi, w->Hs, A_src(), ctx->zeta, w->tau_d, diva ? nullptr : w->Avav,
        diva ? w->A_pow : nullptr, w->ps, w->ks, p.visc_it_relax, p.Glens_flow_law_epsilon_sq_0,
        p.Glens_flow_law_exponent, w->pred_flag);
    if (diva)
      k_diva_shear_b<<<eblocks(w->nTri), kThreads, 0, s>>>(w->nTri, w->nz, w->tau_b, w->eta_3D_b, ctx->zeta,
                                                           p.visc_eff_min, w->duz_b);
    UFE_CUDA(cudaMemsetAsync(w->ks + 1, 0, sizeof(KrylovScalars), s));
    UFE_CUDA(cudaGetLastError());
  }

  void enqueue_picard_pre(bool diva, CondArg inner) {
    if (diva) {
      const int tpb = w->nz <= 40 ? 128 : 64;
      const size_t smem = (size_t)(kMaxNz + w->nz * tpb) * sizeof(double);
      k_vertex_diva<<<pick_blocks(w->nV, tpb, 1 << 20), tpb, smem, s>>>(
          w->nV, w->nTri, w->nz, ba, w->uv, w->uv_base, w->duz_b, w->A_pow, w->Hi, ctx->zeta,
          sliding(), q, w->ps, w->eta_pred_a, w->eta_3D_a, w->N_a, w->F2a1, w->beta_a, w->beta_eff_a);
    } else {
      k_vertex_ssa<<<eblocks(w->nV), kThreads, 0, s>>>(w->nV, ba, w->uv, w->Avav, w->Hi, sliding(), q, w->ps,
                                                       w->eta_pred_a, w->N_a, w->beta_a);
    }
    UFE_CUDA(cudaGetLastError());
    enqueue_assemble(diva ? kFromDIVA : kFromSSA, p.krylov_initial_guess == UFE_X0_CURRENT, inner);
  }

  void enqueue_picard_post(bool diva, CondArg outer) {
    if (diva)
      k_finalize<true><<<eblocks(w->nTri), kThreads, 0, s>>>(w->nTri, w->kv.X, w->uv, q, w->ps, w->ks, w->beta_b,
                                                             w->bfc_b, w->F2b1, w->uv_base, w->tau_b,
                                                             ctx->red.partials, ctx->red.tickets, outer, w->nz,
                                                             w->eta_3D_b, ctx->zeta, w->duz_b);
    else
      k_finalize<false><<<eblocks(w->nTri), kThreads, 0, s>>>(w->nTri, w->kv.X, w->uv, q, w->ps, w->ks, nullptr,
                                                              nullptr, nullptr, nullptr, nullptr,
                                                              ctx->red.partials, ctx->red.tickets, outer);
    UFE_CUDA(cudaGetLastError());
  }
};

// ---- graph construction ----------------------------------------------------------------------
// Capture `fn` into `g` after `deps`; returns the capture's sink nodes.
template <class F>
std::vector<cudaGraphNode_t> capture_into(cudaStream_t s, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                                          F &&fn) {
  UFE_CUDA(cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                         cudaStreamCaptureModeThreadLocal));
  try {
    fn();
  } catch (...) {
    cudaGraph_t dummy;
    cudaStreamEndCapture(s, &dummy);
    throw;
  }
  cudaStreamCaptureStatus st;
  const cudaGraphNode_t *sinks = nullptr;
  size_t nsinks = 0;
  UFE_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &sinks, nullptr, &nsinks));
  std::vector<cudaGraphNode_t> out(sinks, sinks + nsinks);
  cudaGraph_t g2;
  UFE_CUDA(cudaStreamEndCapture(s, &g2));
  return out;
}

// Add a while-node after `deps`; returns (node, body graph).
cudaGraphNode_t add_while(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
                          cudaGraph_t *body) {
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  UFE_CUDA(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &np));
  *body = np.conditional.phGraph_out[0];
  return node;
}

uint64_t params_key(const ufe_solver_params &p, int lanes, int has_bc) {
  const unsigned char *b = reinterpret_cast<const unsigned char *>(&p);
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < sizeof(p); ++i) { h ^= b[i]; h *= 1099511628211ull; }
  h ^= (uint64_t)lanes * 0x9E3779B97F4A7C15ull;
  h ^= (uint64_t)(has_bc + 7) * 0xC2B2AE3D27D4EB4Full;
  return h;
}

// Kernel nodes of a graph (not those inside its conditional bodies).
int32_t count_kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  UFE_CUDA(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  if (n) UFE_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
  int32_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    UFE_CUDA(cudaGraphNodeGetType(nodes[i], &t));
    if (t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

// The whole Picard solve as one graph: prologue -> while(picard){ pre -> while(krylov){...} -> post }
cudaGraphExec_t build_picard_graph(Solver &S, bool diva) {
  cudaGraph_t g;
  UFE_CUDA(cudaGraphCreate(&g, 0));
  try {
    cudaGraphConditionalHandle h_outer;
    UFE_CUDA(cudaGraphConditionalHandleCreate(&h_outer, g, 1, cudaGraphCondAssignDefault));
    auto sinks = capture_into(S.s, g, {}, [&] { S.enqueue_prologue(diva); });
    S.w->graph_kernels_pro[diva] = count_kernel_nodes(g);
    S.w->graph_kernels_it[diva] = -1;
    S.w->graph_kernels_round[diva] = -1;
    cudaGraph_t body;
    add_while(g, sinks, h_outer, &body);
    CondArg outer{h_outer, 1};
    if (S.pair_ok()) {
      // double-word: while(rounds){ persistent double-word solve, FP64 residual, gate }, then the
      // persistent FP64 solve (idle unless the rounds ended unconverged)
      cudaGraphConditionalHandle h_pair;
      UFE_CUDA(cudaGraphConditionalHandleCreate(&h_pair, body, 0, 0));
      CondArg pc{h_pair, 1};
      auto pre = capture_into(S.s, body, {}, [&] { S.enqueue_picard_pre(diva, pc); });
      cudaGraph_t rbody;
      cudaGraphNode_t wr = add_while(body, pre, h_pair, &rbody);
      capture_into(S.s, rbody, {}, [&] { S.pair_round(pc); });
      auto fb = capture_into(S.s, body, {wr}, [&] { S.enqueue_outer_halo64(); });
      capture_into(S.s, body, fb, [&] { S.enqueue_picard_post(diva, outer); });
      S.w->graph_kernels_it[diva] = count_kernel_nodes(body);
      S.w->graph_kernels_round[diva] = count_kernel_nodes(rbody);
      cudaGraphExec_t exec;
      UFE_CUDA(cudaGraphInstantiate(&exec, g, 0));
      cudaGraphDestroy(g);
      return exec;
    }
    if (S.p.precision != UFE_PREC_FP32_REFINE && S.halo64_ok()) {
      // FP64: the whole Krylov solve of a Picard iteration is one persistent launch
      CondArg none{0, 0};
      auto pre = capture_into(S.s, body, {}, [&] { S.enqueue_picard_pre(diva, none); });
      auto ks = capture_into(S.s, body, pre, [&] { S.enqueue_outer_halo64(); });
      capture_into(S.s, body, ks, [&] { S.enqueue_picard_post(diva, outer); });
      S.w->graph_kernels_it[diva] = count_kernel_nodes(body);
      S.w->graph_kernels_round[diva] = 0;
      cudaGraphExec_t exec;
      UFE_CUDA(cudaGraphInstantiate(&exec, g, 0));
      cudaGraphDestroy(g);
      return exec;
    }
    cudaGraphConditionalHandle h_inner;
    UFE_CUDA(cudaGraphConditionalHandleCreate(&h_inner, body, 0, 0));
    CondArg inner{h_inner, 1};
    auto pre = capture_into(S.s, body, {}, [&] { S.enqueue_picard_pre(diva, inner); });
    cudaGraph_t kbody;
    cudaGraphNode_t wk = add_while(body, pre, h_inner, &kbody);
    if (S.p.precision == UFE_PREC_FP32_REFINE) {
      // refinement loop: inner FP32 BiCGStab, then x += d and the FP64 residual test
      cudaGraphNode_t wi;
      if (persistent_krylov() && S.ctx->allow_persistent) {
        CondArg none{0, 0};
        auto ii = capture_into(S.s, kbody, {}, [&] {
          S.enqueue_inner_init(none);
          S.enqueue_inner_persist();
        });
        capture_into(S.s, kbody, ii, [&] { S.enqueue_refine_update(inner); });
      } else {
        cudaGraphConditionalHandle h_in32;   // a handle must belong to a conditional node
        UFE_CUDA(cudaGraphConditionalHandleCreate(&h_in32, kbody, 0, 0));
        CondArg in32{h_in32, 1};
        auto ii = capture_into(S.s, kbody, {}, [&] { S.enqueue_inner_init(in32); });
        cudaGraph_t ibody;
        wi = add_while(kbody, ii, h_in32, &ibody);
        capture_into(S.s, ibody, {}, [&] { S.krylov_iter32(in32); });
        capture_into(S.s, kbody, {wi}, [&] { S.enqueue_refine_update(inner); });
      }
      // FP64 fallback when the refinement loop gave up
      cudaGraphConditionalHandle h_fb;
      UFE_CUDA(cudaGraphConditionalHandleCreate(&h_fb, body, 0, 0));
      CondArg fb{h_fb, 1};
      auto fi = capture_into(S.s, body, {wk}, [&] { S.enqueue_fallback_init(fb); });
      cudaGraph_t fbody;
      wk = add_while(body, fi, h_fb, &fbody);
      capture_into(S.s, fbody, {}, [&] { S.krylov_iter64(fb); });
    } else {
      capture_into(S.s, kbody, {}, [&] { S.krylov_iter64(inner); });
    }
    capture_into(S.s, body, {wk}, [&] { S.enqueue_picard_post(diva, outer); });
    cudaGraphExec_t exec;
    UFE_CUDA(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    return exec;
  } catch (...) {
    cudaGraphDestroy(g);
    throw;
  }
}

// Host-driven loop over the same kernels (UFE_NO_GRAPH=1): for debugging and comparison.
void run_picard_host(Solver &S, bool diva) {
  CondArg none{0, 0};
  Work *w = S.w;
  S.enqueue_prologue(diva);
  for (int it = 0; it < S.p.visc_it_nit + 2; ++it) {
    S.enqueue_picard_pre(diva, none);
    for (;;) {
      if (S.p.precision == UFE_PREC_FP32_REFINE) {
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
        S.enqueue_inner_init(none);
        if (persistent_krylov() && S.ctx->allow_persistent) {
          S.enqueue_inner_persist();
        } else {
          for (;;) {
            for (int c = 0; c < 8; ++c) S.krylov_iter32(none);
            UFE_CUDA(cudaMemcpyAsync(w->ks_host + 1, w->ks + 1, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
            UFE_CUDA(cudaStreamSynchronize(S.s));
            if (!w->ks_host[1].active) break;
          }
        }
        S.enqueue_refine_update(none);
      } else if (S.halo64_ok()) {
        if (S.pair_ok()) S.run_pair_host();
        else S.enqueue_outer_halo64();
        break;
      } else {
        for (int c = 0; c < 8; ++c) S.krylov_iter64(none);
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
      }
    }
    if (S.p.precision == UFE_PREC_FP32_REFINE) {
      S.enqueue_fallback_init(none);
      for (;;) {
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
        for (int c = 0; c < 8; ++c) S.krylov_iter64(none);
      }
    }
    S.enqueue_picard_post(diva, none);
    UFE_CUDA(cudaMemcpyAsync(w->ps_host, w->ps, sizeof(PicardScalars), cudaMemcpyDeviceToHost, S.s));
    UFE_CUDA(cudaStreamSynchronize(S.s));
    if (!w->ps_host->active) break;
  }
}

bool use_graphs() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("UFE_NO_GRAPH");
    v = (e && *e && *e != '0') ? 0 : 1;
  }
  return v == 1;
}

void validate_params(const ufe_solver_params *p) {
  UFE_REQUIRE(p, UFE_ERR_INVALID, "null params");
  UFE_REQUIRE(p->choice_sliding_law >= 0 && p->choice_sliding_law <= UFE_SLIDING_IDEALISED_SSA_ICESTREAM,
              UFE_ERR_INVALID, "unknown sliding law");
  // Schoof only derived his ice-stream solution for n = 3 (Schoof_SSA_solution.f90:40)
  UFE_REQUIRE(p->choice_sliding_law != UFE_SLIDING_IDEALISED_SSA_ICESTREAM || p->Glens_flow_law_exponent == 3.0,
              UFE_ERR_INVALID, "the SSA_icestream sliding law needs Glens_flow_law_exponent = 3");
  UFE_REQUIRE(p->choice_ice_rheology_Glen >= UFE_RHEOLOGY_INPUT &&
                  p->choice_ice_rheology_Glen <= UFE_RHEOLOGY_HUYBRECHTS1992 &&
                  (p->choice_enhancement_factor_transition == UFE_ENH_SEPARATE ||
                   p->choice_enhancement_factor_transition == UFE_ENH_INTERP),
              UFE_ERR_INVALID, "unknown rheology or enhancement-factor choice");
  UFE_REQUIRE(p->visc_it_nit >= 0 && p->krylov_max_it >= 1, UFE_ERR_INVALID, "iteration limits out of range");
  UFE_REQUIRE(p->precision == UFE_PREC_FP64 || p->precision == UFE_PREC_FP32_REFINE ||
                  p->precision == UFE_PREC_FP32_PAIR,
              UFE_ERR_INVALID, "unknown precision mode");
  UFE_REQUIRE(p->krylov_initial_guess == UFE_X0_ZERO || p->krylov_initial_guess == UFE_X0_CURRENT, UFE_ERR_INVALID,
              "unknown initial guess mode");
  const int32_t bcs[8] = {p->BC_u_west, p->BC_u_east, p->BC_u_south, p->BC_u_north,
                          p->BC_v_west, p->BC_v_east, p->BC_v_south, p->BC_v_north};
  for (int i = 0; i < 8; ++i)
    UFE_REQUIRE(bcs[i] == UFE_BC_INFINITE || bcs[i] == UFE_BC_ZERO || (i < 4 && bcs[i] == UFE_BC_INFINITE_SSA_ICESTREAM),
                UFE_ERR_INVALID, "unsupported boundary condition");   // the ice-stream copy is u only (:562)
  UFE_REQUIRE(p->Glens_flow_law_exponent > 0 && p->visc_it_relax > 0 && p->visc_it_relax <= 1, UFE_ERR_INVALID,
              "flow law exponent or relaxation out of range");
  UFE_REQUIRE(p->krylov_inner_rtol > 0 && p->krylov_inner_rtol < 1, UFE_ERR_INVALID, "krylov_inner_rtol out of range");
  UFE_REQUIRE(p->krylov_forcing >= 0 && p->krylov_forcing < 1, UFE_ERR_INVALID, "krylov_forcing out of range");
}

int32_t check_err_flag(Solver &S) {
  int err = 0;
  UFE_CUDA(cudaMemcpyAsync(&err, S.w->err, sizeof(int), cudaMemcpyDeviceToHost, S.s));
  UFE_CUDA(cudaStreamSynchronize(S.s));
  if (err) {
    UFE_CUDA(cudaMemsetAsync(S.w->err, 0, sizeof(int), S.s));
    UFE_REQUIRE(!(err & kErrNoDiag), UFE_ERR_INVALID, "a 2nd-order b_b operator row has no diagonal entry");
    UFE_REQUIRE(!(err & kErrBcNeighbour), UFE_ERR_INVALID,
                "a border triangle's neighbour is missing from its b_b operator row");
    UFE_REQUIRE(false, UFE_ERR_INVALID, "a border triangle has no neighbours");
  }
  return UFE_OK;
}

// A resident Picard solve in two halves: picard_launch queues the whole solve on the context's
// stream (graph or host loop) and the copies of its scalars; picard_collect waits for it and
// reads the result.  Ensembles launch all members before collecting any.
void picard_launch(ufe_ctx *ctx, const ufe_solver_params &p, bool diva) {
  Solver S(ctx, p);
  S.setup_solve_inputs();
  Work *w = S.w;
  UFE_REQUIRE(ctx->nz <= kMaxNz, UFE_ERR_CAPACITY, "nz exceeds 64 layers");
  cudaEventRecord(ctx->ev0, S.s);
  if (use_graphs()) {
    cudaGraphExec_t *gx = diva ? &w->graph_diva : &w->graph_ssa;
    uint64_t *key = diva ? &w->graph_diva_key : &w->graph_ssa_key;
    uint64_t k = params_key(p, S.lanes, w->has_bc) ^ (ctx->allow_persistent ? 0x5bd1e995ull : 0ull);
    if (!*gx || *key != k) {
      if (*gx) cudaGraphExecDestroy(*gx);
      *gx = nullptr;
      *gx = build_picard_graph(S, diva);
      *key = k;
    }
    UFE_CUDA(cudaGraphLaunch(*gx, S.s));
    w->last_kernels_pro = w->graph_kernels_pro[diva];
    w->last_kernels_it = w->graph_kernels_it[diva];
    w->last_kernels_round = w->graph_kernels_round[diva];
  } else {
    run_picard_host(S, diva);
    w->last_kernels_pro = w->last_kernels_it = w->last_kernels_round = -1;
  }
  cudaEventRecord(ctx->ev1, S.s);
  UFE_CUDA(cudaMemcpyAsync(w->ps_host, w->ps, sizeof(PicardScalars), cudaMemcpyDeviceToHost, S.s));
  UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars) * 2, cudaMemcpyDeviceToHost, S.s));
}

int32_t picard_collect(ufe_ctx *ctx, const ufe_solver_params &p, ufe_solve_stats *stats) {
  Solver S(ctx, p);
  Work *w = S.w;
  UFE_CUDA(cudaStreamSynchronize(S.s));
  check_err_flag(S);
  const PicardScalars ps = *w->ps_host;
  const KrylovScalars ks = w->ks_host[0];
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  int32_t total_its = w->ks_host[1].total_its + ks.total_its;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->n_visc_its = ps.it;
    stats->n_Axb_its = total_its;
    stats->n_refinements = ps.n_refine;
    stats->status = ps.status;
    stats->L2_uv = ps.L2;
    stats->visc_it_relax_applied = ps.relax;
    stats->device_ms = ms;
    stats->n_fp64_its = ks.total_its - ks.pair_its;
    stats->n_pair_its = ks.pair_its;
    stats->n_kernels = (w->last_kernels_it >= 0 && w->last_kernels_round >= 0)
                           ? w->last_kernels_pro + ps.it * w->last_kernels_it + ks.pair_rounds_total * w->last_kernels_round
                           : -1;
  }
  return ps.status;
}

// Run a resident Picard solve; fills stats; returns the status.
int32_t run_picard(ufe_ctx *ctx, const ufe_solver_params &p, bool diva, ufe_solve_stats *stats) {
  picard_launch(ctx, p, diva);
  return picard_collect(ctx, p, stats);
}

}  // namespace

// ============================================================================================
// entry points

// caller-ordered vertex field -> internal order (zero when absent)
static void upload_vertex_opt(ufe_ctx *ctx, double *dst, const double *src) {
  if (src) to_internal(ctx, dst, src, false, 1);
  else UFE_CUDA(cudaMemsetAsync(dst, 0, sizeof(double) * ctx->nV, ctx->stream));
}

static void upload_bc(ufe_ctx *ctx, Work *w, const ufe_bc_prescribed *bc) {
  cudaStream_t s = ctx->stream;
  const int nTri = ctx->nTri;
  w->has_bc = 0;
  if (bc && (bc->mask_b || bc->u_b || bc->v_b)) {
    UFE_REQUIRE(bc->mask_b && bc->u_b && bc->v_b, UFE_ERR_INVALID,
                "need to provide prescribed u,v fields and mask");  // SSA_main.f90:147-150
    to_internal_i32(ctx, w->bc_mask, bc->mask_b, true);
    pair_to_internal(ctx, w->bc_uv, bc->u_b, bc->v_b);
    w->has_bc = 1;
  }
}

extern "C" int32_t ufe_ice_upload(ufe_ctx *ctx, const ufe_ice_state *ice, const ufe_bc_prescribed *bc) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ice && ice->Hi && ice->Hs && ice->fraction_gr_b && ice->mask_grounded_ice,
                UFE_ERR_INVALID, "ice state arrays missing");
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    cudaStream_t s = ctx->stream;
    const size_t nV = ctx->nV, nTri = ctx->nTri, nz = ctx->nz;
    to_internal(ctx, w->Hi, ice->Hi, false, 1);
    to_internal(ctx, w->Hs, ice->Hs, false, 1);
    // A_flow may be absent when the solve computes it (calc_ice_rheology_Glen)
    w->has_A = ice->A_flow != nullptr;
    if (ice->A_flow) to_internal(ctx, w->A_flow, ice->A_flow, false, (int)nz);
    else UFE_CUDA(cudaMemsetAsync(w->A_flow, 0, sizeof(double) * nV * nz, s));
    // calc_ice_rheology_Glen inputs: buffers allocated on first use and kept (captured solve
    // graphs hold their addresses); the flags say which were given with this ice state
    auto opt_vertex = [&](double *&dst, int32_t &has, const double *src, int ncols) {
      has = src != nullptr;
      if (!src) return;
      if (!dst) dst = alloc_n<double>(nV * ncols);
      to_internal(ctx, dst, src, false, ncols);
    };
    opt_vertex(w->Ti, w->has_Ti, ice->Ti, (int)nz);
    opt_vertex(w->fgr_v, w->has_fgr_v, ice->fraction_gr, 1);
    opt_vertex(w->Hib, w->has_Hib, ice->Hib, 1);
    opt_vertex(w->SL, w->has_SL, ice->SL, 1);
    w->has_mask_fl = ice->mask_floating_ice != nullptr;
    if (ice->mask_floating_ice) {
      if (!w->mask_fl) w->mask_fl = alloc_n<int32_t>(nV);
      to_internal_i32(ctx, w->mask_fl, ice->mask_floating_ice, false);
    }
    to_internal(ctx, w->fgr_b, ice->fraction_gr_b, true, 1);
    to_internal_i32(ctx, w->mask_gr, ice->mask_grounded_ice, false);
    upload_vertex_opt(ctx, w->beta_sq, ice->beta_sq);
    upload_vertex_opt(ctx, w->alpha_sq, ice->alpha_sq);
    upload_vertex_opt(ctx, w->effp, ice->effective_pressure);
    upload_vertex_opt(ctx, w->tys, ice->till_yield_stress);
    // NaN/Inf in any input field is an error (the reference's do_check_for_NaN checks)
    {
      int *flag = w->err;
      UFE_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      const double *arrs[] = {w->Hi, w->Hs, w->A_flow, w->fgr_b, w->beta_sq, w->alpha_sq, w->effp, w->tys,
                              w->has_Ti ? w->Ti : nullptr, w->has_fgr_v ? w->fgr_v : nullptr,
                              w->has_Hib ? w->Hib : nullptr, w->has_SL ? w->SL : nullptr};
      const size_t lens[] = {nV, nV, nV * nz, nTri, nV, nV, nV, nV, nV * nz, nV, nV, nV};
      for (int k = 0; k < 12; ++k)
        if (arrs[k])
          k_check_finite<<<pick_blocks((int64_t)lens[k], kThreads, 256), kThreads, 0, s>>>(arrs[k], (int64_t)lens[k],
                                                                                          flag);
      UFE_CUDA(cudaGetLastError());
      int hflag = 0;
      UFE_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      UFE_REQUIRE(hflag == 0, UFE_ERR_NAN, "NaN or infinite value in the ice state");
    }
    int any = 0;
    for (size_t v = 0; v < nV && !any; ++v) any = ice->mask_grounded_ice[v] != 0;
    w->any_grounded = any;
    upload_bc(ctx, w, bc);
    UFE_CUDA(cudaStreamSynchronize(s));
    return UFE_OK;
  });
}

static void check_sliding_inputs(const ufe_solver_params *p, const ufe_ice_state *ice) {
  if (!ice) return;
  switch (p->choice_sliding_law) {
    case UFE_SLIDING_WEERTMAN:
      UFE_REQUIRE(ice->beta_sq, UFE_ERR_INVALID, "Weertman sliding needs beta_sq"); break;
    case UFE_SLIDING_COULOMB: case UFE_SLIDING_BUDD:
      UFE_REQUIRE(ice->till_yield_stress, UFE_ERR_INVALID, "Coulomb/Budd sliding needs till_yield_stress"); break;
    case UFE_SLIDING_TSAI2015: case UFE_SLIDING_SCHOOF2005:
      UFE_REQUIRE(ice->beta_sq && ice->alpha_sq && ice->effective_pressure, UFE_ERR_INVALID,
                  "Tsai2015/Schoof2005 sliding needs beta_sq, alpha_sq and effective_pressure");
      break;
    default: break;
  }
}

// A start velocity set from outside the learned start (zero, the caller's, a previous solve's)
// carries no predicted viscosity.
static void disarm_prediction(Work *w, cudaStream_t s) {
  UFE_CUDA(cudaMemsetAsync(w->pred_flag, 0, sizeof(int32_t), s));
}

// Queue a resident solve; false when there is nothing to solve (no grounded ice), in which
// case the zero velocity is already set and the stats are zero.
static bool resident_launch(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start, bool diva) {
  validate_params(p);
  UFE_CUDA(cudaSetDevice(ctx->device));
  Work *w = ensure_work(ctx);
  cudaStream_t s = ctx->stream;
  const int nTri = ctx->nTri;
  if (cold_start) {
    disarm_prediction(w, s);
    UFE_CUDA(cudaMemsetAsync(w->uv, 0, sizeof(double2) * nTri, s));
    if (diva) {
      UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * nTri, s));
      UFE_CUDA(cudaMemsetAsync(w->tau_b, 0, sizeof(double2) * nTri, s));
      UFE_CUDA(cudaMemsetAsync(w->eta_3D_b, 0, sizeof(double) * (size_t)nTri * ctx->nz, s));
    }
  }
  bool skip = !w->any_grounded || (!diva && p->choice_sliding_law == UFE_SLIDING_NO_SLIDING);
  if (skip) {
    UFE_CUDA(cudaMemsetAsync(w->uv, 0, sizeof(double2) * nTri, s));
    if (diva) UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * nTri, s));
    return false;
  }
  picard_launch(ctx, *p, diva);
  return true;
}

static int32_t resident_solve(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start, bool diva,
                              ufe_solve_stats *stats) {
  validate_params(p);
  UFE_CUDA(cudaSetDevice(ctx->device));
  Work *w = ensure_work(ctx);
  cudaStream_t s = ctx->stream;
  const int nTri = ctx->nTri;
  if (cold_start) {
    disarm_prediction(w, s);
    UFE_CUDA(cudaMemsetAsync(w->uv, 0, sizeof(double2) * nTri, s));
    if (diva) {
      UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * nTri, s));
      UFE_CUDA(cudaMemsetAsync(w->tau_b, 0, sizeof(double2) * nTri, s));
      UFE_CUDA(cudaMemsetAsync(w->eta_3D_b, 0, sizeof(double) * (size_t)nTri * ctx->nz, s));
    }
  }
  bool skip = !w->any_grounded || (!diva && p->choice_sliding_law == UFE_SLIDING_NO_SLIDING);
  if (skip) {
    // solve_SSA/solve_DIVA return zero velocities without grounded ice (SSA_main.f90:121-129)
    UFE_CUDA(cudaMemsetAsync(w->uv, 0, sizeof(double2) * nTri, s));
    if (diva) UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * nTri, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    if (stats) memset(stats, 0, sizeof(*stats));
    return UFE_OK;
  }
  return run_picard(ctx, *p, diva, stats);
}

// ---- learned Picard start: the mesh side ------------------------------------------------------
// Features per triangle (16 floats) from the resident ice state, in internal order:
//  0 Hi_b/1e3   1 Hs_b/1e3   2,3 dHs/dx, dHs/dy x100 (clipped to +-10)   4 fraction_gr_b
//  5 log10(max(beta_sq_b,1)) - 4   6,7 driving stress / 1e5   8,9 previous velocity / 1e3
//  10,11 local sliding balance (|tau_d| / beta_sq)^3 along tau_d, times fraction_gr_b, / 1e3
//  12 log10(1 + |that|) / 3   13 ice present (Hi_b > 0)   14,15 zero
__global__ void k_gnn_features(int nTri, OpRow ab, const double *Hi, const double *Hs, const double *beta_sq,
                               const double *fgr_b, const double2 *uv, int use_prev, float *x, float *mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  double Hib = 0.0, Hsb = 0.0, dx = 0.0, dy = 0.0, bb = 0.0;
  for (int k = ab.ptr[t]; k < ab.ptr[t + 1]; ++k) {
    const int v = ab.ind[k];
    Hib += ab.v0[k] * Hi[v];
    Hsb += ab.v0[k] * Hs[v];
    dx += ab.v1[k] * Hs[v];
    dy += ab.v2[k] * Hs[v];
    if (beta_sq) bb += ab.v0[k] * beta_sq[v];
  }
  const double tx = -kIceDensity * kGrav * Hib * dx, ty = -kIceDensity * kGrav * Hib * dy;
  const double tau = sqrt(tx * tx + ty * ty);
  const double fg = fgr_b[t];
  double usl = fg * pow(tau / fmax(bb, 1.0), 3.0);
  usl = fmin(usl, 1e4);
  const double ux = tau > 0.0 ? usl * tx / tau : 0.0, uy = tau > 0.0 ? usl * ty / tau : 0.0;
  float *o = x + t * 16;
  o[0] = (float)(Hib / 1e3);
  o[1] = (float)(Hsb / 1e3);
  o[2] = (float)fmax(-10.0, fmin(10.0, dx * 100.0));
  o[3] = (float)fmax(-10.0, fmin(10.0, dy * 100.0));
  o[4] = (float)fg;
  o[5] = (float)(log10(fmax(bb, 1.0)) - 4.0);
  o[6] = (float)(tx / 1e5);
  o[7] = (float)(ty / 1e5);
  o[8] = use_prev ? (float)(uv[t].x / 1e3) : 0.f;
  o[9] = use_prev ? (float)(uv[t].y / 1e3) : 0.f;
  o[10] = (float)(ux / 1e3);
  o[11] = (float)(uy / 1e3);
  o[12] = (float)(log10(1.0 + usl) / 3.0);
  o[13] = Hib > 0.0 ? 1.f : 0.f;
  o[14] = 0.f;
  o[15] = 0.f;
  if (mask) mask[t] = Hib > 0.0 ? 1.f : 0.f;
}

__global__ void k_gnn_graph(int nTri, const int32_t *TriC, int32_t *nbr) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  for (int q = 0; q < 3; ++q) nbr[t * 3 + q] = TriC[(int64_t)q * nTri + t] - 1;   // 1-based, 0: none
}

__global__ void k_gnn_velocity(int nTri, double2 *uv, float *y, int to_state, const float *mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  float *yt = y + t * kGnnOut;
  if (to_state) {
    const bool ice = !mask || mask[t] > 0.f;
    uv[t] = ice ? make_double2((double)yt[0] * 1e3, (double)yt[1] * 1e3) : make_double2(0.0, 0.0);
  } else {
    yt[0] = (float)(uv[t].x / 1e3);
    yt[1] = (float)(uv[t].y / 1e3);
  }
}

// Training target of the viscosity output: the solve's vertically averaged effective viscosity
// (N_a / max(0.1, Hi) on the vertices, from the last Picard iteration) mapped to the triangles,
// as (log10(eta) - kGnnLogEtaOff) / kGnnLogEtaScale.
__global__ void k_gnn_visc_target(int nTri, OpRow ab, const double *N_a, const double *Hi, float *y) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  double e = 0.0;
  for (int k = ab.ptr[t]; k < ab.ptr[t + 1]; ++k) {
    const int v = ab.ind[k];
    e += ab.v0[k] * (N_a[v] / fmax(0.1, Hi[v]));
  }
  y[t * kGnnOut + 2] = (float)((log10(fmax(e, 1e-30)) - kGnnLogEtaOff) / kGnnLogEtaScale);
}

// The predicted viscosity on the vertices: the b->a map of the log-viscosity output over the
// vertex's triangles with ice (all of them where none has ice), then arms the next solve.
__global__ void k_gnn_visc_pred(int nV, OpRow ba, const float *y, const float *mask, double *eta_a,
                                int32_t *pred_flag) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v == 0) *pred_flag = 1;
  if (v >= nV) return;
  double sw = 0.0, s = 0.0, sa = 0.0;
  for (int k = ba.ptr[v]; k < ba.ptr[v + 1]; ++k) {
    const int t = ba.ind[k];
    const double lv = (double)y[(int64_t)t * kGnnOut + 2];
    sa += ba.v0[k] * lv;
    if (!mask || mask[t] > 0.f) {
      sw += ba.v0[k];
      s += ba.v0[k] * lv;
    }
  }
  const double l = sw > 0.0 ? s / sw : sa;
  eta_a[v] = exp10(kGnnLogEtaScale * l + kGnnLogEtaOff);
}

// one averaging pass over each triangle and its TriC neighbours (ice triangles only)
__global__ void k_smooth_uv(int nTri, const int32_t *TriC, const float *mask, const double2 *in, double2 *out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  if (mask && !(mask[t] > 0.f)) {
    out[t] = in[t];
    return;
  }
  double2 sum = in[t];
  int cnt = 1;
  for (int q = 0; q < 3; ++q) {
    const int32_t j = TriC[(int64_t)q * nTri + t] - 1;
    if (j < 0 || (mask && !(mask[j] > 0.f))) continue;
    sum.x += in[j].x;
    sum.y += in[j].y;
    ++cnt;
  }
  out[t] = make_double2(sum.x / cnt, sum.y / cnt);
}

void gnn_mesh_smooth(ufe_ctx *ctx, cudaStream_t s, int passes, const float *mask) {
  Work *w = ctx->work;
  for (int k = 0; k < passes; ++k) {   // ping-pong through the Krylov scratch vector S
    k_smooth_uv<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, ctx->TriC, mask, w->uv, w->kv.S);
    k_smooth_uv<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, ctx->TriC, mask, w->kv.S, w->uv);
  }
  UFE_CUDA(cudaGetLastError());
}

void gnn_mesh_features(ufe_ctx *ctx, cudaStream_t s, int use_prev, float *x, float *mask) {
  Work *w = ctx->work;
  UFE_REQUIRE(w, UFE_ERR_INVALID, "learned start: upload the ice state first");
  const DevCSR &mab = ctx->ops[UFE_OP_MAP_A_B];
  OpRow ab{mab.ptr, mab.ind, mab.val, ctx->ops[UFE_OP_DDX_A_B].val, ctx->ops[UFE_OP_DDY_A_B].val};
  k_gnn_features<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, ab, w->Hi, w->Hs, w->beta_sq, w->fgr_b, w->uv,
                                                          use_prev, x, mask);
  UFE_CUDA(cudaGetLastError());
}

void gnn_mesh_graph(ufe_ctx *ctx, cudaStream_t s, int32_t *nbr) {
  k_gnn_graph<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, ctx->TriC, nbr);
  UFE_CUDA(cudaGetLastError());
}

void gnn_mesh_velocity(ufe_ctx *ctx, cudaStream_t s, float *y, bool to_state, const float *mask) {
  Work *w = ctx->work;
  UFE_REQUIRE(w, UFE_ERR_INVALID, "learned start: upload the ice state first");
  k_gnn_velocity<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, w->uv, y, to_state ? 1 : 0, mask);
  UFE_CUDA(cudaGetLastError());
  if (to_state) {
    disarm_prediction(w, s);   // a velocity-only prediction; gnn_mesh_viscosity arms the viscosity
    // a predicted start carries no vertical-shear state: DIVA begins its first iteration as from
    // a cold start, but with this velocity
    UFE_CUDA(cudaMemsetAsync(w->uv_base, 0, sizeof(double2) * ctx->nTri, s));
    UFE_CUDA(cudaMemsetAsync(w->tau_b, 0, sizeof(double2) * ctx->nTri, s));
    UFE_CUDA(cudaMemsetAsync(w->eta_3D_b, 0, sizeof(double) * (size_t)ctx->nTri * ctx->nz, s));
  }
}

// to_state: store the predicted viscosity (output 2 of y) on the vertices and arm the next solve's
// first iteration with it; otherwise write the solved viscosity into output 2 of y as the target.
void gnn_mesh_viscosity(ufe_ctx *ctx, cudaStream_t s, float *y, bool to_state, const float *mask) {
  Work *w = ctx->work;
  UFE_REQUIRE(w, UFE_ERR_INVALID, "learned start: upload the ice state first");
  if (to_state) {
    const DevCSR &mba = ctx->ops[UFE_OP_MAP_B_A];
    OpRow ba{mba.ptr, mba.ind, mba.val, nullptr, nullptr};
    k_gnn_visc_pred<<<(ctx->nV + 255) / 256, 256, 0, s>>>(ctx->nV, ba, y, mask, w->eta_pred_a, w->pred_flag);
  } else {
    const DevCSR &mab = ctx->ops[UFE_OP_MAP_A_B];
    OpRow ab{mab.ptr, mab.ind, mab.val, nullptr, nullptr};
    k_gnn_visc_target<<<(ctx->nTri + 255) / 256, 256, 0, s>>>(ctx->nTri, ab, w->N_a, w->Hi, y);
  }
  UFE_CUDA(cudaGetLastError());
}

extern "C" int32_t ufe_solve_ssa_resident(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start,
                                          ufe_solve_stats *stats) {
  return guarded(ctx, [&]() -> int32_t { return resident_solve(ctx, p, cold_start, false, stats); });
}

extern "C" int32_t ufe_solve_diva_resident(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start,
                                           ufe_solve_stats *stats) {
  return guarded(ctx, [&]() -> int32_t { return resident_solve(ctx, p, cold_start, true, stats); });
}

// Many independent members, each a context with its mesh and resident ice state (on one device):
// every member's solve is queued on its own stream before any is waited for, so the members of
// uneven size run side by side.  The persistent FP32 kernel (which needs the whole GPU) is not
// used inside an ensemble.
extern "C" int32_t ufe_ensemble_solve(ufe_ctx *const *ctxs, int32_t n, const ufe_solver_params *p, int32_t diva,
                                      int32_t cold_start, ufe_solve_stats *stats, double *wall_ms) {
  if (!ctxs || n < 1 || !p) return UFE_ERR_INVALID;
  for (int32_t i = 0; i < n; ++i)
    if (!ctxs[i] || ctxs[i]->device != ctxs[0]->device) return UFE_ERR_INVALID;
  std::vector<char> launched(n, 0);
  std::vector<int32_t> rc(n, UFE_OK);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaSetDevice(ctxs[0]->device) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    return UFE_ERR_DEVICE;
  cudaEventRecord(e0, ctxs[0]->stream);
  for (int32_t i = 0; i < n; ++i) {
    ufe_ctx *c = ctxs[i];
    if (i > 0) cudaStreamWaitEvent(c->stream, e0, 0);
    rc[i] = guarded(c, [&]() -> int32_t {
      c->allow_persistent = false;
      launched[i] = resident_launch(c, p, cold_start, diva != 0) ? 1 : 0;
      return UFE_OK;
    });
  }
  for (int32_t i = 0; i < n; ++i) {
    ufe_ctx *c = ctxs[i];
    if (rc[i] < 0) continue;
    rc[i] = guarded(c, [&]() -> int32_t {
      if (!launched[i]) {
        UFE_CUDA(cudaStreamSynchronize(c->stream));
        if (stats) memset(&stats[i], 0, sizeof(ufe_solve_stats));
        return UFE_OK;
      }
      return picard_collect(c, *p, stats ? &stats[i] : nullptr);
    });
    if (i > 0) {
      cudaEvent_t done;
      if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess) {
        cudaEventRecord(done, c->stream);
        cudaStreamWaitEvent(ctxs[0]->stream, done, 0);
        cudaEventDestroy(done);
      }
    }
  }
  for (int32_t i = 0; i < n; ++i) ctxs[i]->allow_persistent = true;
  cudaEventRecord(e1, ctxs[0]->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (wall_ms) *wall_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int32_t worst = UFE_OK;
  for (int32_t i = 0; i < n; ++i) {
    if (rc[i] < 0 && (worst >= 0 || rc[i] < worst)) worst = rc[i];
    else if (worst >= 0 && rc[i] > worst) worst = rc[i];
  }
  return worst;
}

// The autotuner: for this mesh, time the three FP64 Krylov kernels with each rows-per-warp
// choice (1 with the sliced-ELL layout, 2, 4, 8) on the system the last solve assembled, and keep
// the fastest for this context's later solves.  us (optional, 4 entries): the measured
// per-iteration microseconds of each choice.
extern "C" int32_t ufe_autotune(ufe_ctx *ctx, int32_t repeats, int32_t *lanes_out, double *us) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ctx->work, UFE_ERR_INVALID, "autotune: run a solve on this context first");
    const int choices[4] = {1, 2, 4, 8};
    double best = 1e300;
    int best_l = 1;
    for (int c = 0; c < 4; ++c) {
      ctx->lanes = choices[c];
      double t[3] = {0, 0, 0};
      int64_t geo[2];
      const int32_t rc = ufe_profile_krylov_kernels(ctx, UFE_PREC_FP64, repeats > 0 ? repeats : 20, t, geo);
      UFE_REQUIRE(rc == UFE_OK, rc, "autotune: kernel timing failed");
      const double it = t[0] + t[1] + t[2];
      if (us) us[c] = it;
      if (it < best) {
        best = it;
        best_l = choices[c];
      }
    }
    ctx->lanes = best_l;
    if (lanes_out) *lanes_out = best_l;
    return UFE_OK;
  });
}

static void download_pair(ufe_ctx *ctx, const double2 *src, double *a, double *b) {
  pair_to_external(ctx, a, b, src);
}

static void upload_pair(ufe_ctx *ctx, double2 *dst, const double *a, const double *b) {
  pair_to_internal(ctx, dst, a, b);
}

extern "C" int32_t ufe_solve_history(ufe_ctx *ctx, double *out, int32_t cap, int32_t *n) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(out && n && cap >= 0, UFE_ERR_INVALID, "bad history arguments");
    UFE_REQUIRE(ctx->work, UFE_ERR_INVALID, "no solve has run on this context");
    Work *w = ctx->work;
    UFE_CUDA(cudaMemcpyAsync(w->ps_host, w->ps, sizeof(PicardScalars), cudaMemcpyDeviceToHost, ctx->stream));
    UFE_CUDA(cudaStreamSynchronize(ctx->stream));
    int rows = w->ps_host->it < kHistMax ? w->ps_host->it : kHistMax;
    if (rows > cap) rows = cap;
    memcpy(out, w->ps_host->hist, sizeof(double) * rows * kHistCols);
    *n = rows;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_velocity_download(ufe_ctx *ctx, double *u_b, double *v_b) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    download_pair(ctx, w->uv, u_b, v_b);
    return UFE_OK;
  });
}

extern "C" int32_t ufe_solve_ssa(ufe_ctx *ctx, const ufe_solver_params *p, const ufe_ice_state *ice,
                                 const ufe_bc_prescribed *bc, double *u_b, double *v_b, int32_t *n_visc_its,
                                 int32_t *n_Axb_its, ufe_solve_stats *stats) {
  int32_t rc = ufe_ice_upload(ctx, ice, bc);
  if (rc != UFE_OK) return rc;
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(u_b && v_b, UFE_ERR_INVALID, "null velocity arrays");
    validate_params(p);
    check_sliding_inputs(p, ice);
    Work *w = ensure_work(ctx);
    upload_pair(ctx, w->uv, u_b, v_b);
    disarm_prediction(w, ctx->stream);
    ufe_solve_stats st;
    int32_t r = resident_solve(ctx, p, 0, false, &st);
    download_pair(ctx, w->uv, u_b, v_b);
    if (n_visc_its) *n_visc_its = st.n_visc_its;
    if (n_Axb_its) *n_Axb_its = st.n_Axb_its;
    if (stats) *stats = st;
    return r;
  });
}

extern "C" int32_t ufe_solve_diva(ufe_ctx *ctx, const ufe_solver_params *p, const ufe_ice_state *ice,
                                  const ufe_bc_prescribed *bc, ufe_diva_state *ds, int32_t *n_visc_its,
                                  int32_t *n_Axb_its, ufe_solve_stats *stats) {
  int32_t rc = ufe_ice_upload(ctx, ice, bc);
  if (rc != UFE_OK) return rc;
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ds && ds->u_vav_b && ds->v_vav_b && ds->u_base_b && ds->v_base_b && ds->tau_bx_b && ds->tau_by_b &&
                    ds->eta_3D_b,
                UFE_ERR_INVALID, "DIVA state arrays missing");
    validate_params(p);
    check_sliding_inputs(p, ice);
    UFE_REQUIRE(ctx->nz <= kMaxNz, UFE_ERR_CAPACITY, "nz exceeds 64 layers");
    Work *w = ensure_work(ctx);
    cudaStream_t s = ctx->stream;
    const size_t nTri = ctx->nTri, nz = ctx->nz;
    upload_pair(ctx, w->uv, ds->u_vav_b, ds->v_vav_b);
    upload_pair(ctx, w->uv_base, ds->u_base_b, ds->v_base_b);
    upload_pair(ctx, w->tau_b, ds->tau_bx_b, ds->tau_by_b);
    to_internal(ctx, w->eta_3D_b, ds->eta_3D_b, true, (int)nz);
    disarm_prediction(w, s);
    ufe_solve_stats st;
    int32_t r = resident_solve(ctx, p, 0, true, &st);
    download_pair(ctx, w->uv, ds->u_vav_b, ds->v_vav_b);
    download_pair(ctx, w->uv_base, ds->u_base_b, ds->v_base_b);
    download_pair(ctx, w->tau_b, ds->tau_bx_b, ds->tau_by_b);
    to_external(ctx, ds->eta_3D_b, w->eta_3D_b, true, (int)nz);
    if (r >= 0 && ds->u_3D_b && ds->v_3D_b) {
      if (!w->any_grounded) {
        memset(ds->u_3D_b, 0, sizeof(double) * nTri * nz);
        memset(ds->v_3D_b, 0, sizeof(double) * nTri * nz);
      } else {
        double *u3 = (double *)dev_alloc(sizeof(double) * nTri * nz), *v3 = (double *)dev_alloc(sizeof(double) * nTri * nz);
        Solver S(ctx, *p);
        k_diva_F1<<<S.eblocks(ctx->nV), kThreads, 0, s>>>(ctx->nV, ctx->nz, w->eta_3D_a, w->Hi, ctx->zeta, w->F1_3D_a);
        k_diva_u3d<<<S.eblocks((int64_t)nTri * nz), kThreads, 0, s>>>(
            ctx->nV, ctx->nTri, ctx->nz, S.ab, w->F1_3D_a, w->uv_base, w->tau_b, w->bfc_b,
            p->choice_sliding_law == UFE_SLIDING_NO_SLIDING, u3, v3);
        UFE_CUDA(cudaGetLastError());
        to_external(ctx, ds->u_3D_b, u3, true, (int)nz);
        to_external(ctx, ds->v_3D_b, v3, true, (int)nz);
        dev_free(u3);
        dev_free(v3);
      }
    }
    UFE_CUDA(cudaStreamSynchronize(s));
    if (n_visc_its) *n_visc_its = st.n_visc_its;
    if (n_Axb_its) *n_Axb_its = st.n_Axb_its;
    if (stats) *stats = st;
    return r;
  });
}

// Upload the per-triangle inputs of solve_SSA_DIVA_linearised.
static void upload_linearised_inputs(ufe_ctx *ctx, Work *w, const double *N_b, const double *dN_dx_b,
                                     const double *dN_dy_b, const double *beta_b, const double *tau_dx_b,
                                     const double *tau_dy_b, const ufe_bc_prescribed *bc) {
  UFE_REQUIRE(N_b && dN_dx_b && dN_dy_b && beta_b && tau_dx_b && tau_dy_b, UFE_ERR_INVALID,
              "linearised-solve input missing");
  cudaStream_t s = ctx->stream;
  const size_t n = ctx->nTri;
  (void)s; (void)n;
  to_internal(ctx, w->N_b_in, N_b, true, 1);
  to_internal(ctx, w->dNx_b_in, dN_dx_b, true, 1);
  to_internal(ctx, w->dNy_b_in, dN_dy_b, true, 1);
  to_internal(ctx, w->beta_b_in, beta_b, true, 1);
  upload_pair(ctx, w->tau_d, tau_dx_b, tau_dy_b);
  upload_bc(ctx, w, bc);
}

extern "C" int32_t ufe_assemble_linearised(ufe_ctx *ctx, const ufe_solver_params *p, const double *N_b,
                                           const double *dN_dx_b, const double *dN_dy_b,
                                           const double *basal_friction_coefficient_b, const double *tau_dx_b,
                                           const double *tau_dy_b, const double *u_b_prev, const double *v_b_prev,
                                           const ufe_bc_prescribed *bc, int32_t *ptr, int32_t *ind, double *val,
                                           double *bb, int64_t cap, int64_t *nnz_out) {
  return guarded(ctx, [&]() -> int32_t {
    validate_params(p);
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    upload_linearised_inputs(ctx, w, N_b, dN_dx_b, dN_dy_b, basal_friction_coefficient_b, tau_dx_b, tau_dy_b, bc);
    upload_pair(ctx, w->uv, u_b_prev, v_b_prev);   // the 'infinite_SSA_icestream' border rows read it
    Solver S(ctx, *p);
    CondArg none{0, 0};
    S.enqueue_assemble(kFromTriangles, false, none);
    check_err_flag(S);
    const int nTri = ctx->nTri, nrow = 2 * nTri;
    cudaStream_t s = ctx->stream;
    int32_t *rowlen = (int32_t *)dev_alloc(sizeof(int32_t) * (nrow + 1));
    int32_t *dptr = (int32_t *)dev_alloc(sizeof(int32_t) * (nrow + 1));
    UFE_CUDA(cudaMemsetAsync(rowlen, 0, sizeof(int32_t) * (nrow + 1), s));
    const DevCSR &m2 = ctx->ops[UFE_OP_M2_DDX_B_B];
    k_export_len<<<S.eblocks(nTri), kThreads, 0, s>>>(nTri, m2.ptr, ctx->TriBI, ctx->TriC, w->bc_mask, S.q,
                                                       ctx->perm_t, rowlen);
    UFE_CUDA(cudaGetLastError());
    std::vector<int32_t> hl(nrow + 1);
    UFE_CUDA(cudaMemcpyAsync(hl.data(), rowlen, sizeof(int32_t) * (nrow + 1), cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    std::vector<int32_t> hp(nrow + 1, 0);
    for (int i = 0; i < nrow; ++i) hp[i + 1] = hp[i] + hl[i];
    const int64_t nnz = hp[nrow];
    if (nnz_out) *nnz_out = nnz;
    int32_t rc = UFE_OK;
    if (nnz > cap || !ptr || !ind || !val || !bb) {
      rc = UFE_ERR_CAPACITY;
    } else {
      UFE_CUDA(cudaMemcpyAsync(dptr, hp.data(), sizeof(int32_t) * (nrow + 1), cudaMemcpyHostToDevice, s));
      int32_t *dind = (int32_t *)dev_alloc(sizeof(int32_t) * (nnz ? nnz : 1));
      double *dval = (double *)dev_alloc(sizeof(double) * (nnz ? nnz : 1));
      k_export_fill<<<S.eblocks(nTri), kThreads, 0, s>>>(nTri, m2.ptr, m2.ind, ctx->TriBI, ctx->TriC, w->bc_mask,
                                                         S.q, w->blk, ctx->perm_t, dptr, dind, dval);
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaMemcpyAsync(ind, dind, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaMemcpyAsync(val, dval, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      {
        std::vector<double> bu(nTri), bv(nTri);
        pair_to_external(ctx, bu.data(), bv.data(), w->kv.B);
        for (int t = 0; t < nTri; ++t) { bb[2 * t] = bu[t]; bb[2 * t + 1] = bv[t]; }
      }
      dev_free(dind);
      dev_free(dval);
      for (int i = 0; i <= nrow; ++i) ptr[i] = hp[i] + 1;
      for (int64_t k = 0; k < nnz; ++k) ind[k] += 1;
    }
    dev_free(rowlen);
    dev_free(dptr);
    return rc;
  });
}

extern "C" int32_t ufe_solve_linearised(ufe_ctx *ctx, const ufe_solver_params *p, double *u_b, double *v_b,
                                        const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                                        const double *basal_friction_coefficient_b, const double *tau_dx_b,
                                        const double *tau_dy_b, double *u_b_prev, double *v_b_prev,
                                        const ufe_bc_prescribed *bc, int32_t *n_Axb_its) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(u_b && v_b, UFE_ERR_INVALID, "null velocity arrays");
    validate_params(p);
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    const int nTri = ctx->nTri;
    if (u_b_prev) memcpy(u_b_prev, u_b, sizeof(double) * nTri);
    if (v_b_prev) memcpy(v_b_prev, v_b, sizeof(double) * nTri);
    upload_linearised_inputs(ctx, w, N_b, dN_dx_b, dN_dy_b, basal_friction_coefficient_b, tau_dx_b, tau_dy_b, bc);
    upload_pair(ctx, w->uv, u_b, v_b);
    Solver S(ctx, *p);
    CondArg none{0, 0};
    UFE_CUDA(cudaMemsetAsync(w->ks, 0, sizeof(KrylovScalars) * 3, S.s));
    S.enqueue_assemble(kFromTriangles, p->krylov_initial_guess == UFE_X0_CURRENT, none);
    for (;;) {
      if (p->precision == UFE_PREC_FP32_REFINE) {
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
        S.enqueue_inner_init(none);
        if (persistent_krylov() && S.ctx->allow_persistent) {
          S.enqueue_inner_persist();
        } else {
          for (;;) {
            for (int c = 0; c < 8; ++c) S.krylov_iter32(none);
            UFE_CUDA(cudaMemcpyAsync(w->ks_host + 1, w->ks + 1, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
            UFE_CUDA(cudaStreamSynchronize(S.s));
            if (!w->ks_host[1].active) break;
          }
        }
        S.enqueue_refine_update(none);
      } else if (S.pair_ok()) {
        S.run_pair_host();
        break;
      } else {
        for (int c = 0; c < 8; ++c) S.krylov_iter64(none);
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
      }
    }
    if (p->precision == UFE_PREC_FP32_REFINE) {
      S.enqueue_fallback_init(none);
      for (;;) {
        UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, S.s));
        UFE_CUDA(cudaStreamSynchronize(S.s));
        if (!w->ks_host[0].active) break;
        for (int c = 0; c < 8; ++c) S.krylov_iter64(none);
      }
    }
    check_err_flag(S);
    UFE_CUDA(cudaMemcpyAsync(w->ks_host, w->ks, sizeof(KrylovScalars) * 2, cudaMemcpyDeviceToHost, S.s));
    UFE_CUDA(cudaStreamSynchronize(S.s));
    download_pair(ctx, w->kv.X, u_b, v_b);
    if (n_Axb_its)
      *n_Axb_its = (p->precision == UFE_PREC_FP32_REFINE) ? w->ks_host[1].total_its + w->ks_host[0].total_its
                                                          : w->ks_host[0].total_its;
    return w->ks_host[0].status;
  });
}

// Mean microseconds per iteration of the persistent Krylov kernel (FP64 solve, double-word
// solve, or FP32 inner solve) on the system the last solve assembled.  The solve restarts from its usual
// initialisation (x = 0 for the FP64 solve; the current FP64 residual for the inner solve) with
// a zero tolerance, so the kernel runs `iterations` iterations unless the recurrence breaks down.
extern "C" int32_t ufe_profile_krylov_persistent(ufe_ctx *ctx, int32_t precision, int32_t iterations,
                                                 double *us_per_iteration) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(us_per_iteration && iterations >= 1, UFE_ERR_INVALID, "bad profile arguments");
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    UFE_REQUIRE(w->nnzb > 0, UFE_ERR_INVALID, "no assembled system: run a solve first");
    ufe_solver_params p;
    ufe_default_params(&p);
    p.precision = precision;
    p.krylov_max_it = iterations;
    p.krylov_inner_rtol = 1e-300;
    Solver S(ctx, p);
    const bool fp32 = precision == UFE_PREC_FP32_REFINE;
    const bool pair = precision == UFE_PREC_FP32_PAIR;
    UFE_REQUIRE(fp32 ? S.halo_ok() : pair ? S.pair_ok() : S.halo64_ok(), UFE_ERR_INVALID,
                "persistent Krylov kernel not in use");
    cudaStream_t s = S.s;
    CondArg none{0, 0};
    if (fp32) {
      S.enqueue_inner_init(none);
    } else {
      UFE_CUDA(cudaMemsetAsync(w->ks, 0, sizeof(KrylovScalars), s));   // no state of the last solve
      BsrMat<double, double, 1> m = S.mat64<1>();
      k_krylov_init<BsrMat<double, double, 1>><<<krylov_grid(m, kThreads, S.grid), kThreads, 0, s>>>(
          m, S.kv64(), w->ks, 0.0, 0.0, iterations, 1, ctx->red.partials, ctx->red.tickets, none, 0);
      UFE_CUDA(cudaGetLastError());
    }
    KrylovScalars *dks = w->ks + (fp32 ? 1 : 0);
    UFE_CUDA(cudaEventRecord(ctx->ev0, s));
    if (fp32) {
      k_reset_gsync<<<1, 1, 0, s>>>(w->gsync);
      S.inner_halo();
    } else if (pair) {
      S.pair_solve_once();   // conversions in and out included
    } else {
      S.enqueue_outer_halo64();
    }
    UFE_CUDA(cudaEventRecord(ctx->ev1, s));
    UFE_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    UFE_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    KrylovScalars out;
    UFE_CUDA(cudaMemcpy(&out, dks, sizeof(out), cudaMemcpyDeviceToHost));
    UFE_REQUIRE(out.it >= 1, UFE_ERR_DEVICE, "persistent Krylov kernel did not iterate");
    *us_per_iteration = 1000.0 * ms / out.it;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_profile_krylov_kernels(ufe_ctx *ctx, int32_t precision, int32_t repeats, double *us,
                                              int64_t *geometry) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(us && repeats >= 1, UFE_ERR_INVALID, "bad profile arguments");
    UFE_CUDA(cudaSetDevice(ctx->device));
    Work *w = ensure_work(ctx);
    ufe_solver_params p;
    ufe_default_params(&p);
    p.precision = precision;
    Solver S(ctx, p);
    // a live iteration state: the scalars stay active (ttol 0, huge rnorm0 and max_it), so every
    // launch does its full work
    KrylovScalars ks;
    memset(&ks, 0, sizeof(ks));
    ks.active = 1; ks.rho = 1.0; ks.rhoold = 1.0; ks.alpha = 0.5; ks.omega = 0.5; ks.omegaold = 0.5;
    ks.beta = 0.5; ks.ttol = 0.0; ks.rnorm0 = 1e300; ks.max_it = 1 << 30;
    KrylovScalars *dks = w->ks + (precision == UFE_PREC_FP32_REFINE ? 1 : 0);
    cudaStream_t s = S.s;
    auto time_kernel = [&](auto launch) -> double {
      UFE_CUDA(cudaMemcpyAsync(dks, &ks, sizeof(ks), cudaMemcpyHostToDevice, s));
      launch();
      UFE_CUDA(cudaEventRecord(ctx->ev0, s));
      for (int r = 0; r < repeats; ++r) launch();   // the scalars stay active: ttol 0, no max_it
      UFE_CUDA(cudaEventRecord(ctx->ev1, s));
      UFE_CUDA(cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      UFE_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      return 1000.0 * ms / repeats;
    };
    CondArg none{0, 0};
    auto run3 = [&](auto mat, auto v) {
      unsigned g = krylov_grid(mat, kThreads, S.grid);
      unsigned g2 = pick_blocks(mat.items, kThreads, S.grid);
      us[0] = time_kernel([&] { k_p_spmv<decltype(mat)><<<g, kThreads, 0, s>>>(mat, v, dks, ctx->red.partials, ctx->red.tickets); });
      us[1] = time_kernel([&] { k_s_spmv<decltype(mat)><<<g, kThreads, 0, s>>>(mat, v, dks, ctx->red.partials, ctx->red.tickets); });
      us[2] = time_kernel([&] { k_xr<decltype(mat)><<<g2, kThreads, 0, s>>>(mat, v, dks, ctx->red.partials, ctx->red.tickets, none); });
    };
    // the kernels read the matrix and vectors left by the last solve
    if (precision == UFE_PREC_FP32_REFINE) {
      switch (S.lanes) {
        case 1: run3(S.mat32<1>(), S.kv_inner()); break;
        case 2: run3(S.mat32<2>(), S.kv_inner()); break;
        case 8: run3(S.mat32<8>(), S.kv_inner()); break;
        default: run3(S.mat32<4>(), S.kv_inner()); break;
      }
    } else {
      switch (S.lanes) {
        case 1: run3(S.mat64<1>(), S.kv64()); break;
        case 2: run3(S.mat64<2>(), S.kv64()); break;
        case 8: run3(S.mat64<8>(), S.kv64()); break;
        default: run3(S.mat64<4>(), S.kv64()); break;
      }
    }
    UFE_CUDA(cudaGetLastError());
    UFE_CUDA(cudaMemsetAsync(w->ks, 0, sizeof(KrylovScalars) * 2, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    if (geometry) { geometry[0] = ctx->nTri; geometry[1] = w->nnzb; }
    return UFE_OK;
  });
}

// General CSR matrix-equation solve (solve_matrix_equation_CSR_PETSc): same BiCGStab kernels on
// scalar rows, host-checked every few iterations.
static uint64_t bits_of_double(double d) {
  uint64_t u;
  memcpy(&u, &d, sizeof(u));
  return u;
}

// inverse diagonal of a CSR matrix: the row's diagonal entries summed in storage order
__global__ void k_csr_dinv(int m, const int32_t *ptr, const int32_t *ind, const double *val, double *dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double d = 0.0;
  for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k)
    if (ind[k] == i) d += val[k];
  dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
}

void csr_scratch_alloc(CsrSolveScratch &scr, int64_t m) {
  scr.vec = (double *)dev_alloc(sizeof(double) * (size_t)m * 10);
  scr.ks = (KrylovScalars *)dev_alloc(sizeof(KrylovScalars));
  UFE_CUDA(cudaMallocHost(&scr.hks, sizeof(KrylovScalars)));
  scr.cap = m;
}

void csr_scratch_free(CsrSolveScratch &scr) {
  if (scr.graph) cudaGraphExecDestroy(scr.graph);
  dev_free(scr.vec);
  dev_free(scr.ks);
  if (scr.hks) cudaFreeHost(scr.hks);
  scr = CsrSolveScratch{};
}

int32_t solve_csr_device(ufe_ctx *ctx, const DevCSR &A, const double *b, double *x, double rtol, double abstol,
                         int32_t max_it, int32_t *its, CsrSolveScratch *scratch) {
  cudaStream_t s = ctx->stream;
  const int m = A.m;
  CsrSolveScratch own;
  const bool owned = !(scratch && scratch->cap >= m);
  if (owned) csr_scratch_alloc(own, m);
  CsrSolveScratch &scr = owned ? own : *scratch;
  double *vec = scr.vec;
  KrylovScalars *ks = scr.ks;
  KrylovScalars *hks = scr.hks;
  int32_t status = UFE_OK;
  try {
    double *dinv = vec, *R = vec + m, *RP = R + m, *S = RP + m, *T = S + m, *P0 = T + m, *P1 = P0 + m,
           *V0 = P1 + m, *V1 = V0 + m;
    const char *ng = getenv("UFE_NO_GRAPH");
    if (!owned && !(ng && *ng && *ng != '0')) {
      // a caller that solves repeatedly on the same buffers: the whole solve as one graph, its
      // iteration loop a conditional while-node that k_xr keeps open (built once per buffers,
      // sizes and tolerances; the host waits once, at the end)
      uint64_t key = 1469598103934665603ull;
      const uint64_t parts[] = {(uint64_t)(uintptr_t)A.ptr, (uint64_t)(uintptr_t)A.ind, (uint64_t)(uintptr_t)A.val,
                                (uint64_t)(uintptr_t)b, (uint64_t)(uintptr_t)x, (uint64_t)m, (uint64_t)A.nnz,
                                (uint64_t)bits_of_double(rtol), (uint64_t)bits_of_double(abstol),
                                (uint64_t)max_it};
      for (uint64_t q : parts) { key ^= q; key *= 1099511628211ull; }
      if (!scr.graph || scr.key != key) {
        if (scr.graph) { cudaGraphExecDestroy(scr.graph); scr.graph = nullptr; }
        cudaGraph_t g;
        UFE_CUDA(cudaGraphCreate(&g, 0));
        try {
          cudaGraphConditionalHandle h;
          UFE_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
          const CondArg cond{h, 1};
          using M1 = CsrMat;
          M1 mat{m, A.ptr, A.ind, A.val};
          KV<double> v;
          v.X = x; v.R = R; v.RP = RP; v.S = S; v.T = T; v.B = const_cast<double *>(b); v.dinv = dinv;
          v.P[0] = P0; v.P[1] = P1; v.V[0] = V0; v.V[1] = V1;
          const unsigned gk = krylov_grid(mat, kThreads, max_grid(ctx));
          auto deps = capture_into(s, g, {}, [&]() {
            k_csr_dinv<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, A.ptr, A.ind, A.val, dinv);
            UFE_CUDA(cudaMemsetAsync(ks, 0, sizeof(KrylovScalars), s));
            k_krylov_init<M1><<<gk, kThreads, 0, s>>>(mat, v, ks, rtol, abstol, max_it, 0, ctx->red.partials,
                                                      ctx->red.tickets, cond);
            UFE_CUDA(cudaGetLastError());
          });
          cudaGraph_t body;
          add_while(g, deps, h, &body);
          const unsigned gu = (unsigned)pick_blocks(m, kThreads, kMaxReduceBlocks);
          capture_into(s, body, {}, [&]() {   // p and s row by row, then the SpMVs gather them
            k_p_update<double><<<gu, kThreads, 0, s>>>(m, v, ks);
            k_p_spmv<M1><<<gk, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, 1);
            k_s_update<double><<<gu, kThreads, 0, s>>>(m, v, ks);
            k_s_spmv<M1><<<gk, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, 1);
            k_xr<M1><<<gk, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, cond);
            UFE_CUDA(cudaGetLastError());
          });
          UFE_CUDA(cudaGraphInstantiate(&scr.graph, g, 0));
        } catch (...) {
          cudaGraphDestroy(g);
          throw;
        }
        UFE_CUDA(cudaGraphDestroy(g));
        scr.key = key;
      }
      UFE_CUDA(cudaGraphLaunch(scr.graph, s));
      UFE_CUDA(cudaMemcpyAsync(hks, ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      *its = hks->it;
      return hks->status;
    }
    // Jacobi diagonal (PCJACOBI: 1 where the diagonal is zero)
    k_csr_dinv<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, A.ptr, A.ind, A.val, dinv);
    UFE_CUDA(cudaMemsetAsync(ks, 0, sizeof(KrylovScalars), s));
    CsrMat mat{m, A.ptr, A.ind, A.val};
    KV<double> v;
    v.X = x; v.R = R; v.RP = RP; v.S = S; v.T = T; v.B = const_cast<double *>(b); v.dinv = dinv;
    v.P[0] = P0; v.P[1] = P1; v.V[0] = V0; v.V[1] = V1;
    const int grid = max_grid(ctx);
    CondArg none{0, 0};
    k_krylov_init<CsrMat><<<krylov_grid(mat, kThreads, grid), kThreads, 0, s>>>(
        mat, v, ks, rtol, abstol, max_it, 0, ctx->red.partials, ctx->red.tickets, none);
    UFE_CUDA(cudaGetLastError());
    for (;;) {
      const unsigned gu = (unsigned)pick_blocks(m, kThreads, kMaxReduceBlocks);
      for (int c = 0; c < 8; ++c) {
        unsigned g = krylov_grid(mat, kThreads, grid);
        k_p_update<double><<<gu, kThreads, 0, s>>>(m, v, ks);
        k_p_spmv<CsrMat><<<g, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, 1);
        k_s_update<double><<<gu, kThreads, 0, s>>>(m, v, ks);
        k_s_spmv<CsrMat><<<g, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, 1);
        k_xr<CsrMat><<<g, kThreads, 0, s>>>(mat, v, ks, ctx->red.partials, ctx->red.tickets, none);
      }
      UFE_CUDA(cudaGetLastError());
      UFE_CUDA(cudaMemcpyAsync(hks, ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
      UFE_CUDA(cudaStreamSynchronize(s));
      if (!hks->active) break;
    }
    *its = hks->it;
    status = hks->status;
  } catch (...) {
    cudaStreamSynchronize(s);
    if (owned) csr_scratch_free(own);
    throw;
  }
  if (owned) csr_scratch_free(own);
  return status;
}
