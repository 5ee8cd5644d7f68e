// Ice thickness update (conservation of mass) on the GPU: calc_dHi_dt
// (src/UFEMISM/ice_dynamics/conservation_of_mass/conservation_of_mass_main.f90:23-109) with the
// explicit scheme (conservation_of_mass_explicit.f90:22-134, border rule :136-283) and the
// semi-implicit scheme (conservation_of_mass_semiimplicit.f90:23-174, matrix conditions :176-314).
//
// The work runs in the context's internal (Z-ordered) vertex numbering, on its renumbered mesh
// arrays; every row keeps the reference's add_entry layout -- the diagonal, then the connections
// C(vi, 1:nC) in the caller's order, which the renumbering keeps -- so the values are those of
// the caller's numbering and an export only renames rows and columns.  Fields cross the ABI
// through a staging buffer and one gather per array.  One thread per vertex row:
//   k_divq_matrix   M_divQ (calc_ice_flux_divergence_matrix_upwind, conservation_of_mass_utilities.f90:22-132),
//                   the edge velocity of map_velocities_from_b_to_c_2D (map_velocities_to_c_grid.f90:17-69)
//                   read through the precomputed triangle pair of each connection;
//   k_rate          divQ = M_divQ H in row order, dH/dt, and the flux-limited time step's minimum
//                   (calc_flux_limited_timestep, :158-204) as an atomic minimum on the bit patterns
//                   of non-negative doubles (exact and order-free);
//   k_step          H(t+dt) = max(0, H + dH/dt dt) with dt = min(dt, max(dt_ice_min, limit));
//   k_border        one pass of apply_ice_thickness_BC_explicit over the border vertices, reading
//                   the surface elevations as they stood before the pass;
//   k_semi_system   the semi-implicit stiffness row, load vector and initial guess with the
//                   border / prescribed / no-ice rows applied in the reference's order.
// Every expression keeps the reference's operation order, and the library is built without FMA
// contraction, so the explicit step and the assembled system are bit-identical to the oracle's.
// The semi-implicit matrix equation goes to the library's CSR BiCGStab/Jacobi.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ufe_internal.cuh"

constexpr double kIceDensityM = 910.0;        // parameters.f90:23
constexpr double kSeawaterDensityM = 1028.0;  // parameters.f90:25

struct MassWork {
  int32_t nV = 0, nTri = 0, nC_mem = 0;
  int64_t nnz = 0;
  double *A = nullptr, *Cw = nullptr;          // Voronoi areas, connection widths (nV x nC_mem)
  int2 *ct = nullptr;                           // triangles of each connection's edge (nV x nC_mem)
  double *Dc = nullptr;                         // connection lengths D (nV x nC_mem), once per mesh
  int32_t *ptr = nullptr, *ind = nullptr;       // M_divQ pattern, 0-based
  double *valM = nullptr, *valA = nullptr;
  // inputs (nV unless noted)
  double *Hi = nullptr, *Hb = nullptr, *SL = nullptr, *u = nullptr, *v = nullptr;   // u, v: nTri
  double *SMB = nullptr, *BMB = nullptr, *LMB = nullptr, *fm = nullptr, *target = nullptr;
  double *prHi = nullptr, *dprev = nullptr;
  int32_t *noice = nullptr, *prmask = nullptr;
  // outputs and scratch
  double *dHdt = nullptr, *Hit = nullptr, *divQ = nullptr, *AMB = nullptr;
  double *dex = nullptr, *Hex = nullptr, *qex = nullptr, *aex = nullptr;
  double *Hs = nullptr, *Hs_tot = nullptr, *bb = nullptr;
  int32_t *nint = nullptr;
  double *dt = nullptr;                         // [0] dt of the scheme, [1] the explicit part's
  unsigned long long *dtlim = nullptr;          // [0], [1]: bit patterns of the limits
  int32_t *flag = nullptr;                      // negative thickness found
  CsrSolveScratch krylov;                       // the semi-implicit solve's work vectors
  double *stage = nullptr;                      // max(nV, nTri): fields in the caller's order
  int32_t *stagei = nullptr;                    // nV
};

namespace {

__device__ __forceinline__ double opt(const double *a, int64_t i, double d) { return a ? a[i] : d; }

// dst[c*n + i] = src[c*n + map[i]] (caller -> internal with perm, internal -> caller with iperm)
template <class T>
__global__ void k_permute(int64_t n, int ncols, const T *__restrict__ src, const int32_t *__restrict__ map,
                          T *__restrict__ dst) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * ncols) return;
  const int64_t c = e / n, i = e - c * n;
  dst[e] = src[c * n + map[i]];
}

__device__ __forceinline__ double surface_elevation(double Hi, double Hb, double SL) {
  return Hi + fmax(SL - kIceDensityM / kSeawaterDensityM * Hi, Hb);   // ice_geometry_basics.f90:28-41
}
__device__ __forceinline__ double thickness_from_surface(double Hb, double Hs, double SL) {   // :58-82
  const double Hi_float = fmax(0.0, (SL - Hb) * (kSeawaterDensityM / kIceDensityM));
  const double Hs_float = Hb + Hi_float;
  if (Hs > Hs_float) return Hs - Hb;
  return fmin(Hi_float, (Hs - SL) / (1.0 - (kIceDensityM / kSeawaterDensityM)));
}

// the triangles of the edge from vi to each neighbour (the ones among iTri(vi, :) holding vj),
// and the connection length D = sqrt(D_x^2 + D_y^2) (mesh_secondary.f90:333-339)
__global__ void k_conn_tris(int nV, int nTri, int nC_mem, const double *V, const int32_t *nC, const int32_t *C,
                            const int32_t *niTri, const int32_t *iTri, const int32_t *Tri, int2 *ct, double *Dc) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  for (int ci = 0; ci < nC_mem; ++ci) {
    int2 r = make_int2(-1, -1);
    double D = 0.0;
    if (ci < nC[vi]) {
      const int vj = C[(int64_t)ci * nV + vi] - 1;
      const double Dx = V[vj] - V[vi], Dy = V[nV + vj] - V[nV + vi];
      D = sqrt(Dx * Dx + Dy * Dy);
      for (int k = 0; k < niTri[vi]; ++k) {
        const int t = iTri[(int64_t)k * nV + vi] - 1;
        for (int q = 0; q < 3; ++q)
          if (Tri[(int64_t)q * nTri + t] - 1 == vj) {
            if (r.x < 0) r.x = t; else r.y = t;
          }
      }
    }
    ct[(int64_t)ci * nV + vi] = r;
    Dc[(int64_t)ci * nV + vi] = D;
  }
}

struct MeshRef {
  int nV, nTri;
  const double *V;
  const int32_t *nC, *C, *VBI;
};

// The zero half of max(0, u_perp) / min(0, u_perp) is not divided: 0 / A_i is +0, and c0 + 0 is c0,
// so skipping it leaves every value as the reference's expression gives it.
__global__ void k_divq_matrix(MeshRef m, const double *A, const double *Cw, const int2 *ct, const double *Dc,
                              const double *u, const double *v, const double *fm, const int32_t *ptr, double *val) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= m.nV) return;
  const int nV = m.nV;
  const int64_t k0 = ptr[vi];
  const double A_i = A[vi];
  const double xi = m.V[vi], yi = m.V[nV + vi];
  const bool out_i = opt(fm, vi, 1.0) >= 1.0;
  double c0 = 0.0;
  for (int ci = 0; ci < m.nC[vi]; ++ci) {
    const int64_t cix = (int64_t)ci * nV + vi;
    const int vj = m.C[cix] - 1;
    const int2 t = ct[cix];
    double uc, vc;
    if (t.y < 0) {
      uc = u[t.x];
      vc = v[t.x];
    } else {
      uc = (u[t.x] + u[t.y]) / 2.0;
      vc = (v[t.x] + v[t.y]) / 2.0;
    }
    const double L_c = Cw[cix];
    const double Dx = m.V[vj] - xi, Dy = m.V[nV + vj] - yi;
    const double D = Dc[cix];
    const double u_perp = uc * Dx / D + vc * Dy / D;
    if (out_i && u_perp > 0.0) c0 = c0 + L_c * u_perp / A_i;
    val[k0 + 1 + ci] = (u_perp < 0.0 && opt(fm, vj, 1.0) >= 1.0) ? L_c * u_perp / A_i : 0.0;
  }
  val[k0] = c0;
}

struct Inputs {
  const double *Hi, *Hb, *SL, *SMB, *BMB, *LMB, *fm, *target, *prHi, *dprev;
  const int32_t *noice, *prmask;
};

__device__ __forceinline__ double mass_balance(const Inputs &in, int vi) {
  return opt(in.fm, vi, 1.0) * (opt(in.SMB, vi, 0.0) + opt(in.BMB, vi, 0.0) - opt(in.target, vi, 0.0));
}

// divQ, dH/dt (= AMB before the limits) and the time-step limit of every thinning vertex; the
// limits' minimum per block first (one atomic per block: contended per-vertex atomics on one
// address serialise), on the bit patterns, which order non-negative doubles as their values
__global__ void __launch_bounds__(256) k_rate(int nV, const int32_t *ptr, const int32_t *ind, const double *val,
                                              Inputs in, double Hi_min, double *divQ, double *dHdt, double *AMB,
                                              unsigned long long *dtlim) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lim_bits = ~0ull;
  if (vi < nV) {
    double q = 0.0;
    for (int32_t k = ptr[vi]; k < ptr[vi + 1]; ++k) q = q + val[k] * in.Hi[ind[k]];
    divQ[vi] = q;
    const double r = -q + mass_balance(in, vi) + opt(in.LMB, vi, 0.0);
    dHdt[vi] = r;
    AMB[vi] = r;
    if (in.Hi[vi] > Hi_min && r < 0.0) {
      const double lim = in.Hi[vi] / fmax(r, 1e-9);   // as written: a thinning rate gives Hi / 1e-9
      lim_bits = (unsigned long long)__double_as_longlong(lim);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, lim_bits, o);
    lim_bits = other < lim_bits ? other : lim_bits;
  }
  __shared__ unsigned long long wmin[8];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = lim_bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = wmin[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) b = wmin[w] < b ? wmin[w] : b;
    if (b != ~0ull) atomicMin(dtlim, b);
  }
}

__global__ void k_step(int nV, const double *Hi, const double *dHdt, double *dt, const unsigned long long *dtlim,
                       double dt_ice_min, const double *Hb, const double *SL, double *Hit, double *Hs) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  // calc_flux_limited_timestep's minimum, floored at dt_ice_min; dt = min(dt, dt_max).  Thread 0
  // stores it back; a thread that reads the stored value gets the same dt (min is idempotent).
  const double dt_eff = fmin(*dt, fmax(dt_ice_min, __longlong_as_double((long long)*dtlim)));
  if (vi == 0) *dt = dt_eff;
  if (vi >= nV) return;
  const double h = fmax(0.0, Hi[vi] + dHdt[vi] * dt_eff);
  Hit[vi] = h;
  Hs[vi] = surface_elevation(h, Hb[vi], SL[vi]);
}

__global__ void k_surface(int nV, const double *H, const double *Hb, const double *SL, double *Hs) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi < nV) Hs[vi] = surface_elevation(H[vi], Hb[vi], SL[vi]);
}

// calc_n_interior_neighbours (conservation_of_mass_utilities.f90:206-234)
__global__ void k_interior_neighbours(MeshRef m, const int32_t *noice, int32_t *nint) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= m.nV) return;
  int n = 0;
  for (int ci = 0; ci < m.nC[vi]; ++ci) {
    const int vj = m.C[(int64_t)ci * m.nV + vi] - 1;
    if (m.VBI[vj] == 0 && !(noice && noice[vj])) ++n;
  }
  nint[vi] = n;
}

__device__ __forceinline__ int border_bc(int vbi, int4 bc) {   // (west, east, south, north)
  if (vbi == 1 || vbi == 2) return bc.w;
  if (vbi == 3 || vbi == 4) return bc.y;
  if (vbi == 5 || vbi == 6) return bc.z;
  if (vbi == 7 || vbi == 8) return bc.x;
  return -1;
}

// One pass of apply_ice_thickness_BC_explicit: pass 0 sets border vertices with interior
// neighbours to their interior neighbours' mean surface, pass 1 those without to all
// neighbours' mean; 'zero' borders get no ice in both.  Hs_tot is the pass's starting copy.
__global__ void k_border(MeshRef m, int pass, int4 bc, const int32_t *noice, const int32_t *nint, const double *Hb,
                         const double *SL, const double *Hs_tot, double *Hs, double *H) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= m.nV) return;
  const int b = border_bc(m.VBI[vi], bc);
  if (b < 0) return;
  if (b == UFE_BC_H_ZERO) {
    H[vi] = 0.0;
    return;
  }
  const int n = nint[vi];
  if ((pass == 0) != (n > 0)) return;
  double s = 0.0;
  for (int ci = 0; ci < m.nC[vi]; ++ci) {
    const int vj = m.C[(int64_t)ci * m.nV + vi] - 1;
    if (pass == 1 || (m.VBI[vj] == 0 && !(noice && noice[vj]))) s = s + Hs_tot[vj];
  }
  const double av = s / (double)(pass == 0 ? n : m.nC[vi]);
  const double hs = fmax(Hb[vi], av);
  Hs[vi] = hs;
  H[vi] = thickness_from_surface(Hb[vi], hs, SL[vi]);
}

// the rest of calc_dHi_dt_explicit: prescribed thickness, no-ice mask, dH/dt and AMB
__global__ void k_explicit_finish(int nV, Inputs in, const double *dt, double *Hit, double *dHdt, double *AMB) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  double h = Hit[vi];
  if (in.prmask && in.prmask[vi] == 1) h = fmax(0.0, in.prHi[vi]);
  if (in.noice && in.noice[vi]) h = 0.0;
  Hit[vi] = h;
  const double r = (h - in.Hi[vi]) / *dt;
  dHdt[vi] = r;
  AMB[vi] = r - AMB[vi];
}

// calc_dHi_dt_semiimplicit's stiffness row, load vector and initial guess, then
// apply_ice_thickness_BC_matrix: border rows (the explicit solution), prescribed rows, no-ice rows
__global__ void k_semi_system(MeshRef m, const int32_t *ptr, const int32_t *ind, const double *valM, Inputs in,
                              double dt, double fs, const double *Hex, double *valA, double *bb, double *x0,
                              double *divQ) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= m.nV) return;
  const int32_t k1 = ptr[vi], k2 = ptr[vi + 1];
  double q = 0.0;
  for (int32_t k = k1; k < k2; ++k) q = q + valM[k] * in.Hi[ind[k]];
  divQ[vi] = q;
  const double Hi = in.Hi[vi];
  double b = Hi - (dt * (1.0 - fs) * q) + fmax(-1.0 * Hi, dt * (mass_balance(in, vi) + opt(in.LMB, vi, 0.0)));
  double x = Hi + dt * opt(in.dprev, vi, 0.0);
  bool ident = false;
  if (m.VBI[vi] > 0) { ident = true; b = Hex[vi]; x = Hex[vi]; }
  if (in.prmask && in.prmask[vi] == 1) { ident = true; b = in.prHi[vi]; x = in.prHi[vi]; }
  if (in.noice && in.noice[vi]) { ident = true; b = 0.0; x = 0.0; }
  for (int32_t k = k1; k < k2; ++k) {
    const bool diag = ind[k] == vi;
    valA[k] = ident ? (diag ? 1.0 : 0.0) : (diag ? valM[k] * dt * fs + 1.0 : valM[k] * dt * fs);
  }
  bb[vi] = b;
  x0[vi] = x;
}

__global__ void k_semi_finish(int nV, const double *Hi, double dt, const double *Hit, double *dHdt, double *AMB) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  const double a = (Hit[vi] - Hi[vi]) / dt;
  const double r = (Hit[vi] - Hi[vi]) / dt;
  dHdt[vi] = r;
  AMB[vi] = r - a;
}

// calc_dHi_dt after the scheme: negative thickness to zero (and the reference's warning), AMB, dH/dt
__global__ void k_main_finish(int nV, const double *Hi, const double *dt, double Hi_min, double *Hit, double *dHdt,
                              double *AMB, int32_t *flag) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  double h = Hit[vi];
  if (h < 0.0) {
    if (h < -0.1 && Hi[vi] > Hi_min) atomicOr(flag, 1);
    h = 0.0;
  }
  Hit[vi] = h;
  const double d = *dt;
  AMB[vi] = AMB[vi] + (h - Hi[vi]) / d - dHdt[vi];
  dHdt[vi] = (h - Hi[vi]) / d;
}

__global__ void k_none(int nV, const double *Hi, double *Hit, double *dHdt, double *AMB) {
  const int vi = blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nV) return;
  Hit[vi] = Hi[vi];
  dHdt[vi] = 0.0;
  AMB[vi] = 0.0;
}

__global__ void k_set_limit(unsigned long long *dtlim, double v) {
  *dtlim = (unsigned long long)__double_as_longlong(v);
}

unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

MassWork *mass_work(ufe_ctx *ctx) {
  UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "ice thickness: upload a mesh first");
  UFE_REQUIRE(ctx->mass && ctx->mass->A, UFE_ERR_INVALID,
              "ice thickness: upload the mesh's Voronoi areas and connection widths first");
  return ctx->mass;
}

template <class T>
T *alloc_n(size_t n) { return (T *)dev_alloc(sizeof(T) * (n ? n : 1)); }

void alloc_fields(MassWork *w) {
  const size_t nV = w->nV, nT = w->nTri;
  double **vs[] = {&w->Hi, &w->Hb, &w->SL, &w->SMB, &w->BMB, &w->LMB, &w->fm, &w->target, &w->prHi, &w->dprev,
                   &w->dHdt, &w->Hit, &w->divQ, &w->AMB, &w->dex, &w->Hex, &w->qex, &w->aex, &w->Hs, &w->Hs_tot,
                   &w->bb};
  for (double **p : vs) *p = alloc_n<double>(nV);
  w->u = alloc_n<double>(nT);
  w->v = alloc_n<double>(nT);
  w->noice = alloc_n<int32_t>(nV);
  w->prmask = alloc_n<int32_t>(nV);
  w->nint = alloc_n<int32_t>(nV);
  w->dt = alloc_n<double>(2);
  w->dtlim = alloc_n<unsigned long long>(2);
  w->flag = alloc_n<int32_t>(1);
  w->valM = alloc_n<double>(w->nnz);
  w->valA = alloc_n<double>(w->nnz);
  csr_scratch_alloc(w->krylov, w->nV);
  w->stage = alloc_n<double>(std::max(nV, nT));
  w->stagei = alloc_n<int32_t>(nV);
}

MeshRef mesh_ref(ufe_ctx *ctx) { return MeshRef{ctx->nV, ctx->nTri, ctx->V, ctx->nC, ctx->C, ctx->VBI}; }

// upload the fields the caller gave, in the internal numbering; returns the device-side view
// (null where not given)
Inputs upload_inputs(ufe_ctx *ctx, MassWork *w, const ufe_thickness_fields *f) {
  cudaStream_t s = ctx->stream;
  const size_t nV = w->nV, nT = w->nTri;
  auto up = [&](double *d, const double *h, bool tri) -> const double * {
    if (!h) return nullptr;
    const size_t n = tri ? nT : nV;
    UFE_CUDA(cudaMemcpyAsync(w->stage, h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    k_permute<double><<<blocks(n), 256, 0, s>>>((int64_t)n, 1, w->stage, tri ? ctx->perm_t : ctx->perm_v, d);
    return d;
  };
  auto upi = [&](int32_t *d, const int32_t *h) -> const int32_t * {
    if (!h) return nullptr;
    UFE_CUDA(cudaMemcpyAsync(w->stagei, h, sizeof(int32_t) * nV, cudaMemcpyHostToDevice, s));
    k_permute<int32_t><<<blocks(nV), 256, 0, s>>>((int64_t)nV, 1, w->stagei, ctx->perm_v, d);
    return d;
  };
  Inputs in;
  in.Hi = up(w->Hi, f->Hi, false);
  in.Hb = up(w->Hb, f->Hb, false);
  in.SL = up(w->SL, f->SL, false);
  up(w->u, f->u_vav_b, true);
  up(w->v, f->v_vav_b, true);
  in.SMB = up(w->SMB, f->SMB, false);
  in.BMB = up(w->BMB, f->BMB, false);
  in.LMB = up(w->LMB, f->LMB, false);
  in.fm = up(w->fm, f->fraction_margin, false);
  in.target = up(w->target, f->dHi_dt_target, false);
  in.prHi = up(w->prHi, f->BC_prescr_Hi, false);
  in.dprev = up(w->dprev, f->dHi_dt, false);
  in.noice = upi(w->noice, f->mask_noice);
  in.prmask = upi(w->prmask, f->BC_prescr_mask);
  return in;
}

void check_inputs(const ufe_thickness_params *p, const ufe_thickness_fields *f) {
  UFE_REQUIRE(p && f, UFE_ERR_INVALID, "ice thickness: null parameters or fields");
  UFE_REQUIRE(p->choice_ice_integration_method >= UFE_DHI_NONE &&
                  p->choice_ice_integration_method <= UFE_DHI_SEMIIMPLICIT,
              UFE_ERR_INVALID, "unknown choice_ice_integration_method");
  const int32_t bcs[4] = {p->BC_H_west, p->BC_H_east, p->BC_H_south, p->BC_H_north};
  for (int32_t b : bcs)
    UFE_REQUIRE(b == UFE_BC_H_ZERO || b == UFE_BC_H_INFINITE, UFE_ERR_INVALID, "unknown BC_H (zero or infinite)");
  UFE_REQUIRE(f->Hi && f->Hb && f->SL && f->u_vav_b && f->v_vav_b, UFE_ERR_INVALID,
              "ice thickness: Hi, Hb, SL, u_vav_b and v_vav_b are required");
  UFE_REQUIRE((f->BC_prescr_mask == nullptr) == (f->BC_prescr_Hi == nullptr), UFE_ERR_INVALID,
              "need to provide prescribed both Hi and mask");
  UFE_REQUIRE(p->dHi_PETSc_max_it >= 1 && p->dHi_PETSc_rtol >= 0.0 && p->dHi_PETSc_abstol >= 0.0, UFE_ERR_INVALID,
              "ice thickness: bad Krylov tolerances");
}

// calc_dHi_dt_explicit on the device into (dHdt, Hit, divQ, AMB); dt at dt_slot is shortened
void run_explicit(ufe_ctx *ctx, MassWork *w, const ufe_thickness_params *p, const Inputs &in, int dt_slot,
                  double *dHdt, double *Hit, double *divQ, double *AMB) {
  cudaStream_t s = ctx->stream;
  const int nV = w->nV;
  const MeshRef m = mesh_ref(ctx);
  const int4 bc = make_int4(p->BC_H_west, p->BC_H_east, p->BC_H_south, p->BC_H_north);
  k_set_limit<<<1, 1, 0, s>>>(w->dtlim + dt_slot, p->dt_ice_max);
  k_rate<<<blocks(nV), 256, 0, s>>>(nV, w->ptr, w->ind, w->valM, in, p->Hi_min, divQ, dHdt, AMB, w->dtlim + dt_slot);
  k_step<<<blocks(nV), 256, 0, s>>>(nV, in.Hi, dHdt, w->dt + dt_slot, w->dtlim + dt_slot, p->dt_ice_min, in.Hb, in.SL,
                                    Hit, w->Hs);
  for (int pass = 0; pass < 2; ++pass) {
    UFE_CUDA(cudaMemcpyAsync(w->Hs_tot, w->Hs, sizeof(double) * nV, cudaMemcpyDeviceToDevice, s));
    k_border<<<blocks(nV), 256, 0, s>>>(m, pass, bc, in.noice, w->nint, in.Hb, in.SL, w->Hs_tot, w->Hs, Hit);
  }
  k_explicit_finish<<<blocks(nV), 256, 0, s>>>(nV, in, w->dt + dt_slot, Hit, dHdt, AMB);
  UFE_CUDA(cudaGetLastError());
}

// the semi-implicit system (valA, bb, x0) for step dt; x0 is the initial guess
void semi_system(ufe_ctx *ctx, MassWork *w, const ufe_thickness_params *p, const Inputs &in, double dt, double *x0) {
  cudaStream_t s = ctx->stream;
  const int nV = w->nV;
  const MeshRef m = mesh_ref(ctx);
  const int4 bc = make_int4(p->BC_H_west, p->BC_H_east, p->BC_H_south, p->BC_H_north);
  UFE_CUDA(cudaMemcpyAsync(w->dt + 1, &dt, sizeof(double), cudaMemcpyHostToDevice, s));
  run_explicit(ctx, w, p, in, 1, w->dex, w->Hex, w->qex, w->aex);
  // apply_ice_thickness_BC_matrix_domain_border applies the border rule to the explicit solution again
  k_surface<<<blocks(nV), 256, 0, s>>>(nV, w->Hex, in.Hb, in.SL, w->Hs);
  for (int pass = 0; pass < 2; ++pass) {
    UFE_CUDA(cudaMemcpyAsync(w->Hs_tot, w->Hs, sizeof(double) * nV, cudaMemcpyDeviceToDevice, s));
    k_border<<<blocks(nV), 256, 0, s>>>(m, pass, bc, in.noice, w->nint, in.Hb, in.SL, w->Hs_tot, w->Hs, w->Hex);
  }
  k_semi_system<<<blocks(nV), 256, 0, s>>>(m, w->ptr, w->ind, w->valM, in, dt, p->dHi_semiimplicit_fs, w->Hex,
                                           w->valA, w->bb, x0, w->divQ);
  UFE_CUDA(cudaGetLastError());
}

// an internal vertex field into the caller's host array
void download_vertex(ufe_ctx *ctx, MassWork *w, double *h, const double *d) {
  cudaStream_t s = ctx->stream;
  k_permute<double><<<blocks(w->nV), 256, 0, s>>>(w->nV, 1, d, ctx->iperm_v, w->stage);
  UFE_CUDA(cudaMemcpyAsync(h, w->stage, sizeof(double) * w->nV, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));   // the staging buffer is reused by the next field
}

void prepare(ufe_ctx *ctx, MassWork *w, const ufe_thickness_params *p, const Inputs &in) {
  cudaStream_t s = ctx->stream;
  const int nV = w->nV;
  const MeshRef m = mesh_ref(ctx);
  k_divq_matrix<<<blocks(nV), 256, 0, s>>>(m, w->A, w->Cw, w->ct, w->Dc, w->u, w->v, in.fm, w->ptr, w->valM);
  k_interior_neighbours<<<blocks(nV), 256, 0, s>>>(m, in.noice, w->nint);
  UFE_CUDA(cudaGetLastError());
  (void)p;
}

}  // namespace

void free_mass(ufe_ctx *ctx) {
  MassWork *w = ctx->mass;
  if (!w) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  void *ptrs[] = {w->A, w->Cw, w->ct, w->Dc, w->ptr, w->ind, w->valM, w->valA, w->Hi, w->Hb, w->SL, w->u, w->v,
                  w->SMB, w->BMB, w->LMB, w->fm, w->target, w->prHi, w->dprev, w->noice, w->prmask, w->dHdt,
                  w->Hit, w->divQ, w->AMB, w->dex, w->Hex, w->qex, w->aex, w->Hs, w->Hs_tot, w->bb, w->nint,
                  w->dt, w->dtlim, w->flag, w->stage, w->stagei};
  for (void *q : ptrs) dev_free(q);
  csr_scratch_free(w->krylov);
  delete w;
  ctx->mass = nullptr;
}

extern "C" void ufe_default_thickness_params(ufe_thickness_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->choice_ice_integration_method = UFE_DHI_SEMIIMPLICIT;
  p->BC_H_west = p->BC_H_east = p->BC_H_south = p->BC_H_north = UFE_BC_H_ZERO;
  p->dHi_PETSc_max_it = 10000;
  p->dHi_semiimplicit_fs = 1.5;
  p->dHi_PETSc_rtol = 1e-8;
  p->dHi_PETSc_abstol = 1e-6;
  p->dt_ice_max = 10.0;
  p->dt_ice_min = 0.1;
  p->Hi_min = 0.0;
}

extern "C" int32_t ufe_mesh_voronoi_upload(ufe_ctx *ctx, const double *A, const double *Cw) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "upload a mesh first");
    UFE_REQUIRE(A && Cw, UFE_ERR_INVALID, "null Voronoi arrays");
    UFE_CUDA(cudaSetDevice(ctx->device));
    free_mass(ctx);
    cudaStream_t s = ctx->stream;
    MassWork *w = new MassWork;
    ctx->mass = w;
    w->nV = ctx->nV;
    w->nTri = ctx->nTri;
    w->nC_mem = ctx->nC_mem;
    const size_t nc = (size_t)w->nV * w->nC_mem;
    for (int64_t i = 0; i < w->nV; ++i)
      UFE_REQUIRE(A[i] > 0.0 && std::isfinite(A[i]), UFE_ERR_INVALID, "Voronoi cell areas must be positive");
    w->A = alloc_n<double>(w->nV);
    w->Cw = alloc_n<double>(nc);
    w->ct = alloc_n<int2>(nc);
    w->Dc = alloc_n<double>(nc);
    double *tmp = alloc_n<double>(nc);   // the caller's order, then gathered into the internal one
    UFE_CUDA(cudaMemcpyAsync(tmp, A, sizeof(double) * w->nV, cudaMemcpyHostToDevice, s));
    k_permute<double><<<blocks(w->nV), 256, 0, s>>>(w->nV, 1, tmp, ctx->perm_v, w->A);
    UFE_CUDA(cudaMemcpyAsync(tmp, Cw, sizeof(double) * nc, cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    k_permute<double><<<blocks((int64_t)nc), 256, 0, s>>>(w->nV, w->nC_mem, tmp, ctx->perm_v, w->Cw);
    UFE_CUDA(cudaStreamSynchronize(s));
    dev_free(tmp);
    k_conn_tris<<<blocks(w->nV), 256, 0, s>>>(w->nV, w->nTri, w->nC_mem, ctx->V, ctx->nC, ctx->C, ctx->niTri,
                                              ctx->iTri, ctx->Tri, w->ct, w->Dc);
    UFE_CUDA(cudaGetLastError());
    // M_divQ's pattern: row vi = [vi, C(vi, 1:nC)] (calc_ice_flux_divergence_matrix_upwind's add_entry order)
    std::vector<int32_t> nC(w->nV), C(nc);
    UFE_CUDA(cudaMemcpyAsync(nC.data(), ctx->nC, sizeof(int32_t) * w->nV, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(C.data(), ctx->C, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    std::vector<int32_t> ptr(w->nV + 1), ind;
    ind.reserve((size_t)w->nV * 8);
    for (int32_t vi = 0; vi < w->nV; ++vi) {
      ptr[vi] = (int32_t)ind.size();
      ind.push_back(vi);
      for (int ci = 0; ci < nC[vi]; ++ci) ind.push_back(C[(size_t)ci * w->nV + vi] - 1);
    }
    ptr[w->nV] = (int32_t)ind.size();
    w->nnz = (int64_t)ind.size();
    w->ptr = alloc_n<int32_t>(w->nV + 1);
    w->ind = alloc_n<int32_t>(w->nnz);
    UFE_CUDA(cudaMemcpyAsync(w->ptr, ptr.data(), sizeof(int32_t) * (w->nV + 1), cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaMemcpyAsync(w->ind, ind.data(), sizeof(int32_t) * w->nnz, cudaMemcpyHostToDevice, s));
    alloc_fields(w);
    UFE_CUDA(cudaStreamSynchronize(s));
    return UFE_OK;
  });
}

extern "C" int32_t ufe_thickness_assemble(ufe_ctx *ctx, const ufe_thickness_params *p, const ufe_thickness_fields *f,
                                          double dt, int32_t *ptr, int32_t *ind, double *val, double *bb, double *x0,
                                          int64_t cap, int64_t *nnz) {
  return guarded(ctx, [&]() -> int32_t {
    check_inputs(p, f);
    UFE_REQUIRE(ptr && ind && val && bb && x0 && nnz, UFE_ERR_INVALID, "null output arrays");
    UFE_CUDA(cudaSetDevice(ctx->device));
    MassWork *w = mass_work(ctx);
    cudaStream_t s = ctx->stream;
    *nnz = w->nnz;
    UFE_REQUIRE(cap >= w->nnz, UFE_ERR_CAPACITY, "ice thickness: matrix output too small");
    const Inputs in = upload_inputs(ctx, w, f);
    prepare(ctx, w, p, in);
    semi_system(ctx, w, p, in, dt, w->Hit);
    // rows back in the caller's numbering: caller row r is internal row iperm[r], entries in the
    // same order, columns renamed through perm
    const int nV = w->nV;
    std::vector<int32_t> ip(nV + 1), ii(w->nnz);
    std::vector<double> iv(w->nnz);
    UFE_CUDA(cudaMemcpyAsync(ip.data(), w->ptr, sizeof(int32_t) * (nV + 1), cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(ii.data(), w->ind, sizeof(int32_t) * w->nnz, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(iv.data(), w->valA, sizeof(double) * w->nnz, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    const std::vector<int32_t> &pv = ctx->perm_v_h, &iq = ctx->iperm_v_h;
    int64_t k = 0;
    for (int32_t r = 0; r < nV; ++r) {
      ptr[r] = (int32_t)k;
      const int32_t i = iq[r];
      for (int32_t e = ip[i]; e < ip[i + 1]; ++e, ++k) {
        ind[k] = pv[ii[e]];
        val[k] = iv[e];
      }
    }
    ptr[nV] = (int32_t)k;
    download_vertex(ctx, w, bb, w->bb);
    download_vertex(ctx, w, x0, w->Hit);
    return UFE_OK;
  });
}

extern "C" int32_t ufe_calc_dHi_dt(ufe_ctx *ctx, const ufe_thickness_params *p, ufe_thickness_fields *f, double *dt,
                                   ufe_thickness_stats *stats) {
  return guarded(ctx, [&]() -> int32_t {
    check_inputs(p, f);
    UFE_REQUIRE(dt && *dt > 0.0, UFE_ERR_INVALID, "ice thickness: dt must be positive");
    UFE_REQUIRE(f->dHi_dt && f->Hi_tplusdt && f->divQ && f->AMB, UFE_ERR_INVALID, "ice thickness: null outputs");
    UFE_CUDA(cudaSetDevice(ctx->device));
    MassWork *w = mass_work(ctx);
    cudaStream_t s = ctx->stream;
    const int nV = w->nV;
    ufe_thickness_stats st;
    memset(&st, 0, sizeof(st));
    const Inputs in = upload_inputs(ctx, w, f);
    UFE_CUDA(cudaMemcpyAsync(w->dt, dt, sizeof(double), cudaMemcpyHostToDevice, s));
    UFE_CUDA(cudaMemsetAsync(w->flag, 0, sizeof(int32_t), s));
    UFE_CUDA(cudaEventRecord(ctx->ev0, s));
    int32_t status = UFE_OK;
    if (p->choice_ice_integration_method == UFE_DHI_NONE) {
      k_none<<<blocks(nV), 256, 0, s>>>(nV, in.Hi, w->Hit, w->dHdt, w->AMB);
      UFE_CUDA(cudaMemsetAsync(w->divQ, 0, sizeof(double) * nV, s));   // not computed by the reference here
    } else {
      prepare(ctx, w, p, in);
      if (p->choice_ice_integration_method == UFE_DHI_EXPLICIT) {
        run_explicit(ctx, w, p, in, 0, w->dHdt, w->Hit, w->divQ, w->AMB);
      } else {
        semi_system(ctx, w, p, in, *dt, w->Hit);
        DevCSR A;
        A.m = A.n = nV;
        A.nnz = w->nnz;
        A.ptr = w->ptr;
        A.ind = w->ind;
        A.val = w->valA;
        int32_t its = 0;
        status = solve_csr_device(ctx, A, w->bb, w->Hit, p->dHi_PETSc_rtol, p->dHi_PETSc_abstol,
                                  p->dHi_PETSc_max_it, &its, &w->krylov);
        st.n_Axb_its = its;
        st.krylov_status = status;
        k_semi_finish<<<blocks(nV), 256, 0, s>>>(nV, in.Hi, *dt, w->Hit, w->dHdt, w->AMB);
      }
      k_main_finish<<<blocks(nV), 256, 0, s>>>(nV, in.Hi, w->dt, p->Hi_min, w->Hit, w->dHdt, w->AMB, w->flag);
      UFE_CUDA(cudaGetLastError());
    }
    UFE_CUDA(cudaEventRecord(ctx->ev1, s));
    download_vertex(ctx, w, f->dHi_dt, w->dHdt);
    download_vertex(ctx, w, f->Hi_tplusdt, w->Hit);
    download_vertex(ctx, w, f->divQ, w->divQ);
    download_vertex(ctx, w, f->AMB, w->AMB);
    UFE_CUDA(cudaMemcpyAsync(dt, w->dt, sizeof(double), cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(&st.found_negative, w->flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    UFE_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    st.device_ms = ms;
    if (stats) *stats = st;
    return status < 0 ? status : UFE_OK;
  });
}
