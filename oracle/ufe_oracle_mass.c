/* CPU restatement of the reference's ice-thickness update (conservation of mass) -- TEST
 * INFRASTRUCTURE ONLY: the checker for ufe_calc_dHi_dt, never linked into the library.
 *
 * Follows, in the reference tree src/UFEMISM/ice_dynamics/:
 *   conservation_of_mass/conservation_of_mass_main.f90:23-109          calc_dHi_dt
 *   conservation_of_mass/conservation_of_mass_explicit.f90:22-134      calc_dHi_dt_explicit
 *   conservation_of_mass/conservation_of_mass_explicit.f90:136-283     apply_ice_thickness_BC_explicit
 *   conservation_of_mass/conservation_of_mass_semiimplicit.f90:23-174  calc_dHi_dt_semiimplicit
 *   conservation_of_mass/conservation_of_mass_semiimplicit.f90:176-314 apply_ice_thickness_BC_matrix*
 *   conservation_of_mass/conservation_of_mass_utilities.f90:22-132     calc_ice_flux_divergence_matrix_upwind
 *   conservation_of_mass/conservation_of_mass_utilities.f90:158-204    calc_flux_limited_timestep
 *   conservation_of_mass/conservation_of_mass_utilities.f90:206-234    calc_n_interior_neighbours
 *   utilities/map_velocities_to_c_grid.f90:17-69                        map_velocities_from_b_to_c_2D
 * and src/UPSY/basic/math_utilities/ice_geometry_basics.f90:28-82 (ice_surface_elevation,
 * Hi_from_Hb_Hs_and_SL), src/UPSY/mesh/mesh_secondary.f90:300-341 (the connection vectors D_x,
 * D_y, D).  Every expression keeps the reference's operation order; the build turns off FMA
 * contraction, so each multiply and add rounds once as in the Fortran. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ufe_oracle.h"

#define ICE_DENSITY_M 910.0
#define SEAWATER_DENSITY_M 1028.0

void orc_default_thickness_params(ufe_thickness_params *p) {
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

static double surface_elevation(double Hi, double Hb, double SL) {
  return Hi + fmax(SL - ICE_DENSITY_M / SEAWATER_DENSITY_M * Hi, Hb);
}

static double thickness_from_surface(double Hb, double Hs, double SL) {
  double Hi_float = fmax(0.0, (SL - Hb) * (SEAWATER_DENSITY_M / ICE_DENSITY_M));
  double Hs_float = Hb + Hi_float;
  if (Hs > Hs_float) return Hs - Hb;
  return fmin(Hi_float, (Hs - SL) / (1.0 - (ICE_DENSITY_M / SEAWATER_DENSITY_M)));
}

/* the 1 or 2 triangles of the edge from vi to vj (0-based; -1 = none) */
static void edge_triangles(const ufe_mesh_desc *m, int vi, int vj, int *t1, int *t2) {
  *t1 = *t2 = -1;
  for (int k = 0; k < m->niTri[vi]; ++k) {
    int t = m->iTri[(int64_t)k * m->nV + vi] - 1;
    for (int q = 0; q < 3; ++q)
      if (m->Tri[(int64_t)q * m->nTri + t] - 1 == vj) {
        if (*t1 < 0) *t1 = t; else *t2 = t;
      }
  }
}

/* M_divQ (1-based CSR, rows: the diagonal, then C(vi,1:nC) in order) */
static void flux_divergence_matrix(const ufe_mesh_desc *m, const double *A, const double *Cw,
                                   const double *u_b, const double *v_b, const double *fm, orc_csr *M) {
  const int nV = m->nV;
  int64_t nnz = 0;
  for (int vi = 0; vi < nV; ++vi) nnz += 1 + m->nC[vi];
  M->m = M->n = nV;
  M->nnz = M->nnz_max = nnz;
  M->ptr = (int32_t *)malloc(sizeof(int32_t) * (nV + 1));
  M->ind = (int32_t *)malloc(sizeof(int32_t) * nnz);
  M->val = (double *)malloc(sizeof(double) * nnz);
  int64_t k = 0;
  for (int vi = 0; vi < nV; ++vi) {
    M->ptr[vi] = (int32_t)(k + 1);
    const int nC = m->nC[vi];
    double c0 = 0.0;
    int64_t kd = k++;
    for (int ci = 0; ci < nC; ++ci) {
      const int vj = m->C[(int64_t)ci * nV + vi] - 1;
      int t1, t2;
      edge_triangles(m, vi, vj, &t1, &t2);
      double uc, vc;   /* map_velocities_from_b_to_c_2D */
      if (t2 < 0) { uc = u_b[t1]; vc = v_b[t1]; }
      else { uc = (u_b[t1] + u_b[t2]) / 2.0; vc = (v_b[t1] + v_b[t2]) / 2.0; }
      const double A_i = A[vi];
      const double L_c = Cw[(int64_t)ci * nV + vi];
      const double Dx = m->V[vj] - m->V[vi], Dy = m->V[nV + vj] - m->V[nV + vi];
      const double D = sqrt(Dx * Dx + Dy * Dy);
      const double u_perp = uc * Dx / D + vc * Dy / D;
      const double fmi = fm ? fm[vi] : 1.0, fmj = fm ? fm[vj] : 1.0;
      if (fmi >= 1.0) c0 = c0 + L_c * fmax(0.0, u_perp) / A_i;
      double cj = 0.0;
      if (fmj >= 1.0) cj = L_c * fmin(0.0, u_perp) / A_i;
      M->ind[k] = vj + 1;
      M->val[k] = cj;
      ++k;
    }
    M->ind[kd] = vi + 1;
    M->val[kd] = c0;
  }
  M->ptr[nV] = (int32_t)(k + 1);
}

static int bc_of_vertex(const ufe_thickness_params *p, int vbi) {
  if (vbi == 1 || vbi == 2) return p->BC_H_north;
  if (vbi == 3 || vbi == 4) return p->BC_H_east;
  if (vbi == 5 || vbi == 6) return p->BC_H_south;
  if (vbi == 7 || vbi == 8) return p->BC_H_west;
  return -1;
}

/* apply_ice_thickness_BC_explicit: two passes over the border vertices, each reading the surface
 * elevations as they stood before the pass. */
static void bc_explicit(const ufe_mesh_desc *m, const ufe_thickness_params *p, const int32_t *noice,
                        const double *Hb, const double *SL, double *Hi) {
  const int nV = m->nV;
  double *Hs = (double *)malloc(sizeof(double) * nV * 2), *Hs_tot = Hs + nV;
  int *nint = (int *)malloc(sizeof(int) * nV);
  for (int vi = 0; vi < nV; ++vi) Hs[vi] = surface_elevation(Hi[vi], Hb[vi], SL[vi]);
  for (int vi = 0; vi < nV; ++vi) {
    nint[vi] = 0;
    for (int ci = 0; ci < m->nC[vi]; ++ci) {
      int vj = m->C[(int64_t)ci * nV + vi] - 1;
      if (m->VBI[vj] == 0 && !(noice && noice[vj])) nint[vi]++;
    }
  }
  for (int pass = 0; pass < 2; ++pass) {
    memcpy(Hs_tot, Hs, sizeof(double) * nV);
    for (int vi = 0; vi < nV; ++vi) {
      const int bc = bc_of_vertex(p, m->VBI[vi]);
      if (bc < 0) continue;
      if (bc == UFE_BC_H_ZERO) { Hi[vi] = 0.0; continue; }
      if (pass == 0 && nint[vi] > 0) {
        double s = 0.0;
        for (int ci = 0; ci < m->nC[vi]; ++ci) {
          int vj = m->C[(int64_t)ci * nV + vi] - 1;
          if (m->VBI[vj] == 0 && !(noice && noice[vj])) s = s + Hs_tot[vj];
        }
        double av = s / (double)nint[vi];
        Hs[vi] = fmax(Hb[vi], av);
        Hi[vi] = thickness_from_surface(Hb[vi], Hs[vi], SL[vi]);
      } else if (pass == 1 && nint[vi] == 0) {
        double s = 0.0;
        for (int ci = 0; ci < m->nC[vi]; ++ci) s = s + Hs_tot[m->C[(int64_t)ci * nV + vi] - 1];
        double av = s / (double)m->nC[vi];
        Hs[vi] = fmax(Hb[vi], av);
        Hi[vi] = thickness_from_surface(Hb[vi], Hs[vi], SL[vi]);
      }
    }
  }
  free(Hs);
  free(nint);
}

static double nz_or(const double *a, int i, double d) { return a ? a[i] : d; }

/* calc_dHi_dt_explicit: AMB, dHi_dt, Hi_tplusdt, divQ; *dt shortened by the flux limit */
static void explicit_step(const ufe_mesh_desc *m, const orc_csr *M, const ufe_thickness_params *p,
                          const ufe_thickness_fields *f, double *dt, double *dHi_dt, double *Hi_t,
                          double *divQ, double *AMB) {
  const int nV = m->nV;
  orc_spmv(M, f->Hi, divQ, 1);
  for (int vi = 0; vi < nV; ++vi) {
    double mb = nz_or(f->fraction_margin, vi, 1.0) *
                (nz_or(f->SMB, vi, 0.0) + nz_or(f->BMB, vi, 0.0) - nz_or(f->dHi_dt_target, vi, 0.0));
    dHi_dt[vi] = -divQ[vi] + mb + nz_or(f->LMB, vi, 0.0);
    AMB[vi] = dHi_dt[vi];
  }
  /* calc_flux_limited_timestep (max(dHi_dt, 1e-9) of a negative rate is 1e-9, as written) */
  double dt_max = p->dt_ice_max;
  for (int vi = 0; vi < nV; ++vi)
    if (f->Hi[vi] > p->Hi_min && dHi_dt[vi] < 0.0) {
      double lim = f->Hi[vi] / fmax(dHi_dt[vi], 1e-9);
      if (lim < dt_max) dt_max = lim;
    }
  dt_max = fmax(p->dt_ice_min, dt_max);
  *dt = fmin(*dt, dt_max);
  for (int vi = 0; vi < nV; ++vi) Hi_t[vi] = fmax(0.0, f->Hi[vi] + dHi_dt[vi] * *dt);
  bc_explicit(m, p, f->mask_noice, f->Hb, f->SL, Hi_t);
  if (f->BC_prescr_mask)
    for (int vi = 0; vi < nV; ++vi)
      if (f->BC_prescr_mask[vi] == 1) Hi_t[vi] = fmax(0.0, f->BC_prescr_Hi[vi]);
  if (f->mask_noice)
    for (int vi = 0; vi < nV; ++vi)
      if (f->mask_noice[vi]) Hi_t[vi] = 0.0;
  for (int vi = 0; vi < nV; ++vi) {
    dHi_dt[vi] = (Hi_t[vi] - f->Hi[vi]) / *dt;
    AMB[vi] = dHi_dt[vi] - AMB[vi];
  }
}

static void identity_row(orc_csr *A, int vi) {
  for (int32_t k = A->ptr[vi] - 1; k < A->ptr[vi + 1] - 1; ++k) A->val[k] = (A->ind[k] - 1 == vi) ? 1.0 : 0.0;
}

/* calc_dHi_dt_semiimplicit up to the Krylov solve: A, bb and the initial guess x0 */
static void semiimplicit_system(const ufe_mesh_desc *m, const orc_csr *M, const ufe_thickness_params *p,
                                const ufe_thickness_fields *f, const double *dHi_dt_prev, double dt,
                                orc_csr *A, double *bb, double *x0, double *divQ) {
  const int nV = m->nV;
  double *w = (double *)malloc(sizeof(double) * nV * 4);
  double *dex = w, *Hex = w + nV, *qex = w + 2 * nV, *aex = w + 3 * nV;
  double dt_ex = dt;
  explicit_step(m, M, p, f, &dt_ex, dex, Hex, qex, aex);
  orc_spmv(M, f->Hi, divQ, 1);
  *A = *M;
  A->ptr = (int32_t *)malloc(sizeof(int32_t) * (nV + 1));
  A->ind = (int32_t *)malloc(sizeof(int32_t) * M->nnz);
  A->val = (double *)malloc(sizeof(double) * M->nnz);
  memcpy(A->ptr, M->ptr, sizeof(int32_t) * (nV + 1));
  memcpy(A->ind, M->ind, sizeof(int32_t) * M->nnz);
  const double fs = p->dHi_semiimplicit_fs;
  for (int64_t k = 0; k < M->nnz; ++k) A->val[k] = M->val[k] * dt * fs;
  for (int vi = 0; vi < nV; ++vi)
    for (int32_t k = A->ptr[vi] - 1; k < A->ptr[vi + 1] - 1; ++k)
      if (A->ind[k] - 1 == vi) A->val[k] = A->val[k] + 1.0;
  for (int vi = 0; vi < nV; ++vi) {
    double mb = nz_or(f->fraction_margin, vi, 1.0) *
                (nz_or(f->SMB, vi, 0.0) + nz_or(f->BMB, vi, 0.0) - nz_or(f->dHi_dt_target, vi, 0.0));
    bb[vi] = f->Hi[vi] - (dt * (1.0 - fs) * divQ[vi]) + fmax(-1.0 * f->Hi[vi], dt * (mb + nz_or(f->LMB, vi, 0.0)));
    x0[vi] = f->Hi[vi] + dt * nz_or(dHi_dt_prev, vi, 0.0);
  }
  /* apply_ice_thickness_BC_matrix: domain border (the explicit solution, its border rule applied
   * again), prescribed thickness, no-ice mask */
  bc_explicit(m, p, f->mask_noice, f->Hb, f->SL, Hex);
  for (int vi = 0; vi < nV; ++vi)
    if (m->VBI[vi] > 0) { identity_row(A, vi); bb[vi] = Hex[vi]; x0[vi] = Hex[vi]; }
  if (f->BC_prescr_mask)
    for (int vi = 0; vi < nV; ++vi)
      if (f->BC_prescr_mask[vi] == 1) { identity_row(A, vi); bb[vi] = f->BC_prescr_Hi[vi]; x0[vi] = f->BC_prescr_Hi[vi]; }
  if (f->mask_noice)
    for (int vi = 0; vi < nV; ++vi)
      if (f->mask_noice[vi]) { identity_row(A, vi); bb[vi] = 0.0; x0[vi] = 0.0; }
  free(w);
}

static int32_t check_params(const ufe_mesh_desc *m, const ufe_thickness_params *p, const ufe_thickness_fields *f) {
  const int bcs[4] = {p->BC_H_west, p->BC_H_east, p->BC_H_south, p->BC_H_north};
  for (int i = 0; i < 4; ++i)
    if (bcs[i] != UFE_BC_H_ZERO && bcs[i] != UFE_BC_H_INFINITE) return UFE_ERR_INVALID;
  if (p->choice_ice_integration_method < UFE_DHI_NONE || p->choice_ice_integration_method > UFE_DHI_SEMIIMPLICIT)
    return UFE_ERR_INVALID;
  if (!f->Hi || !f->Hb || !f->SL || !f->u_vav_b || !f->v_vav_b || !f->dHi_dt || !f->Hi_tplusdt || !f->divQ || !f->AMB)
    return UFE_ERR_INVALID;
  if ((f->BC_prescr_mask == NULL) != (f->BC_prescr_Hi == NULL)) return UFE_ERR_INVALID;
  (void)m;
  return UFE_OK;
}

int32_t orc_thickness_assemble(const ufe_mesh_desc *m, const double *A_vor, const double *Cw,
                               const ufe_thickness_params *p, const ufe_thickness_fields *f, double dt,
                               orc_csr *A, double *bb, double *x0) {
  int32_t rc = check_params(m, p, f);
  if (rc != UFE_OK) return rc;
  orc_csr M;
  flux_divergence_matrix(m, A_vor, Cw, f->u_vav_b, f->v_vav_b, f->fraction_margin, &M);
  double *divQ = (double *)malloc(sizeof(double) * m->nV);
  semiimplicit_system(m, &M, p, f, f->dHi_dt, dt, A, bb, x0, divQ);
  free(divQ);
  orc_csr_free(&M);
  return UFE_OK;
}

int32_t orc_calc_dHi_dt(const ufe_mesh_desc *m, const double *A_vor, const double *Cw,
                        const ufe_thickness_params *p, ufe_thickness_fields *f, double *dt,
                        ufe_thickness_stats *st) {
  int32_t rc = check_params(m, p, f);
  if (rc != UFE_OK) return rc;
  const int nV = m->nV;
  ufe_thickness_stats dummy;
  if (!st) st = &dummy;
  memset(st, 0, sizeof(*st));
  for (int vi = 0; vi < nV; ++vi) f->AMB[vi] = 0.0;
  if (p->choice_ice_integration_method == UFE_DHI_NONE) {
    for (int vi = 0; vi < nV; ++vi) { f->Hi_tplusdt[vi] = f->Hi[vi]; f->dHi_dt[vi] = 0.0; }
    return UFE_OK;
  }
  orc_csr M;
  flux_divergence_matrix(m, A_vor, Cw, f->u_vav_b, f->v_vav_b, f->fraction_margin, &M);
  if (p->choice_ice_integration_method == UFE_DHI_EXPLICIT) {
    explicit_step(m, &M, p, f, dt, f->dHi_dt, f->Hi_tplusdt, f->divQ, f->AMB);
  } else {
    orc_csr A;
    double *bb = (double *)malloc(sizeof(double) * nV);
    semiimplicit_system(m, &M, p, f, f->dHi_dt, *dt, &A, bb, f->Hi_tplusdt, f->divQ);
    int32_t its = 0;
    int32_t ks = orc_bicgstab(&A, bb, f->Hi_tplusdt, p->dHi_PETSc_rtol, p->dHi_PETSc_abstol, p->dHi_PETSc_max_it, &its);
    st->n_Axb_its = its;
    st->krylov_status = ks;
    for (int vi = 0; vi < nV; ++vi) {
      f->AMB[vi] = (f->Hi_tplusdt[vi] - f->Hi[vi]) / *dt;
      f->dHi_dt[vi] = (f->Hi_tplusdt[vi] - f->Hi[vi]) / *dt;
      f->AMB[vi] = f->dHi_dt[vi] - f->AMB[vi];
    }
    free(bb);
    orc_csr_free(&A);
  }
  orc_csr_free(&M);
  /* calc_dHi_dt: negative thickness to zero (with the reference's warning), AMB, dHi_dt */
  int neg = 0;
  for (int vi = 0; vi < nV; ++vi)
    if (f->Hi_tplusdt[vi] < 0.0) {
      if (f->Hi_tplusdt[vi] < -0.1 && f->Hi[vi] > p->Hi_min) neg = 1;
      f->Hi_tplusdt[vi] = 0.0;
    }
  st->found_negative = neg;
  for (int vi = 0; vi < nV; ++vi) {
    f->AMB[vi] = f->AMB[vi] + (f->Hi_tplusdt[vi] - f->Hi[vi]) / *dt - f->dHi_dt[vi];
    f->dHi_dt[vi] = (f->Hi_tplusdt[vi] - f->Hi[vi]) / *dt;
  }
  return UFE_OK;
}
