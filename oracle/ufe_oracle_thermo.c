/*
 * ufe_oracle_thermo.c -- CPU restatement of UFEMISM 2.0's column temperature solve
 * (TEST INFRASTRUCTURE ONLY: what the GPU library's thermodynamics entry points are compared with).
 *
 * Paths are relative to the UFEMISM2.0 source tree.  Every expression keeps the Fortran
 * evaluation order (left to right for * and /, unary minus applied to the whole product), and
 * the build disables FMA contraction, so the arithmetic rounds as the reference's does.
 *
 * Fortran MIN/MAX on reals: gfortran (9 and later, NaNs honoured) evaluates them as IEEE
 * minNum/maxNum, which ignore a NaN argument; fmin/fmax here have the same semantics.
 */
#include "ufe_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* src/UPSY/basic/parameters.f90:15-23 */
#define TH_PI 3.141592653589793
#define TH_SEC_PER_YEAR 31556943.36
#define TH_T0 273.16
#define TH_CC_GRADIENT 8.7E-04
#define TH_ICE_DENSITY 910.0
/* src/UPSY/basic/math_utilities/shape_functions.f90:13 */
#define TH_Q 1.5

/* calc_shape_functions_1D_reg_2nd_order (shape_functions.f90:17-79) with its two neighbours;
 * the 2x2 inverse is calc_matrix_inverse_2_by_2 (matrix_algebra.f90:110-131). */
static int shape_1d_reg2(double x, const double xc[2], double *Nfx_i, double *Nfxx_i,
                         double Nfx_c[2], double Nfxx_c[2]) {
  double dx[2], w[2];
  for (int ci = 0; ci < 2; ++ci) dx[ci] = xc[ci] - x;
  for (int ci = 0; ci < 2; ++ci) w[ci] = 1.0 / pow(fabs(dx[ci]), TH_Q);
  double A11 = 0.0, A12 = 0.0, A21 = 0.0, A22 = 0.0;
  for (int ci = 0; ci < 2; ++ci) {
    const double w2 = w[ci] * w[ci];
    const double dx2 = dx[ci] * dx[ci];
    A11 = A11 + w2 * dx[ci] * dx[ci];
    A12 = A12 + w2 * dx[ci] * 1.0 / 2.0 * dx2;
    A21 = A21 + w2 * 1.0 / 2.0 * dx2 * dx[ci];
    A22 = A22 + w2 * 1.0 / 2.0 * dx2 * 1.0 / 2.0 * dx2;
  }
  const double det = A11 * A22 - A12 * A21;
  if (fabs(det) < DBL_MIN) return -1;
  const double M11 = A22 / det, M12 = -A12 / det, M21 = -A21 / det, M22 = A11 / det;
  for (int ci = 0; ci < 2; ++ci) {
    const double w2 = w[ci] * w[ci];
    const double dx2 = dx[ci] * dx[ci];
    Nfx_c[ci] = w2 * ((M11 * dx[ci]) + (M12 * 1.0 / 2.0 * dx2));
    Nfxx_c[ci] = w2 * ((M21 * dx[ci]) + (M22 * 1.0 / 2.0 * dx2));
  }
  *Nfx_i = -(Nfx_c[0] + Nfx_c[1]);
  *Nfxx_i = -(Nfxx_c[0] + Nfxx_c[1]);
  return 0;
}

/* calc_vertical_operators_reg_1D (mesh_zeta.f90:288-366) followed by
 * calc_zeta_operators_tridiagonal (:487-605): row k keeps its entries at k-1, k, k+1 (the
 * one-sided end rows drop their second neighbour). */
int32_t orc_zeta_operators(int32_t nz, const double *zeta, double *l1, double *d1, double *u1,
                           double *l2, double *d2, double *u2) {
  if (nz < 3 || !zeta) return UFE_ERR_INVALID;
  for (int k = 0; k < nz; ++k) {
    int ic[2];
    if (k == 0) { ic[0] = 1; ic[1] = 2; }
    else if (k == nz - 1) { ic[0] = nz - 3; ic[1] = nz - 2; }
    else { ic[0] = k - 1; ic[1] = k + 1; }
    const double zc[2] = {zeta[ic[0]], zeta[ic[1]]};
    double fi, fii, fc[2], fcc[2];
    if (shape_1d_reg2(zeta[k], zc, &fi, &fii, fc, fcc) != 0) return UFE_ERR_INVALID;
    l1[k] = 0.0; u1[k] = 0.0; l2[k] = 0.0; u2[k] = 0.0;
    d1[k] = fi;
    d2[k] = fii;
    for (int i = 0; i < 2; ++i) {
      if (ic[i] == k - 1) { l1[k] = fc[i]; l2[k] = fcc[i]; }
      if (ic[i] == k + 1) { u1[k] = fc[i]; u2[k] = fcc[i]; }
    }
  }
  return UFE_OK;
}

/* solve_tridiagonal_matrix_equation (tridiagonal_solver.f90:13-51); b and d are overwritten as
 * the reference's intent(inout) arguments are.  a[0] and c[n-1] are not read. */
void orc_tridiagonal(int32_t n, const double *a, double *b, const double *c, double *d, double *x) {
  for (int i = 1; i < n; ++i) {
    const double w = a[i] / b[i - 1];
    b[i] = b[i] - w * c[i - 1];
    d[i] = d[i] - w * d[i - 1];
  }
  for (int i = 0; i < n; ++i) x[i] = 0.0;
  x[n - 1] = d[n - 1] / b[n - 1];
  for (int i = n - 2; i >= 0; --i) x[i] = (d[i] - c[i] * x[i + 1]) / b[i];
}

int32_t orc_tridiagonal_batched(int32_t n, int32_t nsys, const double *a, const double *b,
                                const double *c, const double *d, double *x) {
  if (n < 1 || nsys < 0) return UFE_ERR_INVALID;
  double *bb = (double *)malloc(sizeof(double) * (size_t)n * 2);
  if (!bb) return UFE_ERR_INVALID;
  for (int64_t j = 0; j < nsys; ++j) {
    memcpy(bb, b + j * n, sizeof(double) * (size_t)n);
    memcpy(bb + n, d + j * n, sizeof(double) * (size_t)n);
    orc_tridiagonal(n, a + j * n, bb, c + j * n, bb + n, x + j * n);
  }
  free(bb);
  return UFE_OK;
}

typedef struct {
  int nz;
  const double *zeta, *l1, *d1, *u1, *l2, *d2, *u2;
} zops;

/* solve_1D_heat_equation (thermodynamics_3D_heat_equation.f90:309-479) for one column.
 * Ti is the current profile; Ki and Cpi come from the temperature at the start of the step.
 * grounded != 0: basal heat flux Q (:405-413); else the floating base T_base_float (:415-423). */
static void solve_1d(const zops *z, const double *Ti, const double *u, const double *v,
                     const double *w, const double *udx, const double *vdy, double T_surf,
                     const double *pmp, const double *Ki, const double *Cpi, const double *dzx,
                     const double *dzy, const double *dzz, const double *dzt, const double *Phi,
                     double dt, double *out, int grounded, double Q, double T_base_float,
                     double *work) {
  const int nz = z->nz;
  double *a = work, *b = work + nz, *c = work + 2 * nz, *d = work + 3 * nz, *x = work + 4 * nz;
  for (int k = 0; k < 4 * nz; ++k) work[k] = 0.0;
  b[0] = 1.0;
  d[0] = fmin(T_surf, TH_T0);
  b[nz - 1] = 1.0;
  if (grounded)
    d[nz - 1] = fmin(pmp[nz - 1], Ti[nz - 2] - (z->zeta[nz - 1] - z->zeta[nz - 2]) * Q / (dzz[nz - 1] * Ki[nz - 1]));
  else
    d[nz - 1] = fmin(T_base_float, pmp[nz - 1]);
  for (int k = 1; k < nz - 1; ++k) {
    const double c_ddzeta = dzt[k] + (u[k] * dzx[k]) + (v[k] * dzy[k]) + (w[k] * dzz[k]);
    const double c_d2dzeta2 = -(Ki[k] / (TH_ICE_DENSITY * Cpi[k]) * (dzz[k] * dzz[k]));
    a[k] = (c_ddzeta * z->l1[k]) + (c_d2dzeta2 * z->l2[k]);
    b[k] = 1.0 / dt + (c_ddzeta * z->d1[k]) + (c_d2dzeta2 * z->d2[k]);
    c[k] = (c_ddzeta * z->u1[k]) + (c_d2dzeta2 * z->u2[k]);
    d[k] = Ti[k] / dt - udx[k] - vdy[k] + Phi[k] / (TH_ICE_DENSITY * Cpi[k]);
  }
  orc_tridiagonal(nz, a, b, c, d, x);
  for (int k = 0; k < nz; ++k) out[k] = fmin(x[k], pmp[k]);
}

/* replace_Ti_with_robin_solution (thermodynamics_utilities.f90:256-337) for column vi. */
static void robin_column(int32_t nz, const double *zeta, double Hi_eff, double Hi_min, int32_t mask,
                         double T_surf_annual, double SMB, double geo, const double *pmp, double *Ti) {
  const double K_R = 9.828 * TH_SEC_PER_YEAR * exp(-(0.0057 * TH_T0));
  const double kappa_R = K_R / (TH_ICE_DENSITY * 2127.5);
  const double grad = -(1.0 * geo / K_R);
  const double Ts = fmin(TH_T0, T_surf_annual);
  if (Hi_eff > Hi_min) {
    if (mask == UFE_COL_GROUNDED || mask == UFE_COL_GL_GR) {
      if (SMB > 0.0) {
        const double L = sqrt(2.0 * kappa_R * Hi_eff / SMB);
        for (int k = 0; k < nz; ++k) {
          const double dist = (1.0 - zeta[k]) * Hi_eff;
          const double erf1 = erf(dist / L);
          const double erf2 = erf(Hi_eff / L);
          Ti[k] = Ts + sqrt(TH_PI) / 2.0 * L * grad * (erf1 - erf2);
        }
      } else {
        for (int k = 0; k < nz; ++k) Ti[k] = Ts + ((TH_T0 - TH_CC_GRADIENT * Hi_eff) - Ts) * zeta[k];
      }
    } else if (mask == UFE_COL_FLOATING) {
      for (int k = 0; k < nz; ++k) Ti[k] = Ts + zeta[k] * (pmp[nz - 1] - Ts);
    }
  } else {
    for (int k = 0; k < nz; ++k) Ti[k] = Ts;
  }
  for (int k = 0; k < nz; ++k) Ti[k] = fmin(Ti[k], pmp[k]);
}

static int column_stable(int nz, const double *T) {
  int ok = 1;
  for (int k = 0; k < nz; ++k) {
    if (T[k] != T[k]) ok = 0;
    if (T[k] < 180.0) ok = 0;
    if (T[k] > TH_T0) ok = 0;
  }
  return ok;
}

/* The column loop of solve_3D_heat_equation (thermodynamics_3D_heat_equation.f90:131-292) with
 * its prelude's outputs as inputs: Cp (thermodynamics_utilities.f90:130-165), K (:167-202) and
 * T_pmp (:204-229) are computed here from the step's starting temperature. */
/* is_unstable (optional, nV): 0 stable at the full dt, 2 stable after dt halving, 1 unstable
 * (Robin profile). */
int32_t orc_thermo_step(const ufe_thermo_params *p, int32_t nV, int32_t nz, const double *zeta,
                        const ufe_thermo_columns *s, double *Ti_next, int32_t *n_unstable_out,
                        int32_t *is_unstable) {
  if (!p || !s || !zeta || !Ti_next || nV < 1 || nz < 3) return UFE_ERR_INVALID;
  if (p->choice_GL_temperature_BC == UFE_GLBC_SUBGRID && !s->fraction_gr) return UFE_ERR_INVALID;
  double *ops = (double *)malloc(sizeof(double) * 6 * (size_t)nz);
  if (!ops) return UFE_ERR_INVALID;
  if (orc_zeta_operators(nz, zeta, ops, ops + nz, ops + 2 * nz, ops + 3 * nz, ops + 4 * nz, ops + 5 * nz) != 0) {
    free(ops);
    return UFE_ERR_INVALID;
  }
  const zops z = {nz, zeta, ops, ops + nz, ops + 2 * nz, ops + 3 * nz, ops + 4 * nz, ops + 5 * nz};
  int32_t n_unstable = 0, bad_mask = 0;
  int32_t *flag = (int32_t *)calloc((size_t)nV, sizeof(int32_t));

#pragma omp parallel reduction(+ : n_unstable, bad_mask)
  {
    double *col = (double *)malloc(sizeof(double) * (size_t)nz * 24);
    double *Ti0 = col, *u = col + nz, *v = col + 2 * nz, *w = col + 3 * nz, *udx = col + 4 * nz,
           *vdy = col + 5 * nz, *dzx = col + 6 * nz, *dzy = col + 7 * nz, *dzz = col + 8 * nz,
           *dzt = col + 9 * nz, *phi = col + 10 * nz, *Ki = col + 11 * nz, *Cpi = col + 12 * nz,
           *pmp = col + 13 * nz, *cur = col + 14 * nz, *x_gr = col + 15 * nz, *x_fl = col + 16 * nz,
           *work = col + 17 * nz;
#pragma omp for schedule(dynamic, 256)
    for (int64_t vi = 0; vi < nV; ++vi) {
      const double Hi_eff = s->Hi_eff[vi];
      if (Hi_eff < p->Hi_min_thermo) {
        for (int k = 0; k < nz; ++k) Ti_next[(int64_t)k * nV + vi] = s->T_surf_annual[vi];
        continue;
      }
      for (int k = 0; k < nz; ++k) {
        const int64_t o = (int64_t)k * nV + vi;
        Ti0[k] = s->Ti[o]; u[k] = s->u_3D[o]; v[k] = s->v_3D[o]; w[k] = s->w_3D[o];
        udx[k] = s->u_times_dTdxp_upwind[o]; vdy[k] = s->v_times_dTdyp_upwind[o];
        dzx[k] = s->dzeta_dx[o]; dzy[k] = s->dzeta_dy[o]; dzz[k] = s->dzeta_dz[o]; dzt[k] = s->dzeta_dt[o];
        phi[k] = s->internal_heating[o];
        Cpi[k] = p->choice_ice_heat_capacity == UFE_CP_UNIFORM ? p->uniform_ice_heat_capacity
                                                               : 2115.3 + 7.79293 * (Ti0[k] - TH_T0);
        Ki[k] = p->choice_ice_thermal_conductivity == UFE_K_UNIFORM ? p->uniform_ice_thermal_conductivity
                                                                    : 3.101E08 * exp(-(0.0057 * Ti0[k]));
        pmp[k] = TH_T0 - TH_CC_GRADIENT * Hi_eff * zeta[k];
        cur[k] = Ti0[k];
      }
      const int32_t mask = s->mask[vi];
      const double Ts = s->T_surf_annual[vi], Q = s->Q_base_grnd[vi], Tbf = pmp[nz - 1];
      if (mask != UFE_COL_GL_GR && mask != UFE_COL_GROUNDED && mask != UFE_COL_FLOATING) {
        bad_mask += 1;
        continue;
      }
      int found = 0, it_dt = 0;
      while (!found && it_dt < 10) {
        it_dt += 1;
        const double dt_applied = p->dt * pow(0.5, (double)(it_dt - 1));
        const int nsub = 1 << (it_dt - 1);
        for (int sub = 0; sub < nsub; ++sub) {
          if (mask == UFE_COL_GL_GR) {
            solve_1d(&z, cur, u, v, w, udx, vdy, Ts, pmp, Ki, Cpi, dzx, dzy, dzz, dzt, phi, dt_applied, x_gr, 1, Q, 0.0, work);
            if (p->choice_GL_temperature_BC == UFE_GLBC_SUBGRID || p->choice_GL_temperature_BC == UFE_GLBC_PMP)
              solve_1d(&z, cur, u, v, w, udx, vdy, Ts, pmp, Ki, Cpi, dzx, dzy, dzz, dzt, phi, dt_applied, x_fl, 0, 0.0, Tbf, work);
            else
              memcpy(x_fl, x_gr, sizeof(double) * (size_t)nz);
            if (p->choice_GL_temperature_BC == UFE_GLBC_SUBGRID) {
              const double fr = s->fraction_gr[vi];
              for (int k = 0; k < nz; ++k) x_gr[k] = fr * x_gr[k] + (1.0 - fr) * x_fl[k];
            } else if (p->choice_GL_temperature_BC == UFE_GLBC_PMP) {
              memcpy(x_gr, x_fl, sizeof(double) * (size_t)nz);
            }
          } else if (mask == UFE_COL_GROUNDED) {
            solve_1d(&z, cur, u, v, w, udx, vdy, Ts, pmp, Ki, Cpi, dzx, dzy, dzz, dzt, phi, dt_applied, x_gr, 1, Q, 0.0, work);
          } else {
            solve_1d(&z, cur, u, v, w, udx, vdy, Ts, pmp, Ki, Cpi, dzx, dzy, dzz, dzt, phi, dt_applied, x_gr, 0, 0.0, Tbf, work);
          }
          memcpy(cur, x_gr, sizeof(double) * (size_t)nz);
        }
        found = column_stable(nz, cur);
      }
      if (!found) {
        flag[vi] = 1;
        n_unstable += 1;
      } else if (it_dt > 1) {
        flag[vi] = 2;   /* stable after dt halving (reported to tests only) */
      }
      for (int k = 0; k < nz; ++k) Ti_next[(int64_t)k * nV + vi] = cur[k];
    }
    free(col);
  }

  int32_t rc = UFE_OK;
  if (bad_mask > 0) {
    rc = UFE_ERR_INVALID;
  } else if ((int64_t)n_unstable < ((int64_t)nV + 99) / 100) {
    /* n_unstable < CEILING(REAL(nV) / 100) (:256) */
    double *pmp = (double *)malloc(sizeof(double) * (size_t)nz);
    double *col = (double *)malloc(sizeof(double) * (size_t)nz);
    for (int64_t vi = 0; vi < nV; ++vi) {
      if (flag[vi] != 1) continue;
      const double Hi_eff = s->Hi_eff[vi];
      for (int k = 0; k < nz; ++k) {
        pmp[k] = TH_T0 - TH_CC_GRADIENT * Hi_eff * zeta[k];
        col[k] = Ti_next[(int64_t)k * nV + vi];
      }
      robin_column(nz, zeta, Hi_eff, p->Hi_min_thermo, s->mask[vi], s->T_surf_annual[vi], s->SMB[vi],
                   s->geothermal_heat_flux[vi], pmp, col);
      for (int k = 0; k < nz; ++k) Ti_next[(int64_t)k * nV + vi] = col[k];
    }
    free(pmp);
    free(col);
  } else {
    rc = UFE_ERR_THERMO_UNSTABLE;
  }
  if (n_unstable_out) *n_unstable_out = n_unstable;
  if (is_unstable) memcpy(is_unstable, flag, sizeof(int32_t) * (size_t)nV);
  free(flag);
  free(ops);
  return rc;
}

/* ---- the prelude on the mesh ------------------------------------------------------------- */

/* solve_3D_heat_equation (thermodynamics_3D_heat_equation.f90:33-307): the prelude -- the
 * vertex zeta gradients of calc_zeta_gradients (zeta_gradients.f90:19, a-grid terms), the upwind
 * products of calc_upwind_heat_flux_derivatives (thermodynamics_utilities.f90:339-434), the
 * annual-mean surface temperature (:118-120) and Q_base_grnd (:131-133) -- then the column loop. */
int32_t orc_ops_solve_3D_heat_equation(orc_ops *h, const ufe_thermo_params *p, const ufe_heat_fields *f,
                                       double *Ti_next, int32_t *n_unstable, int32_t *is_unstable) {
  if (!h || !p || !f || !Ti_next) return UFE_ERR_INVALID;
  const ufe_mesh_desc *m = orc_ops_mesh(h);
  const int64_t nV = m->nV, nTri = m->nTri, nz = m->nz, nCm = m->nC_mem;
  if (nz < 3 || f->n_months < 1) return UFE_ERR_INVALID;
  const orc_csr *Dxaa = orc_ops_op(h, UFE_OP_DDX_A_A), *Dyaa = orc_ops_op(h, UFE_OP_DDY_A_A);
  const orc_csr *Dxab = orc_ops_op(h, UFE_OP_DDX_A_B), *Dyab = orc_ops_op(h, UFE_OP_DDY_A_B);

  const size_t nl = (size_t)nV * (size_t)nz;
  double *dHi_dx = malloc(sizeof(double) * nV), *dHi_dy = malloc(sizeof(double) * nV);
  double *dHs_dx = malloc(sizeof(double) * nV), *dHs_dy = malloc(sizeof(double) * nV);
  double *dzx = malloc(sizeof(double) * nl), *dzy = malloc(sizeof(double) * nl);
  double *dzz = malloc(sizeof(double) * nl), *dzt = malloc(sizeof(double) * nl);
  double *dTdx_b = malloc(sizeof(double) * (size_t)nTri * nz), *dTdy_b = malloc(sizeof(double) * (size_t)nTri * nz);
  double *udx = calloc(nl, sizeof(double)), *vdy = calloc(nl, sizeof(double));
  double *Ts = malloc(sizeof(double) * nV), *Q = malloc(sizeof(double) * nV);

  orc_spmv(Dxaa, f->Hi, dHi_dx, 1);
  orc_spmv(Dyaa, f->Hi, dHi_dy, 1);
  orc_spmv(Dxaa, f->Hs, dHs_dx, 1);
  orc_spmv(Dyaa, f->Hs, dHs_dy, 1);
  for (int64_t vi = 0; vi < nV; ++vi) {
    const double Hi = fmax(10.0, f->Hi[vi]);
    for (int64_t k = 0; k < nz; ++k) {
      const double zeta = m->zeta[k];
      const int64_t o = k * nV + vi;
      dzt[o] = (1.0 / Hi) * (f->dHs_dt[vi] - zeta * f->dHi_dt[vi]);
      dzx[o] = (1.0 / Hi) * (dHs_dx[vi] - zeta * dHi_dx[vi]);
      dzy[o] = (1.0 / Hi) * (dHs_dy[vi] - zeta * dHi_dy[vi]);
      dzz[o] = (-1.0 / Hi);
    }
  }

  orc_spmv(Dxab, f->Ti, dTdx_b, (int32_t)nz);
  orc_spmv(Dyab, f->Ti, dTdy_b, (int32_t)nz);
  int32_t rc = UFE_OK;
  for (int64_t vi = 0; vi < nV && rc == UFE_OK; ++vi) {
    if (f->Hi[vi] < 1.0) continue;   /* udx, vdy stay 0 */
    const double uu[2] = {-f->u_vav[vi], -f->v_vav[vi]};
    int64_t ti_up = -1;
    for (int64_t vti = 0; vti < m->niTri[vi]; ++vti) {
      const int64_t ti = m->iTri[vti * nV + vi] - 1;
      int64_t vib = -1, vic = -1;
      for (int n1 = 0; n1 < 3; ++n1) {
        const int n2 = (n1 + 1) % 3, n3 = (n2 + 1) % 3;
        if (m->Tri[n1 * nTri + ti] - 1 == vi) {
          vib = m->Tri[n2 * nTri + ti] - 1;
          vic = m->Tri[n3 * nTri + ti] - 1;
          break;
        }
      }
      if (vib < 0) continue;
      const double ab[2] = {m->V[vib] - m->V[vi], m->V[nV + vib] - m->V[nV + vi]};
      const double ac[2] = {m->V[vic] - m->V[vi], m->V[nV + vic] - m->V[nV + vi]};
      if ((ab[0] * uu[1]) - (ab[1] * uu[0]) >= 0.0 && (uu[0] * ac[1]) - (uu[1] * ac[0]) >= 0.0) {
        ti_up = ti;
        break;
      }
    }
    if (ti_up < 0) {
      rc = UFE_ERR_INVALID;   /* 'could not find upwind triangle!' */
      break;
    }
    for (int64_t k = 0; k < nz; ++k) {
      udx[k * nV + vi] = f->u_3D_b[k * nTri + ti_up] * dTdx_b[k * nTri + ti_up];
      vdy[k * nV + vi] = f->v_3D_b[k * nTri + ti_up] * dTdy_b[k * nTri + ti_up];
    }
  }
  (void)nCm;

  /* calc_strain_heating (thermodynamics_utilities.f90:24-78) when no internal heating is given */
  double *phi_own = NULL;
  const double *phi = f->internal_heating;
  if (!phi) {
    const double n = f->Glens_flow_law_exponent > 0.0 ? f->Glens_flow_law_exponent : 3.0;
    phi_own = malloc(sizeof(double) * nl);
    for (int64_t vi = 0; vi < nV; ++vi)
      for (int64_t k = 0; k < nz; ++k) {
        const int64_t o = k * nV + vi;
        if (f->Hi[vi] < 0.1) { phi_own[o] = 0.0; continue; }
        const double D = sqrt(0.5 * (f->du_dx_3D[o] * f->du_dx_3D[o] + f->dv_dy_3D[o] * f->dv_dy_3D[o] +
                                     f->dw_dz_3D[o] * f->dw_dz_3D[o] +
                                     0.5 * ((f->du_dy_3D[o] + f->dv_dx_3D[o]) * (f->du_dy_3D[o] + f->dv_dx_3D[o])) +
                                     0.5 * ((f->du_dz_3D[o] + f->dw_dx_3D[o]) * (f->du_dz_3D[o] + f->dw_dx_3D[o])) +
                                     0.5 * ((f->dv_dz_3D[o] + f->dw_dy_3D[o]) * (f->dv_dz_3D[o] + f->dw_dy_3D[o]))));
        phi_own[o] = 2.0 * pow(f->A_flow[o], -1.0 / n) * pow(D, 1.0 / n + 1.0);
      }
    phi = phi_own;
  }
  for (int64_t vi = 0; vi < nV; ++vi) {
    double sum = 0.0;
    for (int32_t mo = 0; mo < f->n_months; ++mo) sum = sum + f->T2m[(int64_t)mo * nV + vi];
    Ts[vi] = sum / (double)f->n_months;
    /* calc_frictional_heating (:80-128) when no frictional heating is given */
    double fric;
    if (f->frictional_heating) fric = f->frictional_heating[vi];
    else if (f->no_sliding) fric = 0.0;
    else if (f->mask[vi] == UFE_COL_GROUNDED || f->mask[vi] == UFE_COL_GL_GR)
      fric = f->basal_friction_coefficient[vi] * f->uabs_base[vi];
    else fric = 0.0;
    Q[vi] = fric + f->geothermal_heat_flux[vi];
  }

  if (rc == UFE_OK) {
    ufe_thermo_columns c;
    c.Ti = f->Ti; c.u_3D = f->u_3D; c.v_3D = f->v_3D; c.w_3D = f->w_3D;
    c.u_times_dTdxp_upwind = udx; c.v_times_dTdyp_upwind = vdy;
    c.dzeta_dx = dzx; c.dzeta_dy = dzy; c.dzeta_dz = dzz; c.dzeta_dt = dzt;
    c.internal_heating = phi; c.Hi_eff = f->Hi_eff; c.T_surf_annual = Ts;
    c.Q_base_grnd = Q; c.mask = f->mask; c.fraction_gr = f->fraction_gr;
    c.geothermal_heat_flux = f->geothermal_heat_flux; c.SMB = f->SMB;
    rc = orc_thermo_step(p, (int32_t)nV, (int32_t)nz, m->zeta, &c, Ti_next, n_unstable, is_unstable);
  }
  free(dHi_dx); free(dHi_dy); free(dHs_dx); free(dHs_dy);
  free(dzx); free(dzy); free(dzz); free(dzt); free(dTdx_b); free(dTdy_b);
  free(udx); free(vdy); free(Ts); free(Q); free(phi_own);
  return rc;
}
