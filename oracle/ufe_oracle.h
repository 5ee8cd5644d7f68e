/*
 * ufe_oracle.h -- CPU restatement of UFEMISM 2.0's velocity-solve path, in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is what the GPU library is compared against (tests,
 * the smoke check and the CPU baseline leg of the benchmark).  Nothing in the product
 * links, loads or calls it.
 *
 * Every function restates the Fortran routine it names (file:line relative to the UFEMISM2.0
 * source tree).  The Krylov solver restates PETSc's KSPBCGS with a Jacobi preconditioner
 * (PETSc is an external, unpinned dependency of the reference; see oracle.c).
 *
 * Matrices use the reference's CSR layout: 1-based ptr/ind, rows appended in order and entries
 * in the order add_entry_CSR_dist appends them (CSR_matrix_basics.f90:251-277).
 */
#ifndef UFE_ORACLE_H
#define UFE_ORACLE_H

#include <stdint.h>
#include "../include/ufe_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t m, n;
  int64_t nnz, nnz_max;
  int32_t *ptr;   /* m+1, 1-based */
  int32_t *ind;   /* nnz, 1-based */
  double  *val;
} orc_csr;

void    orc_csr_free(orc_csr *A);

/* calc_matrix_operators_mesh_{a_a,a_b,b_a,b_b_2nd_order}; ops[UFE_OP_COUNT] receives freshly
 * allocated matrices (free with orc_csr_free). */
int32_t orc_build_operators(const ufe_mesh_desc *mesh, orc_csr *ops);

/* multiply_CSR_matrix_with_vector_1D/2D */
void    orc_spmv(const orc_csr *A, const double *x, double *y, int32_t ncols);

/* solve_SSA_DIVA_linearised's matrix build (rows 2(ti-1)+uv) */
int32_t orc_assemble_linearised(const ufe_mesh_desc *mesh, const orc_csr *ops,
                                const ufe_solver_params *p,
                                const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                                const double *beta_b, const double *tau_dx_b, const double *tau_dy_b,
                                const double *u_prev, const double *v_prev,
                                const ufe_bc_prescribed *bc, orc_csr *A, double *bb);

/* KSPBCGS + PCJACOBI, left preconditioned, preconditioned residual norm */
int32_t orc_bicgstab(const orc_csr *A, const double *b, double *x, double rtol, double abstol,
                     int32_t max_it, int32_t *its);

int32_t orc_solve_ssa(const ufe_mesh_desc *mesh, const orc_csr *ops, const ufe_solver_params *p,
                      const ufe_ice_state *ice, const ufe_bc_prescribed *bc,
                      double *u_b, double *v_b, ufe_solve_stats *st,
                      const double *eta_first /* nV or NULL: first-iteration viscosity */);

int32_t orc_solve_diva(const ufe_mesh_desc *mesh, const orc_csr *ops, const ufe_solver_params *p,
                       const ufe_ice_state *ice, const ufe_bc_prescribed *bc,
                       ufe_diva_state *ds, ufe_solve_stats *st,
                       const double *eta_first /* nV or NULL: first-iteration viscosity */);

/* calc_dHi_dt (conservation_of_mass_main.f90:23-109) and the semi-implicit system before its
 * Krylov solve (A: 1-based CSR, freshly allocated), on the caller's vertex numbering; A_vor and Cw
 * are type_mesh's Voronoi cell areas and connection widths (ufe_oracle_mass.c). */
void    orc_default_thickness_params(ufe_thickness_params *p);
int32_t orc_calc_dHi_dt(const ufe_mesh_desc *m, const double *A_vor, const double *Cw,
                        const ufe_thickness_params *p, ufe_thickness_fields *f, double *dt,
                        ufe_thickness_stats *st);
int32_t orc_thickness_assemble(const ufe_mesh_desc *m, const double *A_vor, const double *Cw,
                               const ufe_thickness_params *p, const ufe_thickness_fields *f, double dt,
                               orc_csr *A, double *bb, double *x0);

/* Convenience for ctypes callers: build operators into an opaque handle. */
typedef struct orc_ops orc_ops;
orc_ops *orc_ops_create(const ufe_mesh_desc *mesh, int32_t *status);
void     orc_ops_destroy(orc_ops *h);
int32_t  orc_ops_info(orc_ops *h, int32_t op, int32_t *m, int32_t *n, int64_t *nnz);
int32_t  orc_ops_export(orc_ops *h, int32_t op, int32_t *ptr, int32_t *ind, double *val);
int32_t  orc_ops_apply(orc_ops *h, int32_t op, const double *x, double *y, int32_t ncols);
int32_t  orc_ops_solve_ssa(orc_ops *h, const ufe_solver_params *p, const ufe_ice_state *ice,
                           const ufe_bc_prescribed *bc, double *u_b, double *v_b, ufe_solve_stats *st);
int32_t  orc_ops_solve_diva(orc_ops *h, const ufe_solver_params *p, const ufe_ice_state *ice,
                            const ufe_bc_prescribed *bc, ufe_diva_state *ds, ufe_solve_stats *st);
int32_t  orc_ops_set_first_viscosity(orc_ops *h, const double *eta_a);
int32_t  orc_ops_calc_dHi_dt(orc_ops *h, const double *A_vor, const double *Cw, const ufe_thickness_params *p,
                             ufe_thickness_fields *f, double *dt, ufe_thickness_stats *st);
int32_t  orc_ops_thickness_assemble(orc_ops *h, const double *A_vor, const double *Cw,
                                    const ufe_thickness_params *p, const ufe_thickness_fields *f, double dt,
                                    int32_t *ptr, int32_t *ind, double *val, double *bb, double *x0,
                                    int64_t cap, int64_t *nnz_out);
int32_t  orc_ops_assemble(orc_ops *h, const ufe_solver_params *p,
                          const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                          const double *beta_b, const double *tau_dx_b, const double *tau_dy_b,
                          const double *u_prev, const double *v_prev, const ufe_bc_prescribed *bc,
                          int32_t *ptr, int32_t *ind, double *val, double *bb, int64_t cap,
                          int64_t *nnz_out);
int32_t  orc_csr_solve(int32_t m, int64_t nnz, const int32_t *ptr, const int32_t *ind,
                       const double *val, const double *b, double *x, double rtol, double abstol,
                       int32_t max_it, int32_t *its);
int32_t  orc_csr_spmv(int32_t m, int32_t n, int64_t nnz, const int32_t *ptr, const int32_t *ind,
                      const double *val, const double *x, double *y, int32_t ncols);

/* Thermodynamics (ufe_oracle_thermo.c) */
int32_t orc_zeta_operators(int32_t nz, const double *zeta, double *l1, double *d1, double *u1,
                           double *l2, double *d2, double *u2);
void    orc_tridiagonal(int32_t n, const double *a, double *b, const double *c, double *d, double *x);
int32_t orc_tridiagonal_batched(int32_t n, int32_t nsys, const double *a, const double *b,
                                const double *c, const double *d, double *x);
int32_t orc_thermo_step(const ufe_thermo_params *p, int32_t nV, int32_t nz, const double *zeta,
                        const ufe_thermo_columns *s, double *Ti_next, int32_t *n_unstable,
                        int32_t *is_unstable);
int32_t orc_ops_solve_3D_heat_equation(orc_ops *h, const ufe_thermo_params *p, const ufe_heat_fields *f,
                                       double *Ti_next, int32_t *n_unstable, int32_t *is_unstable);
const ufe_mesh_desc *orc_ops_mesh(const orc_ops *h);
const orc_csr *orc_ops_op(const orc_ops *h, int32_t op);

#ifdef __cplusplus
}
#endif
#endif
