/*
 * ufe_gpu.h -- C ABI of the GB300 velocity solver for UFEMISM 2.0.
 *
 * The library replaces, behind plain C calls, the part of UFEMISM's ice-dynamics step that
 * computes velocities: the SSA/DIVA Picard loop with its stiffness-matrix assembly and Krylov
 * solve, the mesh CSR operators that loop applies, and the CSR matrix-equation solve that the
 * reference hands to PETSc.  A Fortran caller binds these entry points with ISO_C_BINDING.
 *
 * Conventions
 *   - Every array is a host array in the layout UFEMISM's derived types hold it: 2-D arrays are
 *     column-major (Fortran order), mesh connectivity is 1-based with 0 meaning "none".
 *   - CSR matrices follow type_sparse_matrix_CSR_dp (src/UPSY/basic/CSR_sparse_matrix_type.f90:15-38):
 *     ptr(m+1), ind(nnz), val(nnz); `index_base` says whether ptr/ind are 0- or 1-based.
 *   - Every call returns an int32 status: 0 ok, >0 a warning (the result is usable), <0 an error.
 *     ufe_ctx_last_error() returns the message of the last failure on a context.
 *   - One host thread per context.  Calls are synchronous: work runs on the context's own CUDA
 *     stream and the call returns after the results are in the caller's buffers.
 *   - No entry point falls back to the CPU.  A context that cannot reach a GB300-class device
 *     (sm_103) fails at ufe_ctx_create.
 */
#ifndef UFE_GPU_H
#define UFE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------------------------- */
#define UFE_OK                    0
#define UFE_WARN_PICARD_MAXIT     1   /* viscosity iteration hit visc_it_nit (SSA_main.f90:229-232) */
#define UFE_WARN_KRYLOV_MAXIT     2   /* a Krylov solve stopped before its tolerance (iteration limit,
                                         divergence or breakdown); the Picard loop went on */
#define UFE_ERR_INVALID          -1   /* bad argument or missing setup step */
#define UFE_ERR_NAN              -2   /* NaN/Inf in a result or an input */
#define UFE_ERR_DIVERGED         -3   /* Picard divergence limits (SSA_main.f90:207-213) or Krylov breakdown */
#define UFE_ERR_THERMO_UNSTABLE  -4   /* more than 1% unstable columns (thermodynamics_3D_heat_equation.f90:255-290) */
#define UFE_ERR_DEVICE           -5   /* CUDA error, or no sm_103 device */
#define UFE_ERR_CAPACITY         -6   /* an output buffer is too small, or a mesh exceeds a built-in limit */

typedef struct ufe_ctx ufe_ctx;

/* ---- mesh ---------------------------------------------------------------------------------- */
/* The arrays of type_mesh (src/UPSY/types/mesh_types.f90:57-97) that the velocity solve reads. */
typedef struct {
  int32_t nV, nTri, nC_mem, nz;
  const double  *V;      /* nV x 2                                                  */
  const int32_t *nC;     /* nV                                                      */
  const int32_t *C;      /* nV x nC_mem, counter-clockwise, edge to edge on borders */
  const int32_t *niTri;  /* nV                                                      */
  const int32_t *iTri;   /* nV x nC_mem, counter-clockwise                          */
  const int32_t *VBI;    /* nV, 0..8                                                */
  const int32_t *Tri;    /* nTri x 3, counter-clockwise                             */
  const int32_t *TriC;   /* nTri x 3, neighbour across from vertex n (0 = none)     */
  const int32_t *TriBI;  /* nTri, 0..8                                              */
  const double  *TriGC;  /* nTri x 2, geometric centres                             */
  const double  *zeta;   /* nz, scaled vertical coordinate (0 = surface, 1 = base)  */
} ufe_mesh_desc;

/* Matrix operators of type_mesh (mesh_types.f90:212-231). */
enum ufe_operator {
  UFE_OP_MAP_A_B = 0,  /* M_map_a_b    nTri x nV   */
  UFE_OP_DDX_A_B,      /* M_ddx_a_b                */
  UFE_OP_DDY_A_B,      /* M_ddy_a_b                */
  UFE_OP_MAP_B_A,      /* M_map_b_a    nV x nTri   */
  UFE_OP_DDX_B_A,      /* M_ddx_b_a                */
  UFE_OP_DDY_B_A,      /* M_ddy_b_a                */
  UFE_OP_DDX_A_A,      /* M_ddx_a_a    nV x nV     */
  UFE_OP_DDY_A_A,      /* M_ddy_a_a                */
  UFE_OP_M2_DDX_B_B,   /* M2_ddx_b_b   nTri x nTri */
  UFE_OP_M2_DDY_B_B,   /* M2_ddy_b_b               */
  UFE_OP_M2_D2DX2_B_B, /* M2_d2dx2_b_b             */
  UFE_OP_M2_D2DXDY_B_B,/* M2_d2dxdy_b_b            */
  UFE_OP_M2_D2DY2_B_B, /* M2_d2dy2_b_b             */
  UFE_OP_COUNT
};

/* ---- solver configuration ------------------------------------------------------------------ */
enum ufe_sliding_law {      /* choice_sliding_law (sliding_laws.f90:25-81) */
  UFE_SLIDING_NO_SLIDING = 0,
  UFE_SLIDING_WEERTMAN   = 1,
  UFE_SLIDING_COULOMB    = 2,
  UFE_SLIDING_BUDD       = 3,
  UFE_SLIDING_TSAI2015   = 4,
  UFE_SLIDING_SCHOOF2005 = 5,
  UFE_SLIDING_ZOET_IVERSON = 6,             /* 'Zoet-Iverson' (:353-409), till_yield_stress given  */
  UFE_SLIDING_IDEALISED_SSA_ICESTREAM = 7   /* 'idealised' with choice_idealised_sliding_law =
                                               'SSA_icestream' (:411-485): the till yield stress of
                                               Schoof's (2006) ice stream from the vertex y coordinate */
};
enum ufe_bc {               /* BC_{u,v}_{west,east,south,north} (solve_linearised_SSA_DIVA.f90:481-641) */
  UFE_BC_INFINITE = 0,
  UFE_BC_ZERO     = 1,
  UFE_BC_INFINITE_SSA_ICESTREAM = 2  /* 'infinite_SSA_icestream' (:562-578), u only: the border value
                                        is the relaxed previous velocity at the same y, 1/3 or 2/3
                                        across the domain (find_ti_copy_SSA_icestream_infinite,
                                        src/UPSY/mesh/mesh_utilities.f90:2681-2729)                */
};
enum ufe_precision {
  UFE_PREC_FP64       = 0,  /* FP64 everywhere                                              */
  UFE_PREC_FP32_REFINE = 1, /* FP32 Krylov (matrix, vectors, preconditioner), FP64 residual
                               recomputation and iterative refinement to the same tolerance   */
  UFE_PREC_FP32_PAIR  = 2   /* the Krylov solve in double-word arithmetic: every matrix entry,
                               vector element and recurrence scalar is a pair of FP32 numbers
                               (about 48 significant bits) computed on the FP32 pipe; the
                               Picard loop, assembly and stopping tests stay FP64.  A system
                               with values outside the FP32 exponent range is solved in FP64.
                               Where the persistent Krylov kernel is not used (UFE_NO_PERSIST,
                               UFE_NO_SELL, no room for its shared-memory patches) this mode
                               runs as UFE_PREC_FP64                                          */
};
enum ufe_rheology {         /* choice_ice_rheology_Glen */
  UFE_RHEOLOGY_INPUT         = 0, /* ice->A_flow is the flow factor, enhancement included (no reference
                                     counterpart: the caller ran calc_ice_rheology_Glen itself)          */
  UFE_RHEOLOGY_UNIFORM       = 1, /* 'uniform': uniform_Glens_flow_factor, then the enhancement factors    */
  UFE_RHEOLOGY_HUYBRECHTS1992 = 2 /* 'Huybrechts1992': Arrhenius A(Ti), then the enhancement factors       */
};
enum ufe_enhancement {      /* choice_enhancement_factor_transition */
  UFE_ENH_SEPARATE = 0,     /* 'separate': m_enh_sheet on grounded, m_enh_shelf on floating vertices    */
  UFE_ENH_INTERP   = 1      /* 'interp': by grounded fraction where Hi > 0 and Hib < SL                 */
};
enum ufe_initial_guess {
  UFE_X0_ZERO    = 0,       /* every Krylov solve starts from x = 0, as PETSc does by default  */
  UFE_X0_CURRENT = 1        /* start from the current Picard iterate                          */
};

/* Scalars of model_configuration.f90 that the velocity solve reads (names without _config). */
typedef struct {
  int32_t choice_sliding_law;             /* enum ufe_sliding_law                           */
  int32_t do_include_SSADIVA_crossterms;  /* :276, default 1                                */
  int32_t do_GL_subgrid_friction;         /* :340, default 1                                */
  int32_t BC_u_west, BC_u_east, BC_u_south, BC_u_north;   /* :316-323, default infinite   */
  int32_t BC_v_west, BC_v_east, BC_v_south, BC_v_north;
  int32_t visc_it_nit;                    /* :308, default 50                               */
  double  visc_it_norm_dUV_tol;           /* :307, default 5e-5                             */
  double  visc_it_relax;                  /* :309, default 0.2                              */
  double  visc_eff_min;                   /* :310, default 1e4                              */
  double  vel_max;                        /* :311, default 5000                             */
  double  stress_balance_PETSc_rtol;      /* :312, default 1e-7                             */
  double  stress_balance_PETSc_abstol;    /* :313, default 1e-5                             */
  double  Glens_flow_law_exponent;        /* :591, default 3                                */
  double  Glens_flow_law_epsilon_sq_0;    /* :592, default 1e-8                             */
  double  slid_Weertman_m;                /* :333, default 3                                */
  double  slid_Budd_q_plastic;            /* :334, default 0.3                              */
  double  slid_Budd_u_threshold;          /* :335, default 100                              */
  double  subgrid_friction_exponent_on_B_grid; /* :345, default 2                           */
  double  slid_beta_max;                  /* :348, default 1e20                             */
  double  slid_delta_v;                   /* :349, default 1e-3                             */
  /* Krylov controls of this library (PETSc takes them from its runtime options) */
  int32_t krylov_max_it;                  /* default 10000 (PETSc's default max_it)          */
  int32_t krylov_initial_guess;           /* enum ufe_initial_guess, default UFE_X0_CURRENT  */
  int32_t precision;                      /* enum ufe_precision, default UFE_PREC_FP64       */
  double  krylov_inner_rtol;              /* FP32 inner-solve reduction per refinement step, default 1e-2;
                                             the linear solve finishes in FP64 if the FP32 steps fail */
  double  krylov_forcing;                 /* two-phase inexact Picard iteration (no reference counterpart).
                                             Phase 1: each linear solve also stops once its residual is
                                             below krylov_forcing x its initial residual (the residual of
                                             the current Picard iterate), so iterations far from the fixed
                                             point are not solved to full accuracy.  When the change norm
                                             has met visc_it_norm_dUV_tol in two such iterations in a row,
                                             the next solve runs to the full Krylov tolerance: if the change
                                             norm then meets the tolerance the solve ends, otherwise phase 1
                                             resumes -- a small step from a loosely solved system never
                                             ends the solve.  0 (default) = the fixed tolerance only, as the
                                             reference's PETSc call; otherwise in (0, 1)                   */
  /* calc_ice_rheology_Glen (constitutive_equation.f90:84-163), model_configuration.f90:594-601 */
  int32_t choice_ice_rheology_Glen;       /* enum ufe_rheology, default UFE_RHEOLOGY_INPUT                  */
  int32_t choice_enhancement_factor_transition; /* enum ufe_enhancement, default UFE_ENH_SEPARATE          */
  double  uniform_Glens_flow_factor;      /* :596, default 1e-16 [Pa^-3 yr^-1]                             */
  double  m_enh_sheet;                    /* :600, default 1                                                */
  double  m_enh_shelf;                    /* :601, default 1                                                */
  double  slid_ZI_p;                      /* :336, default 5 (Zoet-Iverson velocity exponent)               */
  double  slid_ZI_ut;                     /* :337, default 200 [m yr^-1] (Zoet-Iverson transition velocity) */
  /* Schoof (2006) ice stream (refgeo_idealised_SSA_icestream_*, :190-193) read by the idealised
     sliding law; its flow factor is uniform_Glens_flow_factor and Glens_flow_law_exponent must be 3.
     Defaults: the reference's suggested values, as its SSA_icestream test sets them                   */
  double  SSA_icestream_Hi;               /* [m], 2000                                                      */
  double  SSA_icestream_dhdx;             /* surface slope, -0.0003                                         */
  double  SSA_icestream_L;                /* [m] ice-stream width, 150e3                                    */
  double  SSA_icestream_m;                /* margin exponent, 1                                             */
  int32_t reserved[8];
} ufe_solver_params;

/* Fields of type_ice_model / type_bed_roughness_model that the velocity solve reads.
 * Bed-roughness fields are taken after any A-grid grounded-fraction scaling
 * (apply_grounded_fractions_to_bed_roughness, sliding_laws.f90:573-641; off by default). */
typedef struct {
  const double  *Hi;                  /* nV       ice thickness [m]                          */
  const double  *Hs;                  /* nV       surface elevation [m]                      */
  const double  *A_flow;              /* nV x nz  Glen flow factor [Pa^-n yr^-1]             */
  const double  *fraction_gr_b;       /* nTri     sub-grid grounded fraction on triangles    */
  const int32_t *mask_grounded_ice;   /* nV       0/1                                        */
  const double  *beta_sq;             /* nV       Weertman/Tsai/Schoof roughness (or NULL)   */
  const double  *alpha_sq;            /* nV       Tsai/Schoof Coulomb coefficient (or NULL)  */
  const double  *effective_pressure;  /* nV       [Pa] (Tsai/Schoof; or NULL)                */
  const double  *till_yield_stress;   /* nV       [Pa] (Coulomb/Budd, already extended; or NULL) */
  /* read by calc_ice_rheology_Glen when choice_ice_rheology_Glen is not UFE_RHEOLOGY_INPUT (then
   * A_flow may be NULL); NULL where the chosen options do not read them */
  const double  *Ti;                  /* nV x nz  ice temperature [K] ('Huybrechts1992')             */
  const int32_t *mask_floating_ice;   /* nV       0/1 (enhancement factors)                          */
  const double  *fraction_gr;         /* nV       grounded fraction on vertices ('interp')           */
  const double  *Hib;                 /* nV       ice base elevation [m] ('interp')                  */
  const double  *SL;                  /* nV       sea level [m] ('interp')                           */
} ufe_ice_state;

/* Prescribed-velocity boundary condition (solve_SSA optional arguments); all NULL = none. */
typedef struct {
  const int32_t *mask_b;  /* nTri, 1 = velocity prescribed */
  const double  *u_b;     /* nTri */
  const double  *v_b;     /* nTri */
} ufe_bc_prescribed;

/* State of type_ice_velocity_solver_DIVA (ice_model_types.f90:63-109) carried between solves. */
typedef struct {
  double *u_vav_b, *v_vav_b;    /* nTri       in/out: vertically averaged velocity          */
  double *u_base_b, *v_base_b;  /* nTri       in/out: basal velocity                        */
  double *tau_bx_b, *tau_by_b;  /* nTri       in/out: basal shear stress                    */
  double *eta_3D_b;             /* nTri x nz  in/out: effective viscosity on triangles      */
  double *u_3D_b, *v_3D_b;      /* nTri x nz  out:    3-D velocity (NULL to skip)            */
} ufe_diva_state;

typedef struct {
  int32_t n_visc_its;       /* Picard iterations                                          */
  int32_t n_Axb_its;        /* Krylov iterations summed over the Picard iterations        */
  int32_t n_refinements;    /* FP64 refinement steps (UFE_PREC_FP32_REFINE)               */
  int32_t status;           /* same value the call returns                               */
  double  L2_uv;            /* last Picard change norm (calc_L2_norm_uv)                  */
  double  visc_it_relax_applied;
  double  device_ms;        /* device time of the solve                                   */
  int32_t n_fp64_its;       /* of n_Axb_its: FP64 BiCGStab iterations (all of them with    */
                            /* UFE_PREC_FP64; the fallback solves with UFE_PREC_FP32_REFINE) */
  int32_t n_kernels;        /* kernels the solve launched, counted from the kernel nodes of  */
                            /* its graph (-1 where loops inside a Picard iteration make the  */
                            /* count data dependent, or without graphs)                      */
  int32_t n_pair_its;       /* of n_Axb_its: double-word iterations (UFE_PREC_FP32_PAIR)    */
  int32_t reserved[3];
} ufe_solve_stats;

/* ---- context ------------------------------------------------------------------------------- */
void        ufe_default_params(ufe_solver_params *p);
int32_t     ufe_ctx_create(int32_t device, ufe_ctx **out);
void        ufe_ctx_destroy(ufe_ctx *ctx);
const char *ufe_ctx_last_error(const ufe_ctx *ctx);
int32_t     ufe_ctx_get_stream(ufe_ctx *ctx, void **cuda_stream);   /* the context's cudaStream_t */
int32_t     ufe_ctx_synchronize(ufe_ctx *ctx);

/* ---- mesh and operators -------------------------------------------------------------------- */
/* Copy a mesh to the device.  Replaces calc_all_secondary_mesh_data's role as the source of the
 * arrays the solver needs; builds the row translation tables tiuv2n/n2tiuv implicitly
 * (mesh_translation_tables.f90:187-197: row = 2(ti-1)+uv). */
int32_t ufe_mesh_upload(ufe_ctx *ctx, const ufe_mesh_desc *mesh);

/* Build every operator of enum ufe_operator on the GPU (calc_all_matrix_operators_mesh,
 * mesh_disc_calc_matrix_operators_2D.f90:26-59, minus the 1st-order b_b pair). */
int32_t ufe_mesh_build_operators(ufe_ctx *ctx);

/* Install a caller-built operator instead (the Fortran mesh%M_* matrix). */
int32_t ufe_mesh_set_operator(ufe_ctx *ctx, int32_t op, int32_t m, int32_t n, int64_t nnz,
                              const int32_t *ptr, const int32_t *ind, const double *val,
                              int32_t index_base);

int32_t ufe_operator_info(ufe_ctx *ctx, int32_t op, int32_t *m, int32_t *n, int64_t *nnz);
/* Copy an operator back in CSR form (ptr m+1, ind/val nnz) with the requested index base. */
int32_t ufe_operator_export(ufe_ctx *ctx, int32_t op, int32_t *ptr, int32_t *ind, double *val,
                            int32_t index_base);

/* map_a_b_2D/3D, ddx_a_b_2D/3D, ..., ddy_b_a_2D/3D (mesh_disc_apply_operators.f90:18-431):
 * y(:,k) = M_op x(:,k) for k = 1..ncols, column-major x (n x ncols) and y (m x ncols). */
int32_t ufe_apply_operator(ufe_ctx *ctx, int32_t op, const double *x, double *y, int32_t ncols);

/* ---- CSR algebra (caller-supplied matrices) ------------------------------------------------ */
/* multiply_CSR_matrix_with_vector_1D/2D (CSR_matrix_vector_multiplication.f90:198-364). */
int32_t ufe_csr_spmv(ufe_ctx *ctx, int32_t m, int32_t n, int64_t nnz, const int32_t *ptr,
                     const int32_t *ind, const double *val, int32_t index_base,
                     const double *x, double *y, int32_t ncols);

/* solve_matrix_equation_CSR_PETSc (petsc_basic.f90:32-64): Jacobi-preconditioned BiCGStab in the
 * form of PETSc's KSPBCGS with left preconditioning; converged when the preconditioned residual
 * norm is <= max(rtol * ||D^-1 b||, abstol).  xx is the initial guess on entry (pass zeros to
 * reproduce PETSc's default zero guess) and the solution on exit. */
int32_t ufe_solve_csr(ufe_ctx *ctx, int32_t m, int64_t nnz, const int32_t *ptr, const int32_t *ind,
                      const double *val, int32_t index_base, const double *bb, double *xx,
                      double rtol, double abstol, int32_t max_it, int32_t *n_Axb_its);

/* ---- linearised SSA/DIVA ------------------------------------------------------------------- */
/* The stiffness matrix and load vector of solve_SSA_DIVA_linearised
 * (solve_linearised_SSA_DIVA.f90:58-153), exported in the reference's own CSR layout: rows
 * 2(ti-1)+uv, entries in the order add_entry_CSR_dist appends them, 1-based.  `cap` is the
 * capacity of ind/val; *nnz_out receives the entry count. */
int32_t ufe_assemble_linearised(ufe_ctx *ctx, const ufe_solver_params *p,
                                const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                                const double *basal_friction_coefficient_b,
                                const double *tau_dx_b, const double *tau_dy_b,
                                const double *u_b_prev, const double *v_b_prev,
                                const ufe_bc_prescribed *bc,
                                int32_t *ptr, int32_t *ind, double *val, double *bb,
                                int64_t cap, int64_t *nnz_out);

/* solve_SSA_DIVA_linearised (solve_linearised_SSA_DIVA.f90:23-178): u_b/v_b are the current
 * solution on entry (initial guess under UFE_X0_CURRENT) and the new solution on exit;
 * u_b_prev/v_b_prev receive the entry values, as gather_to_all does at :54-55. */
int32_t ufe_solve_linearised(ufe_ctx *ctx, const ufe_solver_params *p,
                             double *u_b, double *v_b,
                             const double *N_b, const double *dN_dx_b, const double *dN_dy_b,
                             const double *basal_friction_coefficient_b,
                             const double *tau_dx_b, const double *tau_dy_b,
                             double *u_b_prev, double *v_b_prev,
                             const ufe_bc_prescribed *bc, int32_t *n_Axb_its);

/* ---- full velocity solves ------------------------------------------------------------------ */
/* solve_SSA (SSA_main.f90:87-242): u_b/v_b in/out (warm start in, solution out). */
int32_t ufe_solve_ssa(ufe_ctx *ctx, const ufe_solver_params *p, const ufe_ice_state *ice,
                      const ufe_bc_prescribed *bc, double *u_b, double *v_b,
                      int32_t *n_visc_its, int32_t *n_Axb_its, ufe_solve_stats *stats);

/* solve_DIVA (DIVA_main.f90:88-262). */
int32_t ufe_solve_diva(ufe_ctx *ctx, const ufe_solver_params *p, const ufe_ice_state *ice,
                       const ufe_bc_prescribed *bc, ufe_diva_state *st,
                       int32_t *n_visc_its, int32_t *n_Axb_its, ufe_solve_stats *stats);

/* Device-resident form of the two solves, for callers that keep the ice state on the GPU between
 * time steps: ufe_ice_upload copies the inputs once; ufe_solve_*_resident runs a solve from the
 * resident velocity state (reset to zero when `cold_start` is 1); ufe_velocity_download copies
 * the resident velocity state back (u_b/v_b for SSA, the u_vav/v_vav pair for DIVA). */
int32_t ufe_ice_upload(ufe_ctx *ctx, const ufe_ice_state *ice, const ufe_bc_prescribed *bc);
int32_t ufe_solve_ssa_resident(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start,
                               ufe_solve_stats *stats);
int32_t ufe_solve_diva_resident(ufe_ctx *ctx, const ufe_solver_params *p, int32_t cold_start,
                                ufe_solve_stats *stats);
int32_t ufe_velocity_download(ufe_ctx *ctx, double *u_b, double *v_b);

/* Mean microseconds per iteration of the persistent Krylov kernel (the whole solve in one launch
 * with shared-memory patches: the FP64 solve, the double-word solve with its conversions in and
 * out, or the FP32 inner solve) on the system the last solve on ctx assembled, running
 * `iterations` iterations.  Measurement only. */
int32_t ufe_profile_krylov_persistent(ufe_ctx *ctx, int32_t precision, int32_t iterations, double *us_per_iteration);

/* ---- thermodynamics: implicit column temperature solve ---------------------------------------- */
enum ufe_heat_capacity { UFE_CP_UNIFORM = 0, UFE_CP_POUNDER1965 = 1 };   /* choice_ice_heat_capacity        */
enum ufe_conductivity  { UFE_K_UNIFORM = 0, UFE_K_RITZ1987 = 1 };        /* choice_ice_thermal_conductivity */
enum ufe_gl_temp_bc    { UFE_GLBC_GROUNDED = 0, UFE_GLBC_SUBGRID = 1, UFE_GLBC_PMP = 2 }; /* choice_GL_temperature_BC */
/* Per-vertex column type: the reference's mask_gl_gr (grounded side of the grounding line, which is
 * also grounded), mask_grounded_ice and mask_floating_ice, tested in that order
 * (thermodynamics_3D_heat_equation.f90:168,198,207). */
enum ufe_column_mask   { UFE_COL_NONE = 0, UFE_COL_GROUNDED = 1, UFE_COL_FLOATING = 2, UFE_COL_GL_GR = 3 };

/* Configuration scalars solve_3D_heat_equation reads (model_configuration.f90:578-584). */
typedef struct {
  double  dt;                               /* [yr] thermodynamics time step                        */
  double  Hi_min_thermo;                    /* [m]  default 10                                      */
  int32_t choice_ice_heat_capacity;         /* default UFE_CP_POUNDER1965                           */
  int32_t choice_ice_thermal_conductivity;  /* default UFE_K_RITZ1987                               */
  double  uniform_ice_heat_capacity;        /* [J kg^-1 K^-1]       default 2009                    */
  double  uniform_ice_thermal_conductivity; /* [J m^-1 K^-1 yr^-1]  default 6.626958e7              */
  int32_t choice_GL_temperature_BC;         /* default UFE_GLBC_GROUNDED                            */
  int32_t reserved[7];
} ufe_thermo_params;

void ufe_default_thermo_params(ufe_thermo_params *p);

/* Column level.  The per-column inputs of the column loop of solve_3D_heat_equation
 * (thermodynamics_3D_heat_equation.f90:133-290) once its prelude has run: nV x nz arrays are
 * column-major (layer k of vertex vi at k*nV + vi), as ice%Ti(vi,k) is. */
typedef struct {
  const double  *Ti;                     /* nV x nz  temperature at time t [K]; Cp and K follow it   */
  const double  *u_3D, *v_3D, *w_3D;     /* nV x nz  [m yr^-1]                                       */
  const double  *u_times_dTdxp_upwind;   /* nV x nz  [K yr^-1] (calc_upwind_heat_flux_derivatives)   */
  const double  *v_times_dTdyp_upwind;   /* nV x nz  [K yr^-1]                                       */
  const double  *dzeta_dx, *dzeta_dy;    /* nV x nz  ice%dzeta_dx_ak, dzeta_dy_ak [m^-1]             */
  const double  *dzeta_dz, *dzeta_dt;    /* nV x nz  ice%dzeta_dz_ak [m^-1], dzeta_dt_ak [yr^-1]     */
  const double  *internal_heating;       /* nV x nz  Phi [J kg^-1 yr^-1]                             */
  const double  *Hi_eff;                 /* nV [m]                                                   */
  const double  *T_surf_annual;          /* nV [K]                                                   */
  const double  *Q_base_grnd;            /* nV [J m^-2 yr^-1] frictional + geothermal heating        */
  const int32_t *mask;                   /* nV enum ufe_column_mask                                  */
  const double  *fraction_gr;            /* nV (read for UFE_GLBC_SUBGRID only; may be NULL else)    */
  const double  *geothermal_heat_flux;   /* nV [J m^-2 yr^-1] (Robin profile)                        */
  const double  *SMB;                    /* nV [m yr^-1]      (Robin profile)                        */
} ufe_thermo_columns;

/* One step for nV independent columns (host arrays in and out): per column the implicit solve
 * of solve_1D_heat_equation (:309-479) with the per-column dt halving (up to 10 levels,
 * :163-239) and the stability check (NaN, < 180 K, > T0, :226-232); then the Robin profile
 * (replace_Ti_with_robin_solution, thermodynamics_utilities.f90:256-337) for the columns that
 * stayed unstable when they are fewer than ceil(nV/100), else UFE_ERR_THERMO_UNSTABLE (:251-290).
 * *n_unstable receives the number of such columns.  No mesh needs to be uploaded. */
int32_t ufe_thermo_step(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t nV, int32_t nz,
                        const double *zeta, const ufe_thermo_columns *cols, double *Ti_next,
                        int32_t *n_unstable);

/* Mesh level: the fields solve_3D_heat_equation(mesh, ice, climate, SMB, dt) reads
 * (thermodynamics_3D_heat_equation.f90:33).  The prelude runs on the GPU from these: the zeta
 * gradients of calc_zeta_gradients (zeta_gradients.f90:19, vertex terms), Cp, K and T_pmp
 * (thermodynamics_utilities.f90:130-229), the upwind advection terms of
 * calc_upwind_heat_flux_derivatives (:339-434), the annual-mean surface temperature, and the
 * two heating terms: calc_strain_heating (:24-78) from A_flow and the 3-D strain rates when
 * internal_heating is NULL, calc_frictional_heating (:80-128) from the basal friction coefficient
 * and basal speed when frictional_heating is NULL (a caller that has them can pass them instead). */
typedef struct {
  const double  *Ti;                     /* nV x nz  [K]                                            */
  const double  *Hi, *Hi_eff, *Hs;       /* nV [m]                                                  */
  const double  *dHi_dt, *dHs_dt;        /* nV [m yr^-1]                                            */
  const double  *u_vav, *v_vav;          /* nV [m yr^-1] vertically averaged velocity on vertices  */
  const double  *u_3D, *v_3D, *w_3D;     /* nV x nz   [m yr^-1]                                     */
  const double  *u_3D_b, *v_3D_b;        /* nTri x nz [m yr^-1]                                     */
  const double  *internal_heating;       /* nV x nz   [J kg^-1 yr^-1]                               */
  const double  *frictional_heating;     /* nV [J m^-2 yr^-1]                                       */
  const double  *geothermal_heat_flux;   /* nV [J m^-2 yr^-1]                                       */
  const double  *T2m;                    /* nV x n_months [K] (climate%T2m)                         */
  int32_t        n_months;
  int32_t        pad;
  const double  *SMB;                    /* nV [m yr^-1]                                            */
  const int32_t *mask;                   /* nV enum ufe_column_mask                                 */
  const double  *fraction_gr;            /* nV (UFE_GLBC_SUBGRID only; may be NULL else)            */
  /* calc_strain_heating inputs (read when internal_heating is NULL): Glen's flow factor and the
     3-D strain rates of ice%du_dx_3D ... ice%dw_dz_3D, nV x nz each [Pa^-n yr^-1], [yr^-1]        */
  const double  *A_flow;
  const double  *du_dx_3D, *du_dy_3D, *du_dz_3D;
  const double  *dv_dx_3D, *dv_dy_3D, *dv_dz_3D;
  const double  *dw_dx_3D, *dw_dy_3D, *dw_dz_3D;
  /* calc_frictional_heating inputs (read when frictional_heating is NULL): nV each; grounded
     vertices are those with mask UFE_COL_GROUNDED or UFE_COL_GL_GR                                */
  const double  *basal_friction_coefficient;   /* [Pa yr m^-1]                                     */
  const double  *uabs_base;                    /* [m yr^-1]                                        */
  /* configuration scalars of the two heating terms */
  int32_t        no_sliding;             /* choice_sliding_law is 'no_sliding': no frictional heating
                                            (calc_frictional_heating, :91-95)                        */
  int32_t        pad2;
  double         Glens_flow_law_exponent; /* calc_strain_heating's n (0 is taken as the default 3)   */
} ufe_heat_fields;

/* solve_3D_heat_equation on the uploaded mesh (operators built or set; the mesh's nz and zeta):
 * host fields in, ice%Ti_next out. */
int32_t ufe_solve_3D_heat_equation(ufe_ctx *ctx, const ufe_thermo_params *p, const ufe_heat_fields *f,
                                   double *Ti_next, int32_t *n_unstable);

/* Device-resident time stepping: ufe_heat_upload copies the fields once; each of the `nsteps`
 * steps of ufe_heat_step_resident is one solve_3D_heat_equation followed by Ti <- Ti_next, with
 * velocities, geometry, heating and climate held fixed.  *n_unstable_total sums the Robin
 * columns over the steps; a step with too many unstable columns stops the stepping
 * (UFE_ERR_THERMO_UNSTABLE, the resident Ti left at that step's input).  ufe_heat_download
 * copies the resident temperature out. */
int32_t ufe_heat_upload(ufe_ctx *ctx, const ufe_heat_fields *f);
int32_t ufe_heat_step_resident(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t nsteps,
                               int32_t *n_unstable_total, double *device_ms);
int32_t ufe_heat_download(ufe_ctx *ctx, double *Ti);

/* Time the kernels of one heat-equation step on the resident state of ufe_heat_upload without
 * advancing it: each is launched `repeats` times between two CUDA events on the context's stream.
 * us[0..3] receive the mean microseconds of the column pass, the dt-halving retry pass, the Robin
 * pass and the end-of-step bookkeeping; counts[0..1] the columns with ice (Hi_eff >= Hi_min_thermo)
 * and the columns without.  Measurement only; no reference counterpart. */
int32_t ufe_profile_heat_kernels(ufe_ctx *ctx, const ufe_thermo_params *p, int32_t repeats, double *us,
                                 int64_t *counts);

/* The tridiagonal d/dzeta and d2/dzeta2 operators of the column solve (calc_zeta_operators_tridiagonal,
 * mesh_zeta.f90:487-605, from calc_vertical_operators_reg_1D, :288-366).  Each array has nz
 * entries indexed by row: *_l[k] couples row k to k-1 (*_l[0] = 0), *_u[k] couples k to k+1
 * (*_u[nz-1] = 0).  Host computation. */
int32_t ufe_zeta_operators(int32_t nz, const double *zeta, double *ddz_l, double *ddz_d,
                           double *ddz_u, double *d2dz2_l, double *d2dz2_d, double *d2dz2_u);

/* solve_tridiagonal_matrix_equation (tridiagonal_solver.f90:13-51) for `nsys` systems of size n on
 * the GPU: system j in column j of the n x nsys column-major host arrays a (a[0] unused), b, c
 * (c[n-1] unused) and d; x receives the solutions.  Thomas algorithm, one thread per system. */
int32_t ufe_tridiagonal_solve(ufe_ctx *ctx, int32_t n, int32_t nsys, const double *a, const double *b,
                              const double *c, const double *d, double *x);

/* ---- ensembles ----------------------------------------------------------------------------------- */
/* Solve n independent members, each a context on the same device with its mesh and resident ice
 * state (ufe_ice_upload): every member's resident solve is queued on its own stream before any is
 * waited for, so members of uneven size run side by side.  stats[i] (optional) per member;
 * *wall_ms the time from the first launch to the last completion.  Returns the most severe
 * member status.  No reference counterpart: the reference runs one solve at a time. */
int32_t ufe_ensemble_solve(ufe_ctx *const *ctxs, int32_t n, const ufe_solver_params *p, int32_t diva,
                           int32_t cold_start, ufe_solve_stats *stats, double *wall_ms);

/* Autotuner: time the FP64 Krylov kernels of the system the last solve on ctx assembled with each
 * rows-per-warp choice (1 -- with the sliced-ELL layout --, 2, 4, 8) and keep the fastest for the
 * context's later solves.  *lanes receives the choice; us[0..3] (optional) the measured
 * microseconds per iteration of each. */
int32_t ufe_autotune(ufe_ctx *ctx, int32_t repeats, int32_t *lanes, double *us);

/* ---- learned Picard start: tensor-core building block ----------------------------------------- */
/* Y[M x N] = X[M x K] * W[N x K]^T with BF16 X and W (raw 16-bit patterns, row-major) and FP32 Y,
 * on the tcgen05 tensor cores (one 128-row tile per CTA, accumulator in tensor memory).  M a
 * multiple of 128, N 64 or 128, K a multiple of 64 up to 256.  The network's layers are built on
 * the same tile; this entry point exercises it alone.  No reference counterpart. */
int32_t ufe_umma_gemm_bf16(ufe_ctx *ctx, int32_t M, int32_t N, int32_t K, const uint16_t *X, const uint16_t *W,
                           float *Y);

/* ---- learned Picard start: the mesh-graph network ---------------------------------------------- */
/* A network on the triangle b-grid (nodes: triangles, edges: TriC neighbours) that predicts the
 * velocity and the effective viscosity a Picard solve starts from.  Width 64: an encoder from 16
 * per-triangle features, four message-passing layers h <- h + W2 relu(W1 [h, mean of the
 * neighbours' h] + b1) + b2, and a linear decoder to three outputs: (u, v) / 1000 m/yr and
 * (log10(eta_vav) - 7.5) / 2 with eta_vav the vertically averaged effective viscosity in Pa yr.
 * Forward and backward run in hand-written kernels on the
 * tcgen05 tensor cores (BF16 operands, FP32 accumulation); Adam in FP32.  The solve still iterates
 * to its own tolerance: the prediction only replaces the zero (or previous-step) start.  No
 * reference counterpart; it feeds solve_SSA / solve_DIVA (SSA_main.f90:87, DIVA_main.f90:88). */
typedef struct ufe_gnn ufe_gnn;

int32_t ufe_gnn_param_count(void);
int32_t ufe_gnn_create(ufe_ctx *ctx, uint64_t seed, ufe_gnn **out);   /* lives on ctx's device/stream;  */
void    ufe_gnn_destroy(ufe_gnn *g);                                   /* call other ufe_gnn_* only while ctx lives */
int32_t ufe_gnn_get_params(ufe_gnn *g, float *params);                /* ufe_gnn_param_count() floats */
int32_t ufe_gnn_set_params(ufe_gnn *g, const float *params);          /* also resets the Adam state   */

/* Explicit graphs (host arrays): n nodes, nbr n x 3 row-major (-1: no neighbour; the adjacency must
 * be symmetric), x n x 16 features, y / target n x 3, w n loss weights.  loss = sum_i w_i |y_i - t_i|^2;
 * grad receives its gradient with respect to the parameters. */
int32_t ufe_gnn_forward(ufe_gnn *g, int64_t n, const int32_t *nbr, const float *x, float *y);
int32_t ufe_gnn_loss_grad(ufe_gnn *g, int64_t n, const int32_t *nbr, const float *x, const float *target,
                          const float *w, double *loss, float *grad);

/* Kernels one ufe_gnn_predict_velocity call launches with this many smoothing passes (one more
 * for ufe_gnn_predict_start with with_viscosity = 1). */
int32_t ufe_gnn_predict_kernels(int32_t smooth_passes);

/* The mesh path.  ufe_gnn_features: the 16 features of a mesh context's resident ice state (after
 * ufe_ice_upload), nTri x 16 in the caller's triangle order; use_prev_velocity = 0 zeroes the
 * previous-velocity features (a cold start).  ufe_gnn_dataset_add: store one training member on the
 * device -- the features (given, as taken before the solve, or NULL to take them now with a zero
 * previous velocity) and the context's resident solution (velocity, and the vertically averaged
 * viscosity of its last Picard iteration) as the target; returns the member count.
 * ufe_gnn_train: `epochs` passes over the stored members, one Adam step per member.
 * ufe_gnn_predict_velocity: write the predicted velocity into the context's resident state for a
 * following resident solve with cold_start = 0, after `smooth_passes` (0: none) averaging passes over
 * each triangle and its neighbours (noise in the prediction roughens the first viscosity field).
 * ufe_gnn_predict_start: the same, and with with_viscosity = 1 also the predicted viscosity on the
 * vertices, which the next resident solve with cold_start = 0 uses in its first Picard iteration in
 * place of Glen's law (SSA: the vertex viscosity; DIVA: every layer, a depth-uniform first
 * viscosity), clamped as Glen's law is.  A cold start, a velocity upload or a solve consumes it. */
int32_t ufe_gnn_features(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity, float *x);
int32_t ufe_gnn_dataset_add(ufe_gnn *g, ufe_ctx *mesh_ctx, const float *features_before);
int32_t ufe_gnn_dataset_clear(ufe_gnn *g);
int32_t ufe_gnn_train(ufe_gnn *g, int32_t epochs, float lr, uint64_t seed, float *loss_per_epoch,
                      double *device_ms);
int32_t ufe_gnn_evaluate(ufe_gnn *g, double *mean_loss);
int32_t ufe_gnn_predict_velocity(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity, int32_t smooth_passes,
                                 double *device_ms);
int32_t ufe_gnn_predict_start(ufe_gnn *g, ufe_ctx *mesh_ctx, int32_t use_prev_velocity, int32_t smooth_passes,
                              int32_t with_viscosity, double *device_ms);

/* ---- ice thickness: conservation of mass ------------------------------------------------------ */
/* calc_dHi_dt (src/UFEMISM/ice_dynamics/conservation_of_mass/conservation_of_mass_main.f90:23-109)
 * with the explicit scheme (conservation_of_mass_explicit.f90:22-134) and the semi-implicit one
 * (conservation_of_mass_semiimplicit.f90:23-174): the upwind flux-divergence matrix M_divQ
 * (conservation_of_mass_utilities.f90:22-132, edge velocities as in map_velocities_from_b_to_c_2D,
 * map_velocities_to_c_grid.f90:17-69), the flux-limited time step (:158-204), the domain-border,
 * prescribed-thickness and no-ice conditions, and for the semi-implicit scheme the matrix equation
 * (1 + dt fs M_divQ) H(t+dt) = H(t) - dt (1 - fs) M_divQ H(t) + max(-H(t), dt m), solved with the
 * same BiCGStab/Jacobi as solve_matrix_equation_CSR_PETSc.  Computed on the mesh's own (caller's)
 * vertex numbering; every field is in the caller's order. */

/* The Voronoi geometry of type_mesh the flux divergence reads (mesh_types.f90: A, Cw; built by
 * mesh_secondary.f90): cell areas A (nV) and the lengths Cw of the shared Voronoi boundary of
 * each connection (nV x nC_mem, column-major like C).  Once per mesh, before ufe_calc_dHi_dt. */
int32_t ufe_mesh_voronoi_upload(ufe_ctx *ctx, const double *A, const double *Cw);

enum ufe_ice_integration { UFE_DHI_NONE = 0, UFE_DHI_EXPLICIT = 1, UFE_DHI_SEMIIMPLICIT = 2 };
enum ufe_bc_H { UFE_BC_H_ZERO = 0, UFE_BC_H_INFINITE = 1 };   /* BC_H_* 'zero', 'infinite' */

typedef struct {
  int32_t choice_ice_integration_method;                   /* ufe_ice_integration                  */
  int32_t BC_H_west, BC_H_east, BC_H_south, BC_H_north;    /* ufe_bc_H                             */
  int32_t dHi_PETSc_max_it;                                /* Krylov iteration limit               */
  double dHi_semiimplicit_fs;                              /* 0 explicit .. 1 implicit, >1 over-implicit */
  double dHi_PETSc_rtol, dHi_PETSc_abstol;
  double dt_ice_max, dt_ice_min;                           /* [yr], calc_flux_limited_timestep     */
  double Hi_min;                                           /* [m]                                  */
  int32_t reserved[4];
} ufe_thickness_params;

/* The reference's configuration defaults (model_configuration.f90): semi-implicit, fs 1.5, rtol
 * 1e-8, abstol 1e-6, dt_ice_max 10 yr, dt_ice_min 0.1 yr, Hi_min 0, BC_H 'zero' on all sides. */
void ufe_default_thickness_params(ufe_thickness_params *p);

typedef struct {
  const double *Hi, *Hb, *SL;             /* nV: thickness, bedrock, sea level at t            */
  const double *u_vav_b, *v_vav_b;        /* nTri: vertically averaged velocity [m/yr]          */
  const double *SMB, *BMB, *LMB;          /* nV [m/yr]; NULL = 0                                */
  const double *fraction_margin;          /* nV [0-1]; NULL = 1                                 */
  const int32_t *mask_noice;              /* nV, 1 = no ice allowed; NULL = none                */
  const double *dHi_dt_target;            /* nV [m/yr]; NULL = 0                                */
  const int32_t *BC_prescr_mask;          /* nV, 1 = prescribed; NULL = none (then ...Hi too)   */
  const double *BC_prescr_Hi;             /* nV                                                 */
  double *dHi_dt;                         /* nV in: the previous rate (the semi-implicit
                                             initial guess H + dt dH/dt; NULL in = 0); out       */
  double *Hi_tplusdt, *divQ, *AMB;        /* nV out                                             */
} ufe_thickness_fields;

typedef struct {
  int32_t n_Axb_its;        /* Krylov iterations of the semi-implicit solve                      */
  int32_t krylov_status;    /* UFE_OK or UFE_WARN_KRYLOV_MAXIT                                   */
  int32_t found_negative;   /* the reference's warning: H(t+dt) < -0.1 where H(t) > Hi_min         */
  int32_t pad;
  double device_ms;         /* device time of the step (CUDA events, without the copies)         */
} ufe_thickness_stats;

/* One call of calc_dHi_dt.  *dt is in/out as in the reference (the explicit scheme may shorten it). */
int32_t ufe_calc_dHi_dt(ufe_ctx *ctx, const ufe_thickness_params *p, ufe_thickness_fields *f, double *dt,
                        ufe_thickness_stats *stats);

/* The semi-implicit system after its boundary conditions -- stiffness matrix (0-based CSR in the
 * reference's add_entry order: the diagonal, then the neighbours in C order), load vector and
 * initial guess -- as the semi-implicit scheme hands it to the Krylov solve (for parity checks).
 * cap: entries val/ind can hold; *nnz receives the count. */
int32_t ufe_thickness_assemble(ufe_ctx *ctx, const ufe_thickness_params *p, const ufe_thickness_fields *f, double dt,
                               int32_t *ptr, int32_t *ind, double *val, double *bb, double *x0, int64_t cap,
                               int64_t *nnz);

/* ---- allocation-free solve -------------------------------------------------------------------- */
/* The CSR matrix-equation solve of ufe_solve_csr (same BiCGStab/Jacobi, same convergence test)
 * for callers that cannot let a library allocate device memory -- e.g. a host model whose GPU
 * memory is handed out by its own pool or caching allocator, or a coupled run that fixes its GPU
 * footprint at start-up.  This entry point has no counterpart in the reference.
 *
 * The matrix (d_ptr m+1, d_ind/d_val nnz, `index_base` 0 or 1), right-hand side and solution are
 * the caller's DEVICE buffers; d_xx holds the initial guess on entry and the solution on exit.
 * Work vectors and scalars live in one fixed device array of the library (about 9.1 MiB per GPU):
 * no cudaMalloc or cudaFree happens in the call.  Under CUDA's default lazy module loading the
 * array is reserved on a device by the first call there (with CUDA_MODULE_LOADING=EAGER, when the
 * CUDA context starts) and held until the process exits; later calls take no device memory.
 * Systems with more than 131,072 unknowns are rejected with UFE_ERR_CAPACITY.  The matrix is
 * checked on the device before use (ptr[0] = base, ptr[m] = nnz + base, ptr non-decreasing, every
 * column inside the matrix): a malformed one returns UFE_ERR_INVALID.  Work runs on `cuda_stream`
 * (NULL: the legacy default stream), which must belong to the current device, and the call
 * returns after it finishes.  On entry the call clears any CUDA error left pending by earlier
 * work.  All calls on a device share the array: calls that overlap on the GPU race.  The first
 * call on a device resolves the array's address and should come before any stream capture begins.
 * No context is needed. */
int32_t ufe_solve_csr_noalloc(int32_t m, int64_t nnz, const int32_t *d_ptr, const int32_t *d_ind,
                              const double *d_val, int32_t index_base, const double *d_bb, double *d_xx,
                              double rtol, double abstol, int32_t max_it, int32_t *n_Axb_its,
                              void *cuda_stream);

/* ---- diagnostics ---------------------------------------------------------------------------- */
/* Per-Picard-iteration record of the last solve on this context: `cap` rows of 5 values
 * (L2 change norm, Krylov iterations, Krylov status, final Krylov residual, FP64 refinement
 * steps); *n receives the rows written (at most 128). */
int32_t ufe_solve_history(ufe_ctx *ctx, double *out, int32_t cap, int32_t *n);

/* Time the three BiCGStab kernels on the system assembled by the last solve on this context:
 * each kernel is launched `repeats` times back to back between two CUDA events on the context's
 * stream (the kernels are idempotent for fixed scalars).  us[0..2] receive the mean duration in
 * microseconds of the p-update+SpMV, s-update+SpMV and x/r-update kernels; `precision` picks the
 * FP64 or FP32 kernels.  geometry[0..1] receive the block rows and the stored 2x2 blocks. */
int32_t ufe_profile_krylov_kernels(ufe_ctx *ctx, int32_t precision, int32_t repeats, double *us,
                                   int64_t *geometry);

#ifdef __cplusplus
}
#endif
#endif /* UFE_GPU_H */
