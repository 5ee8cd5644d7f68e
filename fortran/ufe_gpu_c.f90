! ufe_gpu_c -- ISO_C_BINDING mirror of include/ufe_gpu.h: the structs (bind(C) derived types with
! the same members in the same order) and an interface block for every entry point a UFEMISM
! caller uses.  Self-contained (iso_c_binding only), so it compiles on its own; ufe_gpu_mod.f90
! builds the reference-named wrappers on top of it inside the UFEMISM source tree.
!
! Arrays pass as type(c_ptr) members (c_loc of the Fortran arrays, which already have the layout
! the library expects: column-major, 1-based mesh indices) or as assumed-size dummies.
module ufe_gpu_c
  use iso_c_binding
  implicit none
  public

  ! status codes
  integer(c_int32_t), parameter :: UFE_OK = 0, UFE_WARN_PICARD_MAXIT = 1, UFE_WARN_KRYLOV_MAXIT = 2
  integer(c_int32_t), parameter :: UFE_ERR_INVALID = -1, UFE_ERR_NAN = -2, UFE_ERR_DIVERGED = -3
  integer(c_int32_t), parameter :: UFE_ERR_THERMO_UNSTABLE = -4, UFE_ERR_DEVICE = -5, UFE_ERR_CAPACITY = -6
  ! enum ufe_operator
  integer(c_int32_t), parameter :: UFE_OP_MAP_A_B = 0, UFE_OP_DDX_A_B = 1, UFE_OP_DDY_A_B = 2
  integer(c_int32_t), parameter :: UFE_OP_MAP_B_A = 3, UFE_OP_DDX_B_A = 4, UFE_OP_DDY_B_A = 5
  integer(c_int32_t), parameter :: UFE_OP_DDX_A_A = 6, UFE_OP_DDY_A_A = 7
  integer(c_int32_t), parameter :: UFE_OP_M2_DDX_B_B = 8, UFE_OP_M2_DDY_B_B = 9, UFE_OP_M2_D2DX2_B_B = 10
  integer(c_int32_t), parameter :: UFE_OP_M2_D2DXDY_B_B = 11, UFE_OP_M2_D2DY2_B_B = 12
  ! enum ufe_sliding_law, ufe_bc, ufe_rheology, ufe_enhancement, ufe_column_mask
  integer(c_int32_t), parameter :: UFE_SLIDING_NO_SLIDING = 0, UFE_SLIDING_WEERTMAN = 1, UFE_SLIDING_COULOMB = 2
  integer(c_int32_t), parameter :: UFE_SLIDING_BUDD = 3, UFE_SLIDING_TSAI2015 = 4, UFE_SLIDING_SCHOOF2005 = 5
  integer(c_int32_t), parameter :: UFE_SLIDING_ZOET_IVERSON = 6, UFE_SLIDING_IDEALISED_SSA_ICESTREAM = 7
  integer(c_int32_t), parameter :: UFE_BC_INFINITE = 0, UFE_BC_ZERO = 1, UFE_BC_INFINITE_SSA_ICESTREAM = 2
  integer(c_int32_t), parameter :: UFE_RHEOLOGY_INPUT = 0, UFE_RHEOLOGY_UNIFORM = 1, UFE_RHEOLOGY_HUYBRECHTS1992 = 2
  integer(c_int32_t), parameter :: UFE_ENH_SEPARATE = 0, UFE_ENH_INTERP = 1
  integer(c_int32_t), parameter :: UFE_COL_NONE = 0, UFE_COL_GROUNDED = 1, UFE_COL_FLOATING = 2, UFE_COL_GL_GR = 3
  ! enum ufe_ice_integration, ufe_bc_H
  integer(c_int32_t), parameter :: UFE_DHI_NONE = 0, UFE_DHI_EXPLICIT = 1, UFE_DHI_SEMIIMPLICIT = 2
  integer(c_int32_t), parameter :: UFE_BC_H_ZERO = 0, UFE_BC_H_INFINITE = 1

  type, bind(C) :: ufe_mesh_desc
    integer(c_int32_t) :: nV, nTri, nC_mem, nz
    type(c_ptr) :: V, nC, C, niTri, iTri, VBI, Tri, TriC, TriBI, TriGC, zeta
  end type

  type, bind(C) :: ufe_solver_params
    integer(c_int32_t) :: choice_sliding_law, do_include_SSADIVA_crossterms, do_GL_subgrid_friction
    integer(c_int32_t) :: BC_u_west, BC_u_east, BC_u_south, BC_u_north
    integer(c_int32_t) :: BC_v_west, BC_v_east, BC_v_south, BC_v_north
    integer(c_int32_t) :: visc_it_nit
    real(c_double) :: visc_it_norm_dUV_tol, visc_it_relax, visc_eff_min, vel_max
    real(c_double) :: stress_balance_PETSc_rtol, stress_balance_PETSc_abstol
    real(c_double) :: Glens_flow_law_exponent, Glens_flow_law_epsilon_sq_0, slid_Weertman_m
    real(c_double) :: slid_Budd_q_plastic, slid_Budd_u_threshold, subgrid_friction_exponent_on_B_grid
    real(c_double) :: slid_beta_max, slid_delta_v
    integer(c_int32_t) :: krylov_max_it, krylov_initial_guess, precision
    real(c_double) :: krylov_inner_rtol, krylov_forcing
    integer(c_int32_t) :: choice_ice_rheology_Glen, choice_enhancement_factor_transition
    real(c_double) :: uniform_Glens_flow_factor, m_enh_sheet, m_enh_shelf
    real(c_double) :: slid_ZI_p, slid_ZI_ut
    real(c_double) :: SSA_icestream_Hi, SSA_icestream_dhdx, SSA_icestream_L, SSA_icestream_m
    integer(c_int32_t) :: reserved(8)
  end type

  type, bind(C) :: ufe_ice_state
    type(c_ptr) :: Hi, Hs, A_flow, fraction_gr_b, mask_grounded_ice
    type(c_ptr) :: beta_sq, alpha_sq, effective_pressure, till_yield_stress
    type(c_ptr) :: Ti, mask_floating_ice, fraction_gr, Hib, SL
  end type

  type, bind(C) :: ufe_bc_prescribed
    type(c_ptr) :: mask_b, u_b, v_b
  end type

  type, bind(C) :: ufe_diva_state
    type(c_ptr) :: u_vav_b, v_vav_b, u_base_b, v_base_b, tau_bx_b, tau_by_b, eta_3D_b, u_3D_b, v_3D_b
  end type

  type, bind(C) :: ufe_solve_stats
    integer(c_int32_t) :: n_visc_its, n_Axb_its, n_refinements, status
    real(c_double) :: L2_uv, visc_it_relax_applied, device_ms
    integer(c_int32_t) :: n_fp64_its, n_kernels, n_pair_its
    integer(c_int32_t) :: reserved(3)
  end type

  type, bind(C) :: ufe_thermo_params
    real(c_double) :: dt, Hi_min_thermo
    integer(c_int32_t) :: choice_ice_heat_capacity, choice_ice_thermal_conductivity
    real(c_double) :: uniform_ice_heat_capacity, uniform_ice_thermal_conductivity
    integer(c_int32_t) :: choice_GL_temperature_BC
    integer(c_int32_t) :: reserved(7)
  end type

  type, bind(C) :: ufe_heat_fields
    type(c_ptr) :: Ti, Hi, Hi_eff, Hs, dHi_dt, dHs_dt, u_vav, v_vav, u_3D, v_3D, w_3D, u_3D_b, v_3D_b
    type(c_ptr) :: internal_heating, frictional_heating, geothermal_heat_flux, T2m
    integer(c_int32_t) :: n_months, pad
    type(c_ptr) :: SMB, mask, fraction_gr
    type(c_ptr) :: A_flow, du_dx_3D, du_dy_3D, du_dz_3D, dv_dx_3D, dv_dy_3D, dv_dz_3D, dw_dx_3D, dw_dy_3D, dw_dz_3D
    type(c_ptr) :: basal_friction_coefficient, uabs_base
    integer(c_int32_t) :: no_sliding, pad2
    real(c_double) :: Glens_flow_law_exponent
  end type

  type, bind(C) :: ufe_thickness_params
    integer(c_int32_t) :: choice_ice_integration_method, BC_H_west, BC_H_east, BC_H_south, BC_H_north
    integer(c_int32_t) :: dHi_PETSc_max_it
    real(c_double) :: dHi_semiimplicit_fs, dHi_PETSc_rtol, dHi_PETSc_abstol, dt_ice_max, dt_ice_min, Hi_min
    integer(c_int32_t) :: reserved(4)
  end type

  type, bind(C) :: ufe_thickness_fields
    type(c_ptr) :: Hi, Hb, SL, u_vav_b, v_vav_b, SMB, BMB, LMB, fraction_margin, mask_noice, dHi_dt_target
    type(c_ptr) :: BC_prescr_mask, BC_prescr_Hi, dHi_dt, Hi_tplusdt, divQ, AMB
  end type

  type, bind(C) :: ufe_thickness_stats
    integer(c_int32_t) :: n_Axb_its, krylov_status, found_negative, pad
    real(c_double) :: device_ms
  end type

  interface
    subroutine ufe_default_thickness_params(p) bind(C, name='ufe_default_thickness_params')
      import :: ufe_thickness_params
      type(ufe_thickness_params), intent(out) :: p
    end subroutine
    integer(c_int32_t) function ufe_mesh_voronoi_upload(ctx, A, Cw) bind(C, name='ufe_mesh_voronoi_upload')
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: A(*), Cw(*)
    end function
    integer(c_int32_t) function ufe_calc_dHi_dt(ctx, p, f, dt, st) bind(C, name='ufe_calc_dHi_dt')
      import :: c_int32_t, c_ptr, c_double, ufe_thickness_params, ufe_thickness_fields, ufe_thickness_stats
      type(c_ptr), value :: ctx
      type(ufe_thickness_params), intent(in) :: p
      type(ufe_thickness_fields), intent(in) :: f
      real(c_double), intent(inout) :: dt
      type(ufe_thickness_stats), intent(out) :: st
    end function
    subroutine ufe_default_params(p) bind(C, name='ufe_default_params')
      import :: ufe_solver_params
      type(ufe_solver_params), intent(out) :: p
    end subroutine
    subroutine ufe_default_thermo_params(p) bind(C, name='ufe_default_thermo_params')
      import :: ufe_thermo_params
      type(ufe_thermo_params), intent(out) :: p
    end subroutine
    integer(c_int32_t) function ufe_ctx_create(device, ctx) bind(C, name='ufe_ctx_create')
      import :: c_int32_t, c_ptr
      integer(c_int32_t), value :: device
      type(c_ptr), intent(out) :: ctx
    end function
    subroutine ufe_ctx_destroy(ctx) bind(C, name='ufe_ctx_destroy')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    type(c_ptr) function ufe_ctx_last_error(ctx) bind(C, name='ufe_ctx_last_error')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int32_t) function ufe_mesh_upload(ctx, m) bind(C, name='ufe_mesh_upload')
      import :: c_int32_t, c_ptr, ufe_mesh_desc
      type(c_ptr), value :: ctx
      type(ufe_mesh_desc), intent(in) :: m
    end function
    integer(c_int32_t) function ufe_mesh_build_operators(ctx) bind(C, name='ufe_mesh_build_operators')
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int32_t) function ufe_mesh_set_operator(ctx, op, m, n, nnz, ptr, ind, val, index_base) &
        bind(C, name='ufe_mesh_set_operator')
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: op, m, n, index_base
      integer(c_int64_t), value :: nnz
      integer(c_int32_t), intent(in) :: ptr(*), ind(*)
      real(c_double), intent(in) :: val(*)
    end function
    integer(c_int32_t) function ufe_apply_operator(ctx, op, x, y, ncols) bind(C, name='ufe_apply_operator')
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: op, ncols
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(out) :: y(*)
    end function
    integer(c_int32_t) function ufe_csr_spmv(ctx, m, n, nnz, ptr, ind, val, index_base, x, y, ncols) &
        bind(C, name='ufe_csr_spmv')
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: m, n, index_base, ncols
      integer(c_int64_t), value :: nnz
      integer(c_int32_t), intent(in) :: ptr(*), ind(*)
      real(c_double), intent(in) :: val(*), x(*)
      real(c_double), intent(out) :: y(*)
    end function
    integer(c_int32_t) function ufe_solve_csr(ctx, m, nnz, ptr, ind, val, index_base, bb, xx, rtol, abstol, &
        max_it, n_Axb_its) bind(C, name='ufe_solve_csr')
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: m, index_base, max_it
      integer(c_int64_t), value :: nnz
      integer(c_int32_t), intent(in) :: ptr(*), ind(*)
      real(c_double), intent(in) :: val(*), bb(*)
      real(c_double), intent(inout) :: xx(*)
      real(c_double), value :: rtol, abstol
      integer(c_int32_t), intent(out) :: n_Axb_its
    end function
    integer(c_int32_t) function ufe_solve_ssa(ctx, p, ice, bc, u_b, v_b, n_visc, n_axb, st) &
        bind(C, name='ufe_solve_ssa')
      import :: c_int32_t, c_ptr, c_double, ufe_solver_params, ufe_ice_state, ufe_solve_stats
      type(c_ptr), value :: ctx, bc
      type(ufe_solver_params), intent(in) :: p
      type(ufe_ice_state), intent(in) :: ice
      real(c_double), intent(inout) :: u_b(*), v_b(*)
      integer(c_int32_t), intent(out) :: n_visc, n_axb
      type(ufe_solve_stats), intent(out) :: st
    end function
    integer(c_int32_t) function ufe_solve_diva(ctx, p, ice, bc, ds, n_visc, n_axb, st) &
        bind(C, name='ufe_solve_diva')
      import :: c_int32_t, c_ptr, ufe_solver_params, ufe_ice_state, ufe_diva_state, ufe_solve_stats
      type(c_ptr), value :: ctx, bc
      type(ufe_solver_params), intent(in) :: p
      type(ufe_ice_state), intent(in) :: ice
      type(ufe_diva_state), intent(in) :: ds
      integer(c_int32_t), intent(out) :: n_visc, n_axb
      type(ufe_solve_stats), intent(out) :: st
    end function
    integer(c_int32_t) function ufe_solve_3D_heat_equation(ctx, p, f, Ti_next, n_unstable) &
        bind(C, name='ufe_solve_3D_heat_equation')
      import :: c_int32_t, c_ptr, c_double, ufe_thermo_params, ufe_heat_fields
      type(c_ptr), value :: ctx
      type(ufe_thermo_params), intent(in) :: p
      type(ufe_heat_fields), intent(in) :: f
      real(c_double), intent(out) :: Ti_next(*)
      integer(c_int32_t), intent(out) :: n_unstable
    end function
    integer(c_int32_t) function ufe_tridiagonal_solve(ctx, n, nsys, a, b, c, d, x) &
        bind(C, name='ufe_tridiagonal_solve')
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: n, nsys
      real(c_double), intent(in) :: a(*), b(*), c(*), d(*)
      real(c_double), intent(out) :: x(*)
    end function
  end interface

contains

  ! The C string of ufe_ctx_last_error as a Fortran string (for crash messages).
  function ufe_last_error(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: s(:)
    integer :: n
    interface
      integer(c_size_t) function strlen(p) bind(C, name='strlen')
        import :: c_ptr, c_size_t
        type(c_ptr), value :: p
      end function
    end interface
    type(c_ptr) :: p
    p = ufe_ctx_last_error(ctx)
    n = int(strlen(p))
    call c_f_pointer(p, s, [n])
    allocate(character(len=n) :: msg)
    msg = transfer(s(1:n), msg)
  end function

end module ufe_gpu_c
