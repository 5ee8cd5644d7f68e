! ufe_gpu_mod -- the GB300 library behind UFEMISM's own routine names.
!
! Compiled inside the UFEMISM2.0 source tree (it uses the model's types and configuration).  Each
! wrapper keeps the argument list of the routine it replaces, fills the C structs of ufe_gpu_c
! with c_loc pointers to the model's arrays (no copies on the Fortran side) and maps the library's
! status codes onto the model's crash/warning handling.  A model region owns one context, created
! with the mesh (ufe_attach_mesh, called from initialise_model_region and after every remesh).
!
! Replaces:
!   solve_SSA                         SSA_main.f90:87-242
!   solve_DIVA                        DIVA_main.f90:88-262
!   solve_matrix_equation_CSR_PETSc   src/UPSY/basic/petsc_basic.f90:32-64
!   map_a_b_2D ... ddy_b_a_3D         src/UPSY/mesh/discretisation/mesh_disc_apply_operators.f90:121-431
!   solve_3D_heat_equation            src/UFEMISM/thermodynamics/thermodynamics_3D_heat_equation.f90:33-307
!   solve_tridiagonal_matrix_equation src/UPSY/basic/math_utilities/tridiagonal_solver.f90:13-51
! The wrappers carry a gpu_ prefix so that both implementations can sit in one build while a
! model is switched over; renaming them to the plain names makes them a drop-in.
module ufe_gpu_mod
  use iso_c_binding
  use ufe_gpu_c
  use precisions, only: dp
  use parameters, only: pi
  use mesh_types, only: type_mesh
  use ice_model_types, only: type_ice_model, type_ice_velocity_solver_SSA, type_ice_velocity_solver_DIVA
  use bed_roughness_model_types, only: type_bed_roughness_model
  use climate_model_types, only: type_climate_model
  use SMB_model_types, only: type_SMB_model
  use CSR_sparse_matrix_type, only: type_sparse_matrix_CSR_dp
  use model_configuration, only: C
  use control_resources_and_error_messaging, only: crash, warning
  implicit none

  private
  public :: ufe_attach_mesh, ufe_detach, gpu_solve_SSA, gpu_solve_DIVA, gpu_solve_matrix_equation_CSR_PETSc
  public :: gpu_map_a_b_2D, gpu_ddx_a_b_2D, gpu_ddy_a_b_2D, gpu_map_b_a_2D, gpu_ddx_b_a_2D, gpu_ddy_b_a_2D
  public :: gpu_map_a_b_3D, gpu_map_b_a_3D, gpu_solve_3D_heat_equation, gpu_solve_tridiagonal_matrix_equation
  public :: gpu_calc_dHi_dt

  type(c_ptr), save :: ctx = c_null_ptr
  logical, save :: voronoi_uploaded = .false.    ! mesh%A, mesh%Cw sent for the attached mesh

contains

  subroutine check(rc, what)
    integer(c_int32_t), intent(in) :: rc
    character(len=*), intent(in) :: what
    if (rc < 0) call crash(what // ': ' // ufe_last_error(ctx))
    if (rc > 0) call warning(what // ': viscosity or Krylov iteration did not reach its tolerance')
  end subroutine

  subroutine ufe_attach_mesh(mesh)
    type(type_mesh), target, intent(in) :: mesh
    type(ufe_mesh_desc) :: d
    if (.not. c_associated(ctx)) then
      if (ufe_ctx_create(0_c_int32_t, ctx) /= UFE_OK) call crash('no GB300 device for the velocity solve')
    end if
    d = ufe_mesh_desc(mesh%nV, mesh%nTri, mesh%nC_mem, mesh%nz, c_loc(mesh%V), c_loc(mesh%nC), c_loc(mesh%C), &
      c_loc(mesh%niTri), c_loc(mesh%iTri), c_loc(mesh%VBI), c_loc(mesh%Tri), c_loc(mesh%TriC), &
      c_loc(mesh%TriBI), c_loc(mesh%TriGC), c_loc(mesh%zeta))
    call check(ufe_mesh_upload(ctx, d), 'ufe_mesh_upload')
    call check(ufe_mesh_build_operators(ctx), 'ufe_mesh_build_operators')
    voronoi_uploaded = .false.
  end subroutine

  subroutine ufe_detach()
    if (c_associated(ctx)) call ufe_ctx_destroy(ctx)
    ctx = c_null_ptr
  end subroutine

  integer(c_int32_t) function bc_code(s)
    character(len=*), intent(in) :: s
    select case (trim(s))
    case ('infinite');               bc_code = UFE_BC_INFINITE
    case ('zero');                   bc_code = UFE_BC_ZERO
    case ('infinite_SSA_icestream'); bc_code = UFE_BC_INFINITE_SSA_ICESTREAM
    case default
      call crash('boundary condition "' // trim(s) // '" is not offered by the GPU solve')
      bc_code = -1
    end select
  end function

  ! model_configuration -> ufe_solver_params (the fields the velocity solve reads)
  subroutine params_from_config(p, rtol, abstol)
    type(ufe_solver_params), intent(out) :: p
    real(dp), intent(in) :: rtol, abstol
    call ufe_default_params(p)
    select case (trim(C%choice_sliding_law))
    case ('no_sliding');   p%choice_sliding_law = UFE_SLIDING_NO_SLIDING
    case ('Weertman');     p%choice_sliding_law = UFE_SLIDING_WEERTMAN
    case ('Coulomb');      p%choice_sliding_law = UFE_SLIDING_COULOMB
    case ('Budd');         p%choice_sliding_law = UFE_SLIDING_BUDD
    case ('Tsai2015');     p%choice_sliding_law = UFE_SLIDING_TSAI2015
    case ('Schoof2005');   p%choice_sliding_law = UFE_SLIDING_SCHOOF2005
    case ('Zoet-Iverson'); p%choice_sliding_law = UFE_SLIDING_ZOET_IVERSON
    case ('idealised')
      if (trim(C%choice_idealised_sliding_law) /= 'SSA_icestream') &
        call crash('idealised sliding law "' // trim(C%choice_idealised_sliding_law) // '" is not offered on the GPU')
      p%choice_sliding_law = UFE_SLIDING_IDEALISED_SSA_ICESTREAM
    case default
      call crash('unknown choice_sliding_law "' // trim(C%choice_sliding_law) // '"')
    end select
    p%do_include_SSADIVA_crossterms = merge(1, 0, C%do_include_SSADIVA_crossterms)
    p%do_GL_subgrid_friction = merge(1, 0, C%do_GL_subgrid_friction)
    p%BC_u_west = bc_code(C%BC_u_west);   p%BC_u_east = bc_code(C%BC_u_east)
    p%BC_u_south = bc_code(C%BC_u_south); p%BC_u_north = bc_code(C%BC_u_north)
    p%BC_v_west = bc_code(C%BC_v_west);   p%BC_v_east = bc_code(C%BC_v_east)
    p%BC_v_south = bc_code(C%BC_v_south); p%BC_v_north = bc_code(C%BC_v_north)
    p%visc_it_nit = C%visc_it_nit
    p%visc_it_norm_dUV_tol = C%visc_it_norm_dUV_tol
    p%visc_it_relax = C%visc_it_relax
    p%visc_eff_min = C%visc_eff_min
    p%vel_max = C%vel_max
    p%stress_balance_PETSc_rtol = rtol
    p%stress_balance_PETSc_abstol = abstol
    p%Glens_flow_law_exponent = C%Glens_flow_law_exponent
    p%Glens_flow_law_epsilon_sq_0 = C%Glens_flow_law_epsilon_sq_0
    p%slid_Weertman_m = C%slid_Weertman_m
    p%slid_Budd_q_plastic = C%slid_Budd_q_plastic
    p%slid_Budd_u_threshold = C%slid_Budd_u_threshold
    p%subgrid_friction_exponent_on_B_grid = C%subgrid_friction_exponent_on_B_grid
    p%slid_beta_max = C%slid_beta_max
    p%slid_delta_v = C%slid_delta_v
    p%slid_ZI_p = C%slid_ZI_p
    p%slid_ZI_ut = C%slid_ZI_ut
    p%SSA_icestream_Hi = C%refgeo_idealised_SSA_icestream_Hi
    p%SSA_icestream_dhdx = C%refgeo_idealised_SSA_icestream_dhdx
    p%SSA_icestream_L = C%refgeo_idealised_SSA_icestream_L
    p%SSA_icestream_m = C%refgeo_idealised_SSA_icestream_m
    ! calc_ice_rheology_Glen runs inside the GPU solve
    select case (trim(C%choice_ice_rheology_Glen))
    case ('uniform');        p%choice_ice_rheology_Glen = UFE_RHEOLOGY_UNIFORM
    case ('Huybrechts1992'); p%choice_ice_rheology_Glen = UFE_RHEOLOGY_HUYBRECHTS1992
    case default
      p%choice_ice_rheology_Glen = UFE_RHEOLOGY_INPUT      ! other choices: the model computes ice%A_flow
    end select
    p%choice_enhancement_factor_transition = merge(UFE_ENH_INTERP, UFE_ENH_SEPARATE, &
      trim(C%choice_enhancement_factor_transition) == 'interp')
    p%uniform_Glens_flow_factor = C%uniform_Glens_flow_factor
    p%m_enh_sheet = C%m_enh_sheet
    p%m_enh_shelf = C%m_enh_shelf
  end subroutine

  ! The ice-state struct over the model's arrays; the logical masks become int32 copies.
  subroutine ice_from_model(ice, bed_roughness, st, mask_gr, mask_fl)
    type(type_ice_model), target, intent(inout) :: ice
    type(type_bed_roughness_model), target, intent(in) :: bed_roughness
    type(ufe_ice_state), intent(out) :: st
    integer(c_int32_t), allocatable, target, intent(inout) :: mask_gr(:), mask_fl(:)
    mask_gr = merge(1_c_int32_t, 0_c_int32_t, ice%mask_grounded_ice)
    mask_fl = merge(1_c_int32_t, 0_c_int32_t, ice%mask_floating_ice)
    st%Hi = c_loc(ice%Hi)
    st%Hs = c_loc(ice%Hs)
    st%A_flow = c_loc(ice%A_flow)
    st%fraction_gr_b = c_loc(ice%fraction_gr_b)
    st%mask_grounded_ice = c_loc(mask_gr)
    st%beta_sq = c_loc(bed_roughness%beta_sq)
    st%alpha_sq = c_loc(bed_roughness%alpha_sq)
    st%effective_pressure = c_loc(ice%effective_pressure)
    st%till_yield_stress = c_loc(ice%till_yield_stress)
    st%Ti = c_loc(ice%Ti)
    st%mask_floating_ice = c_loc(mask_fl)
    st%fraction_gr = c_loc(ice%fraction_gr)
    st%Hib = c_loc(ice%Hib)
    st%SL = c_loc(ice%SL)
  end subroutine

  subroutine prescribed_bc(bc, mask_b, BC_prescr_mask_b, BC_prescr_u_b, BC_prescr_v_b)
    type(ufe_bc_prescribed), target, intent(out) :: bc
    integer(c_int32_t), allocatable, target, intent(inout) :: mask_b(:)
    integer,  dimension(:), optional, intent(in) :: BC_prescr_mask_b
    real(dp), dimension(:), optional, target, intent(in) :: BC_prescr_u_b, BC_prescr_v_b
    bc = ufe_bc_prescribed(c_null_ptr, c_null_ptr, c_null_ptr)
    if (present(BC_prescr_mask_b) .or. present(BC_prescr_u_b) .or. present(BC_prescr_v_b)) then
      if (.not. (present(BC_prescr_mask_b) .and. present(BC_prescr_u_b) .and. present(BC_prescr_v_b))) &
        call crash('need to provide prescribed u,v fields and mask!')
      mask_b = int(BC_prescr_mask_b, c_int32_t)
      bc = ufe_bc_prescribed(c_loc(mask_b), c_loc(BC_prescr_u_b), c_loc(BC_prescr_v_b))
    end if
  end subroutine

  ! solve_SSA (SSA_main.f90:87-100): same arguments
  subroutine gpu_solve_SSA(mesh, ice, bed_roughness, SSA, n_visc_its, n_Axb_its, &
      BC_prescr_mask_b, BC_prescr_u_b, BC_prescr_v_b)
    type(type_mesh), intent(in) :: mesh
    type(type_ice_model), target, intent(inout) :: ice
    type(type_bed_roughness_model), target, intent(in) :: bed_roughness
    type(type_ice_velocity_solver_SSA), target, intent(inout) :: SSA
    integer, intent(out) :: n_visc_its, n_Axb_its
    integer,  dimension(:), optional, intent(in) :: BC_prescr_mask_b
    real(dp), dimension(:), optional, target, intent(in) :: BC_prescr_u_b, BC_prescr_v_b
    type(ufe_solver_params) :: p
    type(ufe_ice_state) :: st
    type(ufe_bc_prescribed), target :: bc
    type(ufe_solve_stats) :: stats
    integer(c_int32_t), allocatable, target :: mask_gr(:), mask_fl(:), mask_b(:)
    integer(c_int32_t) :: nv, na
    type(c_ptr) :: pbc
    call params_from_config(p, C%stress_balance_PETSc_rtol, C%stress_balance_PETSc_abstol)
    call ice_from_model(ice, bed_roughness, st, mask_gr, mask_fl)
    call prescribed_bc(bc, mask_b, BC_prescr_mask_b, BC_prescr_u_b, BC_prescr_v_b)
    pbc = merge(c_loc(bc), c_null_ptr, c_associated(bc%mask_b))
    call check(ufe_solve_ssa(ctx, p, st, pbc, SSA%u_b, SSA%v_b, nv, na, stats), 'solve_SSA')
    n_visc_its = nv
    n_Axb_its = na
  end subroutine

  ! solve_DIVA (DIVA_main.f90:88-101): same arguments
  subroutine gpu_solve_DIVA(mesh, ice, bed_roughness, DIVA, n_visc_its, n_Axb_its, &
      BC_prescr_mask_b, BC_prescr_u_b, BC_prescr_v_b)
    type(type_mesh), intent(in) :: mesh
    type(type_ice_model), target, intent(inout) :: ice
    type(type_bed_roughness_model), target, intent(in) :: bed_roughness
    type(type_ice_velocity_solver_DIVA), target, intent(inout) :: DIVA
    integer, intent(out) :: n_visc_its, n_Axb_its
    integer,  dimension(:), optional, intent(in) :: BC_prescr_mask_b
    real(dp), dimension(:), optional, target, intent(in) :: BC_prescr_u_b, BC_prescr_v_b
    type(ufe_solver_params) :: p
    type(ufe_ice_state) :: st
    type(ufe_bc_prescribed), target :: bc
    type(ufe_diva_state) :: ds
    type(ufe_solve_stats) :: stats
    integer(c_int32_t), allocatable, target :: mask_gr(:), mask_fl(:), mask_b(:)
    integer(c_int32_t) :: nv, na
    type(c_ptr) :: pbc
    call params_from_config(p, C%stress_balance_PETSc_rtol, C%stress_balance_PETSc_abstol)
    call ice_from_model(ice, bed_roughness, st, mask_gr, mask_fl)
    call prescribed_bc(bc, mask_b, BC_prescr_mask_b, BC_prescr_u_b, BC_prescr_v_b)
    pbc = merge(c_loc(bc), c_null_ptr, c_associated(bc%mask_b))
    ds = ufe_diva_state(c_loc(DIVA%u_vav_b), c_loc(DIVA%v_vav_b), c_loc(DIVA%u_base_b), c_loc(DIVA%v_base_b), &
      c_loc(DIVA%tau_bx_b), c_loc(DIVA%tau_by_b), c_loc(DIVA%eta_3D_b), c_loc(DIVA%u_3D_b), c_loc(DIVA%v_3D_b))
    call check(ufe_solve_diva(ctx, p, st, pbc, ds, nv, na, stats), 'solve_DIVA')
    n_visc_its = nv
    n_Axb_its = na
  end subroutine

  ! solve_matrix_equation_CSR_PETSc (petsc_basic.f90:32-41): BiCGStab + Jacobi on the GPU
  subroutine gpu_solve_matrix_equation_CSR_PETSc(AA, bb, xx, rtol, abstol, n_Axb_its)
    type(type_sparse_matrix_CSR_dp), intent(in) :: AA
    real(dp), dimension(:), intent(in) :: bb
    real(dp), dimension(:), intent(inout) :: xx
    real(dp), intent(in) :: rtol, abstol
    integer, intent(out) :: n_Axb_its
    integer(c_int32_t) :: its
    call check(ufe_solve_csr(ctx, int(AA%m, c_int32_t), int(AA%nnz, c_int64_t), AA%ptr, AA%ind, AA%val, 1_c_int32_t, &
      bb, xx, rtol, abstol, 10000_c_int32_t, its), 'solve_matrix_equation_CSR_PETSc')
    n_Axb_its = its
  end subroutine

  ! mesh_disc_apply_operators.f90: each is one SpMV with the GPU-resident operator
  subroutine apply(op, d_in, d_out, ncols)
    integer(c_int32_t), intent(in) :: op, ncols
    real(dp), dimension(*), intent(in) :: d_in
    real(dp), dimension(*), intent(out) :: d_out
    call check(ufe_apply_operator(ctx, op, d_in, d_out, ncols), 'apply operator')
  end subroutine
  subroutine gpu_map_a_b_2D(mesh, d_a, d_b)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_a
    real(dp), dimension(:), intent(out) :: d_b
    call apply(UFE_OP_MAP_A_B, d_a, d_b, 1_c_int32_t)
  end subroutine
  subroutine gpu_ddx_a_b_2D(mesh, d_a, d_b)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_a
    real(dp), dimension(:), intent(out) :: d_b
    call apply(UFE_OP_DDX_A_B, d_a, d_b, 1_c_int32_t)
  end subroutine
  subroutine gpu_ddy_a_b_2D(mesh, d_a, d_b)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_a
    real(dp), dimension(:), intent(out) :: d_b
    call apply(UFE_OP_DDY_A_B, d_a, d_b, 1_c_int32_t)
  end subroutine
  subroutine gpu_map_b_a_2D(mesh, d_b, d_a)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_b
    real(dp), dimension(:), intent(out) :: d_a
    call apply(UFE_OP_MAP_B_A, d_b, d_a, 1_c_int32_t)
  end subroutine
  subroutine gpu_ddx_b_a_2D(mesh, d_b, d_a)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_b
    real(dp), dimension(:), intent(out) :: d_a
    call apply(UFE_OP_DDX_B_A, d_b, d_a, 1_c_int32_t)
  end subroutine
  subroutine gpu_ddy_b_a_2D(mesh, d_b, d_a)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:), intent(in) :: d_b
    real(dp), dimension(:), intent(out) :: d_a
    call apply(UFE_OP_DDY_B_A, d_b, d_a, 1_c_int32_t)
  end subroutine
  subroutine gpu_map_a_b_3D(mesh, d_a, d_b)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:,:), intent(in) :: d_a
    real(dp), dimension(:,:), intent(out) :: d_b
    call apply(UFE_OP_MAP_A_B, d_a, d_b, int(size(d_a, 2), c_int32_t))
  end subroutine
  subroutine gpu_map_b_a_3D(mesh, d_b, d_a)
    type(type_mesh), intent(in) :: mesh
    real(dp), dimension(:,:), intent(in) :: d_b
    real(dp), dimension(:,:), intent(out) :: d_a
    call apply(UFE_OP_MAP_B_A, d_b, d_a, int(size(d_b, 2), c_int32_t))
  end subroutine

  ! solve_3D_heat_equation (thermodynamics_3D_heat_equation.f90:33): prelude and heating terms on
  ! the GPU; ice%Ti_next receives the new temperature
  subroutine gpu_solve_3D_heat_equation(mesh, ice, climate, SMB, dt)
    type(type_mesh), intent(in) :: mesh
    type(type_ice_model), target, intent(inout) :: ice
    type(type_climate_model), target, intent(in) :: climate
    type(type_SMB_model), target, intent(in) :: SMB
    real(dp), intent(in) :: dt
    type(ufe_thermo_params) :: p
    type(ufe_heat_fields) :: f
    integer(c_int32_t), allocatable, target :: mask(:)
    integer(c_int32_t) :: n_unstable, rc
    call ufe_default_thermo_params(p)
    p%dt = dt
    p%Hi_min_thermo = C%Hi_min_thermo
    p%choice_ice_heat_capacity = merge(1, 0, trim(C%choice_ice_heat_capacity) == 'Pounder1965')
    p%choice_ice_thermal_conductivity = merge(1, 0, trim(C%choice_ice_thermal_conductivity) == 'Ritz1987')
    p%uniform_ice_heat_capacity = C%uniform_ice_heat_capacity
    p%uniform_ice_thermal_conductivity = C%uniform_ice_thermal_conductivity
    select case (trim(C%choice_GL_temperature_BC))
    case ('subgrid'); p%choice_GL_temperature_BC = 1
    case ('pmp');     p%choice_GL_temperature_BC = 2
    case default;     p%choice_GL_temperature_BC = 0
    end select
    ! column types in the order the reference tests them (:168,198,207)
    mask = merge(UFE_COL_GL_GR, merge(UFE_COL_GROUNDED, merge(UFE_COL_FLOATING, UFE_COL_NONE, &
      ice%mask_floating_ice), ice%mask_grounded_ice), ice%mask_gl_gr)
    f%Ti = c_loc(ice%Ti); f%Hi = c_loc(ice%Hi); f%Hi_eff = c_loc(ice%Hi_eff); f%Hs = c_loc(ice%Hs)
    f%dHi_dt = c_loc(ice%dHi_dt); f%dHs_dt = c_loc(ice%dHs_dt)
    f%u_vav = c_loc(ice%u_vav); f%v_vav = c_loc(ice%v_vav)
    f%u_3D = c_loc(ice%u_3D); f%v_3D = c_loc(ice%v_3D); f%w_3D = c_loc(ice%w_3D)
    f%u_3D_b = c_loc(ice%u_3D_b); f%v_3D_b = c_loc(ice%v_3D_b)
    f%internal_heating = c_null_ptr            ! calc_strain_heating on the GPU
    f%frictional_heating = c_null_ptr          ! calc_frictional_heating on the GPU
    f%geothermal_heat_flux = c_loc(ice%geothermal_heat_flux)
    f%T2m = c_loc(climate%T2m); f%n_months = int(size(climate%T2m, 2), c_int32_t); f%pad = 0
    f%SMB = c_loc(SMB%SMB); f%mask = c_loc(mask); f%fraction_gr = c_loc(ice%fraction_gr)
    f%A_flow = c_loc(ice%A_flow)
    f%du_dx_3D = c_loc(ice%du_dx_3D); f%du_dy_3D = c_loc(ice%du_dy_3D); f%du_dz_3D = c_loc(ice%du_dz_3D)
    f%dv_dx_3D = c_loc(ice%dv_dx_3D); f%dv_dy_3D = c_loc(ice%dv_dy_3D); f%dv_dz_3D = c_loc(ice%dv_dz_3D)
    f%dw_dx_3D = c_loc(ice%dw_dx_3D); f%dw_dy_3D = c_loc(ice%dw_dy_3D); f%dw_dz_3D = c_loc(ice%dw_dz_3D)
    f%basal_friction_coefficient = c_loc(ice%basal_friction_coefficient)
    f%uabs_base = c_loc(ice%uabs_base)
    f%no_sliding = merge(1, 0, trim(C%choice_sliding_law) == 'no_sliding'); f%pad2 = 0
    f%Glens_flow_law_exponent = C%Glens_flow_law_exponent
    rc = ufe_solve_3D_heat_equation(ctx, p, f, ice%Ti_next, n_unstable)
    if (rc == UFE_ERR_THERMO_UNSTABLE) call crash('heat equation solver unstable for more than 1% of vertices!')
    call check(rc, 'solve_3D_heat_equation')
  end subroutine

  ! solve_tridiagonal_matrix_equation (tridiagonal_solver.f90:13-51): a(2:n), b(1:n), c(1:n-1), d(1:n);
  ! the library takes n-long sub- and super-diagonals (first and last entry unused)
  subroutine gpu_solve_tridiagonal_matrix_equation(n, a, b, c, d, x)
    integer, intent(in) :: n
    real(dp), dimension(2:n), intent(in) :: a
    real(dp), dimension(1:n), intent(in) :: b, d
    real(dp), dimension(1:n-1), intent(in) :: c
    real(dp), dimension(1:n), intent(out) :: x
    real(dp), dimension(1:n) :: a_n, c_n
    a_n(1) = 0._dp
    a_n(2:n) = a
    c_n(1:n-1) = c
    c_n(n) = 0._dp
    call check(ufe_tridiagonal_solve(ctx, int(n, c_int32_t), 1_c_int32_t, a_n, b, c_n, d, x), &
      'solve_tridiagonal_matrix_equation')
  end subroutine

  ! calc_dHi_dt (conservation_of_mass_main.f90:23-109) with the same arguments; the mesh's Voronoi
  ! geometry (mesh%A, mesh%Cw) goes to the GPU on the first call after each ufe_attach_mesh
  subroutine gpu_calc_dHi_dt(mesh, Hi, Hb, SL, u_vav_b, v_vav_b, SMB, BMB, LMB, AMB, fraction_margin, &
      mask_noice, dt, dHi_dt, Hi_tplusdt, divQ, dHi_dt_target, BC_prescr_mask, BC_prescr_Hi)
    type(type_mesh), target, intent(in) :: mesh
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(in) :: Hi, Hb, SL, SMB, BMB, LMB, fraction_margin
    real(dp), dimension(mesh%ti1:mesh%ti2), target, intent(in) :: u_vav_b, v_vav_b
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(inout) :: AMB
    logical, dimension(mesh%vi1:mesh%vi2), intent(in) :: mask_noice
    real(dp), intent(inout) :: dt
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(inout) :: dHi_dt    ! in: the previous rate
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(out) :: Hi_tplusdt, divQ
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(in) :: dHi_dt_target
    integer, dimension(mesh%vi1:mesh%vi2), target, intent(in), optional :: BC_prescr_mask
    real(dp), dimension(mesh%vi1:mesh%vi2), target, intent(in), optional :: BC_prescr_Hi
    type(ufe_thickness_params) :: p
    type(ufe_thickness_fields) :: f
    type(ufe_thickness_stats) :: st
    integer(c_int32_t), allocatable, target :: noice(:), prescr(:)
    if (.not. voronoi_uploaded) then
      call check(ufe_mesh_voronoi_upload(ctx, mesh%A, mesh%Cw), 'ufe_mesh_voronoi_upload')
      voronoi_uploaded = .true.
    end if
    call ufe_default_thickness_params(p)
    select case (trim(C%choice_ice_integration_method))
    case ('none');          p%choice_ice_integration_method = UFE_DHI_NONE
    case ('explicit');      p%choice_ice_integration_method = UFE_DHI_EXPLICIT
    case ('semi-implicit'); p%choice_ice_integration_method = UFE_DHI_SEMIIMPLICIT
    case default; call crash('unknown choice_ice_integration_method "' // trim(C%choice_ice_integration_method) // '"!')
    end select
    p%BC_H_west = bc_H_code(C%BC_H_west); p%BC_H_east = bc_H_code(C%BC_H_east)
    p%BC_H_south = bc_H_code(C%BC_H_south); p%BC_H_north = bc_H_code(C%BC_H_north)
    p%dHi_semiimplicit_fs = C%dHi_semiimplicit_fs
    p%dHi_PETSc_rtol = C%dHi_PETSc_rtol; p%dHi_PETSc_abstol = C%dHi_PETSc_abstol
    p%dt_ice_max = C%dt_ice_max; p%dt_ice_min = C%dt_ice_min; p%Hi_min = C%Hi_min
    noice = merge(1_c_int32_t, 0_c_int32_t, mask_noice)
    f%Hi = c_loc(Hi); f%Hb = c_loc(Hb); f%SL = c_loc(SL); f%u_vav_b = c_loc(u_vav_b); f%v_vav_b = c_loc(v_vav_b)
    f%SMB = c_loc(SMB); f%BMB = c_loc(BMB); f%LMB = c_loc(LMB); f%fraction_margin = c_loc(fraction_margin)
    f%mask_noice = c_loc(noice); f%dHi_dt_target = c_loc(dHi_dt_target)
    f%BC_prescr_mask = c_null_ptr; f%BC_prescr_Hi = c_null_ptr
    if (present(BC_prescr_mask) .or. present(BC_prescr_Hi)) then
      if (.not. (present(BC_prescr_mask) .and. present(BC_prescr_Hi))) call crash('need to provide prescribed both Hi and mask!')
      prescr = int(BC_prescr_mask, c_int32_t)
      f%BC_prescr_mask = c_loc(prescr); f%BC_prescr_Hi = c_loc(BC_prescr_Hi)
    end if
    f%dHi_dt = c_loc(dHi_dt); f%Hi_tplusdt = c_loc(Hi_tplusdt); f%divQ = c_loc(divQ); f%AMB = c_loc(AMB)
    call check(ufe_calc_dHi_dt(ctx, p, f, dt, st), 'calc_dHi_dt')
    if (st%found_negative /= 0) call warning('encountered negative values for Hi_tplusdt - time step too large?')
  end subroutine

  integer(c_int32_t) function bc_H_code(s)
    character(len=*), intent(in) :: s
    select case (trim(s))
    case ('zero');     bc_H_code = UFE_BC_H_ZERO
    case ('infinite'); bc_H_code = UFE_BC_H_INFINITE
    case default
      call crash('unknown BC_H "' // trim(s) // '"')
      bc_H_code = -1
    end select
  end function

end module ufe_gpu_mod
