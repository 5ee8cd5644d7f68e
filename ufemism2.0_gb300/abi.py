"""ctypes mirror of include/ufe_gpu.h and the loader of the in-tree GB300 library.

The library is loaded from ``_build/libufe_gpu.so`` next to this package.  There is no fallback:
if the shared object is missing, :func:`load_library` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libufe_gpu.so")

# status codes
UFE_OK = 0
UFE_WARN_PICARD_MAXIT = 1
UFE_WARN_KRYLOV_MAXIT = 2
UFE_ERR_INVALID = -1
UFE_ERR_NAN = -2
UFE_ERR_DIVERGED = -3
UFE_ERR_THERMO_UNSTABLE = -4
UFE_ERR_DEVICE = -5
UFE_ERR_CAPACITY = -6

# operators (enum ufe_operator)
OPERATORS = ["MAP_A_B", "DDX_A_B", "DDY_A_B", "MAP_B_A", "DDX_B_A", "DDY_B_A", "DDX_A_A", "DDY_A_A",
             "M2_DDX_B_B", "M2_DDY_B_B", "M2_D2DX2_B_B", "M2_D2DXDY_B_B", "M2_D2DY2_B_B"]
OP = {name: i for i, name in enumerate(OPERATORS)}

SLIDING = {"no_sliding": 0, "Weertman": 1, "Coulomb": 2, "Budd": 3, "Tsai2015": 4, "Schoof2005": 5,
           "Zoet-Iverson": 6, "idealised_SSA_icestream": 7}
BC = {"infinite": 0, "zero": 1, "infinite_SSA_icestream": 2}
PREC_FP64, PREC_FP32_REFINE, PREC_FP32_PAIR = 0, 1, 2
X0_ZERO, X0_CURRENT = 0, 1
RHEOLOGY = {"input": 0, "uniform": 1, "Huybrechts1992": 2}
ENHANCEMENT = {"separate": 0, "interp": 1}

dptr = C.POINTER(C.c_double)
iptr = C.POINTER(C.c_int32)
fptr = C.POINTER(C.c_float)


class MeshDesc(C.Structure):
    _fields_ = [("nV", C.c_int32), ("nTri", C.c_int32), ("nC_mem", C.c_int32), ("nz", C.c_int32),
                ("V", dptr), ("nC", iptr), ("C", iptr), ("niTri", iptr), ("iTri", iptr), ("VBI", iptr),
                ("Tri", iptr), ("TriC", iptr), ("TriBI", iptr), ("TriGC", dptr), ("zeta", dptr)]


class SolverParams(C.Structure):
    _fields_ = [("choice_sliding_law", C.c_int32), ("do_include_SSADIVA_crossterms", C.c_int32),
                ("do_GL_subgrid_friction", C.c_int32),
                ("BC_u_west", C.c_int32), ("BC_u_east", C.c_int32), ("BC_u_south", C.c_int32), ("BC_u_north", C.c_int32),
                ("BC_v_west", C.c_int32), ("BC_v_east", C.c_int32), ("BC_v_south", C.c_int32), ("BC_v_north", C.c_int32),
                ("visc_it_nit", C.c_int32),
                ("visc_it_norm_dUV_tol", C.c_double), ("visc_it_relax", C.c_double), ("visc_eff_min", C.c_double),
                ("vel_max", C.c_double), ("stress_balance_PETSc_rtol", C.c_double),
                ("stress_balance_PETSc_abstol", C.c_double), ("Glens_flow_law_exponent", C.c_double),
                ("Glens_flow_law_epsilon_sq_0", C.c_double), ("slid_Weertman_m", C.c_double),
                ("slid_Budd_q_plastic", C.c_double), ("slid_Budd_u_threshold", C.c_double),
                ("subgrid_friction_exponent_on_B_grid", C.c_double), ("slid_beta_max", C.c_double),
                ("slid_delta_v", C.c_double),
                ("krylov_max_it", C.c_int32), ("krylov_initial_guess", C.c_int32), ("precision", C.c_int32),
                ("krylov_inner_rtol", C.c_double), ("krylov_forcing", C.c_double),
                ("choice_ice_rheology_Glen", C.c_int32), ("choice_enhancement_factor_transition", C.c_int32),
                ("uniform_Glens_flow_factor", C.c_double), ("m_enh_sheet", C.c_double), ("m_enh_shelf", C.c_double),
                ("slid_ZI_p", C.c_double), ("slid_ZI_ut", C.c_double),
                ("SSA_icestream_Hi", C.c_double), ("SSA_icestream_dhdx", C.c_double),
                ("SSA_icestream_L", C.c_double), ("SSA_icestream_m", C.c_double),
                ("reserved", C.c_int32 * 8)]


class IceState(C.Structure):
    _fields_ = [("Hi", dptr), ("Hs", dptr), ("A_flow", dptr), ("fraction_gr_b", dptr),
                ("mask_grounded_ice", iptr), ("beta_sq", dptr), ("alpha_sq", dptr),
                ("effective_pressure", dptr), ("till_yield_stress", dptr),
                ("Ti", dptr), ("mask_floating_ice", iptr), ("fraction_gr", dptr), ("Hib", dptr), ("SL", dptr)]


class BCPrescribed(C.Structure):
    _fields_ = [("mask_b", iptr), ("u_b", dptr), ("v_b", dptr)]


class DivaState(C.Structure):
    _fields_ = [("u_vav_b", dptr), ("v_vav_b", dptr), ("u_base_b", dptr), ("v_base_b", dptr),
                ("tau_bx_b", dptr), ("tau_by_b", dptr), ("eta_3D_b", dptr), ("u_3D_b", dptr), ("v_3D_b", dptr)]


class SolveStats(C.Structure):
    _fields_ = [("n_visc_its", C.c_int32), ("n_Axb_its", C.c_int32), ("n_refinements", C.c_int32),
                ("status", C.c_int32), ("L2_uv", C.c_double), ("visc_it_relax_applied", C.c_double),
                ("device_ms", C.c_double), ("n_fp64_its", C.c_int32), ("n_kernels", C.c_int32),
                ("n_pair_its", C.c_int32), ("reserved", C.c_int32 * 3)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


def default_params(**overrides) -> SolverParams:
    """The defaults of UFEMISM's model_configuration.f90 (same values as ufe_default_params)."""
    p = SolverParams()
    p.choice_sliding_law = SLIDING["Weertman"]
    p.do_include_SSADIVA_crossterms = 1
    p.do_GL_subgrid_friction = 1
    for side in ("west", "east", "south", "north"):
        setattr(p, f"BC_u_{side}", BC["infinite"])
        setattr(p, f"BC_v_{side}", BC["infinite"])
    p.visc_it_nit = 50
    p.visc_it_norm_dUV_tol = 5e-5
    p.visc_it_relax = 0.2
    p.visc_eff_min = 1e4
    p.vel_max = 5000.0
    p.stress_balance_PETSc_rtol = 1e-7
    p.stress_balance_PETSc_abstol = 1e-5
    p.Glens_flow_law_exponent = 3.0
    p.Glens_flow_law_epsilon_sq_0 = 1e-8
    p.slid_Weertman_m = 3.0
    p.slid_Budd_q_plastic = 0.3
    p.slid_Budd_u_threshold = 100.0
    p.subgrid_friction_exponent_on_B_grid = 2.0
    p.slid_beta_max = 1e20
    p.slid_delta_v = 1e-3
    p.krylov_max_it = 10000
    p.krylov_initial_guess = X0_CURRENT
    p.precision = PREC_FP64
    p.krylov_inner_rtol = 1e-2
    p.krylov_forcing = 0.0
    p.choice_ice_rheology_Glen = RHEOLOGY["input"]
    p.choice_enhancement_factor_transition = ENHANCEMENT["separate"]
    p.uniform_Glens_flow_factor = 1e-16
    p.m_enh_sheet = 1.0
    p.m_enh_shelf = 1.0
    p.slid_ZI_p = 5.0
    p.slid_ZI_ut = 200.0
    p.SSA_icestream_Hi = 2000.0
    p.SSA_icestream_dhdx = -0.0003
    p.SSA_icestream_L = 150e3
    p.SSA_icestream_m = 1.0
    names = {"choice_sliding_law": SLIDING, "choice_ice_rheology_Glen": RHEOLOGY,
             "choice_enhancement_factor_transition": ENHANCEMENT}
    names.update({f"BC_{c}_{side}": BC for c in "uv" for side in ("west", "east", "south", "north")})
    for k, v in overrides.items():
        if k in names and isinstance(v, str):
            v = names[k][v]
        setattr(p, k, v)
    return p


# -- thermodynamics ------------------------------------------------------------------------------
CP = {"uniform": 0, "Pounder1965": 1}
KI = {"uniform": 0, "Ritz1987": 1}
GLBC = {"grounded": 0, "subgrid": 1, "pmp": 2}
COL_NONE, COL_GROUNDED, COL_FLOATING, COL_GL_GR = 0, 1, 2, 3


class ThermoParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("Hi_min_thermo", C.c_double),
                ("choice_ice_heat_capacity", C.c_int32), ("choice_ice_thermal_conductivity", C.c_int32),
                ("uniform_ice_heat_capacity", C.c_double), ("uniform_ice_thermal_conductivity", C.c_double),
                ("choice_GL_temperature_BC", C.c_int32), ("reserved", C.c_int32 * 7)]


class ThermoColumns(C.Structure):
    _fields_ = [(n, dptr) for n in ("Ti", "u_3D", "v_3D", "w_3D", "u_times_dTdxp_upwind", "v_times_dTdyp_upwind",
                                    "dzeta_dx", "dzeta_dy", "dzeta_dz", "dzeta_dt", "internal_heating", "Hi_eff",
                                    "T_surf_annual", "Q_base_grnd")] + \
              [("mask", iptr), ("fraction_gr", dptr), ("geothermal_heat_flux", dptr), ("SMB", dptr)]


class HeatFields(C.Structure):
    _fields_ = [(n, dptr) for n in ("Ti", "Hi", "Hi_eff", "Hs", "dHi_dt", "dHs_dt", "u_vav", "v_vav", "u_3D",
                                    "v_3D", "w_3D", "u_3D_b", "v_3D_b", "internal_heating", "frictional_heating",
                                    "geothermal_heat_flux", "T2m")] + \
              [("n_months", C.c_int32), ("pad", C.c_int32), ("SMB", dptr), ("mask", iptr), ("fraction_gr", dptr)] + \
              [(n, dptr) for n in ("A_flow", "du_dx_3D", "du_dy_3D", "du_dz_3D", "dv_dx_3D", "dv_dy_3D", "dv_dz_3D",
                                    "dw_dx_3D", "dw_dy_3D", "dw_dz_3D", "basal_friction_coefficient", "uabs_base")] + \
              [("no_sliding", C.c_int32), ("pad2", C.c_int32), ("Glens_flow_law_exponent", C.c_double)]


def default_thermo_params(**overrides) -> ThermoParams:
    """The defaults of UFEMISM's model_configuration.f90 (same values as ufe_default_thermo_params)."""
    p = ThermoParams()
    p.dt = 1.0
    p.Hi_min_thermo = 10.0
    p.choice_ice_heat_capacity = CP["Pounder1965"]
    p.choice_ice_thermal_conductivity = KI["Ritz1987"]
    p.uniform_ice_heat_capacity = 2009.0
    p.uniform_ice_thermal_conductivity = 6.626958e7
    p.choice_GL_temperature_BC = GLBC["grounded"]
    names = {"choice_ice_heat_capacity": CP, "choice_ice_thermal_conductivity": KI, "choice_GL_temperature_BC": GLBC}
    for k, v in overrides.items():
        if k in names and isinstance(v, str):
            v = names[k][v]
        setattr(p, k, v)
    return p


def _fcol(a):
    """Column-major float64 copy of an (n, nz) or (n,) array; None stays None."""
    if a is None:
        return None
    return np.asfortranarray(a, dtype=np.float64)


def thermo_columns(cols: dict) -> tuple[ThermoColumns, list]:
    """ThermoColumns over a dict of the ufe_thermo_columns fields (numpy arrays, (nV, nz) or (nV,))."""
    keep, vals = [], {}
    for name, typ in ThermoColumns._fields_:
        a = cols.get(name)
        if a is None:
            vals[name] = None
            continue
        a = np.asfortranarray(a, dtype=np.int32) if typ is iptr else _fcol(a)
        keep.append(a)
        vals[name] = a.ctypes.data_as(typ)
    return ThermoColumns(**vals), keep


def heat_fields(f: dict) -> tuple[HeatFields, list]:
    """HeatFields over a dict of the ufe_heat_fields fields (T2m as (nV, n_months))."""
    keep, vals = [], {}
    for name, typ in HeatFields._fields_:
        if name in ("n_months", "pad", "pad2"):
            continue
        if name in ("no_sliding", "Glens_flow_law_exponent"):
            vals[name] = f.get(name, 0)
            continue
        a = f.get(name)
        if a is None:
            vals[name] = None
            continue
        a = np.asfortranarray(a, dtype=np.int32) if typ is iptr else _fcol(a)
        keep.append(a)
        vals[name] = a.ctypes.data_as(typ)
    T2m = np.asarray(f["T2m"])
    vals["n_months"] = T2m.shape[1] if T2m.ndim == 2 else 1
    vals["pad"] = 0
    vals["pad2"] = 0
    return HeatFields(**vals), keep


# -- ice thickness (conservation of mass) -------------------------------------------------------
DHI = {"none": 0, "explicit": 1, "semi-implicit": 2}
BC_H = {"zero": 0, "infinite": 1}


class ThicknessParams(C.Structure):
    _fields_ = [("choice_ice_integration_method", C.c_int32), ("BC_H_west", C.c_int32), ("BC_H_east", C.c_int32),
                ("BC_H_south", C.c_int32), ("BC_H_north", C.c_int32), ("dHi_PETSc_max_it", C.c_int32),
                ("dHi_semiimplicit_fs", C.c_double), ("dHi_PETSc_rtol", C.c_double), ("dHi_PETSc_abstol", C.c_double),
                ("dt_ice_max", C.c_double), ("dt_ice_min", C.c_double), ("Hi_min", C.c_double),
                ("reserved", C.c_int32 * 4)]


class ThicknessFields(C.Structure):
    _fields_ = [("Hi", dptr), ("Hb", dptr), ("SL", dptr), ("u_vav_b", dptr), ("v_vav_b", dptr),
                ("SMB", dptr), ("BMB", dptr), ("LMB", dptr), ("fraction_margin", dptr), ("mask_noice", iptr),
                ("dHi_dt_target", dptr), ("BC_prescr_mask", iptr), ("BC_prescr_Hi", dptr),
                ("dHi_dt", dptr), ("Hi_tplusdt", dptr), ("divQ", dptr), ("AMB", dptr)]


class ThicknessStats(C.Structure):
    _fields_ = [("n_Axb_its", C.c_int32), ("krylov_status", C.c_int32), ("found_negative", C.c_int32),
                ("pad", C.c_int32), ("device_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


def default_thickness_params(**overrides) -> ThicknessParams:
    """The defaults of model_configuration.f90 (same values as ufe_default_thickness_params);
    string choices ('semi-implicit', 'infinite', ...) are accepted for the enum fields."""
    p = ThicknessParams()
    p.choice_ice_integration_method = DHI["semi-implicit"]
    for side in ("west", "east", "south", "north"):
        setattr(p, f"BC_H_{side}", BC_H["zero"])
    p.dHi_PETSc_max_it = 10000
    p.dHi_semiimplicit_fs = 1.5
    p.dHi_PETSc_rtol = 1e-8
    p.dHi_PETSc_abstol = 1e-6
    p.dt_ice_max = 10.0
    p.dt_ice_min = 0.1
    p.Hi_min = 0.0
    for k, v in overrides.items():
        if k == "choice_ice_integration_method" and isinstance(v, str):
            v = DHI[v]
        elif k.startswith("BC_H_") and isinstance(v, str):
            v = BC_H[v]
        setattr(p, k, v)
    return p


THICKNESS_INPUTS = ("Hi", "Hb", "SL", "u_vav_b", "v_vav_b", "SMB", "BMB", "LMB", "fraction_margin", "mask_noice",
                    "dHi_dt_target", "BC_prescr_mask", "BC_prescr_Hi")
THICKNESS_OUTPUTS = ("dHi_dt", "Hi_tplusdt", "divQ", "AMB")


def thickness_fields(f: dict) -> tuple[ThicknessFields, list]:
    """ThicknessFields over a dict of arrays (inputs as named in THICKNESS_INPUTS; the outputs in
    THICKNESS_OUTPUTS must be present, dHi_dt holding the previous rate)."""
    keep = [v for v in f.values() if isinstance(v, np.ndarray)]
    vals = {}
    for k, _ in ThicknessFields._fields_:
        a = f.get(k)
        vals[k] = (as_i(a) if k in ("mask_noice", "BC_prescr_mask") else as_d(a)) if a is not None else None
    return ThicknessFields(**vals), keep


# -- numpy <-> ctypes helpers -------------------------------------------------------------------
def as_d(a):
    """Pointer to a contiguous float64 buffer (Fortran-ordered arrays are flattened column-major)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous), "float64 contiguous array needed"
    return a.ctypes.data_as(dptr)


def as_i(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and (a.flags.f_contiguous or a.flags.c_contiguous), "int32 contiguous array needed"
    return a.ctypes.data_as(iptr)


def mesh_desc(mesh) -> tuple[MeshDesc, list]:
    """A MeshDesc over a :class:`mesh.Mesh`; the returned list keeps the arrays alive."""
    keep = [mesh.V, mesh.nC, mesh.C, mesh.niTri, mesh.iTri, mesh.VBI, mesh.Tri, mesh.TriC, mesh.TriBI,
            mesh.TriGC, mesh.zeta]
    d = MeshDesc(mesh.nV, mesh.nTri, mesh.nC_mem, mesh.nz, as_d(mesh.V), as_i(mesh.nC), as_i(mesh.C),
                 as_i(mesh.niTri), as_i(mesh.iTri), as_i(mesh.VBI), as_i(mesh.Tri), as_i(mesh.TriC),
                 as_i(mesh.TriBI), as_d(mesh.TriGC), as_d(mesh.zeta))
    return d, keep


def ice_state(ice: dict) -> tuple[IceState, list]:
    """An IceState over a dict of arrays.  A_flow may be absent when the solve computes the flow
    factor (choice_ice_rheology_Glen 'uniform' or 'Huybrechts1992'); Ti, mask_floating_ice,
    fraction_gr, Hib and SL are passed when present."""
    keep = [v for v in ice.values() if isinstance(v, np.ndarray)]
    s = IceState(as_d(ice["Hi"]), as_d(ice["Hs"]), as_d(ice.get("A_flow")), as_d(ice["fraction_gr_b"]),
                 as_i(ice["mask_grounded_ice"]), as_d(ice.get("beta_sq")), as_d(ice.get("alpha_sq")),
                 as_d(ice.get("effective_pressure")), as_d(ice.get("till_yield_stress")),
                 as_d(ice.get("Ti")), as_i(ice.get("mask_floating_ice")), as_d(ice.get("fraction_gr")),
                 as_d(ice.get("Hib")), as_d(ice.get("SL")))
    return s, keep


def bc_prescribed(bc: dict | None):
    if not bc:
        return None, []
    b = BCPrescribed(as_i(bc["mask_b"]), as_d(bc["u_b"]), as_d(bc["v_b"]))
    return b, [bc["mask_b"], bc["u_b"], bc["v_b"]]


# -- the library ---------------------------------------------------------------------------------
EXPORTS = {
    "ufe_default_params": (None, [C.POINTER(SolverParams)]),
    "ufe_default_thickness_params": (None, [C.POINTER(ThicknessParams)]),
    "ufe_mesh_voronoi_upload": (C.c_int32, [C.c_void_p, dptr, dptr]),
    "ufe_calc_dHi_dt": (C.c_int32, [C.c_void_p, C.POINTER(ThicknessParams), C.POINTER(ThicknessFields), dptr,
                                    C.POINTER(ThicknessStats)]),
    "ufe_thickness_assemble": (C.c_int32, [C.c_void_p, C.POINTER(ThicknessParams), C.POINTER(ThicknessFields),
                                           C.c_double, iptr, iptr, dptr, dptr, dptr, C.c_int64,
                                           C.POINTER(C.c_int64)]),
    "ufe_ctx_create": (C.c_int32, [C.c_int32, C.POINTER(C.c_void_p)]),
    "ufe_ctx_destroy": (None, [C.c_void_p]),
    "ufe_ctx_last_error": (C.c_char_p, [C.c_void_p]),
    "ufe_ctx_get_stream": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "ufe_ctx_synchronize": (C.c_int32, [C.c_void_p]),
    "ufe_mesh_upload": (C.c_int32, [C.c_void_p, C.POINTER(MeshDesc)]),
    "ufe_mesh_build_operators": (C.c_int32, [C.c_void_p]),
    "ufe_mesh_set_operator": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int64, iptr, iptr, dptr,
                                          C.c_int32]),
    "ufe_operator_info": (C.c_int32, [C.c_void_p, C.c_int32, iptr, iptr, C.POINTER(C.c_int64)]),
    "ufe_operator_export": (C.c_int32, [C.c_void_p, C.c_int32, iptr, iptr, dptr, C.c_int32]),
    "ufe_apply_operator": (C.c_int32, [C.c_void_p, C.c_int32, dptr, dptr, C.c_int32]),
    "ufe_csr_spmv": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, iptr, iptr, dptr, C.c_int32, dptr,
                                 dptr, C.c_int32]),
    "ufe_solve_csr": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64, iptr, iptr, dptr, C.c_int32, dptr, dptr,
                                  C.c_double, C.c_double, C.c_int32, iptr]),
    "ufe_assemble_linearised": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), dptr, dptr, dptr, dptr, dptr, dptr,
                                            dptr, dptr, C.POINTER(BCPrescribed), iptr, iptr, dptr, dptr, C.c_int64,
                                            C.POINTER(C.c_int64)]),
    "ufe_solve_linearised": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), dptr, dptr, dptr, dptr, dptr, dptr,
                                         dptr, dptr, dptr, dptr, C.POINTER(BCPrescribed), iptr]),
    "ufe_solve_ssa": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), C.POINTER(IceState), C.POINTER(BCPrescribed),
                                  dptr, dptr, iptr, iptr, C.POINTER(SolveStats)]),
    "ufe_solve_diva": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), C.POINTER(IceState), C.POINTER(BCPrescribed),
                                   C.POINTER(DivaState), iptr, iptr, C.POINTER(SolveStats)]),
    "ufe_ice_upload": (C.c_int32, [C.c_void_p, C.POINTER(IceState), C.POINTER(BCPrescribed)]),
    "ufe_solve_ssa_resident": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), C.c_int32, C.POINTER(SolveStats)]),
    "ufe_solve_diva_resident": (C.c_int32, [C.c_void_p, C.POINTER(SolverParams), C.c_int32, C.POINTER(SolveStats)]),
    "ufe_velocity_download": (C.c_int32, [C.c_void_p, dptr, dptr]),
    "ufe_solve_csr_noalloc": (C.c_int32, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                          C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32, iptr,
                                          C.c_void_p]),
    "ufe_solve_history": (C.c_int32, [C.c_void_p, dptr, C.c_int32, iptr]),
    "ufe_profile_krylov_kernels": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, dptr, C.POINTER(C.c_int64)]),
    "ufe_gnn_predict_kernels": (C.c_int32, [C.c_int32]),
    "ufe_profile_krylov_persistent": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, dptr]),
    "ufe_default_thermo_params": (None, [C.POINTER(ThermoParams)]),
    "ufe_thermo_step": (C.c_int32, [C.c_void_p, C.POINTER(ThermoParams), C.c_int32, C.c_int32, dptr,
                                    C.POINTER(ThermoColumns), dptr, iptr]),
    "ufe_solve_3D_heat_equation": (C.c_int32, [C.c_void_p, C.POINTER(ThermoParams), C.POINTER(HeatFields), dptr, iptr]),
    "ufe_heat_upload": (C.c_int32, [C.c_void_p, C.POINTER(HeatFields)]),
    "ufe_heat_step_resident": (C.c_int32, [C.c_void_p, C.POINTER(ThermoParams), C.c_int32, iptr, dptr]),
    "ufe_heat_download": (C.c_int32, [C.c_void_p, dptr]),
    "ufe_zeta_operators": (C.c_int32, [C.c_int32, dptr, dptr, dptr, dptr, dptr, dptr, dptr]),
    "ufe_profile_heat_kernels": (C.c_int32, [C.c_void_p, C.POINTER(ThermoParams), C.c_int32, dptr,
                                             C.POINTER(C.c_int64)]),
    "ufe_tridiagonal_solve": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, dptr, dptr, dptr, dptr, dptr]),
    "ufe_umma_gemm_bf16": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "ufe_ensemble_solve": (C.c_int32, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(SolverParams), C.c_int32,
                                       C.c_int32, C.POINTER(SolveStats), dptr]),
    "ufe_autotune": (C.c_int32, [C.c_void_p, C.c_int32, iptr, dptr]),
    "ufe_gnn_param_count": (C.c_int32, []),
    "ufe_gnn_create": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "ufe_gnn_destroy": (None, [C.c_void_p]),
    "ufe_gnn_get_params": (C.c_int32, [C.c_void_p, fptr]),
    "ufe_gnn_set_params": (C.c_int32, [C.c_void_p, fptr]),
    "ufe_gnn_forward": (C.c_int32, [C.c_void_p, C.c_int64, iptr, fptr, fptr]),
    "ufe_gnn_loss_grad": (C.c_int32, [C.c_void_p, C.c_int64, iptr, fptr, fptr, fptr, dptr, fptr]),
    "ufe_gnn_features": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, fptr]),
    "ufe_gnn_dataset_add": (C.c_int32, [C.c_void_p, C.c_void_p, fptr]),
    "ufe_gnn_dataset_clear": (C.c_int32, [C.c_void_p]),
    "ufe_gnn_train": (C.c_int32, [C.c_void_p, C.c_int32, C.c_float, C.c_uint64, fptr, dptr]),
    "ufe_gnn_evaluate": (C.c_int32, [C.c_void_p, dptr]),
    "ufe_gnn_predict_velocity": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, dptr]),
    "ufe_gnn_predict_start": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, dptr]),
}

_LIB = None


def load_library(path: str = LIB_PATH):
    """Load libufe_gpu.so and declare every entry point of include/ufe_gpu.h."""
    global _LIB
    if _LIB is not None and path == LIB_PATH:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"GB300 library not built: {path} is missing (run build())")
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _LIB = lib
    return lib
