"""calc_ice_rheology_Glen (constitutive_equation.f90:84-163) inside the solve, and the sliding laws
added beside it: the oracle against a numpy restatement of the formulas (CPU), the GPU against the
oracle (gpu).  Tolerances: 1e-12 relative L2 where only the host libm's exp differs, 1e-8 for
GPU-vs-oracle solves with Krylov run to 1e-12."""
import numpy as np
import pytest

from helpers import rel_l2


def _copy(pkg, p, **kw):
    q = pkg.abi.default_params(**{k: getattr(p, k) for k, _ in p._fields_ if k != "reserved"})
    for k, v in kw.items():
        setattr(q, k, pkg.abi.RHEOLOGY[v] if k == "choice_ice_rheology_Glen" else
                pkg.abi.ENHANCEMENT[v] if k == "choice_enhancement_factor_transition" else
                pkg.abi.SLIDING[v] if k == "choice_sliding_law" else v)
    return q


def _thermal_dome(pkg, seed=1):
    """The small dome with a temperature field (colder at the surface and inland) and a band of
    'floating' vertices for the enhancement factors; the flow factor is left to the solve."""
    mesh, ice, params = pkg.geometry.small_dome(seed=seed)
    r = np.hypot(mesh.V[:, 0], mesh.V[:, 1]) / 500e3
    zeta = mesh.zeta
    Ti = np.asfortranarray(235.0 + 30.0 * np.clip(r, 0, 1)[:, None] + 8.0 * zeta[None, :])
    fl = ((r > 0.8) & (r < 0.9)).astype(np.int32)
    ice = dict(ice)
    ice.pop("A_flow")
    ice.update(Ti=Ti, mask_floating_ice=np.ascontiguousarray(fl),
               fraction_gr=np.ascontiguousarray(np.clip(1.5 - r, 0.0, 1.0)),
               Hib=np.ascontiguousarray(np.where(r > 0.7, -50.0, 10.0)), SL=np.zeros(mesh.nV))
    params.stress_balance_PETSc_rtol = 1e-12
    params.stress_balance_PETSc_abstol = 0.0
    params.visc_it_nit = 30
    return mesh, ice, params


def _huybrechts(Ti):
    return np.where(Ti < 263.15, 1.14e-5 * np.exp(-6.0e4 / (8.314 * Ti)), 5.47e10 * np.exp(-13.9e4 / (8.314 * Ti)))


def _enhanced(ice, A, m_sheet, m_shelf, interp):
    A = A.copy()
    for vi in range(A.shape[0]):
        if interp and ice["Hi"][vi] > 0 and ice["Hib"][vi] < ice["SL"][vi]:
            f = ice["fraction_gr"][vi] * m_sheet + (1.0 - ice["fraction_gr"][vi]) * m_shelf
        elif ice["mask_grounded_ice"][vi]:
            f = m_sheet
        elif ice["mask_floating_ice"][vi]:
            f = m_shelf
        else:
            continue
        A[vi, :] = A[vi, :] * f
    return np.asfortranarray(A)


@pytest.mark.parametrize("rheo,enh", [("uniform", "separate"), ("Huybrechts1992", "separate"),
                                      ("Huybrechts1992", "interp")])
def test_oracle_rheology_equals_given_flow_factor(pkg, oracle_mod, rheo, enh):
    mesh, ice, params = _thermal_dome(pkg)
    ice["mask_grounded_ice"] = np.ascontiguousarray(ice["mask_grounded_ice"] * (1 - ice["mask_floating_ice"]))
    kw = dict(choice_ice_rheology_Glen=rheo, choice_enhancement_factor_transition=enh, m_enh_sheet=2.0,
              m_enh_shelf=0.5, uniform_Glens_flow_factor=3e-17, visc_it_nit=8)
    p = _copy(pkg, params, **kw)
    A = np.full(ice["Ti"].shape, 3e-17) if rheo == "uniform" else _huybrechts(ice["Ti"])
    given = dict(ice, A_flow=_enhanced(ice, A, 2.0, 0.5, enh == "interp"))
    orc = oracle_mod.Oracle(mesh)
    a, b = pkg.new_ssa_state(mesh.nTri), pkg.new_ssa_state(mesh.nTri)
    nva, _, sa = orc.solve_SSA(ice, a, p)
    nvb, _, sb = orc.solve_SSA(given, b, _copy(pkg, p, choice_ice_rheology_Glen="input"))
    assert nva == nvb and sa["status"] == sb["status"]
    assert rel_l2(np.r_[a["u_b"], a["v_b"]], np.r_[b["u_b"], b["v_b"]]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("rheo,enh,diva", [("Huybrechts1992", "separate", False), ("Huybrechts1992", "interp", False),
                                           ("uniform", "separate", True), ("Huybrechts1992", "interp", True)])
def test_gpu_rheology_matches_oracle(pkg, oracle_mod, gpu_lib, rheo, enh, diva):
    if diva:
        mesh, ice, params = pkg.geometry.small_channel(sliding="Schoof2005")
        params.stress_balance_PETSc_rtol = 1e-12
        params.stress_balance_PETSc_abstol = 0.0
        params.visc_it_nit = 12
        x = mesh.V[:, 0] / 640e3
        ice = dict(ice)
        ice.pop("A_flow")
        ice.update(Ti=np.asfortranarray(250.0 + 15.0 * x[:, None] + 5.0 * mesh.zeta[None, :]),
                   mask_floating_ice=np.ascontiguousarray((1 - ice["mask_grounded_ice"]).astype(np.int32)),
                   fraction_gr=np.ascontiguousarray(np.clip(1.2 - x, 0, 1)), Hib=np.ascontiguousarray(ice["Hb"]),
                   SL=np.ascontiguousarray(ice["SL"]))
    else:
        mesh, ice, params = _thermal_dome(pkg)
    p = _copy(pkg, params, choice_ice_rheology_Glen=rheo, choice_enhancement_factor_transition=enh,
              m_enh_sheet=1.5, m_enh_shelf=0.8, uniform_Glens_flow_factor=2e-17)
    orc = oracle_mod.Oracle(mesh)
    with pkg.VelocitySolver(mesh, operators=orc.operators()) as g:
        if diva:
            a, b = pkg.new_diva_state(mesh.nTri, mesh.nz), pkg.new_diva_state(mesh.nTri, mesh.nz)
            nvg, _, sg = g.solve_DIVA(ice, a, p)
            nvo, _, so = orc.solve_DIVA(ice, b, p)
            keys = ("u_vav_b", "v_vav_b", "eta_3D_b", "u_3D_b")
        else:
            a, b = pkg.new_ssa_state(mesh.nTri), pkg.new_ssa_state(mesh.nTri)
            nvg, _, sg = g.solve_SSA(ice, a, p)
            nvo, _, so = orc.solve_SSA(ice, b, p)
            keys = ("u_b", "v_b")
    assert nvg == nvo and sg["status"] == so["status"]
    for k in keys:
        assert rel_l2(a[k], b[k]) < 1e-8, k


@pytest.mark.gpu
def test_gpu_zoet_iverson_matches_oracle(pkg, oracle_mod, gpu_lib):
    mesh, ice, params = pkg.geometry.small_dome(seed=2)
    ice = dict(ice, till_yield_stress=np.ascontiguousarray(5e4 + 2e4 * np.cos(mesh.V[:, 0] / 1e5)))
    p = _copy(pkg, params, choice_sliding_law="Zoet-Iverson", stress_balance_PETSc_rtol=1e-12,
              stress_balance_PETSc_abstol=0.0, visc_it_nit=20)
    orc = oracle_mod.Oracle(mesh)
    a, b = pkg.new_ssa_state(mesh.nTri), pkg.new_ssa_state(mesh.nTri)
    with pkg.VelocitySolver(mesh, operators=orc.operators()) as g:
        nvg, _, sg = g.solve_SSA(ice, a, p)
    nvo, _, so = orc.solve_SSA(ice, b, p)
    assert nvg == nvo and sg["status"] == so["status"]
    assert rel_l2(np.r_[a["u_b"], a["v_b"]], np.r_[b["u_b"], b["v_b"]]) < 1e-8


@pytest.mark.gpu
def test_gpu_missing_rheology_inputs_rejected(pkg, gpu_lib):
    mesh, ice, params = pkg.geometry.small_dome(seed=1)
    no_A = {k: v for k, v in ice.items() if k != "A_flow"}
    with pkg.VelocitySolver(mesh) as g:
        for p in (params, _copy(pkg, params, choice_ice_rheology_Glen="Huybrechts1992")):
            with pytest.raises(pkg.UfeError) as e:
                g.solve_SSA(no_A, pkg.new_ssa_state(mesh.nTri), p)
            assert e.value.code == pkg.abi.UFE_ERR_INVALID
