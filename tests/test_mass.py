"""Ice thickness (conservation of mass): calc_dHi_dt on the GPU against the oracle's restatement of
conservation_of_mass_{main,explicit,semiimplicit,utilities}.f90.

Tolerances: the Voronoi geometry tiles the domain to round-off; the explicit step, the flux
divergence and the assembled semi-implicit system (matrix, load vector, initial guess) are
bit-identical to the oracle's; the semi-implicit solution agrees to 1e-10 relative when both
BiCGStab runs go to rtol 1e-13 from the same start (their reductions sum in different orders)."""
import numpy as np
import pytest


def _fields(f, mesh, **over):
    g = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in f.items()}
    g.update(over)
    for k in ("Hi_tplusdt", "divQ", "AMB"):
        g[k] = np.zeros(mesh.nV)
    if g.get("dHi_dt") is None:
        g["dHi_dt"] = np.zeros(mesh.nV)
    return g


@pytest.fixture(scope="module")
def case(pkg):
    mesh, f, p = pkg.geometry.thickness_case()
    A, Cw = pkg.mesh.voronoi_geometry(mesh)
    return mesh, f, p, A, Cw


def test_voronoi_cells_tile_the_domain(pkg, case):
    mesh, _, _, A, Cw = case
    assert abs(A.sum() - (mesh.xmax - mesh.xmin) * (mesh.ymax - mesh.ymin)) < 1e-9 * A.sum()
    assert (A > 0).all()
    C = np.asarray(mesh.C) - 1
    for vi in range(0, mesh.nV, 7):                      # the shared boundary is the same seen from both cells
        for ci in range(mesh.nC[vi]):
            vj = C[vi, ci]
            cj = list(C[vj, :mesh.nC[vj]]).index(vi)
            assert abs(Cw[vi, ci] - Cw[vj, cj]) <= 1e-9 * Cw[vi, ci]


def test_oracle_flux_divergence_conserves_mass(pkg, oracle_mod, case):
    """Upwind fluxes leave one cell and enter its neighbour (conservation_of_mass_utilities.f90:63-77):
    with every margin cell full, the area-weighted divergence sums to zero up to the flux through
    the domain border, which this velocity field (decaying away from the dome) makes negligible."""
    mesh, f, p, A, Cw = case
    q = _fields(f, mesh, fraction_margin=None)
    p.choice_ice_integration_method = pkg.abi.DHI["explicit"]
    oracle_mod.Oracle(mesh).calc_dHi_dt(A, Cw, p, q, 5.0)
    w = A * q["divQ"]
    assert abs(w.sum()) < 1e-12 * np.abs(w).sum()


def test_oracle_semiimplicit_with_fs0_is_the_explicit_step(pkg, oracle_mod, case):
    """f_s = 0 makes the semi-implicit matrix the identity (conservation_of_mass_semiimplicit.f90:37-56):
    its solution is the explicit update wherever neither scheme clips the thickness or the melt."""
    mesh, f, p, A, Cw = case
    orc = oracle_mod.Oracle(mesh)
    pe = pkg.abi.default_thickness_params(**{k: getattr(p, k) for k, _ in p._fields_ if k != "reserved"})
    pe.choice_ice_integration_method = pkg.abi.DHI["explicit"]
    ps = pkg.abi.default_thickness_params(**{k: getattr(p, k) for k, _ in p._fields_ if k != "reserved"})
    ps.choice_ice_integration_method = pkg.abi.DHI["semi-implicit"]
    ps.dHi_semiimplicit_fs = 0.0
    ps.dHi_PETSc_rtol, ps.dHi_PETSc_abstol = 1e-14, 0.0
    e, s = _fields(f, mesh), _fields(f, mesh)
    orc.calc_dHi_dt(A, Cw, pe, e, 2.0)
    orc.calc_dHi_dt(A, Cw, ps, s, 2.0)
    # the semi-implicit load vector limits the applied mass balance to the ice there is,
    # max(-H, dt m); the explicit step does not
    m = f["fraction_margin"] * (f["SMB"] + f["BMB"] - f["dHi_dt_target"]) + f["LMB"]
    free = ((np.asarray(mesh.VBI) == 0) & (f["mask_noice"] == 0) & (f["BC_prescr_mask"] == 0)
            & (e["Hi_tplusdt"] > 1.0) & (2.0 * m >= -f["Hi"]))
    d = np.abs(e["Hi_tplusdt"] - s["Hi_tplusdt"])[free]
    assert d.max() < 1e-9 * e["Hi_tplusdt"][free].max()
    np.testing.assert_array_equal(e["divQ"], s["divQ"])


def test_oracle_explicit_flux_limited_step_and_masks(pkg, oracle_mod, case):
    mesh, f, p, A, Cw = case
    pe = pkg.abi.default_thickness_params(**{k: getattr(p, k) for k, _ in p._fields_ if k != "reserved"})
    pe.choice_ice_integration_method = pkg.abi.DHI["explicit"]
    pe.dt_ice_max = 3.0
    q = _fields(f, mesh)
    dt, st = oracle_mod.Oracle(mesh).calc_dHi_dt(A, Cw, pe, q, 5.0)
    assert dt == 3.0                                             # min(dt, dt_ice_max)
    assert (q["Hi_tplusdt"][f["mask_noice"] == 1] == 0).all()
    pr = (f["BC_prescr_mask"] == 1) & (f["mask_noice"] == 0)
    np.testing.assert_array_equal(q["Hi_tplusdt"][pr], np.maximum(0.0, f["BC_prescr_Hi"][pr]))
    np.testing.assert_allclose(q["dHi_dt"], (q["Hi_tplusdt"] - f["Hi"]) / dt, rtol=0, atol=1e-12)
    east = np.isin(np.asarray(mesh.VBI), [3, 4]) & (f["mask_noice"] == 0)
    assert (q["Hi_tplusdt"][east] == 0).all()                   # 'zero' border


# ---- GPU ---------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def gpu_mass(pkg, gpu_lib, case):
    mesh = case[0]
    s = pkg.VelocitySolver(mesh)
    s.voronoi_upload(case[3], case[4])
    yield s
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["explicit", "none"])
def test_gpu_thickness_step_bitexact(pkg, oracle_mod, case, gpu_mass, method):
    mesh, f, p, A, Cw = case
    p.choice_ice_integration_method = pkg.abi.DHI[method]
    p.dt_ice_max = 4.0
    q = _fields(f, mesh)
    dto, _ = oracle_mod.Oracle(mesh).calc_dHi_dt(A, Cw, p, q, 5.0)
    g = gpu_mass.calc_dHi_dt(p, f, 5.0)
    assert g["dt"] == dto
    for k in ("Hi_tplusdt", "dHi_dt", "AMB") + (("divQ",) if method != "none" else ()):
        np.testing.assert_array_equal(g[k], q[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["infinite", "zero"])
def test_gpu_semiimplicit_system_bitexact(pkg, oracle_mod, case, gpu_mass, bc):
    """The stiffness matrix in the reference's add_entry layout, load vector and initial guess after
    the border, prescribed and no-ice rows."""
    mesh, f, p, A, Cw = case
    pp = pkg.abi.default_thickness_params(BC_H_west=bc, BC_H_east="infinite", BC_H_south="zero", BC_H_north=bc)
    ptr, ind, val, bb, x0 = gpu_mass.thickness_assemble(pp, f, 3.0)
    po, io, vo, bo, xo = oracle_mod.Oracle(mesh).thickness_assemble(A, Cw, pp, _fields(f, mesh), 3.0)
    np.testing.assert_array_equal(ptr, po)
    np.testing.assert_array_equal(ind, io)
    np.testing.assert_array_equal(val, vo)
    np.testing.assert_array_equal(bb, bo)
    np.testing.assert_array_equal(x0, xo)


@pytest.mark.gpu
def test_gpu_semiimplicit_solve_matches_oracle(pkg, oracle_mod, case, gpu_mass):
    """Both solves run to rtol 1e-13, so their difference measures the arithmetic, not the stop."""
    mesh, f, p, A, Cw = case
    p = pkg.abi.default_thickness_params(**{k: getattr(p, k) for k, _ in p._fields_ if k != "reserved"})
    p.choice_ice_integration_method = pkg.abi.DHI["semi-implicit"]
    p.dHi_PETSc_rtol, p.dHi_PETSc_abstol = 1e-13, 0.0
    q = _fields(f, mesh)
    _, sto = oracle_mod.Oracle(mesh).calc_dHi_dt(A, Cw, p, q, 5.0)
    g = gpu_mass.calc_dHi_dt(p, f, 5.0)
    assert g["stats"]["krylov_status"] == 0 and g["stats"]["n_Axb_its"] > 0
    assert abs(g["stats"]["n_Axb_its"] - sto["n_Axb_its"]) <= 2
    rel = np.linalg.norm(g["Hi_tplusdt"] - q["Hi_tplusdt"]) / np.linalg.norm(q["Hi_tplusdt"])
    assert rel < 1e-10, rel
    np.testing.assert_array_equal(g["divQ"], q["divQ"])


@pytest.mark.gpu
def test_gpu_thickness_at_size(pkg, gpu_lib):
    """A 250k-vertex mesh, where the oracle is not run: the area-weighted flux divergence sums to
    round-off (mass conservation) and the semi-implicit solution satisfies the exported system to
    the Krylov tolerance."""
    import scipy.sparse as sp
    mesh, f, p = pkg.geometry.thickness_case(res=1.6e3, seed=3)
    assert mesh.nV > 200_000
    with pkg.VelocitySolver(mesh) as s:
        A, Cw = s.voronoi_upload()
        pe = pkg.abi.default_thickness_params(choice_ice_integration_method="explicit")
        g = s.calc_dHi_dt(pe, dict(f, fraction_margin=None), 1.0)
        w = A * g["divQ"]
        assert abs(w.sum()) < 1e-11 * np.abs(w).sum()
        g = s.calc_dHi_dt(p, f, 1.0)
        assert g["stats"]["krylov_status"] == 0
        ptr, ind, val, bb, x0 = s.thickness_assemble(p, f, 1.0)
    M = sp.csr_matrix((val, ind, ptr), shape=(mesh.nV, mesh.nV))
    x = g["Hi_tplusdt"]
    unclipped = x > 0
    r = (M @ x - bb)[unclipped]
    assert np.linalg.norm(r) <= 1e-7 * np.linalg.norm(bb) + 1e-6 * np.sqrt(mesh.nV)


# ---- Halfar dome: the reference's integrated test for the thickness step ----------------------
def _oracle_step(oracle_mod, mesh, A, Cw):
    orc = oracle_mod.Oracle(mesh)

    def step(p, f, dt):
        q = _fields(f, mesh)
        q["dt"], _ = orc.calc_dHi_dt(A, Cw, p, q, dt)
        return q
    return step


def test_oracle_halfar_dome_converges(pkg, oracle_mod):
    """500 years of the semi-implicit thickness step (f_s 1.5, dt 10 yr) with Halfar's (1983)
    shallow-ice velocity prescribed at each step, as the reference's Halfar_dome integrated test
    runs it with its SIA solve: the RMSE of H against Halfar's solution falls with resolution (the
    reference's scoreboard: 18.0 m at 10 km, SIA included)."""
    rmse = []
    for res in (40e3, 20e3):
        mesh, f, p = pkg.geometry.halfar_case(res=res)
        A, Cw = pkg.mesh.voronoi_geometry(mesh)
        _, e, n = pkg.geometry.halfar_run(_oracle_step(oracle_mod, mesh, A, Cw), mesh, f, p)
        assert n == 50
        rmse.append(e)
    assert rmse[1] < 0.85 * rmse[0] and rmse[1] < 30.0, rmse


@pytest.mark.gpu
def test_gpu_halfar_dome_matches_oracle(pkg, oracle_mod, gpu_lib):
    mesh, f, p = pkg.geometry.halfar_case(res=20e3)
    A, Cw = pkg.mesh.voronoi_geometry(mesh)
    Ho, eo, _ = pkg.geometry.halfar_run(_oracle_step(oracle_mod, mesh, A, Cw), mesh, f, p)
    with pkg.VelocitySolver(mesh) as s:
        s.voronoi_upload(A, Cw)
        Hg, eg, n = pkg.geometry.halfar_run(s.calc_dHi_dt, mesh, f, p)
    assert n == 50
    # each step's semi-implicit solve stops at rtol 1e-8 on both sides (their reductions sum in
    # different orders), so 50 steps agree to about that, not bitwise
    assert abs(eg - eo) < 1e-4 * eo, (eg, eo)
    assert np.linalg.norm(Hg - Ho) < 1e-6 * np.linalg.norm(Ho)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["explicit", "semi-implicit"])
def test_gpu_thickness_minimal_inputs(pkg, oracle_mod, case, gpu_mass, method):
    """Only the required fields (no mass balance, margin fraction, masks or prescribed thickness;
    the library takes 0, 1 and none for them) and 'infinite' borders on all four sides."""
    mesh, f, _, A, Cw = case
    p = pkg.abi.default_thickness_params(choice_ice_integration_method=method, BC_H_west="infinite",
                                         BC_H_east="infinite", BC_H_south="infinite", BC_H_north="infinite")
    if method == "semi-implicit":
        p.dHi_PETSc_rtol, p.dHi_PETSc_abstol = 1e-13, 0.0
    g_in = {k: f[k] for k in ("Hi", "Hb", "SL", "u_vav_b", "v_vav_b", "dHi_dt")}
    q = _fields(g_in, mesh)
    dto, _ = oracle_mod.Oracle(mesh).calc_dHi_dt(A, Cw, p, q, 2.0)
    g = gpu_mass.calc_dHi_dt(p, g_in, 2.0)
    assert g["dt"] == dto
    if method == "explicit":
        for k in ("Hi_tplusdt", "dHi_dt", "AMB", "divQ"):
            np.testing.assert_array_equal(g[k], q[k], err_msg=k)
    else:
        np.testing.assert_array_equal(g["divQ"], q["divQ"])
        rel = np.linalg.norm(g["Hi_tplusdt"] - q["Hi_tplusdt"]) / np.linalg.norm(q["Hi_tplusdt"])
        assert rel < 1e-10, rel


def test_halfar_solution_is_consistent(pkg):
    """geometry.halfar (the published similarity solution) checked against itself: the dome's
    volume is constant in time, and its thickness and shallow-ice velocity satisfy the continuity
    equation dH/dt = -div(H u) inside the margin (central differences)."""
    G = pkg.geometry
    x = np.linspace(-800e3, 800e3, 1601)
    X, Y = np.meshgrid(x, x)
    vol = [G.halfar(X, Y, t)[0].sum() * (x[1] - x[0]) ** 2 for t in (0.0, 500.0, 5000.0)]
    assert max(abs(v - vol[0]) for v in vol) < 2e-3 * vol[0], vol
    rng = np.random.default_rng(0)
    r = rng.uniform(50e3, 350e3, 20)
    th = rng.uniform(0.0, 2 * np.pi, 20)
    px, py = r * np.cos(th), r * np.sin(th)
    t, dt, h = 200.0, 0.05, 50.0
    dHdt = (G.halfar(px, py, t + dt)[0] - G.halfar(px, py, t - dt)[0]) / (2 * dt)

    def flux(qx, qy):
        H, u, v = G.halfar(qx, qy, t)
        return H * u, H * v
    div = ((flux(px + h, py)[0] - flux(px - h, py)[0]) + (flux(px, py + h)[1] - flux(px, py - h)[1])) / (2 * h)
    np.testing.assert_allclose(dHdt, -div, rtol=2e-3, atol=1e-6)
