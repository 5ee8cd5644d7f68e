"""Column temperature solve: the oracle against analytic and dense-solve checks (CPU), and the
GPU library against the oracle (GPU).

The reference holds no test for the heat equation or the Thomas solver, so the oracle is pinned
by an analytic steady state (pure vertical diffusion between fixed temperatures gives a profile
linear in depth), by the exactness of the zeta operators on polynomials, and by a dense solve
of the same tridiagonal systems."""
import numpy as np
import pytest

from helpers import rel_l2  # noqa: F401


def _cols_copy(cols):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in cols.items()}


# ---- CPU: oracle and host logic -------------------------------------------------------------
def test_zeta_operators_exact_on_polynomials(pkg, oracle_mod):
    zeta = pkg.geometry.quadratic_zeta(30)
    l1, d1, u1, l2, d2, u2 = oracle_mod.zeta_operators(zeta)
    inner = slice(1, 29)
    for f, df, d2f in ((zeta, np.ones(30), np.zeros(30)), (zeta ** 2, 2 * zeta, 2 * np.ones(30))):
        fl, fu = np.roll(f, 1), np.roll(f, -1)
        np.testing.assert_allclose((l1 * fl + d1 * f + u1 * fu)[inner], df[inner], rtol=0, atol=1e-9)
        np.testing.assert_allclose((l2 * fl + d2 * f + u2 * fu)[inner], d2f[inner], rtol=0, atol=1e-6)
    assert l1[0] == 0 and u1[-1] == 0 and l2[0] == 0 and u2[-1] == 0


def test_library_zeta_operators_match_oracle(pkg, oracle_mod, gpu_lib):
    """ufe_zeta_operators is host code: no device needed."""
    for nz in (3, 12, 30, 61):
        zeta = pkg.geometry.quadratic_zeta(nz)
        a = pkg.zeta_operators(zeta)
        b = oracle_mod.zeta_operators(zeta)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_tridiagonal_matches_dense_solve(oracle_mod):
    rng = np.random.default_rng(3)
    n, nsys = 30, 50
    a, c = rng.normal(size=(n, nsys)), rng.normal(size=(n, nsys))
    b = 4.0 + np.abs(rng.normal(size=(n, nsys)))
    d = rng.normal(size=(n, nsys))
    x = oracle_mod.tridiagonal(a, b, c, d)
    for j in range(nsys):
        A = np.diag(b[:, j]) + np.diag(a[1:, j], -1) + np.diag(c[:-1, j], 1)
        np.testing.assert_allclose(x[:, j], np.linalg.solve(A, d[:, j]), rtol=1e-12, atol=1e-12)


def test_heat_steady_state_is_linear(pkg, oracle_mod):
    """Pure diffusion, floating columns (fixed base temperature), no advection or heating,
    uniform K and Cp: steps far longer than the diffusion time H^2/kappa (~3e5 yr) reach the
    steady state, T linear in zeta."""
    nV, nz = 8, 20
    zeta = pkg.geometry.quadratic_zeta(nz)
    _, cols = pkg.geometry.random_columns(nV, nz, seed=5)
    H = np.linspace(500.0, 3500.0, nV)
    cols["Hi_eff"] = H
    cols["mask"] = np.full(nV, pkg.abi.COL_FLOATING, np.int32)
    for k in ("u_3D", "v_3D", "w_3D", "u_times_dTdxp_upwind", "v_times_dTdyp_upwind", "dzeta_dx", "dzeta_dy",
              "dzeta_dt", "internal_heating"):
        cols[k] = np.zeros((nV, nz), order="F")
    cols["dzeta_dz"] = np.asfortranarray(np.repeat((-1.0 / H)[:, None], nz, axis=1))
    p = pkg.abi.default_thermo_params(dt=1e9, choice_ice_heat_capacity="uniform",
                                      choice_ice_thermal_conductivity="uniform")
    T = cols["Ti"]
    for _ in range(4):
        cols["Ti"] = T
        T, n, rc, _ = oracle_mod.thermo_step(p, zeta, cols)
        assert rc == 0 and n == 0
    Ts = np.minimum(cols["T_surf_annual"], 273.16)
    Tb = 273.16 - 8.7e-4 * H
    expect = Ts[:, None] + (Tb - Ts)[:, None] * zeta[None, :]
    np.testing.assert_allclose(T, expect, rtol=0, atol=1e-8)


def test_oracle_retry_and_robin_paths(pkg, oracle_mod):
    """The stiff random columns exercise dt halving (flag 2) and the Robin profile (flag 1);
    a small batch with the same columns exceeds the 1 % limit."""
    p = pkg.abi.default_thermo_params(dt=10.0)
    zeta, cols = pkg.geometry.random_columns(4000, 30, seed=1, stiff_frac=0.3, stiffness=3000.0)
    T, n, rc, flags = oracle_mod.thermo_step(p, zeta, cols)
    assert rc == 0 and n == int((flags == 1).sum()) and n > 0 and (flags == 2).sum() > 0
    assert n < 40
    assert np.isfinite(T).all() and (T <= 273.16).all()
    zeta, cols = pkg.geometry.random_columns(400, 30, seed=1, stiff_frac=0.3, stiffness=3000.0)
    _, n, rc, _ = oracle_mod.thermo_step(p, zeta, cols)
    assert n >= 4 and rc == pkg.abi.UFE_ERR_THERMO_UNSTABLE


def test_oracle_heat_equation_on_mesh(pkg, oracle_mod):
    mesh, fields, p = pkg.geometry.small_thermo()
    o = oracle_mod.Oracle(mesh)
    T, n, rc, flags = o.solve_3D_heat_equation(fields, p)
    assert rc == 0 and n == 0
    thin = fields["Hi_eff"] < 10.0
    assert thin.sum() > 0
    np.testing.assert_allclose(T[thin], np.repeat(fields["T2m"][thin].mean(axis=1)[:, None], mesh.nz, axis=1),
                               rtol=0, atol=1e-10)
    assert np.isfinite(T).all() and (T > 180.0).all() and (T <= 273.16).all()
    # the upwind term matters: without advection the result differs
    f2 = dict(fields)
    f2["u_3D_b"] = np.zeros_like(fields["u_3D_b"])
    f2["v_3D_b"] = np.zeros_like(fields["v_3D_b"])
    T2, _, rc2, _ = o.solve_3D_heat_equation(f2, p)
    assert rc2 == 0 and np.abs(T2 - T).max() > 1e-6


# ---- GPU: the library against the oracle -----------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("cp,k", [("uniform", "uniform"), ("Pounder1965", "Ritz1987")])
@pytest.mark.parametrize("glbc", ["grounded", "subgrid", "pmp"])
def test_thermo_step_matches_oracle(pkg, oracle_mod, gpu_lib, cp, k, glbc):
    p = pkg.abi.default_thermo_params(dt=10.0, choice_ice_heat_capacity=cp, choice_ice_thermal_conductivity=k,
                                      choice_GL_temperature_BC=glbc)
    zeta, cols = pkg.geometry.random_columns(4000, 30, seed=1, stiff_frac=0.3, stiffness=3000.0)
    T_o, n_o, rc_o, flags = oracle_mod.thermo_step(p, zeta, _cols_copy(cols))
    assert rc_o == 0 and (flags == 2).sum() > 0 and n_o > 0
    with pkg.ColumnSolver() as s:
        T_g, n_g = s.thermo_step(p, zeta, cols)
    assert n_g == n_o
    robin, retried = flags == 1, flags == 2
    plain = ~robin & ~retried
    if cp == "uniform":
        # same arithmetic, same roundings, for columns solved at the full step
        assert np.array_equal(T_g[plain], T_o[plain])
    else:
        # exp (Ritz conductivity) is the device's: last-bit differences, carried through the solve
        np.testing.assert_allclose(T_g[plain], T_o[plain], rtol=0, atol=1e-9)
    # the dt-halving retries evaluate the Thomas recurrences as warp-parallel scans (reassociated
    # sums), and the Robin profile uses the device's erf/exp: within 1e-9 K
    np.testing.assert_allclose(T_g[retried], T_o[retried], rtol=0, atol=1e-9)
    np.testing.assert_allclose(T_g[robin], T_o[robin], rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_thermo_step_too_many_unstable_is_an_error(pkg, oracle_mod, gpu_lib):
    p = pkg.abi.default_thermo_params(dt=10.0)
    zeta, cols = pkg.geometry.random_columns(400, 30, seed=1, stiff_frac=0.3, stiffness=3000.0)
    _, n_o, rc_o, _ = oracle_mod.thermo_step(p, zeta, _cols_copy(cols))
    assert rc_o == pkg.abi.UFE_ERR_THERMO_UNSTABLE
    with pkg.ColumnSolver() as s:
        with pytest.raises(pkg.UfeError) as e:
            s.thermo_step(p, zeta, cols)
        assert e.value.code == pkg.abi.UFE_ERR_THERMO_UNSTABLE
        # the context stays usable
        zeta, cols = pkg.geometry.random_columns(300, 12, seed=2)
        T, n = s.thermo_step(p, zeta, cols)
        assert n == 0 and np.isfinite(T).all()


@pytest.mark.gpu
def test_tridiagonal_batched_matches_oracle(pkg, oracle_mod, gpu_lib):
    rng = np.random.default_rng(4)
    n, nsys = 37, 1000
    a, c = rng.normal(size=(n, nsys)), rng.normal(size=(n, nsys))
    b = 4.0 + np.abs(rng.normal(size=(n, nsys)))
    d = rng.normal(size=(n, nsys))
    with pkg.ColumnSolver() as s:
        x = s.solve_tridiagonal_matrix_equation(a, b, c, d)
    assert np.array_equal(x, oracle_mod.tridiagonal(a, b, c, d))


def _heat_setup(pkg, oracle_mod, seed=3):
    mesh, fields, p = pkg.geometry.small_thermo(seed=seed)
    o = oracle_mod.Oracle(mesh)
    ops = {name: o.operator(name) for name in pkg.abi.OPERATORS}
    return mesh, fields, p, o, ops


@pytest.mark.gpu
@pytest.mark.parametrize("uniform", [True, False])
def test_heat_equation_on_mesh_matches_oracle(pkg, oracle_mod, gpu_lib, uniform):
    mesh, fields, p, o, ops = _heat_setup(pkg, oracle_mod)
    if uniform:
        p.choice_ice_heat_capacity = pkg.abi.CP["uniform"]
        p.choice_ice_thermal_conductivity = pkg.abi.KI["uniform"]
    T_o, n_o, rc_o, _ = o.solve_3D_heat_equation(fields, p)
    assert rc_o == 0
    with pkg.VelocitySolver(mesh, operators=ops) as s:   # the oracle's operators: identical upwind terms
        T_g, n_g = s.solve_3D_heat_equation(fields, p)
    assert n_g == n_o
    if uniform and n_o == 0:
        assert np.array_equal(T_g, T_o)
    else:
        np.testing.assert_allclose(T_g, T_o, rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_heat_equation_gpu_operators_close_to_oracle(pkg, oracle_mod, gpu_lib):
    mesh, fields, p, o, _ = _heat_setup(pkg, oracle_mod, seed=2)
    T_o, _, rc_o, _ = o.solve_3D_heat_equation(fields, p)
    with pkg.VelocitySolver(mesh) as s:                    # operators built on the GPU
        T_g, _ = s.solve_3D_heat_equation(fields, p)
    assert rc_o == 0
    np.testing.assert_allclose(T_g, T_o, rtol=0, atol=1e-7)


@pytest.mark.gpu
def test_heat_resident_stepping_matches_oracle(pkg, oracle_mod, gpu_lib):
    mesh, fields, p, o, ops = _heat_setup(pkg, oracle_mod, seed=3)
    p.choice_ice_heat_capacity = pkg.abi.CP["uniform"]
    p.choice_ice_thermal_conductivity = pkg.abi.KI["uniform"]
    f = dict(fields)
    for _ in range(5):
        T, n, rc, _ = o.solve_3D_heat_equation(f, p)
        assert rc == 0
        f = dict(f, Ti=T)
    with pkg.VelocitySolver(mesh, operators=ops) as s:
        s.heat_upload(fields)
        n_tot, ms = s.heat_step_resident(p, 5)
        T_g = s.heat_download()
    assert n_tot == 0 and ms > 0
    # bit-exact unless a column needed the dt-halving retries (warp-parallel recurrences, < 1e-9 K)
    np.testing.assert_allclose(T_g, T, rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_heat_resident_stepping_with_robin_columns(pkg, oracle_mod, gpu_lib):
    """20 steps of a case whose floating and grounding-line columns go unstable (Robin profile,
    under the 1 % limit) with the default Pounder/Ritz Cp and K."""
    mesh, fields, p, o, ops = _heat_setup(pkg, oracle_mod, seed=2)
    f = dict(fields)
    n_o = 0
    for _ in range(20):
        T, n, rc, _ = o.solve_3D_heat_equation(f, p)
        assert rc == 0
        n_o += n
        f = dict(f, Ti=T)
    assert n_o > 0
    with pkg.VelocitySolver(mesh, operators=ops) as s:
        s.heat_upload(fields)
        n_g, _ = s.heat_step_resident(p, 20)
        T_g = s.heat_download()
    assert n_g == n_o
    np.testing.assert_allclose(T_g, T, rtol=0, atol=1e-7)


def _heating_inputs(mesh, fields, seed=5):
    """Flow factor, 3-D strain rates and basal sliding fields for calc_strain_heating /
    calc_frictional_heating, smooth in space and depth."""
    rng = np.random.default_rng(seed)
    x, y = mesh.V[:, 0] / 1e6, mesh.V[:, 1] / 1e6
    z = mesh.zeta[None, :]
    out = {"A_flow": np.asfortranarray(1e-16 * (1.0 + 0.5 * np.sin(3 * x)[:, None]) * (1.0 + z))}
    for i, name in enumerate(("du_dx_3D", "du_dy_3D", "du_dz_3D", "dv_dx_3D", "dv_dy_3D", "dv_dz_3D",
                              "dw_dx_3D", "dw_dy_3D", "dw_dz_3D")):
        a, b = rng.normal(size=2)
        scale = 1e-2 if name.endswith("dz_3D") else 1e-3
        out[name] = np.asfortranarray(scale * (np.sin(a + 5 * x + 3 * y)[:, None] * (0.5 + z) + 0.2 * b))
    out["basal_friction_coefficient"] = np.ascontiguousarray(1e3 * (1.5 + np.cos(4 * y)))
    out["uabs_base"] = np.ascontiguousarray(50.0 * (1.0 + np.sin(2 * x) ** 2))
    return out


def _heating_given(pkg, mesh, fields, h):
    """The two heating terms in numpy, the way calc_strain_heating and calc_frictional_heating form
    them (thermodynamics_utilities.f90:24-128)."""
    D = np.sqrt(0.5 * (h["du_dx_3D"] ** 2 + h["dv_dy_3D"] ** 2 + h["dw_dz_3D"] ** 2
                       + 0.5 * (h["du_dy_3D"] + h["dv_dx_3D"]) ** 2 + 0.5 * (h["du_dz_3D"] + h["dw_dx_3D"]) ** 2
                       + 0.5 * (h["dv_dz_3D"] + h["dw_dy_3D"]) ** 2))
    phi = 2.0 * h["A_flow"] ** (-1.0 / 3.0) * D ** (1.0 / 3.0 + 1.0)
    phi[fields["Hi"] < 0.1, :] = 0.0
    grounded = np.isin(fields["mask"], [pkg.abi.COL_GROUNDED, pkg.abi.COL_GL_GR])
    fric = np.where(grounded, h["basal_friction_coefficient"] * h["uabs_base"], 0.0)
    return np.asfortranarray(phi), np.ascontiguousarray(fric)


def test_oracle_heating_terms_equal_given_terms(pkg, oracle_mod):
    """The oracle's strain and frictional heating, computed inside solve_3D_heat_equation, against
    the same terms computed in numpy and passed in (the host libm's pow is the only difference)."""
    mesh, fields, p = pkg.geometry.small_thermo(seed=4)
    h = _heating_inputs(mesh, fields)
    o = oracle_mod.Oracle(mesh)
    computed = {k: v for k, v in fields.items() if k not in ("internal_heating", "frictional_heating")}
    computed.update(h)
    T_c, n_c, rc_c, _ = o.solve_3D_heat_equation(computed, p)
    phi, fric = _heating_given(pkg, mesh, fields, h)
    T_g, n_g, rc_g, _ = o.solve_3D_heat_equation(dict(fields, internal_heating=phi, frictional_heating=fric), p)
    assert rc_c == rc_g == 0 and n_c == n_g
    np.testing.assert_allclose(T_c, T_g, rtol=0, atol=1e-10)
    # without sliding there is no frictional heating
    T_ns, _, _, _ = o.solve_3D_heat_equation(dict(computed, no_sliding=1), p)
    T_z, _, _, _ = o.solve_3D_heat_equation(dict(fields, internal_heating=phi, frictional_heating=0 * fric), p)
    np.testing.assert_allclose(T_ns, T_z, rtol=0, atol=1e-10)


@pytest.mark.gpu
def test_heating_terms_on_gpu_match_oracle(pkg, oracle_mod, gpu_lib):
    """calc_strain_heating and calc_frictional_heating inside ufe_solve_3D_heat_equation, against the
    oracle doing the same (CUDA's pow against the host libm: below 1e-9 K)."""
    mesh, fields, p, o, ops = _heat_setup(pkg, oracle_mod, seed=4)
    h = _heating_inputs(mesh, fields)
    computed = {k: v for k, v in fields.items() if k not in ("internal_heating", "frictional_heating")}
    computed.update(h)
    T_o, n_o, rc_o, _ = o.solve_3D_heat_equation(computed, p)
    with pkg.VelocitySolver(mesh, operators=ops) as s:
        T_g, n_g = s.solve_3D_heat_equation(computed, p)
    assert rc_o == 0 and n_g == n_o
    np.testing.assert_allclose(T_g, T_o, rtol=0, atol=1e-9)
