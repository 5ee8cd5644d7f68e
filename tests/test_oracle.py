"""The CPU oracle, pinned against the reference's own known answers and exactness properties."""
import numpy as np
import pytest

from helpers import kat_csr, load_kats, load_small_dome, rel_l2


@pytest.mark.parametrize("name", ["spmv_6x6", "spmv_7x7_1", "spmv_7x7_2"])
def test_spmv_kats(pkg, oracle_mod, name):
    """ut_petsc.f90:83-150 and ut_mpi_CSR_matrix_vector_multiplication.f90:180-321 (exact)."""
    k = load_kats()[name]
    y = oracle_mod.csr_spmv(kat_csr(pkg, k), np.array(k["x"], float))
    assert np.array_equal(y, np.array(k["y"], float))


def test_spmv_2d_loops_columns(pkg, oracle_mod):
    """multiply_CSR_matrix_with_vector_2D = the 1-D product per column (:355-359)."""
    k = load_kats()["spmv_7x7_2"]
    A = kat_csr(pkg, k)
    X = np.asfortranarray(np.random.default_rng(0).normal(size=(7, 4)))
    Y = oracle_mod.csr_spmv(A, X)
    for c in range(4):
        assert np.array_equal(Y[:, c], oracle_mod.csr_spmv(A, X[:, c].copy()))


def test_poisson_kat(pkg, oracle_mod):
    """ut_mpi_CSR_matrix_solving.f90:193-273: 1-D Poisson with a known solution, to 1e-5."""
    k = load_kats()["poisson_7"]
    x, its, st = oracle_mod.csr_solve(kat_csr(pkg, k), np.array(k["b"]), np.zeros(7), 1e-12, 0.0)
    assert st == 0
    assert np.max(np.abs(x - np.array(k["x"]))) < k["tol"]


def test_bicgstab_matches_direct_solve(pkg, oracle_mod):
    """BiCGStab/Jacobi to rtol 1e-13 agrees with scipy's direct solve on a nonsymmetric system."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    rng = np.random.default_rng(3)
    n = 300
    A = sp.random(n, n, density=0.02, random_state=4, format="csr")
    A = A + sp.diags(np.abs(A).sum(1).A1 + 1.0 + rng.random(n))
    b = rng.normal(size=n)
    x, its, st = oracle_mod.csr_solve(pkg.CSR.from_scipy(A), b, np.zeros(n), 1e-13, 0.0)
    assert st == 0 and its > 0
    assert rel_l2(x, spla.spsolve(A.tocsc(), b)) < 1e-10


def test_bicgstab_zero_rhs_zero_iterations(pkg, oracle_mod):
    k = load_kats()["poisson_7"]
    x, its, st = oracle_mod.csr_solve(kat_csr(pkg, k), np.zeros(7), np.zeros(7), 1e-8, 1e-5)
    assert st == 0 and its == 0 and not x.any()


def test_operators_exact_on_linear_and_quadratic(pkg, oracle_mod):
    """Operator accuracy as the reference's component tests score it
    (ct_discretisation_mapping_derivatives.f90): mapping and 1st derivatives exact for linear
    fields; the 2nd-order b_b operators exact for quadratics on interior rows (TriBI == 0)."""
    mesh, _, _, _, _ = load_small_dome(pkg)
    orc = oracle_mod.Oracle(mesh)
    x, y = mesh.V[:, 0] / 1e5, mesh.V[:, 1] / 1e5
    gx, gy = mesh.TriGC[:, 0] / 1e5, mesh.TriGC[:, 1] / 1e5
    lin = 2.0 * x - 3.0 * y + 1.0
    assert np.max(np.abs(orc.apply("MAP_A_B", lin) - (2 * gx - 3 * gy + 1))) < 1e-12
    assert np.max(np.abs(orc.apply("DDX_A_B", lin) * 1e5 - 2.0)) < 1e-10
    assert np.max(np.abs(orc.apply("DDY_A_B", lin) * 1e5 + 3.0)) < 1e-10
    linb = 2.0 * gx - 3.0 * gy + 1.0
    assert np.max(np.abs(orc.apply("MAP_B_A", linb) - lin)) < 1e-12
    assert np.max(np.abs(orc.apply("DDX_B_A", linb) * 1e5 - 2.0)) < 1e-10
    assert np.max(np.abs(orc.apply("DDX_A_A", lin) * 1e5 - 2.0)) < 1e-10
    q = gx ** 2 + 0.5 * gx * gy - 2 * gy ** 2
    inner = mesh.TriBI == 0
    checks = {"M2_DDX_B_B": (2 * gx + 0.5 * gy) / 1e5, "M2_DDY_B_B": (0.5 * gx - 4 * gy) / 1e5,
              "M2_D2DX2_B_B": np.full_like(gx, 2.0 / 1e10), "M2_D2DXDY_B_B": np.full_like(gx, 0.5 / 1e10),
              "M2_D2DY2_B_B": np.full_like(gx, -4.0 / 1e10)}
    for name, exact in checks.items():
        err = np.abs(orc.apply(name, q) - exact)[inner].max() / np.abs(exact).max()
        assert err < 1e-9, (name, err)


def test_operator_structure_follows_flood_fill(pkg, oracle_mod):
    """Row layout of calc_matrix_operators_mesh_*: a_b rows are the triangle's three vertices in
    Tri order; b_a rows start with iTri in order; 2nd-order b_b rows start with the diagonal,
    then the TriC neighbours in order."""
    mesh, _, _, _, _ = load_small_dome(pkg)
    orc = oracle_mod.Oracle(mesh)
    A = orc.operator("MAP_A_B")
    assert np.array_equal(np.diff(A.ptr), np.full(mesh.nTri, 3))
    assert np.array_equal(A.ind.reshape(-1, 3), mesh.Tri)
    B = orc.operator("MAP_B_A")
    for vi in range(mesh.nV):
        row = B.ind[B.ptr[vi] - 1:B.ptr[vi + 1] - 1]
        n = mesh.niTri[vi]
        assert np.array_equal(row[:n], mesh.iTri[vi, :n])
    M = orc.operator("M2_DDX_B_B")
    for ti in range(mesh.nTri):
        row = M.ind[M.ptr[ti] - 1:M.ptr[ti + 1] - 1]
        assert row[0] == ti + 1
        nb = [t for t in mesh.TriC[ti] if t > 0]
        assert list(row[1:1 + len(nb)]) == nb


def test_golden_small_dome_regenerates(pkg, oracle_mod):
    """The oracle rebuilds the stored operators bit for bit and the stored SSA solution."""
    mesh, ice, params, ops, sol = load_small_dome(pkg)
    orc = oracle_mod.Oracle(mesh)
    for name, A in ops.items():
        B = orc.operator(name)
        assert np.array_equal(A.ptr, B.ptr) and np.array_equal(A.ind, B.ind), name
        assert np.array_equal(A.val, B.val), name
    ssa = pkg.new_ssa_state(mesh.nTri)
    nv, na, st = orc.solve_SSA(ice, ssa, params)
    assert [nv, na, st["status"]] == list(sol["its"])
    assert rel_l2(np.r_[ssa["u_b"], ssa["v_b"]], np.r_[sol["u_b"], sol["v_b"]]) < 1e-12


def test_assembly_layout(pkg, oracle_mod):
    """Stiffness rows of solve_linearised_SSA_DIVA.f90: free rows carry 2 entries per M2 entry
    (u column then v column); 'infinite' border rows carry the TriC neighbours then the diagonal
    -n_neighbours (:512-529)."""
    mesh, ice, params, ops, _ = load_small_dome(pkg)
    orc = oracle_mod.Oracle(mesh)
    rng = np.random.default_rng(1)
    nT = mesh.nTri
    args = [rng.uniform(1e10, 1e12, nT), rng.normal(0, 1e7, nT), rng.normal(0, 1e7, nT),
            rng.uniform(0, 1e4, nT), rng.normal(0, 1e5, nT), rng.normal(0, 1e5, nT)]
    A, bb = orc.assemble_linearised(params, *args)
    M = ops["M2_DDX_B_B"]
    for ti in range(nT):
        for uv in (1, 2):
            row = 2 * ti + uv
            cols = A.ind[A.ptr[row - 1] - 1:A.ptr[row] - 1]
            vals = A.val[A.ptr[row - 1] - 1:A.ptr[row] - 1]
            if mesh.TriBI[ti] > 0:
                nb = [t for t in mesh.TriC[ti] if t > 0]
                assert list(cols) == [2 * (t - 1) + uv for t in nb] + [row]
                assert vals[-1] == -len(nb) and np.all(vals[:-1] == 1.0)
                assert bb[row - 1] == 0.0
            else:
                m2 = M.ind[M.ptr[ti] - 1:M.ptr[ti + 1] - 1]
                assert list(cols) == [c for t in m2 for c in (2 * t - 1, 2 * t)]
                assert bb[row - 1] == -(args[4] if uv == 1 else args[5])[ti]


def test_oracle_ssa_converges_on_dome(pkg, oracle_mod):
    mesh, ice, params = pkg.geometry.small_dome()
    orc = oracle_mod.Oracle(mesh)
    ssa = pkg.new_ssa_state(mesh.nTri)
    nv, na, st = orc.solve_SSA(ice, ssa, params)
    assert st["status"] == 0 and st["L2_uv"] < params.visc_it_norm_dUV_tol
    speed = np.hypot(ssa["u_b"], ssa["v_b"])
    assert speed.max() <= params.vel_max + 1e-9 and speed.mean() > 10.0


def test_oracle_diva_converges_on_channel(pkg, oracle_mod):
    mesh, ice, params = pkg.geometry.small_channel()
    orc = oracle_mod.Oracle(mesh)
    d = pkg.new_diva_state(mesh.nTri, mesh.nz)
    nv, na, st = orc.solve_DIVA(ice, d, params)
    assert st["status"] in (0, 1), st
    assert np.isfinite(d["u_3D_b"]).all()
    # the 3-D profile's vertical average reproduces the depth-averaged velocity (Lipscomb 2019)
    z = mesh.zeta
    uav = np.sum(0.5 * (d["u_3D_b"][:, 1:] + d["u_3D_b"][:, :-1]) * np.diff(z), axis=1)
    grounded = np.abs(d["u_vav_b"]) > 1.0
    assert rel_l2(uav[grounded], d["u_vav_b"][grounded]) < 0.2


def test_oracle_first_iteration_viscosity(pkg, oracle_mod):
    """The learned start's first-iteration viscosity in the oracle: it changes the Picard path,
    the solve still converges to its tolerance near the plain solve, and the next solve consumes it
    (no reference counterpart; the GPU path is compared with this in tests/test_gnn.py)."""
    mesh, ice, params = pkg.geometry.small_dome()
    orc = oracle_mod.Oracle(mesh)
    a, b, c = (pkg.new_ssa_state(mesh.nTri) for _ in range(3))
    nva, _, sta = orc.solve_SSA(ice, a, params)
    orc.set_first_viscosity(np.full(mesh.nV, 3e8))
    nvb, _, stb = orc.solve_SSA(ice, b, params)
    nvc, _, stc = orc.solve_SSA(ice, c, params)          # consumed: the plain solve again
    assert sta["status"] == stb["status"] == stc["status"] == 0
    assert (nvb != nva) or not np.array_equal(a["u_b"], b["u_b"])
    assert nvc == nva and np.array_equal(a["u_b"], c["u_b"]) and np.array_equal(a["v_b"], c["v_b"])
    assert rel_l2(np.r_[b["u_b"], b["v_b"]], np.r_[a["u_b"], a["v_b"]]) < 0.05


def test_picard_maxit_warning(pkg, oracle_mod):
    mesh, ice, params = pkg.geometry.small_dome()
    params.visc_it_nit = 2
    orc = oracle_mod.Oracle(mesh)
    ssa = pkg.new_ssa_state(mesh.nTri)
    nv, na, st = orc.solve_SSA(ice, ssa, params)
    assert st["status"] == 1 and nv == 3


def test_no_grounded_ice_gives_zero_velocity(pkg, oracle_mod):
    mesh, ice, params = pkg.geometry.small_dome()
    ice = dict(ice)
    ice["mask_grounded_ice"] = np.zeros(mesh.nV, np.int32)
    orc = oracle_mod.Oracle(mesh)
    ssa = {"u_b": np.ones(mesh.nTri), "v_b": np.ones(mesh.nTri)}
    nv, na, st = orc.solve_SSA(ice, ssa, params)
    assert nv == 0 and not ssa["u_b"].any() and not ssa["v_b"].any()
