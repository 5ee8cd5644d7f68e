"""Learned Picard start: the tensor-core tile, the network against its CPU restatement, and the
warm start against the plain start."""
import ctypes as C

import numpy as np
import pytest


def bf16_bits(x):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def bf16_value(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 64, 128), (384, 128, 256), (128, 128, 64)])
def test_umma_gemm_tile(pkg, gpu_lib, M, N, K):
    rng = np.random.default_rng(M + N + K)
    X = bf16_bits(rng.normal(size=(M, K)).astype(np.float32))
    W = bf16_bits(rng.normal(size=(N, K)).astype(np.float32))
    Y = np.zeros((M, N), np.float32)
    with pkg.ColumnSolver() as s:
        rc = gpu_lib.ufe_umma_gemm_bf16(s.ctx, M, N, K, X.ctypes.data_as(C.c_void_p), W.ctypes.data_as(C.c_void_p),
                                        Y.ctypes.data_as(C.c_void_p))
        assert rc == 0, gpu_lib.ufe_ctx_last_error(s.ctx)
    ref = bf16_value(X).astype(np.float64) @ bf16_value(W).astype(np.float64).T
    err = np.abs(Y - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


# ---- the network: CPU restatement pinned by finite differences -----------------------------------
def _net_case(G, n=300, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    nbr = G.random_graph(n, seed)
    x = rng.normal(size=(n, G.FIN)) * scale
    p = rng.normal(size=G.NPARAMS) * 0.15
    tgt = rng.normal(size=(n, G.OUT))
    w = rng.uniform(0.0, 1.0, n)
    w /= w.sum()
    return nbr, x, p, tgt, w


def test_gnn_oracle_gradient_matches_finite_differences():
    import gnn_oracle as G
    nbr, x, p, tgt, w = _net_case(G, n=60, seed=1)
    loss, g = G.loss_grad(p, nbr, x, tgt, w, bf=False)
    rng = np.random.default_rng(2)
    idx = rng.choice(G.NPARAMS, 40, replace=False)
    for name in ("We", "be", "W1_0", "b1_3", "W2_2", "Wd", "bd"):   # every kind of parameter
        o, s = G.OFFSETS[name]
        idx = np.r_[idx, o + rng.integers(0, int(np.prod(s)), 3)]
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (G.loss_grad(pp, nbr, x, tgt, w, bf=False)[0] - G.loss_grad(pm, nbr, x, tgt, w, bf=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [128, 300, 1000])
def test_gnn_forward_and_gradient_match_oracle(pkg, gpu_lib, n):
    """BF16 tensor-core forward/backward against the oracle with the same BF16 roundings."""
    import gnn_oracle as G
    nbr, x, p, tgt, w = _net_case(G, n=n, seed=n)
    nbr[nbr == 7] = -1                # node 7 isolated (mean over no neighbours); stays symmetric
    nbr[7] = -1
    with pkg.ColumnSolver() as s:
        net = pkg.LearnedStart(s)
        net.set_params(p.astype(np.float32))
        pf = net.get_params().astype(np.float64)
        y = net.forward(nbr, x)
        y_ref, _ = G.forward(pf, nbr, x.astype(np.float32), bf=True)
        loss, g = net.loss_grad(nbr, x, tgt, w)
        loss_ref, g_ref = G.loss_grad(pf, nbr, x.astype(np.float32).astype(np.float64), tgt.astype(np.float32),
                                      w.astype(np.float32), bf=True)
        net.close()
    # The GPU keeps activations in FP32 and accumulates in FP32, the oracle in FP64: an operand
    # that sits at a BF16 rounding boundary can round the other way (2^-8 relative) and the
    # difference travels through the layers.  Tolerances are set by that, not by the accumulation.
    errs = {name: _rel(g[o:o + int(np.prod(shp))], g_ref[o:o + int(np.prod(shp))])
            for name, (o, shp) in G.OFFSETS.items()}
    assert _rel(y, y_ref) < 3e-3, _rel(y, y_ref)
    assert abs(loss - loss_ref) <= 3e-3 * loss_ref, (loss, loss_ref)
    assert _rel(g, g_ref) < 5e-3, (_rel(g, g_ref), errs)
    assert max(errs.values()) < 3e-2, errs


@pytest.mark.gpu
def test_gnn_warm_start_saves_picard_iterations(pkg, gpu_lib):
    """Train on GPU-generated solutions of a small ensemble; on held-out geometries the learned start
    meets the same Picard criterion in fewer iterations than the cold start.

    The criterion (L2 of the relative change < 1e-4, SSA_DIVA_utilities.f90:179) stops this
    slowly contracting Picard iteration some way from its fixed point, from whichever side it
    comes; so both starts are compared with a tightly converged solve (1e-10), and the learned
    start must land no farther from it than the cold start does (within 50 %)."""
    mesh = pkg.geometry.ensemble_mesh(nV=3000, seed=0)
    T = mesh.Tri - 1
    with pkg.VelocitySolver(mesh) as s:
        net = pkg.LearnedStart(s, seed=1)
        for m in range(24):
            ice, p = pkg.geometry.ensemble_member(mesh, m)
            s.ice_upload(ice)
            x = net.features(s)
            st = s.solve_resident(p, diva=False, cold_start=True)
            assert st["status"] >= 0
            net.dataset_add(s, x)
        losses, _ = net.train(epochs=40, lr=2e-3)
        assert losses[-1] < 0.5 * losses[0]
        cold, warm, e_cold, e_warm = [], [], [], []
        for m in range(100, 104):
            ice, p = pkg.geometry.ensemble_member(mesh, m)
            on_ice = (ice["Hi"][T] > 0).all(axis=1)
            sel = np.r_[on_ice, on_ice]
            s.ice_upload(ice)
            a = s.solve_resident(p, diva=False, cold_start=True)
            uc = np.r_[s.velocity_download()]
            # the reference solution: the same solve to a tight Picard tolerance (near round-off
            # the reference's divergence control cuts the relaxation, so fall back to a looser one)
            tight = pkg.abi.default_params(**{f: getattr(p, f) for f, _ in p._fields_ if f != "reserved"})
            tight.visc_it_nit = 400
            for tol in (1e-8, 1e-7, 1e-6):   # near round-off the divergence control may stop a tighter one
                tight.visc_it_norm_dUV_tol = tol
                try:
                    s.ice_upload(ice)
                    s.solve_resident(tight, diva=False, cold_start=True)
                    break
                except pkg.UfeError:
                    continue
            ut = np.r_[s.velocity_download()]
            s.ice_upload(ice)
            net.predict(s)
            b = s.solve_resident(p, diva=False, cold_start=False)
            uw = np.r_[s.velocity_download()]
            assert a["status"] == 0 and b["status"] == 0
            cold.append(a["n_visc_its"])
            warm.append(b["n_visc_its"])
            e_cold.append(np.linalg.norm((uc - ut)[sel]) / np.linalg.norm(ut[sel]))
            e_warm.append(np.linalg.norm((uw - ut)[sel]) / np.linalg.norm(ut[sel]))
        assert sum(warm) < 0.8 * sum(cold), (cold, warm)
        assert np.mean(e_warm) <= 1.5 * np.mean(e_cold), (e_cold, e_warm)
        net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("diva", [False, True])
def test_predicted_viscosity_start_matches_oracle(pkg, oracle_mod, gpu_lib, diva):
    """ufe_gnn_predict_start with the viscosity: a network whose decoder is constant predicts the
    start velocity (u0, v0) on the ice triangles and a uniform viscosity.  The GPU solve from that
    start, whose first Picard iteration takes the predicted viscosity in place of Glen's law (every
    layer for DIVA), matches the oracle's solve from the same velocity with the same first-iteration
    viscosity: same Picard count, velocities within 1e-8."""
    import gnn_oracle as G
    if diva:
        mesh, ice, params = pkg.geometry.small_channel(sliding="Schoof2005")
        params.visc_it_nit = 12
    else:
        mesh, ice, params = pkg.geometry.small_dome(seed=1)
    params.stress_balance_PETSc_rtol = 1e-12
    params.stress_balance_PETSc_abstol = 0.0
    orc = oracle_mod.Oracle(mesh)
    u0, v0, c = 30.0, -4.0, 0.55                     # c = (log10(eta) - 7.5) / 2
    with pkg.VelocitySolver(mesh, operators=orc.operators()) as g:
        net = pkg.LearnedStart(g)
        P = G.unpack(net.get_params().astype(np.float64))
        P["Wd"][:] = 0.0
        P["bd"][:] = [u0 / 1e3, v0 / 1e3, c]
        net.set_params(G.pack(P).astype(np.float32))
        g.ice_upload(ice)
        net.predict(g, viscosity=True)
        st = g.solve_resident(params, diva=diva, cold_start=False)
        ug = np.r_[g.velocity_download()]
        # a velocity-only prediction leaves Glen's law in the first iteration
        g.ice_upload(ice)
        net.predict(g, viscosity=False)
        st_v = g.solve_resident(params, diva=diva, cold_start=False)
        uv_only = np.r_[g.velocity_download()]
        net.close()
    on_ice = orc.apply("MAP_A_B", ice["Hi"]) > 0
    f32 = lambda a: float(np.float32(a))
    u_start = np.where(on_ice, f32(u0 / 1e3) * 1e3, 0.0)
    v_start = np.where(on_ice, f32(v0 / 1e3) * 1e3, 0.0)
    eta = np.full(mesh.nV, 10.0 ** (2.0 * f32(c) + 7.5))
    if diva:
        b = pkg.new_diva_state(mesh.nTri, mesh.nz)
        b["u_vav_b"][:], b["v_vav_b"][:] = u_start, v_start
        orc.set_first_viscosity(eta)
        nvo, _, sto = orc.solve_DIVA(ice, b, params)
        uo = np.r_[b["u_vav_b"], b["v_vav_b"]]
    else:
        b = pkg.new_ssa_state(mesh.nTri)
        b["u_b"][:], b["v_b"][:] = u_start, v_start
        orc.set_first_viscosity(eta)
        nvo, _, sto = orc.solve_SSA(ice, b, params)
        uo = np.r_[b["u_b"], b["v_b"]]
    assert st["status"] == sto["status"] and st["n_visc_its"] == nvo, (st, nvo, sto)
    assert _rel(ug, uo) < 1e-8, _rel(ug, uo)
    # the predicted viscosity changed the iteration: the velocity-only start follows another path
    assert st_v["n_visc_its"] != st["n_visc_its"] or _rel(uv_only, ug) > 1e-12
