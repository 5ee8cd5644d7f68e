"""Synthetic ice geometries for the velocity-solve workloads.

Each builder returns ``(mesh, ice, params)``: a :class:`mesh.Mesh`, a dict of the ice-state arrays
the solver reads (``Hi, Hs, A_flow, fraction_gr_b, mask_grounded_ice`` and the sliding fields),
and an :class:`abi.SolverParams`.

* :func:`dome_case` -- plain SSA on a radially symmetric dome: 800 km x 800 km square,
  ~8,000 vertices (10 km near the r = 500 km margin, 40 km inside), flat bed at 0 m,
  H(r) = 3000 m (1 - (r/500 km)^(4/3))^(3/7) (the t = 0 Halfar shape of
  src/UFEMISM/reference_geometries/idealised_geometries.f90:110-143), Glen n = 3, A = 1e-16,
  Weertman m = 3 with beta^2 = 1e4, Picard to 1e-4, BiCGStab/Jacobi to 1e-8.
* :func:`channel_case` -- DIVA on a MISMIP+-shaped channel: 640 km x 80 km, bed of
  idealised_geometries.f90:357-401 (B0 = -150, B2 = -728.8, B4 = 343.91, B6 = -50.57 m,
  xbar = 300 km, walls of 500 m height and 4 km width at y = +-24 km, floor at -720 m),
  ~60,000 vertices refined where the ice is near flotation, A = 2e-17, n = 3, nz = 12,
  Coulomb-limited Weertman friction (Schoof2005), the boundary conditions of the reference's
  MISMIP+ runs (u = 0 on the west border, v = 0 on all borders).  The thickness stands in for "a uniform 100 m
  start advanced 500 yr at 0.3 m/yr": the accumulation without flux divergence, H = 250 m.

Constants: ice 910, sea water 1028 kg m^-3, g = 9.81 (src/UPSY/basic/parameters.f90).
"""
from __future__ import annotations

import numpy as np

from . import abi
from .mesh import generate_mesh

ICE_DENSITY = 910.0
SEAWATER_DENSITY = 1028.0
GRAV = 9.81


def _tri_vertices(mesh):
    T = mesh.Tri - 1
    return T[:, 0], T[:, 1], T[:, 2]


def grounded_fraction_b(mesh, taf_fn, nsub=6):
    """Area fraction of each triangle where the thickness above flotation is positive.

    The reference computes sub-grid grounded fractions from bilinear TAF interpolation and bedrock
    CDFs (choice_subgrid_grounded_fraction); this stand-in samples TAF at nsub*(nsub+1)/2
    barycentric points of every triangle."""
    a, b, c = _tri_vertices(mesh)
    V = mesh.V
    pts = []
    for i in range(nsub):
        for j in range(nsub - i):
            l1 = (i + 1 / 3) / nsub
            l2 = (j + 1 / 3) / nsub
            pts.append((l1, l2, 1 - l1 - l2))
    cnt = np.zeros(mesh.nTri)
    for l1, l2, l3 in pts:
        x = l1 * V[a, 0] + l2 * V[b, 0] + l3 * V[c, 0]
        y = l1 * V[a, 1] + l2 * V[b, 1] + l3 * V[c, 1]
        cnt += taf_fn(x, y) > 0
    return np.ascontiguousarray(cnt / len(pts))


def surface_elevation(Hi, Hb, SL):
    """ice_surface_elevation: grounded Hb + Hi, floating SL + Hi (1 - rho_i/rho_sw)."""
    return np.maximum(Hb + Hi, SL + Hi * (1.0 - ICE_DENSITY / SEAWATER_DENSITY))


def thickness_above_flotation(Hi, Hb, SL):
    return Hi - np.maximum(0.0, SL - Hb) * (SEAWATER_DENSITY / ICE_DENSITY)


# -- SSA dome (~8,500 vertices) -----------------------------------------------------------------
def dome_thickness(x, y, H0=3000.0, R=500e3):
    r = np.hypot(x, y)
    s = np.clip(1.0 - (r / R) ** (4.0 / 3.0), 0.0, None)
    return np.where(r < R, H0 * s ** (3.0 / 7.0), 0.0)


def dome_resolution(band=140e3, ramp=200e3, fine=10e3, coarse=40e3, R=500e3):
    def res(x, y):
        r = np.hypot(x, y)
        return fine + (coarse - fine) * np.clip((np.abs(r - R) - band) / ramp, 0.0, 1.0)
    return res


def dome_case(seed=0, nz=12, L=800e3, res_scale=1.0, A=1e-16, beta_sq=1e4, H0=3000.0, R=500e3):
    """The SSA dome, ~8,500 vertices (or a coarser copy with res_scale > 1 for quick tests; H0, R and beta_sq vary it
    for the learned start's training set)."""
    res = dome_resolution(band=140e3 * min(res_scale, 1.0) if res_scale < 1 else 140e3,
                          fine=10e3 * res_scale, coarse=40e3 * res_scale, R=R)
    mesh = generate_mesh(-L / 2, L / 2, -L / 2, L / 2, res, seed=seed, nz=nz)
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    Hi = np.ascontiguousarray(dome_thickness(x, y, H0=H0, R=R))
    Hb = np.zeros(mesh.nV)
    SL = np.full(mesh.nV, -10000.0)   # no ocean (idealised_geometries.f90:140)
    Hs = np.ascontiguousarray(surface_elevation(Hi, Hb, SL))
    ice = dict(
        Hi=Hi, Hs=Hs, Hb=Hb, SL=SL,
        A_flow=np.asfortranarray(np.full((mesh.nV, nz), A)),
        fraction_gr_b=np.ones(mesh.nTri),
        mask_grounded_ice=np.ascontiguousarray((Hi > 0).astype(np.int32)),
        beta_sq=np.full(mesh.nV, beta_sq),
    )
    params = abi.default_params(choice_sliding_law="Weertman", slid_Weertman_m=3.0,
                                visc_it_norm_dUV_tol=1e-4, stress_balance_PETSc_rtol=1e-8)
    return mesh, ice, params


# -- DIVA channel (~58k vertices) ---------------------------------------------------------------
def mismip_bed(x, y):
    """calc_idealised_geometry_MISMIPplus bed (idealised_geometries.f90:357-401)."""
    B0, B2, B4, B6 = -150.0, -728.8, 343.91, -50.57
    xbar, fc, dc, wc, zbdeep = 300e3, 4e3, 500.0, 24e3, -720.0
    xt = x / xbar
    Bx = B0 + B2 * xt ** 2 + B4 * xt ** 4 + B6 * xt ** 6
    By = dc / (1 + np.exp(-2.0 * (y - wc) / fc)) + dc / (1 + np.exp(2.0 * (y + wc) / fc))
    return np.maximum(Bx + By, zbdeep)


def channel_resolution(H=250.0, fine=0.9e3, coarse=1.35e3, taf_band=120.0):
    def res(x, y):
        taf = thickness_above_flotation(H, mismip_bed(x, y), 0.0)
        return fine + (coarse - fine) * np.clip(np.abs(taf) / taf_band, 0.0, 1.0)
    return res


def channel_case(seed=0, nz=12, H=250.0, A=2e-17, res_scale=1.0, sliding="Schoof2005"):
    """The DIVA channel, ~58k vertices (or a coarser copy with res_scale > 1)."""
    res = channel_resolution(H=H, fine=0.9e3 * res_scale, coarse=1.35e3 * res_scale)
    mesh = generate_mesh(0.0, 640e3, -40e3, 40e3, res, seed=seed, nz=nz)
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    Hb = mismip_bed(x, y)
    SL = np.zeros(mesh.nV)
    Hi = np.full(mesh.nV, float(H))
    Hs = surface_elevation(Hi, Hb, SL)
    taf = thickness_above_flotation(Hi, Hb, SL)
    effp = np.maximum(0.0, ICE_DENSITY * GRAV * Hi - SEAWATER_DENSITY * GRAV * np.maximum(0.0, SL - Hb))
    fgr_b = grounded_fraction_b(mesh, lambda xx, yy: thickness_above_flotation(H, mismip_bed(xx, yy), 0.0))
    ice = dict(
        Hi=np.ascontiguousarray(Hi), Hs=np.ascontiguousarray(Hs), Hb=Hb, SL=SL,
        A_flow=np.asfortranarray(np.full((mesh.nV, nz), A)),
        fraction_gr_b=fgr_b,
        mask_grounded_ice=np.ascontiguousarray(((taf > 0) & (Hi > 0)).astype(np.int32)),
        beta_sq=np.full(mesh.nV, 1e4),
        alpha_sq=np.full(mesh.nV, 0.5),
        effective_pressure=np.ascontiguousarray(effp),
    )
    # boundary conditions of the reference's MISMIP+ runs
    # (automated_testing/integrated_tests/idealised/MISMIPplus/config_02_5km_spinup.cfg)
    params = abi.default_params(choice_sliding_law=sliding, slid_Weertman_m=3.0,
                                visc_it_norm_dUV_tol=1e-4, stress_balance_PETSc_rtol=1e-8,
                                BC_u_west=abi.BC["zero"], BC_v_west=abi.BC["zero"], BC_v_east=abi.BC["zero"],
                                BC_v_south=abi.BC["zero"], BC_v_north=abi.BC["zero"])
    return mesh, ice, params


# -- Schoof (2006) ice stream: the reference's SSA_icestream integrated test ---------------------
def schoof2006_u(y, A=1e-18, H=2000.0, tantheta=-0.0003, L=150e3, m=1.0):
    """Along-stream velocity of Schoof's (2006) ice stream on an inclined plane with a weak band of
    width L along y = 0 (Schoof2006_icestream, src/UPSY/basic/analytical_solutions/
    Schoof_SSA_solution.f90:15-64, n = 3): zero beyond the half-width W = L (m+1)^(1/m)."""
    y = np.asarray(y, float)
    f = -ICE_DENSITY * GRAV * H * tantheta
    B = A ** (-1.0 / 3.0)
    W = L * (m + 1.0) ** (1.0 / m)
    a = np.abs(y / L)
    ua = -2.0 * f ** 3 * L ** 4 / (B ** 3 * H ** 3)
    ub = 0.25 * ((y / L) ** 4 - (m + 1.0) ** (4.0 / m))
    uc = (-3.0 / ((m + 1.0) * (m + 4.0))) * (a ** (m + 4.0) - (m + 1.0) ** (1.0 + 4.0 / m))
    ud = (3.0 / ((m + 1.0) ** 2 * (2.0 * m + 4.0))) * (a ** (2.0 * m + 4.0) - (m + 1.0) ** (2.0 + 4.0 / m))
    ue = (-1.0 / ((m + 1.0) ** 3 * (3.0 * m + 4.0))) * (a ** (3.0 * m + 4.0) - (m + 1.0) ** (3.0 + 4.0 / m))
    u = ua * (ub + uc + ud + ue)
    return np.where(np.abs(y) > W, 0.0, u)


def icestream_case(res=32e3, seed=0, nz=12):
    """The SSA_icestream integrated test of the reference
    (automated_testing/integrated_tests/idealised/SSA_icestream/config_0*_*km.cfg): an 800 km x 800 km
    slab, 2000 m thick on a bed sloping at -0.0003 in x, uniform resolution `res` (32, 16, 8 or 4 km
    in the reference's four runs), all grounded (sea level -10 km); SSA with the idealised
    SSA_icestream sliding law, uniform A = 1e-18, eps0^2 = 1e-10, Picard relaxation 0.3 to 5e-8
    (up to 5000 iterations), Krylov rtol 1e-7 / abstol 1e-5, u copied across the west and east
    borders ('infinite_SSA_icestream'), u = 0 on the south and north borders, v = 0 on every border.
    The flow factor is computed by the solve (choice_ice_rheology_Glen 'uniform'), so no A_flow is
    passed.  Mesh: this package's generator at uniform resolution (the reference refines with its
    own Ruppert scheme), so the error against Schoof's solution is comparable, not identical."""
    L = 400e3
    mesh = generate_mesh(-L, L, -L, L, lambda x, y: np.full(np.shape(x), float(res)), seed=seed, nz=nz)
    x = mesh.V[:, 0]
    Hi = np.full(mesh.nV, 2000.0)
    Hb = -0.0003 * x                                   # calc_idealised_geometry_SSA_icestream
    SL = np.full(mesh.nV, -10000.0)
    Hs = surface_elevation(Hi, Hb, SL)
    ice = dict(Hi=np.ascontiguousarray(Hi), Hs=np.ascontiguousarray(Hs), Hb=Hb, SL=SL,
               fraction_gr_b=np.ones(mesh.nTri), mask_grounded_ice=np.ones(mesh.nV, np.int32))
    params = abi.default_params(choice_sliding_law="idealised_SSA_icestream", visc_it_norm_dUV_tol=5e-8,
                                visc_it_nit=5000, visc_it_relax=0.3, visc_eff_min=1e4,
                                stress_balance_PETSc_rtol=1e-7, stress_balance_PETSc_abstol=1e-5,
                                Glens_flow_law_epsilon_sq_0=1e-10, choice_ice_rheology_Glen="uniform",
                                uniform_Glens_flow_factor=1e-18,
                                BC_u_west="infinite_SSA_icestream", BC_u_east="infinite_SSA_icestream",
                                BC_u_south="zero", BC_u_north="zero", BC_v_west="zero", BC_v_east="zero",
                                BC_v_south="zero", BC_v_north="zero")
    return mesh, ice, params


def transect_values(mesh, values_a, x0=0.0, dy=1e3):
    """A field on the vertices sampled along the south-north transect x = x0 of the reference's
    transect output ('southnorth,dx=1e3'): linear interpolation in the triangle holding each
    point.  Returns (y, values)."""
    from scipy.spatial import cKDTree
    ymin, ymax = mesh.V[:, 1].min(), mesh.V[:, 1].max()
    y = np.arange(ymin, ymax + 0.5 * dy, dy)
    pts = np.stack([np.full_like(y, x0), y], axis=1)
    T = mesh.Tri - 1
    tree = cKDTree(mesh.TriGC)
    _, cand = tree.query(pts, k=min(12, mesh.nTri))
    out = np.full(len(y), np.nan)
    for i, p in enumerate(pts):
        for t in np.atleast_1d(cand[i]):
            a, b, c = mesh.V[T[t, 0]], mesh.V[T[t, 1]], mesh.V[T[t, 2]]
            det = (b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1])
            l1 = ((b[0] - p[0]) * (c[1] - p[1]) - (c[0] - p[0]) * (b[1] - p[1])) / det
            l2 = ((c[0] - p[0]) * (a[1] - p[1]) - (a[0] - p[0]) * (c[1] - p[1])) / det
            l3 = 1.0 - l1 - l2
            if min(l1, l2, l3) >= -1e-9:
                out[i] = l1 * values_a[T[t, 0]] + l2 * values_a[T[t, 1]] + l3 * values_a[T[t, 2]]
                break
    return y, out


def thickness_case(seed=0, L=800e3, res=20e3, H0=3000.0, R=330e3, U0=400.0, nz=3):
    """An ice-thickness (conservation of mass) workload on a generated mesh: a dome of thickness
    H0 and radius R over a bed of relief around sea level (part of the margin floats), a radial
    outflow velocity rising to U0 m/yr at the margin on the triangles, surface mass balance
    falling with distance, basal melt under floating ice, a band of partly filled margin cells
    (fraction_margin < 1), a no-ice mask near the domain border, a few prescribed-thickness
    vertices, 'infinite' thickness borders west/south and 'zero' east/north.  Returns
    (mesh, fields, thickness params); `res` the mesh spacing in m."""
    mesh = generate_mesh(-L / 2, L / 2, -L / 2, L / 2, lambda x, y: np.full(np.shape(x), float(res)),
                         seed=seed, nz=nz)
    rng = np.random.default_rng(seed)
    x, y = np.asarray(mesh.V[:, 0]), np.asarray(mesh.V[:, 1])
    r = np.hypot(x, y)
    Hi = np.ascontiguousarray(dome_thickness(x, y, H0=H0, R=R))
    Hb = np.ascontiguousarray(-150.0 + 400.0 * np.cos(2 * np.pi * x / 300e3) * np.cos(2 * np.pi * y / 250e3)
                              - 300.0 * (r / R) ** 2)
    SL = np.zeros(mesh.nV)
    gc = np.asarray(mesh.TriGC)
    rt = np.maximum(np.hypot(gc[:, 0], gc[:, 1]), 1.0)
    speed = U0 * np.clip(rt / R, 0.0, 1.2) ** 2 * np.exp(-np.clip(rt - R, 0.0, None) / 50e3)
    speed = speed * (1.0 + 0.2 * rng.standard_normal(mesh.nTri))
    u = np.ascontiguousarray(speed * gc[:, 0] / rt)
    v = np.ascontiguousarray(speed * gc[:, 1] / rt)
    floating = thickness_above_flotation(Hi, Hb, SL) < 0.0
    fields = dict(
        Hi=Hi, Hb=Hb, SL=SL, u_vav_b=u, v_vav_b=v,
        SMB=np.ascontiguousarray(0.5 - 1.5 * (r / (L / 2)) ** 2),
        BMB=np.ascontiguousarray(np.where(floating & (Hi > 0), -2.0, 0.0)),
        LMB=np.zeros(mesh.nV),
        fraction_margin=np.ascontiguousarray(np.where(np.abs(r - R) < 15e3, 0.6, 1.0)),
        mask_noice=np.ascontiguousarray((np.maximum(np.abs(x), np.abs(y)) > 0.45 * L).astype(np.int32)),
        dHi_dt_target=np.zeros(mesh.nV),
        BC_prescr_mask=np.ascontiguousarray((rng.random(mesh.nV) < 0.002).astype(np.int32)),
        BC_prescr_Hi=np.ascontiguousarray(Hi + 10.0),
        dHi_dt=np.ascontiguousarray(0.01 * rng.standard_normal(mesh.nV)),
    )
    params = abi.default_thickness_params(BC_H_west="infinite", BC_H_south="infinite",
                                          BC_H_east="zero", BC_H_north="zero")
    return mesh, fields, params


def halfar(x, y, t, A=1e-16, n=3.0, H0=3000.0, R0=500e3):
    """Halfar's (1981, 1983) similarity solution of the isothermal shallow-ice dome on a flat bed,
    in the form of Bueler et al. (2005, J. Glaciol. 51(173), eqs. 10-11): the thickness H and the
    vertically averaged shallow-ice velocity u = -Gamma H^(n+1) |grad H|^(n-1) grad H,
    Gamma = 2 A (rho g)^n / (n+2), at t years after the moment the dome has height H0 and radius
    R0 (similarity time t0 + t).  Returns (H, u, v) at the points (x, y)."""
    rho_g = 910.0 * 9.81
    gam = 2.0 * A * rho_g ** n / (n + 2.0)
    t0 = 1.0 / ((5.0 * n + 3.0) * gam) * ((2.0 * n + 1.0) / (n + 1.0)) ** n * R0 ** (n + 1.0) / H0 ** (2.0 * n + 1.0)
    T = (t0 + t) / t0
    alpha, beta = 2.0 / (5.0 * n + 3.0), 1.0 / (5.0 * n + 3.0)
    p3, p4 = (n + 1.0) / n, n / (2.0 * n + 1.0)
    x, y = np.asarray(x, float), np.asarray(y, float)
    r = np.hypot(x, y)
    s = np.minimum(T ** (-beta) * r / R0, 1.0)
    f = 1.0 - s ** p3
    H = H0 * T ** (-alpha) * np.where(f > 0.0, f, 0.0) ** p4
    # dH/dr = H0 T^-alpha p4 f^(p4 - 1) (-p3 s^(p3 - 1)) T^-beta / R0 inside the dome
    inside = (f > 0.0) & (r > 0.0)
    dHdr = np.zeros_like(r)
    fi = np.where(inside, f, 1.0)
    dHdr[inside] = (H0 * T ** (-alpha) * p4 * fi[inside] ** (p4 - 1.0) * (-p3) * s[inside] ** (p3 - 1.0)
                    * T ** (-beta) / R0)
    speed = -gam * H ** (n + 1.0) * np.abs(dHdr) ** (n - 1.0) * dHdr   # radial, outward
    rr = np.where(r > 0.0, r, 1.0)
    return H, np.where(inside, speed * x / rr, 0.0), np.where(inside, speed * y / rr, 0.0)


def halfar_case(res=20e3, seed=0, L=1000e3, nz=3, **kw):
    """The reference's Halfar_dome integrated test (automated_testing/integrated_tests/idealised/
    Halfar_dome/config_Halfar_*.cfg: H0 3000 m, R0 500 km, A 1e-16, n 3, a +-1000 km domain,
    'zero' thickness borders, semi-implicit f_s 1.5, dt_ice_max 10 yr) for the thickness step
    alone: the mesh, the thickness fields at t = 0 with Halfar's velocity, and the parameters."""
    mesh = generate_mesh(-L, L, -L, L, lambda x, y: np.full(np.shape(x), float(res)), seed=seed, nz=nz)
    H, _, _ = halfar(mesh.V[:, 0], mesh.V[:, 1], 0.0, **kw)
    gc = np.asarray(mesh.TriGC)
    _, u, v = halfar(gc[:, 0], gc[:, 1], 0.0, **kw)
    fields = dict(Hi=np.ascontiguousarray(H), Hb=np.zeros(mesh.nV), SL=np.full(mesh.nV, -10000.0),
                  u_vav_b=np.ascontiguousarray(u), v_vav_b=np.ascontiguousarray(v), dHi_dt=np.zeros(mesh.nV))
    params = abi.default_thickness_params(dt_ice_max=10.0)
    return mesh, fields, params


def halfar_run(step, mesh, fields, params, years=500.0, dt=10.0, **kw):
    """Step the thickness equation over `years` with Halfar's velocity at each step's start time;
    step(params, fields, dt) -> dict (a calc_dHi_dt).  Returns (H at the end, RMSE against Halfar's
    H there [m], steps)."""
    gc = np.asarray(mesh.TriGC)
    f = dict(fields)
    t, n = 0.0, 0
    while t < years - 1e-9:
        _, u, v = halfar(gc[:, 0], gc[:, 1], t, **kw)
        f["u_vav_b"], f["v_vav_b"] = np.ascontiguousarray(u), np.ascontiguousarray(v)
        out = step(params, f, min(dt, years - t))
        t += out["dt"]
        f["Hi"], f["dHi_dt"] = out["Hi_tplusdt"], out["dHi_dt"]
        n += 1
    Ha, _, _ = halfar(mesh.V[:, 0], mesh.V[:, 1], t, **kw)
    return f["Hi"], float(np.sqrt(np.mean((f["Hi"] - Ha) ** 2))), n


def small_dome(seed=0, nz=12):
    """A ~1,000-vertex dome for tests the CPU oracle finishes in seconds."""
    return dome_case(seed=seed, nz=nz, res_scale=3.0)


def small_channel(seed=0, nz=8, sliding="Schoof2005"):
    """A ~2,000-vertex channel for DIVA tests."""
    return channel_case(seed=seed, nz=nz, res_scale=6.5, sliding=sliding)


# ---- thermodynamics workloads ----------------------------------------------------------------
SEC_PER_YEAR = 31556943.36
T0 = 273.16
CC_GRADIENT = 8.7e-4


def quadratic_zeta(nz):
    """nz zeta values from 0 (surface) to 1 (base), spaced quadratically closer toward the base."""
    s = np.linspace(0.0, 1.0, nz)
    return 1.0 - (1.0 - s) ** 2


def smooth_field(x, y, corr_len, seed, n_modes=96):
    """A smooth, roughly standard-normal random field: a sum of random plane waves whose
    wavenumbers are drawn with scale 1/corr_len."""
    rng = np.random.default_rng(seed)
    k = rng.normal(0.0, 1.0 / corr_len, size=(n_modes, 2))
    ph = rng.uniform(0.0, 2.0 * np.pi, n_modes)
    f = np.zeros(np.shape(x))
    for j in range(n_modes):
        f += np.cos(k[j, 0] * x + k[j, 1] * y + ph[j])
    return f * np.sqrt(2.0 / n_modes)


def _uniform_marginal(f):
    """Map a field to values uniform in (0, 1) by rank."""
    r = np.empty(f.size)
    r[np.argsort(f, kind="stable")] = np.arange(f.size)
    return (r + 0.5) / f.size


def thermo_case(nV=200_000, nz=30, seed=0, corr_len=50e3, thick_corr_len=200e3, dt=10.0):
    """Batched column thermodynamics: a mesh of about ``nV`` vertices (6.8 km inside a central
    disk, 13.7 km outside it, so that the explicit horizontal advection keeps u dt / dx < 1;
    3,500 km x 3,500 km at 200,000 vertices) with ``nz`` quadratic zeta layers; thickness
    uniform in [0, 4000] m with 15 % of the columns ice-free (and a taper to zero over the 40 km
    next to the domain border); surface
    temperature uniform in [-50, -10] degC; geothermal flux normal(55, 10) mW m^-2; velocities from
    smooth random fields with ``corr_len`` correlation, |u| <= 500 m/yr; thickness and the
    floating mask vary over ``thick_corr_len``; about a sixth of the ice floating, with
    grounding-line columns between.  Returns (mesh, fields, params): the fields of
    ufe_heat_fields and an abi.ThermoParams with the given dt [yr]."""
    # explicit horizontal advection (calc_upwind_heat_flux_derivatives) needs u dt / dx < 1:
    # 500 m/yr x 10 yr against cells of L/512 = 6.8 km inside a disk and L/256 outside it; the
    # disk's radius sets the vertex count.
    L = 3500e3 * np.sqrt(nV / 200_000.0)
    fine, coarse = _levels(nV, L)

    def make_res(radius):
        return lambda x, y: np.where(np.hypot(x, y) < radius, fine, coarse)

    res = _calibrated_resolution(make_res, nV, 0.0, L, L, seed=seed)
    mesh = generate_mesh(-L / 2, L / 2, -L / 2, L / 2, res, seed=seed, nz=nz, zeta=quadratic_zeta(nz))
    n = mesh.nV
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    zeta = mesh.zeta
    q = _uniform_marginal(smooth_field(x, y, thick_corr_len, seed + 1))
    H = 4000.0 * np.clip((q - 0.15) / 0.85, 0.0, 1.0)
    # the ice thins to zero over the 40 km next to the domain border (no ice on the border, where
    # an upwind triangle can be missing)
    dist = np.minimum(np.minimum(x + L / 2, L / 2 - x), np.minimum(y + L / 2, L / 2 - y))
    H *= np.clip((dist - 0.5 * coarse) / 40e3, 0.0, 1.0)
    H[mesh.VBI > 0] = 0.0
    ice = H > 0.0
    floating = (smooth_field(x, y, thick_corr_len, seed + 2) > 1.0) & ice
    grounded = ice & ~floating
    # grounded vertices with a floating neighbour: the grounded side of the grounding line
    C = mesh.C - 1
    has_fl_nb = np.zeros(n, bool)
    for c in range(mesh.nC_mem):
        nb = C[:, c]
        ok = (c < mesh.nC) & (nb >= 0)
        has_fl_nb |= ok & floating[np.where(ok, nb, 0)]
    gl = grounded & has_fl_nb
    mask = np.zeros(n, np.int32)
    mask[grounded] = abi.COL_GROUNDED
    mask[floating] = abi.COL_FLOATING
    mask[gl] = abi.COL_GL_GR
    Hs = np.where(floating, H * (1.0 - ICE_DENSITY / SEAWATER_DENSITY), H)

    T_surf = 273.15 - 50.0 + 40.0 * _uniform_marginal(smooth_field(x, y, corr_len, seed + 3))
    months = np.arange(12)
    T2m = T_surf[:, None] + 10.0 * np.cos(2.0 * np.pi * (months[None, :] + 0.5) / 12.0)
    geo = (55.0 + 10.0 * smooth_field(x, y, corr_len, seed + 4)) * 1e-3 * SEC_PER_YEAR
    u = smooth_field(x, y, corr_len, seed + 5)
    v = smooth_field(x, y, corr_len, seed + 6)
    scale = 495.0 / max(np.sqrt(u * u + v * v).max(), 1e-12)
    u_vav, v_vav = u * scale, v * scale
    SMB = 0.3 + 0.4 * smooth_field(x, y, corr_len, seed + 7)
    shape = 1.1 - 0.5 * zeta ** 4                       # vertical mean 1
    u_3D = np.asfortranarray(u_vav[:, None] * shape[None, :])
    v_3D = np.asfortranarray(v_vav[:, None] * shape[None, :])
    w_3D = np.asfortranarray(-SMB[:, None] * (1.0 - zeta[None, :]))
    T = mesh.Tri - 1
    u_3D_b = np.asfortranarray(u_3D[T].mean(axis=1))
    v_3D_b = np.asfortranarray(v_3D[T].mean(axis=1))
    speed = np.sqrt(u_vav ** 2 + v_vav ** 2) / 500.0
    phi = np.asfortranarray(2000.0 * speed[:, None] * zeta[None, :] ** 4)
    fric = np.where(mask == abi.COL_FLOATING, 0.0, 0.05 * speed * SEC_PER_YEAR)
    fric[~ice] = 0.0
    dHi_dt = 0.05 * smooth_field(x, y, corr_len, seed + 8)
    dHs_dt = np.where(floating, 0.115 * dHi_dt, 0.05 * smooth_field(x, y, corr_len, seed + 9))
    fr = np.where(mask == abi.COL_FLOATING, 0.0, 1.0)
    fr[gl] = 0.5 + 0.5 * _uniform_marginal(smooth_field(x, y, corr_len, seed + 10))[gl]
    fr[~ice] = 0.0
    Ts = np.minimum(T_surf, T0)
    pmp_b = T0 - CC_GRADIENT * H
    Tb = np.minimum(pmp_b, Ts + 25.0 + 5.0 * smooth_field(x, y, corr_len, seed + 11))
    Ti = np.asfortranarray(Ts[:, None] + (Tb - Ts)[:, None] * zeta[None, :])
    Ti[H < 10.0, :] = T_surf[H < 10.0, None]
    fields = dict(Ti=Ti, Hi=H, Hi_eff=H.copy(), Hs=Hs, dHi_dt=dHi_dt, dHs_dt=dHs_dt, u_vav=u_vav, v_vav=v_vav,
                  u_3D=u_3D, v_3D=v_3D, w_3D=w_3D, u_3D_b=u_3D_b, v_3D_b=v_3D_b, internal_heating=phi,
                  frictional_heating=fric, geothermal_heat_flux=geo, T2m=np.asfortranarray(T2m), SMB=SMB,
                  mask=mask, fraction_gr=fr)
    params = abi.default_thermo_params(dt=dt)
    return mesh, fields, params


def small_thermo(seed=0, nz=30, nV=3000):
    """A ~3,000-vertex thermodynamics case for tests the CPU oracle finishes in seconds."""
    return thermo_case(nV=nV, nz=nz, seed=seed)


def random_columns(nV, nz, seed=0, stiff_frac=0.0, stiffness=300.0):
    """Per-column inputs of ufe_thermo_columns without a mesh (random but physical values); a
    fraction ``stiff_frac`` of the ice columns gets vertical velocities ``stiffness`` times larger,
    which makes some of them need dt halving and some fail the stability check."""
    rng = np.random.default_rng(seed)
    zeta = quadratic_zeta(nz)
    H = rng.uniform(0.0, 4000.0, nV)
    H[rng.random(nV) < 0.15] = rng.uniform(0.0, 9.0, 1)[0]
    mask = np.where(rng.random(nV) < 0.7, abi.COL_GROUNDED, abi.COL_FLOATING).astype(np.int32)
    mask[rng.random(nV) < 0.1] = abi.COL_GL_GR
    T_surf = rng.uniform(223.15, 263.15, nV)
    Ts = np.minimum(T_surf, T0)
    pmp = T0 - CC_GRADIENT * H[:, None] * zeta[None, :]
    Tb = np.minimum(pmp[:, -1], Ts + rng.uniform(5.0, 40.0, nV))
    Ti = Ts[:, None] + (Tb - Ts)[:, None] * zeta[None, :]
    Hc = np.maximum(H, 10.0)
    u = rng.uniform(-300, 300, nV)[:, None] * (1.1 - 0.5 * zeta[None, :] ** 4)
    v = rng.uniform(-300, 300, nV)[:, None] * (1.1 - 0.5 * zeta[None, :] ** 4)
    w = -rng.uniform(-0.2, 0.6, nV)[:, None] * (1.0 - zeta[None, :])
    stiff = (rng.random(nV) < stiff_frac) & (H >= 10.0)
    w[stiff] *= stiffness * rng.uniform(0.5, 2.0, stiff.sum())[:, None]
    gx, gy = rng.normal(0, 2e-3, nV), rng.normal(0, 2e-3, nV)
    hx, hy = rng.normal(0, 2e-3, nV), rng.normal(0, 2e-3, nV)
    dzx = (gx[:, None] - zeta[None, :] * hx[:, None]) / Hc[:, None]
    dzy = (gy[:, None] - zeta[None, :] * hy[:, None]) / Hc[:, None]
    dzz = np.repeat((-1.0 / Hc)[:, None], nz, axis=1)
    dzt = (rng.normal(0, 0.05, nV)[:, None] - zeta[None, :] * rng.normal(0, 0.05, nV)[:, None]) / Hc[:, None]
    udx = rng.normal(0, 2e-3, (nV, nz))
    vdy = rng.normal(0, 2e-3, (nV, nz))
    phi = rng.uniform(0, 3000, nV)[:, None] * zeta[None, :] ** 4
    geo = rng.normal(55.0, 10.0, nV) * 1e-3 * SEC_PER_YEAR
    fric = np.where(mask == abi.COL_FLOATING, 0.0, rng.uniform(0, 0.05, nV) * SEC_PER_YEAR)
    cols = dict(Ti=Ti, u_3D=u, v_3D=v, w_3D=w, u_times_dTdxp_upwind=udx, v_times_dTdyp_upwind=vdy, dzeta_dx=dzx,
                dzeta_dy=dzy, dzeta_dz=dzz, dzeta_dt=dzt, internal_heating=phi, Hi_eff=H, T_surf_annual=T_surf,
                Q_base_grnd=fric + geo, mask=mask, fraction_gr=rng.uniform(0.0, 1.0, nV), geothermal_heat_flux=geo,
                SMB=rng.uniform(-0.5, 1.0, nV))
    return zeta, {k: (np.asfortranarray(v) if isinstance(v, np.ndarray) else v) for k, v in cols.items()}


# ---- learned-start SSA ensemble (30k-vertex mesh) ---------------------------------------------
def grounded_fraction_b_vertex(mesh, taf, nsub=6):
    """grounded_fraction_b with the thickness above flotation given at vertices (linear within
    each triangle)."""
    a, b, c = _tri_vertices(mesh)
    cnt = np.zeros(mesh.nTri)
    npts = 0
    for i in range(nsub):
        for j in range(nsub - i):
            l1 = (i + 1 / 3) / nsub
            l2 = (j + 1 / 3) / nsub
            cnt += (l1 * taf[a] + l2 * taf[b] + (1 - l1 - l2) * taf[c]) > 0
            npts += 1
    return np.ascontiguousarray(cnt / npts)


def _levels(target, L):
    """Resolutions (fine, coarse) of the two quadtree levels whose uniform point counts bracket
    `target` on an L x L domain (a cell of size L/2^k is split when it is larger than the
    resolution, so the resolutions sit just above the cell sizes)."""
    k = max(1, int(np.floor(np.log(max(target, 4)) / np.log(4.0))))
    return L / 2 ** (k + 1) * 1.01, L / 2 ** k * 1.01


def _calibrated_resolution(make_res, target, lo, hi, L, seed=0, iters=14):
    """The quadtree point generator places points on power-of-two cells, so a uniform resolution
    gives vertex counts four times apart.  `make_res(a)` returns a resolution function whose
    fine region grows with `a`; bisect `a` in [lo, hi] so that the point count is near `target`."""
    from .mesh import generate_points
    a0, a1 = lo, hi
    for _ in range(iters):
        a = 0.5 * (a0 + a1)
        n = len(generate_points(-L / 2, L / 2, -L / 2, L / 2, make_res(a), seed=seed))
        if n < target:
            a0 = a
        else:
            a1 = a
    return make_res(0.5 * (a0 + a1))


def ensemble_mesh(nV=30_000, L=1500e3, seed=0, nz=12, R=600e3):
    """One mesh of about nV vertices over an L x L domain: fine quadtree cells within a band around
    the dome margin r = R (where the ice is thin, floating and fast), cells twice as large
    elsewhere (L/256 and L/128 at 30,000 vertices); the band's width sets the vertex count."""
    fine, coarse = _levels(nV, L)

    def make_res(band):
        def res(x, y):
            r = np.hypot(x, y)
            return np.where(np.abs(r - R) < band, fine, coarse)
        return res

    res = _calibrated_resolution(make_res, nV, 0.0, L, L, seed=seed)
    return generate_mesh(-L / 2, L / 2, -L / 2, L / 2, res, seed=seed, nz=nz)


def ensemble_member(mesh, member, A=1e-16, H0=3000.0, R=600e3, bed_sigma=400.0, bed_corr=20e3,
                    beta_mu=np.log(1e4), beta_sigma=0.5, beta_corr=50e3):
    """Geometry `member` of the learned-start ensemble on `mesh`: bed -200 m plus a Gaussian random
    field (sigma 400 m, correlation 20 km, seeded by the member), the dome thickness of the SSA dome case
    with R = 600 km, floating where the ice is thinner than flotation (sea level 0), and a
    log-normal friction coefficient beta^2 (log-mean ln 1e4, log-sd 0.5, correlation 50 km).
    Returns (ice, params) for an SSA solve (Weertman m = 3, n = 3, A = 1e-16, Picard 1e-4,
    BiCGStab 1e-8)."""
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    bed = -200.0 + bed_sigma * smooth_field(x, y, bed_corr, 1000 + member)
    Hi = np.ascontiguousarray(dome_thickness(x, y, H0=H0, R=R))
    SL = np.zeros(mesh.nV)
    taf = thickness_above_flotation(Hi, bed, SL)
    Hs = np.ascontiguousarray(surface_elevation(Hi, bed, SL))
    grounded = (Hi > 0) & (taf > 0)
    fgr = grounded_fraction_b_vertex(mesh, np.where(Hi > 0, taf, -1.0))
    beta_sq = np.exp(beta_mu + beta_sigma * smooth_field(x, y, beta_corr, 2000 + member))
    ice = dict(Hi=Hi, Hs=Hs, Hb=bed, SL=SL,
               A_flow=np.asfortranarray(np.full((mesh.nV, mesh.nz), A)),
               fraction_gr_b=fgr, mask_grounded_ice=np.ascontiguousarray(grounded.astype(np.int32)),
               beta_sq=np.ascontiguousarray(beta_sq))
    params = abi.default_params(choice_sliding_law="Weertman", slid_Weertman_m=3.0,
                                visc_it_norm_dUV_tol=1e-4, stress_balance_PETSc_rtol=1e-8)
    return ice, params


# ---- mixed-size DIVA ensemble (64 members, 20k-400k vertices) ---------------------------------
MIXED_L = 6000e3      # domain side [m]
MIXED_R = 2200e3      # dome radius [m]


def fractal_field(x, y, seed, slope=-2.0, L=MIXED_L, kmax_len=10e3, n_modes=512):
    """A random field with power spectrum ~ k^slope between wavelengths L and kmax_len: random
    plane waves with wavenumbers log-uniform in [2 pi / L, 2 pi / kmax_len], random directions
    and phases, amplitudes k^(slope/2) times the square root of each mode's share of the
    log-wavenumber band (so the spectral density follows the power law); scaled to zero mean
    and unit RMS over the points given."""
    rng = np.random.default_rng(seed)
    k = np.exp(rng.uniform(np.log(2.0 * np.pi / L), np.log(2.0 * np.pi / kmax_len), n_modes))
    th = rng.uniform(0.0, 2.0 * np.pi, n_modes)
    ph = rng.uniform(0.0, 2.0 * np.pi, n_modes)
    amp = k ** (0.5 * slope) * np.sqrt(k)   # log-uniform k: density ~ 1/k, so weight by sqrt(k)
    f = np.zeros(np.shape(x))
    for j in range(n_modes):
        f += amp[j] * np.cos(k[j] * (np.cos(th[j]) * x + np.sin(th[j]) * y) + ph[j])
    f = f - f.mean()
    return f / np.sqrt(np.mean(f * f))


def mixed_ensemble_mesh(nV, seed=0, nz=12):
    """A mesh of about nV vertices over the 6,000 km domain, fine cells in a band around the
    dome margin r = 2,200 km (the grounding zone), cells twice as large elsewhere."""
    return ensemble_mesh(nV=nV, L=MIXED_L, seed=seed, nz=nz, R=MIXED_R)


def mixed_ensemble_member(mesh, member, A=1e-16, H0=4000.0, bed_rms=800.0, bed_mean=-300.0):
    """Member `member` of the mixed-size DIVA ensemble: a fractal bed (spectral slope -2, RMS
    800 m, mean -300 m, seeded by the member), a dome of thickness H0 = 4,000 m and radius 2,200 km,
    floating where thinner than flotation, log-normal beta^2 as in the learned-start ensemble.
    Returns (ice, params) for a DIVA solve (Weertman m = 3, n = 3, A = 1e-16, Picard 1e-4,
    BiCGStab 1e-8)."""
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    bed = bed_mean + bed_rms * fractal_field(x, y, 3000 + member)
    Hi = np.ascontiguousarray(dome_thickness(x, y, H0=H0, R=MIXED_R))
    SL = np.zeros(mesh.nV)
    taf = thickness_above_flotation(Hi, bed, SL)
    Hs = np.ascontiguousarray(surface_elevation(Hi, bed, SL))
    grounded = (Hi > 0) & (taf > 0)
    fgr = grounded_fraction_b_vertex(mesh, np.where(Hi > 0, taf, -1.0))
    beta_sq = np.exp(np.log(1e4) + 0.5 * smooth_field(x, y, 150e3, 4000 + member))
    ice = dict(Hi=Hi, Hs=Hs, Hb=bed, SL=SL,
               A_flow=np.asfortranarray(np.full((mesh.nV, mesh.nz), A)),
               fraction_gr_b=fgr, mask_grounded_ice=np.ascontiguousarray(grounded.astype(np.int32)),
               beta_sq=np.ascontiguousarray(beta_sq))
    return ice, mixed_ensemble_params()


def mixed_ensemble_params():
    """Solver parameters of the mixed-size DIVA ensemble (the same for every member)."""
    return abi.default_params(choice_sliding_law="Weertman", slid_Weertman_m=3.0,
                              visc_it_norm_dUV_tol=1e-4, stress_balance_PETSc_rtol=1e-8)


def mixed_ensemble_sizes(n=64, lo=20_000, hi=400_000, seed=18):
    """Vertex counts of the mixed-size ensemble: log-uniform in [lo, hi], seeded (seed 18: 8.10M
    vertices in all, the log-uniform mean of 127k per member)."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(int)
