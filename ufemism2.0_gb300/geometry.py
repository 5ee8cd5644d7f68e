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


# -- config 0: SSA dome ------------------------------------------------------------------------
def dome_thickness(x, y, H0=3000.0, R=500e3):
    r = np.hypot(x, y)
    s = np.clip(1.0 - (r / R) ** (4.0 / 3.0), 0.0, None)
    return np.where(r < R, H0 * s ** (3.0 / 7.0), 0.0)


def dome_resolution(band=140e3, ramp=200e3, fine=10e3, coarse=40e3, R=500e3):
    def res(x, y):
        r = np.hypot(x, y)
        return fine + (coarse - fine) * np.clip((np.abs(r - R) - band) / ramp, 0.0, 1.0)
    return res


def dome_case(seed=0, nz=12, L=800e3, res_scale=1.0, A=1e-16, beta_sq=1e4):
    """Config 0 (or a coarser copy with res_scale > 1 for quick tests)."""
    res = dome_resolution(band=140e3 * min(res_scale, 1.0) if res_scale < 1 else 140e3,
                          fine=10e3 * res_scale, coarse=40e3 * res_scale)
    mesh = generate_mesh(-L / 2, L / 2, -L / 2, L / 2, res, seed=seed, nz=nz)
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    Hi = np.ascontiguousarray(dome_thickness(x, y))
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


# -- config 1: DIVA channel --------------------------------------------------------------------
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
    """Config 1 (or a coarser copy with res_scale > 1)."""
    res = channel_resolution(H=H, fine=0.9e3 * res_scale, coarse=1.35e3 * res_scale)
    mesh = generate_mesh(0.0, 640e3, -40e3, 40e3, res, seed=seed, nz=nz)
    x, y = mesh.V[:, 0], mesh.V[:, 1]
    Hb = mismip_bed(x, y)
    SL = np.zeros(mesh.nV)
    Hi = np.full(mesh.nV, H)
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


def small_dome(seed=0, nz=12):
    """A ~1,000-vertex dome for tests the CPU oracle finishes in seconds."""
    return dome_case(seed=seed, nz=nz, res_scale=3.0)


def small_channel(seed=0, nz=8, sliding="Schoof2005"):
    """A ~2,000-vertex channel for DIVA tests."""
    return channel_case(seed=seed, nz=nz, res_scale=6.5, sliding=sliding)
