"""Host-side mirror of UFEMISM's velocity-solve interfaces over the GB300 C ABI.

:class:`VelocitySolver` holds one device context with one mesh and its operators, and exposes the
reference's routine names with the reference's argument meaning:

* operator application -- ``map_a_b_2D/3D``, ``ddx_a_b_2D/3D``, ``ddy_a_b_2D/3D``,
  ``map_b_a_2D/3D``, ``ddx_b_a_2D/3D``, ``ddy_b_a_2D/3D``, ``ddx_a_a_2D``, ``ddy_a_a_2D``
  (src/UPSY/mesh/discretisation/mesh_disc_apply_operators.f90:18-431)
* ``multiply_CSR_matrix_with_vector_1D/2D``
  (src/UPSY/basic/CSR_matrix_algebra/CSR_matrix_vector_multiplication.f90:198-364)
* ``solve_matrix_equation_CSR_PETSc`` (src/UPSY/basic/petsc_basic.f90:32-64)
* ``solve_SSA_DIVA_linearised``
  (src/UFEMISM/ice_dynamics/conservation_of_momentum/SSA_DIVA/solve_linearised_SSA_DIVA.f90:23-178)
* ``solve_SSA`` (.../SSA_DIVA/SSA_main.f90:87-242) and ``solve_DIVA`` (.../DIVA_main.f90:88-262)
* ``calc_dHi_dt`` (src/UFEMISM/ice_dynamics/conservation_of_mass/conservation_of_mass_main.f90:23-109),
  after ``voronoi_upload`` of the mesh's cell areas and connection widths

Errors: a negative status raises :class:`UfeError` (the reference's ``crash``); positive statuses
are warnings (the reference's ``warning``) and are returned.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class UfeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ufe status {code}: {msg}")
        self.code = code


class CSR:
    """A CSR matrix in UFEMISM's layout (type_sparse_matrix_CSR_dp): ptr(m+1), ind, val, 1-based."""

    def __init__(self, m, n, ptr, ind, val, index_base=1):
        self.m, self.n = int(m), int(n)
        self.ptr = np.ascontiguousarray(ptr, dtype=np.int32)
        self.ind = np.ascontiguousarray(ind, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self.index_base = int(index_base)

    @property
    def nnz(self):
        return int(self.ind.size)

    @classmethod
    def from_scipy(cls, A):
        A = A.tocsr()
        return cls(A.shape[0], A.shape[1], A.indptr, A.indices, A.data, index_base=0)

    def to_scipy(self):
        import scipy.sparse as sp
        b = self.index_base
        return sp.csr_matrix((self.val, self.ind - b, self.ptr - b), shape=(self.m, self.n))


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class VelocitySolver:
    """GB300 velocity solve for one mesh.  ``operators`` (optional) installs caller-built
    operator matrices (dict name -> CSR) instead of building them on the GPU."""

    def __init__(self, mesh, device: int = 0, operators: dict | None = None):
        self.lib = abi.load_library()
        self.mesh = mesh
        ctx = C.c_void_p()
        rc = self.lib.ufe_ctx_create(device, C.byref(ctx))
        if rc != 0:
            raise UfeError(rc, "cannot create a context on a GB300 (sm_103) device")
        self.ctx = ctx
        desc, keep = abi.mesh_desc(mesh)
        self._check(self.lib.ufe_mesh_upload(self.ctx, C.byref(desc)))
        if operators:
            for name, A in operators.items():
                self.set_operator(name, A)
        else:
            self._check(self.lib.ufe_mesh_build_operators(self.ctx))

    # -- plumbing ----------------------------------------------------------------------------
    def close(self):
        for child in list(getattr(self, "_children", [])):   # networks created on this context first
            child.close()
        if getattr(self, "ctx", None):
            self.lib.ufe_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> int:
        if rc < 0:
            msg = self.lib.ufe_ctx_last_error(self.ctx)
            raise UfeError(rc, msg.decode() if msg else "")
        return rc

    def stream_handle(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.ufe_ctx_get_stream(self.ctx, C.byref(s)))
        return s.value or 0

    # -- operators ---------------------------------------------------------------------------
    def set_operator(self, name: str, A: CSR):
        self._check(self.lib.ufe_mesh_set_operator(self.ctx, abi.OP[name], A.m, A.n, A.nnz, abi.as_i(A.ptr),
                                                   abi.as_i(A.ind), abi.as_d(A.val), A.index_base))

    def operator(self, name: str, index_base: int = 1) -> CSR:
        op = abi.OP[name]
        m, n, nnz = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(self.lib.ufe_operator_info(self.ctx, op, C.byref(m), C.byref(n), C.byref(nnz)))
        ptr = np.zeros(m.value + 1, np.int32)
        ind = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value, np.float64)
        self._check(self.lib.ufe_operator_export(self.ctx, op, abi.as_i(ptr), abi.as_i(ind), abi.as_d(val), index_base))
        return CSR(m.value, n.value, ptr, ind, val, index_base)

    def apply(self, name: str, x):
        op = abi.OP[name]
        x = np.asfortranarray(x, dtype=np.float64)
        ncols = 1 if x.ndim == 1 else x.shape[1]
        m = C.c_int32()
        self._check(self.lib.ufe_operator_info(self.ctx, op, C.byref(m), None, None))
        y = np.zeros((m.value, ncols), order="F") if x.ndim == 2 else np.zeros(m.value)
        self._check(self.lib.ufe_apply_operator(self.ctx, op, abi.as_d(x), abi.as_d(y), ncols))
        return y

    def map_a_b_2D(self, d): return self.apply("MAP_A_B", d)
    def ddx_a_b_2D(self, d): return self.apply("DDX_A_B", d)
    def ddy_a_b_2D(self, d): return self.apply("DDY_A_B", d)
    def map_b_a_2D(self, d): return self.apply("MAP_B_A", d)
    def ddx_b_a_2D(self, d): return self.apply("DDX_B_A", d)
    def ddy_b_a_2D(self, d): return self.apply("DDY_B_A", d)
    def ddx_a_a_2D(self, d): return self.apply("DDX_A_A", d)
    def ddy_a_a_2D(self, d): return self.apply("DDY_A_A", d)
    map_a_b_3D = map_a_b_2D
    ddx_a_b_3D = ddx_a_b_2D
    ddy_a_b_3D = ddy_a_b_2D
    map_b_a_3D = map_b_a_2D
    ddx_b_a_3D = ddx_b_a_2D
    ddy_b_a_3D = ddy_b_a_2D

    # -- CSR algebra -------------------------------------------------------------------------
    def multiply_CSR_matrix_with_vector_1D(self, A: CSR, x):
        x = _d(x)
        y = np.zeros(A.m)
        self._check(self.lib.ufe_csr_spmv(self.ctx, A.m, A.n, A.nnz, abi.as_i(A.ptr), abi.as_i(A.ind),
                                          abi.as_d(A.val), A.index_base, abi.as_d(x), abi.as_d(y), 1))
        return y

    def multiply_CSR_matrix_with_vector_2D(self, A: CSR, x):
        x = np.asfortranarray(x, dtype=np.float64)
        y = np.zeros((A.m, x.shape[1]), order="F")
        self._check(self.lib.ufe_csr_spmv(self.ctx, A.m, A.n, A.nnz, abi.as_i(A.ptr), abi.as_i(A.ind),
                                          abi.as_d(A.val), A.index_base, abi.as_d(x), abi.as_d(y), x.shape[1]))
        return y

    def solve_matrix_equation_CSR_PETSc(self, A: CSR, bb, xx, rtol, abstol, max_it=10000):
        """Returns (solution, n_Axb_its, status); xx is the initial guess."""
        b = _d(bb)
        x = _d(xx).copy()
        its = C.c_int32()
        st = self._check(self.lib.ufe_solve_csr(self.ctx, A.m, A.nnz, abi.as_i(A.ptr), abi.as_i(A.ind),
                                                abi.as_d(A.val), A.index_base, abi.as_d(b), abi.as_d(x),
                                                rtol, abstol, max_it, C.byref(its)))
        return x, its.value, st

    # -- linearised SSA/DIVA -----------------------------------------------------------------
    def assemble_linearised(self, params, N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b,
                            u_prev=None, v_prev=None, BC=None):
        """The stiffness matrix and load vector in the reference's CSR layout."""
        nT = self.mesh.nTri
        args = [_d(a) for a in (N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b)]
        bc, keep = abi.bc_prescribed(BC)
        cap = 40 * 2 * nT
        ptr = np.zeros(2 * nT + 1, np.int32)
        ind = np.zeros(cap, np.int32)
        val = np.zeros(cap, np.float64)
        bb = np.zeros(2 * nT)
        nnz = C.c_int64()
        up = _d(u_prev) if u_prev is not None else None
        vp = _d(v_prev) if v_prev is not None else None
        self._check(self.lib.ufe_assemble_linearised(self.ctx, C.byref(params), *[abi.as_d(a) for a in args],
                                                     abi.as_d(up), abi.as_d(vp), C.byref(bc) if bc else None,
                                                     abi.as_i(ptr),
                                                     abi.as_i(ind), abi.as_d(val), abi.as_d(bb), cap, C.byref(nnz)))
        n = nnz.value
        return CSR(2 * nT, 2 * nT, ptr, ind[:n].copy(), val[:n].copy(), 1), bb

    def solve_SSA_DIVA_linearised(self, params, u_b, v_b, N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b,
                                  BC=None):
        """u_b, v_b are updated in place; returns (u_b_prev, v_b_prev, n_Axb_its, status)."""
        nT = self.mesh.nTri
        up, vp = np.zeros(nT), np.zeros(nT)
        args = [_d(a) for a in (N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b)]
        bc, keep = abi.bc_prescribed(BC)
        its = C.c_int32()
        st = self._check(self.lib.ufe_solve_linearised(self.ctx, C.byref(params), abi.as_d(u_b), abi.as_d(v_b),
                                                       *[abi.as_d(a) for a in args], abi.as_d(up), abi.as_d(vp),
                                                       C.byref(bc) if bc else None, C.byref(its)))
        return up, vp, its.value, st

    # -- full solves -------------------------------------------------------------------------
    def solve_SSA(self, ice: dict, SSA: dict, params, BC=None):
        """SSA = {'u_b', 'v_b'} updated in place; returns (n_visc_its, n_Axb_its, stats)."""
        st, keep = abi.ice_state(ice)
        bc, keep2 = abi.bc_prescribed(BC)
        nv, na = C.c_int32(), C.c_int32()
        stats = abi.SolveStats()
        self._check(self.lib.ufe_solve_ssa(self.ctx, C.byref(params), C.byref(st), C.byref(bc) if bc else None,
                                           abi.as_d(SSA["u_b"]), abi.as_d(SSA["v_b"]), C.byref(nv), C.byref(na),
                                           C.byref(stats)))
        return nv.value, na.value, stats.as_dict()

    def solve_DIVA(self, ice: dict, DIVA: dict, params, BC=None):
        """DIVA holds u_vav_b, v_vav_b, u_base_b, v_base_b, tau_bx_b, tau_by_b, eta_3D_b and
        optionally u_3D_b, v_3D_b (nTri x nz, Fortran order); updated in place."""
        st, keep = abi.ice_state(ice)
        bc, keep2 = abi.bc_prescribed(BC)
        ds = abi.DivaState(*[abi.as_d(DIVA.get(k)) for k in
                             ("u_vav_b", "v_vav_b", "u_base_b", "v_base_b", "tau_bx_b", "tau_by_b", "eta_3D_b",
                              "u_3D_b", "v_3D_b")])
        nv, na = C.c_int32(), C.c_int32()
        stats = abi.SolveStats()
        self._check(self.lib.ufe_solve_diva(self.ctx, C.byref(params), C.byref(st), C.byref(bc) if bc else None,
                                            C.byref(ds), C.byref(nv), C.byref(na), C.byref(stats)))
        return nv.value, na.value, stats.as_dict()

    # -- device-resident form (time stepping / benchmarking) ------------------------------------
    def ice_upload(self, ice: dict, BC=None):
        st, keep = abi.ice_state(ice)
        bc, keep2 = abi.bc_prescribed(BC)
        self._check(self.lib.ufe_ice_upload(self.ctx, C.byref(st), C.byref(bc) if bc else None))

    def solve_resident(self, params, diva: bool, cold_start: bool = True):
        stats = abi.SolveStats()
        fn = self.lib.ufe_solve_diva_resident if diva else self.lib.ufe_solve_ssa_resident
        self._check(fn(self.ctx, C.byref(params), 1 if cold_start else 0, C.byref(stats)))
        return stats.as_dict()

    def history(self):
        """Per-Picard-iteration rows (L2, Krylov its, Krylov status, final residual, refinements)."""
        out = np.zeros((128, 5))
        n = C.c_int32()
        self._check(self.lib.ufe_solve_history(self.ctx, abi.as_d(out), 128, C.byref(n)))
        return out[:n.value]

    def profile_krylov_kernels(self, precision: int, repeats: int = 50):
        """Mean device time [us] of the three BiCGStab kernels on the last assembled system,
        plus (block rows, stored 2x2 blocks)."""
        us = np.zeros(3)
        geo = (C.c_int64 * 2)()
        self._check(self.lib.ufe_profile_krylov_kernels(self.ctx, precision, repeats, abi.as_d(us), geo))
        return us, (geo[0], geo[1])

    def profile_krylov_persistent(self, precision: int, iterations: int = 200):
        """Microseconds per iteration of the persistent Krylov kernel on the last assembled system."""
        us = C.c_double()
        self._check(self.lib.ufe_profile_krylov_persistent(self.ctx, precision, iterations, C.byref(us)))
        return us.value

    def autotune(self, repeats: int = 20):
        """Pick the rows per warp of the Krylov kernels for this mesh (after a solve); returns
        (choice, microseconds per iteration for 1, 2, 4, 8)."""
        lanes = C.c_int32()
        us = np.zeros(4)
        self._check(self.lib.ufe_autotune(self.ctx, repeats, C.byref(lanes), abi.as_d(us)))
        return lanes.value, us

    def velocity_download(self):
        u, v = np.zeros(self.mesh.nTri), np.zeros(self.mesh.nTri)
        self._check(self.lib.ufe_velocity_download(self.ctx, abi.as_d(u), abi.as_d(v)))
        return u, v

    # -- thermodynamics on this mesh ---------------------------------------------------------
    # -- ice thickness (conservation of mass) -------------------------------------------------
    def voronoi_upload(self, A=None, Cw=None):
        """The mesh's Voronoi cell areas and connection widths (type_mesh's A and Cw); computed by
        mesh.voronoi_geometry when not given."""
        if A is None or Cw is None:
            from .mesh import voronoi_geometry
            A, Cw = voronoi_geometry(self.mesh)
        self._voronoi = (_d(A), np.asfortranarray(Cw, dtype=np.float64))
        self._check(self.lib.ufe_mesh_voronoi_upload(self.ctx, abi.as_d(self._voronoi[0]), abi.as_d(self._voronoi[1])))
        return self._voronoi

    def calc_dHi_dt(self, params, fields: dict, dt: float):
        """calc_dHi_dt: fields holds the inputs (Hi, Hb, SL, u_vav_b, v_vav_b and the optional SMB,
        BMB, LMB, fraction_margin, mask_noice, dHi_dt_target, BC_prescr_mask/Hi) and, when present,
        dHi_dt (the previous rate, the semi-implicit initial guess).  Returns a dict with dHi_dt,
        Hi_tplusdt, divQ, AMB, dt (the time step used) and the stats."""
        nV = self.mesh.nV
        f = {k: fields[k] for k in abi.THICKNESS_INPUTS if fields.get(k) is not None}
        for k in ("mask_noice", "BC_prescr_mask"):
            if k in f:
                f[k] = np.ascontiguousarray(f[k], dtype=np.int32)
        for k in f:
            if k not in ("mask_noice", "BC_prescr_mask"):
                f[k] = _d(f[k])
        prev = fields.get("dHi_dt")
        out = {"dHi_dt": _d(prev).copy() if prev is not None else np.zeros(nV),
               "Hi_tplusdt": np.zeros(nV), "divQ": np.zeros(nV), "AMB": np.zeros(nV)}
        f.update(out)
        tf, keep = abi.thickness_fields(f)
        d = C.c_double(dt)
        st = abi.ThicknessStats()
        self._check(self.lib.ufe_calc_dHi_dt(self.ctx, C.byref(params), C.byref(tf), C.byref(d), C.byref(st)))
        out["dt"] = d.value
        out["stats"] = st.as_dict()
        return out

    def thickness_assemble(self, params, fields: dict, dt: float):
        """The semi-implicit system before its solve: (ptr, ind, val) 0-based, load vector, initial guess."""
        nV = self.mesh.nV
        f = {k: fields[k] for k in abi.THICKNESS_INPUTS if fields.get(k) is not None}
        for k in list(f):
            f[k] = np.ascontiguousarray(f[k], dtype=np.int32 if k in ("mask_noice", "BC_prescr_mask") else np.float64)
        prev = fields.get("dHi_dt")
        f.update({"dHi_dt": _d(prev).copy() if prev is not None else np.zeros(nV), "Hi_tplusdt": np.zeros(nV),
                  "divQ": np.zeros(nV), "AMB": np.zeros(nV)})
        tf, keep = abi.thickness_fields(f)
        cap = int(nV + np.asarray(self.mesh.nC).sum())
        ptr, ind = np.zeros(nV + 1, np.int32), np.zeros(cap, np.int32)
        val, bb, x0 = np.zeros(cap), np.zeros(nV), np.zeros(nV)
        nnz = C.c_int64()
        self._check(self.lib.ufe_thickness_assemble(self.ctx, C.byref(params), C.byref(tf), dt, abi.as_i(ptr),
                                                    abi.as_i(ind), abi.as_d(val), abi.as_d(bb), abi.as_d(x0), cap,
                                                    C.byref(nnz)))
        return ptr, ind[:nnz.value], val[:nnz.value], bb, x0

    def solve_3D_heat_equation(self, fields: dict, params):
        """solve_3D_heat_equation (thermodynamics_3D_heat_equation.f90:33): the prelude and the
        column loop on the GPU; returns (Ti_next (nV, nz), n_unstable)."""
        f, keep = abi.heat_fields(fields)
        out = np.zeros((self.mesh.nV, self.mesh.nz), order="F")
        n = C.c_int32()
        self._check(self.lib.ufe_solve_3D_heat_equation(self.ctx, C.byref(params), C.byref(f), abi.as_d(out),
                                                        C.byref(n)))
        return out, n.value

    def heat_upload(self, fields: dict):
        f, keep = abi.heat_fields(fields)
        self._check(self.lib.ufe_heat_upload(self.ctx, C.byref(f)))

    def heat_step_resident(self, params, nsteps: int):
        """Advance the resident temperature nsteps steps; returns (n_unstable_total, device_ms)."""
        n, ms = C.c_int32(), C.c_double()
        self._check(self.lib.ufe_heat_step_resident(self.ctx, C.byref(params), nsteps, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def profile_heat_kernels(self, params, repeats: int = 20):
        """Mean device time [us] of the column, retry, Robin and bookkeeping kernels of one step on
        the resident state, plus (columns with ice, columns without)."""
        us = np.zeros(4)
        counts = (C.c_int64 * 2)()
        self._check(self.lib.ufe_profile_heat_kernels(self.ctx, C.byref(params), repeats, abi.as_d(us), counts))
        return us, (counts[0], counts[1])

    def heat_download(self):
        out = np.zeros((self.mesh.nV, self.mesh.nz), order="F")
        self._check(self.lib.ufe_heat_download(self.ctx, abi.as_d(out)))
        return out


def new_ssa_state(nTri):
    return {"u_b": np.zeros(nTri), "v_b": np.zeros(nTri)}


def new_diva_state(nTri, nz, with_3d=True):
    d = {k: np.zeros(nTri) for k in ("u_vav_b", "v_vav_b", "u_base_b", "v_base_b", "tau_bx_b", "tau_by_b")}
    d["eta_3D_b"] = np.zeros((nTri, nz), order="F")
    if with_3d:
        d["u_3D_b"] = np.zeros((nTri, nz), order="F")
        d["v_3D_b"] = np.zeros((nTri, nz), order="F")
    return d


def ensemble_solve(solvers, params, diva: bool, cold_start: bool = True):
    """ufe_ensemble_solve over VelocitySolvers with their ice states uploaded; returns
    (list of stats dicts, wall milliseconds).  A negative status raises UfeError."""
    lib = abi.load_library()
    n = len(solvers)
    arr = (C.c_void_p * n)(*[sv.ctx.value for sv in solvers])
    stats = (abi.SolveStats * n)()
    wall = C.c_double()
    rc = lib.ufe_ensemble_solve(arr, n, C.byref(params), 1 if diva else 0, 1 if cold_start else 0, stats,
                                C.byref(wall))
    if rc < 0:
        msgs = [(lib.ufe_ctx_last_error(sv.ctx) or b"").decode() for sv in solvers]
        raise UfeError(rc, "; ".join(m for m in msgs if m))
    return [st.as_dict() for st in stats], wall.value
