"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates UFEMISM's velocity-solve routines in C (oracle/ufe_oracle.c).  Tests, the
smoke check and the benchmark's CPU-baseline leg compare the GPU results with it; the product
never imports this module.  :class:`Oracle` mirrors the method names of the product's ``VelocitySolver``.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libufe_oracle.so")


def _pkg():
    if "ufemism_gb300" in sys.modules:
        return sys.modules["ufemism_gb300"]
    d = os.path.join(ROOT, "ufemism2.0_gb300")
    spec = importlib.util.spec_from_file_location("ufemism_gb300", os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ufemism_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def build():
    """Compile the oracle (make, gcc) into oracle/_build/."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    abi = _pkg().abi
    lib = C.CDLL(LIB)
    dp, ip, vp = abi.dptr, abi.iptr, C.c_void_p
    sig = {
        "orc_ops_create": (vp, [C.POINTER(abi.MeshDesc), ip]),
        "orc_ops_destroy": (None, [vp]),
        "orc_ops_info": (C.c_int32, [vp, C.c_int32, ip, ip, C.POINTER(C.c_int64)]),
        "orc_ops_export": (C.c_int32, [vp, C.c_int32, ip, ip, dp]),
        "orc_ops_apply": (C.c_int32, [vp, C.c_int32, dp, dp, C.c_int32]),
        "orc_ops_solve_ssa": (C.c_int32, [vp, C.POINTER(abi.SolverParams), C.POINTER(abi.IceState),
                                          C.POINTER(abi.BCPrescribed), dp, dp, C.POINTER(abi.SolveStats)]),
        "orc_ops_solve_diva": (C.c_int32, [vp, C.POINTER(abi.SolverParams), C.POINTER(abi.IceState),
                                           C.POINTER(abi.BCPrescribed), C.POINTER(abi.DivaState),
                                           C.POINTER(abi.SolveStats)]),
        "orc_ops_set_first_viscosity": (C.c_int32, [vp, dp]),
        "orc_ops_calc_dHi_dt": (C.c_int32, [vp, dp, dp, C.POINTER(abi.ThicknessParams),
                                            C.POINTER(abi.ThicknessFields), dp, C.POINTER(abi.ThicknessStats)]),
        "orc_ops_thickness_assemble": (C.c_int32, [vp, dp, dp, C.POINTER(abi.ThicknessParams),
                                                   C.POINTER(abi.ThicknessFields), C.c_double, ip, ip, dp, dp, dp,
                                                   C.c_int64, C.POINTER(C.c_int64)]),
        "orc_ops_assemble": (C.c_int32, [vp, C.POINTER(abi.SolverParams), dp, dp, dp, dp, dp, dp, dp, dp,
                                         C.POINTER(abi.BCPrescribed), ip, ip, dp, dp, C.c_int64,
                                         C.POINTER(C.c_int64)]),
        "orc_csr_solve": (C.c_int32, [C.c_int32, C.c_int64, ip, ip, dp, dp, dp, C.c_double, C.c_double,
                                      C.c_int32, ip]),
        "orc_csr_spmv": (C.c_int32, [C.c_int32, C.c_int32, C.c_int64, ip, ip, dp, dp, dp, C.c_int32]),
        "orc_zeta_operators": (C.c_int32, [C.c_int32, dp, dp, dp, dp, dp, dp, dp]),
        "orc_tridiagonal_batched": (C.c_int32, [C.c_int32, C.c_int32, dp, dp, dp, dp, dp]),
        "orc_thermo_step": (C.c_int32, [C.POINTER(abi.ThermoParams), C.c_int32, C.c_int32, dp,
                                        C.POINTER(abi.ThermoColumns), dp, ip, ip]),
        "orc_ops_solve_3D_heat_equation": (C.c_int32, [vp, C.POINTER(abi.ThermoParams), C.POINTER(abi.HeatFields),
                                                       dp, ip, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"oracle status {code} {msg}")
        self.code = code


def _one_based(A):
    """(ptr, ind, val) of a CSR-like object, converted to 1-based int32/float64 arrays."""
    b = getattr(A, "index_base", 1)
    ptr = np.ascontiguousarray(A.ptr, dtype=np.int32) + (1 - b)
    ind = np.ascontiguousarray(A.ind, dtype=np.int32) + (1 - b)
    return ptr.astype(np.int32), ind.astype(np.int32), _d(A.val)


def csr_spmv(A, x):
    """multiply_CSR_matrix_with_vector_1D/2D on a 1-based CSR."""
    lib = load()
    abi = _pkg().abi
    ptr, ind, val = _one_based(A)
    x = np.asfortranarray(x, dtype=np.float64)
    ncols = 1 if x.ndim == 1 else x.shape[1]
    y = np.zeros((A.m, ncols), order="F") if x.ndim == 2 else np.zeros(A.m)
    lib.orc_csr_spmv(A.m, A.n, ind.size, abi.as_i(ptr), abi.as_i(ind), abi.as_d(val), abi.as_d(x), abi.as_d(y), ncols)
    return y


def csr_solve(A, b, x0, rtol, abstol, max_it=10000):
    """BiCGStab/Jacobi in PETSc's KSPBCGS form; returns (x, its, status)."""
    lib = load()
    abi = _pkg().abi
    ptr, ind, val = _one_based(A)
    b = _d(b)
    x = _d(x0).copy()
    its = C.c_int32()
    st = lib.orc_csr_solve(A.m, ind.size, abi.as_i(ptr), abi.as_i(ind), abi.as_d(val), abi.as_d(b), abi.as_d(x),
                           rtol, abstol, max_it, C.byref(its))
    return x, its.value, st


class Oracle:
    """CPU restatement for one mesh; same method names as the product's VelocitySolver."""

    def __init__(self, mesh):
        self.lib = load()
        self.abi = _pkg().abi
        self.mesh = mesh
        self._desc, self._keep = self.abi.mesh_desc(mesh)
        st = C.c_int32()
        self.h = self.lib.orc_ops_create(C.byref(self._desc), C.byref(st))
        if not self.h:
            raise OracleError(st.value, "operator construction failed")

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_ops_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def operator(self, name):
        CSR = _pkg().CSR
        op = self.abi.OP[name]
        m, n, nnz = C.c_int32(), C.c_int32(), C.c_int64()
        self.lib.orc_ops_info(self.h, op, C.byref(m), C.byref(n), C.byref(nnz))
        ptr = np.zeros(m.value + 1, np.int32)
        ind = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        self.lib.orc_ops_export(self.h, op, self.abi.as_i(ptr), self.abi.as_i(ind), self.abi.as_d(val))
        return CSR(m.value, n.value, ptr, ind, val, 1)

    def operators(self):
        return {name: self.operator(name) for name in self.abi.OPERATORS}

    def apply(self, name, x):
        A = self.operator(name)
        return csr_spmv(A, x)

    def assemble_linearised(self, params, N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b, u_prev=None,
                            v_prev=None, BC=None):
        CSR = _pkg().CSR
        nT = self.mesh.nTri
        args = [_d(a) for a in (N_b, dN_dx_b, dN_dy_b, beta_b, tau_dx_b, tau_dy_b)]
        up = _d(u_prev if u_prev is not None else np.zeros(nT))
        vp = _d(v_prev if v_prev is not None else np.zeros(nT))
        bc, keep = self.abi.bc_prescribed(BC)
        cap = 40 * 2 * nT
        ptr = np.zeros(2 * nT + 1, np.int32)
        ind = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        bb = np.zeros(2 * nT)
        nnz = C.c_int64()
        rc = self.lib.orc_ops_assemble(self.h, C.byref(params), *[self.abi.as_d(a) for a in args], self.abi.as_d(up),
                                       self.abi.as_d(vp), C.byref(bc) if bc else None, self.abi.as_i(ptr),
                                       self.abi.as_i(ind), self.abi.as_d(val), self.abi.as_d(bb), cap, C.byref(nnz))
        if rc < 0:
            raise OracleError(rc)
        n = nnz.value
        return CSR(2 * nT, 2 * nT, ptr, ind[:n].copy(), val[:n].copy(), 1), bb

    def set_first_viscosity(self, eta_a=None):
        """Viscosity per vertex for the first Picard iteration of the next solve (the learned
        start's prediction; no reference counterpart), or None to clear it."""
        arr = None if eta_a is None else np.ascontiguousarray(eta_a, dtype=np.float64)
        rc = self.lib.orc_ops_set_first_viscosity(self.h, None if arr is None else self.abi.as_d(arr))
        if rc < 0:
            raise OracleError(rc)

    def calc_dHi_dt(self, A, Cw, params, fields: dict, dt: float):
        """orc_ops_calc_dHi_dt: fills the output arrays of `fields` (dHi_dt, Hi_tplusdt, divQ, AMB;
        dHi_dt holds the previous rate on entry); returns (dt, stats)."""
        f, keep = self.abi.thickness_fields(fields)
        A, Cw = np.ascontiguousarray(A, np.float64), np.asfortranarray(Cw, np.float64)
        d = C.c_double(dt)
        st = self.abi.ThicknessStats()
        rc = self.lib.orc_ops_calc_dHi_dt(self.h, self.abi.as_d(A), self.abi.as_d(Cw), C.byref(params), C.byref(f),
                                          C.byref(d), C.byref(st))
        if rc < 0:
            raise OracleError(rc)
        return d.value, st.as_dict()

    def thickness_assemble(self, A, Cw, params, fields: dict, dt: float):
        """The semi-implicit system (0-based CSR, load vector, initial guess) before its solve."""
        f, keep = self.abi.thickness_fields(fields)
        A, Cw = np.ascontiguousarray(A, np.float64), np.asfortranarray(Cw, np.float64)
        nV = self.mesh.nV
        cap = int(nV + self.mesh.nC.sum())
        ptr, ind = np.zeros(nV + 1, np.int32), np.zeros(cap, np.int32)
        val, bb, x0 = np.zeros(cap), np.zeros(nV), np.zeros(nV)
        nnz = C.c_int64()
        rc = self.lib.orc_ops_thickness_assemble(self.h, self.abi.as_d(A), self.abi.as_d(Cw), C.byref(params),
                                                 C.byref(f), dt, self.abi.as_i(ptr), self.abi.as_i(ind),
                                                 self.abi.as_d(val), self.abi.as_d(bb), self.abi.as_d(x0), cap,
                                                 C.byref(nnz))
        if rc < 0:
            raise OracleError(rc)
        return ptr, ind[:nnz.value], val[:nnz.value], bb, x0

    def solve_SSA(self, ice, SSA, params, BC=None):
        st, keep = self.abi.ice_state(ice)
        bc, keep2 = self.abi.bc_prescribed(BC)
        stats = self.abi.SolveStats()
        rc = self.lib.orc_ops_solve_ssa(self.h, C.byref(params), C.byref(st), C.byref(bc) if bc else None,
                                        self.abi.as_d(SSA["u_b"]), self.abi.as_d(SSA["v_b"]), C.byref(stats))
        if rc < 0:
            raise OracleError(rc)
        return stats.n_visc_its, stats.n_Axb_its, stats.as_dict()

    def solve_DIVA(self, ice, DIVA, params, BC=None):
        st, keep = self.abi.ice_state(ice)
        bc, keep2 = self.abi.bc_prescribed(BC)
        ds = self.abi.DivaState(*[self.abi.as_d(DIVA.get(k)) for k in
                                  ("u_vav_b", "v_vav_b", "u_base_b", "v_base_b", "tau_bx_b", "tau_by_b",
                                   "eta_3D_b", "u_3D_b", "v_3D_b")])
        stats = self.abi.SolveStats()
        rc = self.lib.orc_ops_solve_diva(self.h, C.byref(params), C.byref(st), C.byref(bc) if bc else None,
                                         C.byref(ds), C.byref(stats))
        if rc < 0:
            raise OracleError(rc)
        return stats.n_visc_its, stats.n_Axb_its, stats.as_dict()

    def solve_3D_heat_equation(self, fields: dict, params):
        """orc_ops_solve_3D_heat_equation on this mesh: (Ti_next, n_unstable, status, flags)."""
        f, keep = self.abi.heat_fields(fields)
        out = np.zeros((self.mesh.nV, self.mesh.nz), order="F")
        n = C.c_int32()
        flags = np.zeros(self.mesh.nV, np.int32)
        rc = self.lib.orc_ops_solve_3D_heat_equation(self.h, C.byref(params), C.byref(f), self.abi.as_d(out),
                                                     C.byref(n), self.abi.as_i(flags))
        return out, n.value, rc, flags


# -- thermodynamics ------------------------------------------------------------------------------
def zeta_operators(zeta):
    """orc_zeta_operators: (ddz_l, ddz_d, ddz_u, d2_l, d2_d, d2_u) indexed by row."""
    lib = load()
    zeta = _d(zeta)
    out = [np.zeros(zeta.size) for _ in range(6)]
    rc = lib.orc_zeta_operators(zeta.size, zeta.ctypes.data_as(_pkg().abi.dptr),
                                *[o.ctypes.data_as(_pkg().abi.dptr) for o in out])
    if rc != 0:
        raise OracleError(rc, "zeta operators")
    return tuple(out)


def tridiagonal(a, b, c, d):
    """solve_tridiagonal_matrix_equation for each column of the (n, nsys) arrays."""
    lib = load()
    abi = _pkg().abi
    arrs = [np.asfortranarray(v, dtype=np.float64) for v in (a, b, c, d)]
    n = arrs[0].shape[0]
    nsys = 1 if arrs[0].ndim == 1 else arrs[0].shape[1]
    x = np.zeros_like(arrs[1], order="F")
    rc = lib.orc_tridiagonal_batched(n, nsys, *[v.ctypes.data_as(abi.dptr) for v in arrs], x.ctypes.data_as(abi.dptr))
    if rc != 0:
        raise OracleError(rc, "tridiagonal")
    return x


def thermo_step(params, zeta, cols: dict):
    """orc_thermo_step: returns (Ti_next, n_unstable, status, flags); flags per column are
    0 stable, 2 stable after dt halving, 1 unstable (Robin profile)."""
    lib = load()
    abi = _pkg().abi
    zeta = _d(zeta)
    nV, nz = np.asarray(cols["Ti"]).shape
    st, keep = abi.thermo_columns(cols)
    out = np.zeros((nV, nz), order="F")
    n = C.c_int32()
    flags = np.zeros(nV, np.int32)
    rc = lib.orc_thermo_step(C.byref(params), nV, nz, zeta.ctypes.data_as(abi.dptr), C.byref(st),
                             out.ctypes.data_as(abi.dptr), C.byref(n), flags.ctypes.data_as(abi.iptr))
    return out, n.value, rc, flags
