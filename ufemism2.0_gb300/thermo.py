"""Host-side mirror of UFEMISM's thermodynamics column solve over the GB300 C ABI.

* :class:`ColumnSolver` -- a device context without a mesh: ``thermo_step`` runs the column loop
  of ``solve_3D_heat_equation`` (src/UFEMISM/thermodynamics/thermodynamics_3D_heat_equation.f90:
  131-292) on precomputed per-column inputs, and ``solve_tridiagonal_matrix_equation``
  (src/UPSY/basic/math_utilities/tridiagonal_solver.f90:13-51) solves a batch of tridiagonal
  systems.
* :func:`zeta_operators` -- the tridiagonal d/dzeta, d2/dzeta2 operators
  (src/UPSY/mesh/mesh_zeta.f90:288-366, 487-605).
* The mesh-level ``solve_3D_heat_equation(fields, params)`` and its resident form
  (``heat_upload`` / ``heat_step_resident`` / ``heat_download``) are methods of
  :class:`VelocitySolver`, which owns the mesh and its operators.

Arrays of shape (nV, nz) are passed column-major (layer k of vertex vi at k*nV + vi), as the
reference stores ice%Ti(vi,k).  A negative status raises :class:`UfeError` (the reference's
``crash``, e.g. more than 1 % of the columns unstable).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .solver import UfeError


def zeta_operators(zeta):
    """(ddz_l, ddz_d, ddz_u, d2_l, d2_d, d2_u), each of length nz, indexed by row."""
    lib = abi.load_library()
    zeta = np.ascontiguousarray(zeta, dtype=np.float64)
    nz = zeta.size
    out = [np.zeros(nz) for _ in range(6)]
    rc = lib.ufe_zeta_operators(nz, abi.as_d(zeta), *[abi.as_d(o) for o in out])
    if rc != 0:
        raise UfeError(rc, "zeta operators: need 3 <= nz <= 256 distinct zeta values")
    return tuple(out)


class ColumnSolver:
    """GB300 column solves without a mesh (one device context)."""

    def __init__(self, device: int = 0):
        self.lib = abi.load_library()
        ctx = C.c_void_p()
        rc = self.lib.ufe_ctx_create(device, C.byref(ctx))
        if rc != 0:
            raise UfeError(rc, "cannot create a context on a GB300 (sm_103) device")
        self.ctx = ctx

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

    def thermo_step(self, params, zeta, cols: dict):
        """One step for all columns; returns (Ti_next (nV, nz), n_unstable)."""
        zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        Ti = np.asarray(cols["Ti"])
        nV, nz = Ti.shape
        st, keep = abi.thermo_columns(cols)
        out = np.zeros((nV, nz), order="F")
        n = C.c_int32()
        self._check(self.lib.ufe_thermo_step(self.ctx, C.byref(params), nV, nz, abi.as_d(zeta), C.byref(st),
                                             abi.as_d(out), C.byref(n)))
        return out, n.value

    def solve_tridiagonal_matrix_equation(self, a, b, c, d):
        """Batched Thomas solve: arrays (n,) or (n, nsys), system j in column j; returns x."""
        arrs = [np.asfortranarray(v, dtype=np.float64) for v in (a, b, c, d)]
        n = arrs[0].shape[0]
        nsys = 1 if arrs[0].ndim == 1 else arrs[0].shape[1]
        x = np.zeros_like(arrs[1], order="F")
        self._check(self.lib.ufe_tridiagonal_solve(self.ctx, n, nsys, *[abi.as_d(v) for v in arrs], abi.as_d(x)))
        return x
