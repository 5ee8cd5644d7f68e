"""Learned Picard start: a mesh-graph network that predicts the velocity and the effective viscosity
an SSA/DIVA solve starts from, trained on solutions the plain GPU solver generates
(include/ufe_gpu.h, ufe_gnn_*).

Every solve still iterates to its own Picard tolerance; the network only replaces the zero (cold)
or previous-step start, so a poor prediction costs iterations, never accuracy.

    net = LearnedStart(solver)              # on the solver's GPU context
    for member in training_members:
        solver.ice_upload(ice)
        x = net.features(solver)            # before the solve: previous velocity = 0
        solver.solve_resident(params, diva=False)
        net.dataset_add(solver, x)          # features + the converged velocity as the target
    net.train(epochs=60, lr=1e-3)
    solver.ice_upload(new_ice)
    net.predict(solver, viscosity=True)     # resident velocity (and first viscosity) <- prediction
    solver.solve_resident(params, diva=False, cold_start=False)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .solver import UfeError

FEATURES = 16
OUTPUTS = 3        # u / 1e3, v / 1e3 (m/yr), (log10(eta_vav) - 7.5) / 2 (Pa yr)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class LearnedStart:
    """The network, on the GPU context of `solver` (a VelocitySolver or ColumnSolver)."""

    def __init__(self, solver, seed: int = 0):
        self.lib = abi.load_library()
        self.solver = solver
        h = C.c_void_p()
        rc = self.lib.ufe_gnn_create(solver.ctx, seed, C.byref(h))
        if rc != 0:
            raise UfeError(rc, (self.lib.ufe_ctx_last_error(solver.ctx) or b"").decode())
        self.h = h
        self.nparams = self.lib.ufe_gnn_param_count()
        if not hasattr(solver, "_children"):
            solver._children = []
        solver._children.append(self)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ufe_gnn_destroy(self.h)
            self.h = None
            try:
                self.solver._children.remove(self)
            except (AttributeError, ValueError):
                pass

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc < 0:
            msg = self.lib.ufe_ctx_last_error(self.solver.ctx)
            raise UfeError(rc, msg.decode() if msg else "")
        return rc

    # -- parameters --------------------------------------------------------------------------
    def get_params(self):
        p = np.zeros(self.nparams, np.float32)
        self._check(self.lib.ufe_gnn_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = _f(p)
        assert p.size == self.nparams
        self._check(self.lib.ufe_gnn_set_params(self.h, _fp(p)))

    # -- explicit graphs ---------------------------------------------------------------------
    def forward(self, nbr, x):
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        x = _f(x)
        y = np.zeros((x.shape[0], OUTPUTS), np.float32)
        self._check(self.lib.ufe_gnn_forward(self.h, x.shape[0], abi.as_i(nbr), _fp(x), _fp(y)))
        return y

    def loss_grad(self, nbr, x, target, w):
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        x, target, w = _f(x), _f(target), _f(w)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_double()
        self._check(self.lib.ufe_gnn_loss_grad(self.h, x.shape[0], abi.as_i(nbr), _fp(x), _fp(target), _fp(w),
                                               C.byref(loss), _fp(g)))
        return loss.value, g

    # -- the mesh path -----------------------------------------------------------------------
    def features(self, solver, use_prev_velocity: bool = False):
        x = np.zeros((solver.mesh.nTri, FEATURES), np.float32)
        self._check(self.lib.ufe_gnn_features(self.h, solver.ctx, 1 if use_prev_velocity else 0, _fp(x)))
        return x

    def dataset_add(self, solver, features_before=None):
        fb = None if features_before is None else _f(features_before)
        return self._check(self.lib.ufe_gnn_dataset_add(self.h, solver.ctx, None if fb is None else _fp(fb)))

    def dataset_clear(self):
        self._check(self.lib.ufe_gnn_dataset_clear(self.h))

    def train(self, epochs: int, lr: float = 1e-3, seed: int = 0):
        """Returns (mean training loss per epoch, device milliseconds)."""
        losses = np.zeros(max(epochs, 1), np.float32)
        ms = C.c_double()
        self._check(self.lib.ufe_gnn_train(self.h, epochs, lr, seed, _fp(losses), C.byref(ms)))
        return losses[:epochs], ms.value

    def evaluate(self):
        l = C.c_double()
        self._check(self.lib.ufe_gnn_evaluate(self.h, C.byref(l)))
        return l.value

    def predict(self, solver, use_prev_velocity: bool = False, smooth_passes: int = 0, viscosity: bool = False):
        """Store the predicted velocity as the solver's resident velocity and, with `viscosity`, the
        predicted viscosity for the next solve's first Picard iteration; returns device ms."""
        ms = C.c_double()
        self._check(self.lib.ufe_gnn_predict_start(self.h, solver.ctx, 1 if use_prev_velocity else 0,
                                                   smooth_passes, 1 if viscosity else 0, C.byref(ms)))
        return ms.value
