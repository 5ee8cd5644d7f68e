"""The persistent Krylov kernel's two-reduction form of BiCGStab against PETSc's three-reduction
KSPBCGS recurrence (Jacobi, left preconditioned), both written out in numpy FP64 on the same
system: the same iterates, iteration count and solution.

The two-reduction form takes rho_{k+1} = (s, r^) - omega (t, r^) and
|r_{k+1}|^2 = (s, s) - omega (2 (s, t) - omega (t, t)) from the s-phase reduction and applies the
x/r update of iteration k while staging p for iteration k+1 (k_bicgstab_halo in
ufemism2.0_gb300/csrc/ufe_krylov.cuh); only rounding separates it from the direct form.
"""
import numpy as np
import pytest


def _system(n, seed):
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for i in range(n):   # a banded, non-symmetric operator with a dominant diagonal
        for j in range(max(0, i - 3), min(n, i + 4)):
            A[i, j] = rng.normal()
        A[i, i] = 4.0 + abs(rng.normal())
    b = rng.normal(size=n)
    return A, b


def _init(A, b, x0, rtol, abstol, max_it):
    d = 1.0 / np.diag(A)
    r = d * (b - A @ x0)
    rnorm0 = np.linalg.norm(d * b)
    st = dict(rho=r @ r, alpha=1.0, omega=1.0, omegaold=1.0, beta=r @ r, it=0,
              ttol=max(rtol * rnorm0, abstol), rnorm0=rnorm0, max_it=max_it, dp=np.linalg.norm(r))
    return d, r, st


def bcgs_three(A, b, x0, rtol=1e-10, abstol=0.0, max_it=500):
    """PETSc's recurrence: three reductions per iteration (v,r^); (s,t),(t,t); (r,r^),(r,r)."""
    d, r, st = _init(A, b, x0, rtol, abstol, max_it)
    x, rp = x0.copy(), r.copy()
    p = np.zeros_like(b)
    v = np.zeros_like(b)
    hist = []
    while True:
        p = r - st["beta"] * st["omegaold"] * v + st["beta"] * p
        v = d * (A @ p)
        st["alpha"] = st["rho"] / (v @ rp)
        s = r - st["alpha"] * v
        t = d * (A @ s)
        st["omega"] = (s @ t) / (t @ t)
        x = x + st["alpha"] * p + st["omega"] * s
        r = s - st["omega"] * t
        rho_new = r @ rp
        dp = np.linalg.norm(r)
        st["it"] += 1
        hist.append(dp)
        st["omegaold"] = st["omega"]
        if dp <= st["ttol"] or st["it"] >= st["max_it"]:
            return x, st["it"], np.array(hist)
        st["beta"] = (rho_new / st["rho"]) * (st["alpha"] / st["omega"])
        st["rho"] = rho_new


def bcgs_two(A, b, x0, rtol=1e-10, abstol=0.0, max_it=500):
    """The kernel's form: two reductions per iteration, the x/r update deferred into the next p."""
    d, r0, st = _init(A, b, x0, rtol, abstol, max_it)
    x, rp, R = x0.copy(), r0.copy(), r0.copy()
    P = np.zeros_like(b)
    V = np.zeros_like(b)
    S = T = None
    pending, finish = False, False
    ap = wp = 0.0
    hist = []
    while True:
        # p staging (+ the previous iteration's x/r update)
        if pending:
            r = S - wp * T
            x = x + ap * P + wp * S
            R = r
        pn = R - st["beta"] * st["omegaold"] * V + st["beta"] * P
        finish = False
        P = pn
        V = d * (A @ P)
        st["alpha"] = st["rho"] / (V @ rp)
        # s phase with five dot products
        S = R - st["alpha"] * V
        T = d * (A @ S)
        st_, tt, ss, sr, tr = S @ T, T @ T, S @ S, S @ rp, T @ rp
        w = st_ / tt
        finish = True
        st["it"] += 1
        rho_new = sr - w * tr
        dp = np.sqrt(max(ss - w * (2.0 * st_ - w * tt), 0.0))
        hist.append(dp)
        st["omegaold"] = w
        ap, wp = st["alpha"], w
        if dp <= st["ttol"] or st["it"] >= st["max_it"]:
            break
        st["beta"] = (rho_new / st["rho"]) * (st["alpha"] / w)
        st["rho"] = rho_new
        pending = True
    if finish:
        x = x + ap * P + wp * S
    return x, st["it"], np.array(hist)


@pytest.mark.parametrize("n,seed", [(60, 1), (200, 2), (400, 3)])
def test_two_reduction_form_matches_petsc_recurrence(n, seed):
    A, b = _system(n, seed)
    x0 = np.zeros(n)
    x3, it3, h3 = bcgs_three(A, b, x0)
    x2, it2, h2 = bcgs_two(A, b, x0)
    assert it2 == it3
    np.testing.assert_allclose(h2, h3, rtol=1e-6, atol=1e-13 * h3[0])
    xe = np.linalg.solve(A, b)
    assert np.linalg.norm(x2 - x3) <= 1e-10 * np.linalg.norm(xe)
    assert np.linalg.norm(x2 - xe) <= 1e-8 * np.linalg.norm(xe)


def test_two_reduction_form_from_a_warm_start():
    A, b = _system(150, 7)
    xe = np.linalg.solve(A, b)
    x0 = xe + 1e-3 * np.random.default_rng(8).normal(size=150)
    x3, it3, _ = bcgs_three(A, b, x0, rtol=1e-12)
    x2, it2, _ = bcgs_two(A, b, x0, rtol=1e-12)
    assert it2 == it3
    assert np.linalg.norm(x2 - xe) <= 1e-9 * np.linalg.norm(xe)
