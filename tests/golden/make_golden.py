"""Regenerate the golden fixtures of this directory.

kats.json
    Known-answer tests of UFEMISM's own unit tests for the CSR path, transcribed as data:
    * spmv_6x6   src/UPSY/validation/unit_tests/ut_petsc.f90:83-150
    * spmv_7x7_1 src/UPSY/validation/unit_tests/ut_mpi_CSR_matrix_vector_multiplication.f90:180-246
    * spmv_7x7_2 same file :248-321
    * poisson_7  src/UPSY/validation/unit_tests/ut_mpi_CSR_matrix_solving.f90:193-273
      (checked there to 1e-5 after the solve, :105-114)
    Matrices are 1-based CSR in add_entry order.

small_dome.npz
    A ~740-vertex dome mesh (seed 0), the oracle's 13 operators on it, and the oracle's SSA solve
    (Weertman, Krylov rtol 1e-12 and abstol 0, 10 Picard iterations), so GPU tests on another host compare
    against the same mesh and numbers.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def csr_from_entries(m, entries):
    """entries: list of (row, col, val) 1-based in append order -> (ptr, ind, val) 1-based."""
    ptr = [1] * (m + 1)
    ind, val = [], []
    for r in range(1, m + 1):
        for (i, j, v) in entries:
            if i == r:
                ind.append(j)
                val.append(v)
        ptr[r] = len(ind) + 1
    return ptr, ind, val


def kats():
    out = {}
    e = [(1, 1, 1.0), (2, 1, 2.0), (2, 2, 3.0), (3, 2, 4.0), (3, 4, 5.0), (4, 4, 6.0), (4, 5, 7.0),
         (5, 5, 8.0), (6, 5, 9.0), (6, 6, 10.0)]
    ptr, ind, val = csr_from_entries(6, e)
    out["spmv_6x6"] = dict(m=6, n=6, ptr=ptr, ind=ind, val=val, x=[1, 2, 3, 4, 5, 6],
                           y=[1, 8, 28, 59, 40, 105])
    e = [(1, 1, 1.0), (2, 2, 2.0), (2, 3, 3.0), (3, 2, 4.0), (3, 5, 1.0), (4, 3, 2.0), (4, 4, 3.0), (4, 6, 4.0),
         (5, 4, 1.0), (5, 5, 2.0), (6, 5, 3.0), (6, 7, 4.0), (7, 6, 1.0), (7, 7, 2.0)]
    ptr, ind, val = csr_from_entries(7, e)
    out["spmv_7x7_1"] = dict(m=7, n=7, ptr=ptr, ind=ind, val=val, x=[1, 2, 3, 4, 1, 2, 3],
                             y=[1, 13, 9, 26, 6, 15, 8])
    e = [(1, 1, 1.0), (1, 5, 5.0), (2, 2, 2.0), (2, 3, 3.0), (2, 6, 6.0), (3, 2, 4.0), (3, 5, 1.0),
         (4, 1, 5.0), (4, 3, 2.0), (4, 4, 3.0), (4, 6, 4.0), (4, 7, 5.0), (5, 2, 6.0), (5, 4, 1.0), (5, 5, 2.0),
         (6, 1, 5.0), (6, 5, 3.0), (6, 7, 4.0), (7, 2, 6.0), (7, 6, 1.0), (7, 7, 2.0)]
    ptr, ind, val = csr_from_entries(7, e)
    out["spmv_7x7_2"] = dict(m=7, n=7, ptr=ptr, ind=ind, val=val, x=[1, 2, 3, 4, 1, 2, 3],
                             y=[6, 25, 9, 46, 18, 20, 20])
    e = [(1, 1, 1.0)]
    for r in range(2, 7):
        e += [(r, r - 1, -1.0), (r, r, 2.0), (r, r + 1, -1.0)]
    e += [(7, 7, 1.0)]
    ptr, ind, val = csr_from_entries(7, e)
    out["poisson_7"] = dict(m=7, n=7, ptr=ptr, ind=ind, val=val, b=[1.0] * 7,
                            x=[1.0, 3.5, 5.0, 5.5, 5.0, 3.5, 1.0], tol=1e-5)
    return out


def small_dome():
    import __graft_entry__
    import oracle

    pkg = __graft_entry__.load_package()
    mesh, ice, params = pkg.geometry.small_dome(seed=0)
    orc = oracle.Oracle(mesh)
    arrays = {f"mesh_{k}": v for k, v in mesh.arrays().items()}
    arrays["mesh_box"] = np.array([mesh.xmin, mesh.xmax, mesh.ymin, mesh.ymax])
    for name in pkg.abi.OPERATORS:
        A = orc.operator(name)
        arrays[f"op_{name}_ptr"] = A.ptr
        arrays[f"op_{name}_ind"] = A.ind
        arrays[f"op_{name}_val"] = A.val
    for k in ("Hi", "Hs", "fraction_gr_b", "mask_grounded_ice", "beta_sq"):
        arrays[f"ice_{k}"] = ice[k]
    arrays["ice_A"] = np.array([ice["A_flow"][0, 0]])
    params.stress_balance_PETSc_rtol = 1e-12
    params.stress_balance_PETSc_abstol = 0.0
    params.visc_it_nit = 10
    ssa = pkg.new_ssa_state(mesh.nTri)
    nv, na, st = orc.solve_SSA(ice, ssa, params)
    arrays["ssa_u_b"] = ssa["u_b"]
    arrays["ssa_v_b"] = ssa["v_b"]
    arrays["ssa_its"] = np.array([nv, na, st["status"]])
    np.savez_compressed(os.path.join(HERE, "small_dome.npz"), **arrays)
    return mesh.nV, mesh.nTri, nv, na


if __name__ == "__main__":
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats(), f, indent=1)
    print("small_dome", small_dome())
