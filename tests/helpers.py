"""Shared test helpers: golden fixtures and comparisons."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_kats():
    with open(os.path.join(GOLDEN, "kats.json")) as f:
        return json.load(f)


def kat_csr(pkg, k):
    return pkg.CSR(k["m"], k["n"], np.array(k["ptr"], np.int32), np.array(k["ind"], np.int32),
                   np.array(k["val"], np.float64), 1)


def load_small_dome(pkg):
    """(mesh, ice, params, operators, ssa_solution) of tests/golden/small_dome.npz."""
    z = np.load(os.path.join(GOLDEN, "small_dome.npz"))
    names = ["V", "nC", "C", "niTri", "iTri", "VBI", "Tri", "TriC", "TriBI", "TriGC", "zeta"]
    mesh = pkg.mesh.Mesh.from_arrays(*[z[f"mesh_{n}"] for n in names], z["mesh_box"])
    ice = {k: np.ascontiguousarray(z[f"ice_{k}"]) for k in ("Hi", "Hs", "fraction_gr_b", "mask_grounded_ice", "beta_sq")}
    ice["A_flow"] = np.asfortranarray(np.full((mesh.nV, mesh.nz), float(z["ice_A"][0])))
    params = pkg.abi.default_params(choice_sliding_law="Weertman", visc_it_norm_dUV_tol=1e-4,
                                    stress_balance_PETSc_rtol=1e-12, stress_balance_PETSc_abstol=0.0,
                                    visc_it_nit=10)
    ops = {}
    for name in pkg.abi.OPERATORS:
        ops[name] = pkg.CSR(0, 0, z[f"op_{name}_ptr"], z[f"op_{name}_ind"], z[f"op_{name}_val"], 1)
        shape = {"A_B": (mesh.nTri, mesh.nV), "B_A": (mesh.nV, mesh.nTri), "A_A": (mesh.nV, mesh.nV),
                 "B_B": (mesh.nTri, mesh.nTri)}[name[-3:]]
        ops[name].m, ops[name].n = shape
    sol = dict(u_b=z["ssa_u_b"], v_b=z["ssa_v_b"], its=z["ssa_its"])
    return mesh, ice, params, ops, sol


def rel_l2(a, b):
    a = np.asarray(a, float).ravel()
    b = np.asarray(b, float).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def same_structure(A, B):
    return np.array_equal(A.ptr - A.index_base, B.ptr - B.index_base) and \
        np.array_equal(A.ind - A.index_base, B.ind - B.index_base)
