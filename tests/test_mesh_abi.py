"""Mesh conventions and the C ABI (library loads, symbols, struct layout) -- no GPU needed."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import load_small_dome

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ufe_gpu.h")


def test_mesh_conventions(pkg):
    mesh = pkg.mesh.uniform_mesh(100e3, 15e3, seed=2)
    T = mesh.Tri - 1
    assert np.all(mesh.tri_area() > 0)                       # Tri counter-clockwise
    for ti in range(mesh.nTri):
        for n in range(3):
            tj = mesh.TriC[ti, n]
            if tj:
                shared = set(T[ti]) & set(T[tj - 1])
                assert shared == set(T[ti]) - {T[ti, n]}      # across from vertex n
    for vi in range(mesh.nV):
        nc, nt = mesh.nC[vi], mesh.niTri[vi]
        Cv = mesh.C[vi, :nc] - 1
        ang = np.unwrap(np.arctan2(mesh.V[Cv, 1] - mesh.V[vi, 1], mesh.V[Cv, 0] - mesh.V[vi, 0]))
        assert np.all(np.diff(ang) > 0)                      # counter-clockwise
        for k in range(nt):
            verts = set(T[mesh.iTri[vi, k] - 1])
            assert {vi, Cv[k], Cv[(k + 1) % nc]} == verts     # iTri(k) between C(k), C(k+1)
        assert (mesh.VBI[vi] > 0) == (nt == nc - 1)          # edge to edge on borders
    assert sorted(np.bincount(mesh.VBI)[[2, 4, 6, 8]]) == [1, 1, 1, 1]
    tb = mesh.TriBI
    border_tris = {int(t) - 1 for vi in np.nonzero(mesh.VBI)[0] for t in mesh.iTri[vi, :mesh.niTri[vi]]}
    assert set(np.nonzero(tb)[0]) == border_tris
    assert np.allclose(mesh.TriGC, mesh.V[T].mean(axis=1), rtol=0, atol=1e-9)


def test_dome_workload_size(pkg):
    mesh, ice, params = pkg.geometry.dome_case()
    assert 7000 < mesh.nV < 9500                              # ~8,000 vertices
    assert ice["Hi"].max() == pytest.approx(3000.0, rel=2e-2)


def test_benchmark_workload_sizes(pkg):
    """The synthetic workloads the benchmark measures have the sizes their descriptions state."""
    G = pkg.geometry
    mesh, ice, params = G.channel_case(seed=0)                 # DIVA channel: ~58k vertices, nz 12
    assert 55_000 < mesh.nV < 62_000 and mesh.nz == 12
    x = mesh.V[:, 0]
    assert x.max() - x.min() == pytest.approx(640e3, rel=1e-6)
    mesh3 = G.ensemble_mesh(nV=30_000, seed=0)                # SSA ensemble: ~30k vertices
    assert 28_500 < mesh3.nV < 31_500
    mesh2, fields, tp = G.thermo_case()                       # thermodynamics: ~200k columns x 30
    assert 190_000 < mesh2.nV < 210_000 and mesh2.nz == 30
    frac_free = np.mean(fields["Hi"] <= 0.0)
    assert 0.12 < frac_free < 0.2                              # ~15% of the columns ice-free


def _header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ufe_[a-z0-9_]+)\s*\(", src)))


def test_integration_guide_covers_every_entry_point():
    """Every function of the C ABI appears in the integration guide (what it replaces or serves)."""
    guide = open(os.path.join(os.path.dirname(HEADER), "..", "INTEGRATION.md")).read()
    missing = [f for f in _header_functions() if f not in guide]
    assert not missing, missing


def test_library_exports_every_header_symbol(gpu_lib):
    for name in _header_functions():
        assert hasattr(gpu_lib, name), name


def test_library_has_no_cpu_fallback(gpu_lib, pkg):
    """Without a GB300 the context cannot be created: the product refuses instead of computing."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    ctx = C.c_void_p()
    assert gpu_lib.ufe_ctx_create(0, C.byref(ctx)) == pkg.abi.UFE_ERR_DEVICE
    assert not ctx.value


def test_default_params_match(gpu_lib, pkg):
    p = pkg.abi.SolverParams()
    gpu_lib.ufe_default_params(C.byref(p))
    q = pkg.abi.default_params()
    assert bytes(p) == bytes(q)


def test_default_thermo_params_match(gpu_lib, pkg):
    p = pkg.abi.ThermoParams()
    gpu_lib.ufe_default_thermo_params(C.byref(p))
    q = pkg.abi.default_thermo_params()
    assert bytes(p) == bytes(q)


def test_default_thickness_params_match(gpu_lib, pkg):
    p = pkg.abi.ThicknessParams()
    gpu_lib.ufe_default_thickness_params(C.byref(p))
    q = pkg.abi.default_thickness_params()
    assert bytes(p) == bytes(q)


def test_struct_layout_matches_header(pkg, tmp_path):
    """Compile a C probe against include/ufe_gpu.h and compare sizes/offsets with ctypes."""
    abi = pkg.abi
    structs = {"ufe_mesh_desc": abi.MeshDesc, "ufe_solver_params": abi.SolverParams, "ufe_ice_state": abi.IceState,
               "ufe_bc_prescribed": abi.BCPrescribed, "ufe_diva_state": abi.DivaState,
               "ufe_solve_stats": abi.SolveStats, "ufe_thermo_params": abi.ThermoParams,
               "ufe_thermo_columns": abi.ThermoColumns, "ufe_heat_fields": abi.HeatFields,
               "ufe_thickness_params": abi.ThicknessParams, "ufe_thickness_fields": abi.ThicknessFields,
               "ufe_thickness_stats": abi.ThicknessStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                          check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(out[cname]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, (cname, f)


def test_golden_fixture_loads(pkg):
    mesh, ice, params, ops, sol = load_small_dome(pkg)
    assert mesh.nV == 741 and mesh.nTri == 1372
    assert ops["M2_DDX_B_B"].m == mesh.nTri
