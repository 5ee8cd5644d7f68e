"""The allocation-free CSR solve (ufe_solve_csr_noalloc) against ufe_solve_csr.

The entry point serves callers that cannot let a library allocate device memory (their GPU memory
comes from their own pool, or their footprint is fixed at start-up): they pass device buffers, and
the solver's work vectors live in a fixed device array of the library.  This file runs last, so a
failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

MAX_ROWS = 131072


def _system(n, seed):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=5.0 / n, random_state=seed, format="csr")
    A = (A + sp.diags(np.abs(A).sum(1).A1 + 1.0 + rng.random(n))).tocsr()
    A.sort_indices()
    return A, rng.normal(size=n)


def _reference(lib, pkg, A, b):
    """ufe_solve_csr (host arrays, allocating) on a fresh context."""
    ctx = C.c_void_p()
    assert lib.ufe_ctx_create(0, C.byref(ctx)) == 0
    try:
        n = A.shape[0]
        ptr = np.ascontiguousarray(A.indptr, np.int32)
        ind = np.ascontiguousarray(A.indices, np.int32)
        val = np.ascontiguousarray(A.data, np.float64)
        x = np.zeros(n)
        its = C.c_int32()
        rc = lib.ufe_solve_csr(ctx, n, ind.size, pkg.abi.as_i(ptr), pkg.abi.as_i(ind), pkg.abi.as_d(val), 0,
                               pkg.abi.as_d(np.ascontiguousarray(b)), pkg.abi.as_d(x), 1e-12, 0.0, 10000, C.byref(its))
        assert rc == 0
        return x, its.value
    finally:
        lib.ufe_ctx_destroy(ctx)


def test_noalloc_solve_matches_allocating_solve_twice(gpu_lib, pkg):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    # two calls in a row: the second reuses the scratch the first left behind
    for seed, n, base in ((3, 3000, 0), (4, 5000, 1)):
        A, b = _system(n, seed)
        x_ref, its_ref = _reference(lib, pkg, A, b)
        d_ptr = torch.tensor(A.indptr.astype(np.int32) + base, device=dev)
        d_ind = torch.tensor(A.indices.astype(np.int32) + base, device=dev)
        d_val = torch.tensor(A.data, dtype=torch.float64, device=dev)
        d_b = torch.tensor(b, dtype=torch.float64, device=dev)
        d_x = torch.zeros(n, dtype=torch.float64, device=dev)
        its = C.c_int32()
        torch.cuda.synchronize()
        rc = lib.ufe_solve_csr_noalloc(n, A.nnz, d_ptr.data_ptr(), d_ind.data_ptr(), d_val.data_ptr(), base,
                                       d_b.data_ptr(), d_x.data_ptr(), 1e-12, 0.0, 10000, C.byref(its),
                                       C.c_void_p(stream.cuda_stream))
        assert rc == 0
        x = d_x.cpu().numpy()
        assert rel_l2(x, x_ref) < 1e-8
        assert abs(its.value - its_ref) <= 2


def test_noalloc_rejects_oversized_system(gpu_lib, pkg):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    n = MAX_ROWS + 1
    d_ptr = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    d = torch.zeros(n, dtype=torch.float64, device=dev)
    its = C.c_int32()
    rc = gpu_lib.ufe_solve_csr_noalloc(n, 0, d_ptr.data_ptr(), d_ptr.data_ptr(), d.data_ptr(), 0, d.data_ptr(),
                                       d.data_ptr(), 1e-8, 0.0, 10, C.byref(its), None)
    assert rc == pkg.abi.UFE_ERR_CAPACITY
