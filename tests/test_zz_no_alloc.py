"""The allocation-free CSR solve (ufe_solve_csr_noalloc) against ufe_solve_csr and a direct solve.

The entry point serves callers that cannot let a library allocate device memory: a model whose GPU
memory comes from its own pool or caching allocator, or a coupled run that fixes its GPU footprint
at start-up.  They pass device buffers, and the solver's work vectors live in a fixed device array
of the library.  This file runs last, so a failure here comes after every other test has run; its
tests pass alone in a fresh process as well as after the others.
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


def _device_system(torch, dev, A, b, base):
    return (torch.tensor(A.indptr.astype(np.int32) + base, device=dev),
            torch.tensor(A.indices.astype(np.int32) + base, device=dev),
            torch.tensor(A.data, dtype=torch.float64, device=dev),
            torch.tensor(b, dtype=torch.float64, device=dev),
            torch.zeros(A.shape[0], dtype=torch.float64, device=dev))


def _call(lib, n, nnz, d, base, stream, its, rtol=1e-12):
    d_ptr, d_ind, d_val, d_b, d_x = d
    return lib.ufe_solve_csr_noalloc(n, nnz, d_ptr.data_ptr(), d_ind.data_ptr(), d_val.data_ptr(), base,
                                     d_b.data_ptr(), d_x.data_ptr(), rtol, 0.0, 10000, C.byref(its),
                                     C.c_void_p(stream.cuda_stream) if stream is not None else None)


def test_noalloc_solve_matches_allocating_solve_twice(gpu_lib, pkg):
    torch = pytest.importorskip("torch")
    from scipy.sparse.linalg import spsolve
    lib = gpu_lib
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    # two calls in a row: the second reuses the scratch the first left behind
    for call, (seed, n, base) in enumerate(((3, 3000, 0), (4, 5000, 1))):
        A, b = _system(n, seed)
        x_ref, its_ref = _reference(lib, pkg, A, b)
        x_direct = spsolve(A.tocsc(), b)
        d = _device_system(torch, dev, A, b, base)
        its = C.c_int32()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        stats_before = torch.cuda.memory_stats(dev).get("allocation.all.allocated", 0)
        rc = _call(lib, n, A.nnz, d, base, stream, its)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        stats_after = torch.cuda.memory_stats(dev).get("allocation.all.allocated", 0)
        assert rc == 0
        x = d[4].cpu().numpy()
        assert rel_l2(x, x_ref) < 1e-8
        assert rel_l2(x, x_direct) < 1e-8
        assert abs(its.value - its_ref) <= 2
        if call == 1:
            # after the first call on the device (which loads the library's device module and its
            # fixed array), a call takes no device memory at all
            assert free_after == free_before
            assert stats_after == stats_before


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


def test_noalloc_rejects_malformed_matrix_on_device(gpu_lib, pkg):
    """A column index outside the matrix, or row pointers that disagree with nnz, are found by the
    device-side check before any kernel indexes through them; a good system solves afterwards."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    A, b = _system(2000, 7)
    its = C.c_int32()
    for base in (0, 1):
        bad_col = A.copy()
        bad_col.indices = bad_col.indices.copy()
        bad_col.indices[A.nnz // 2] = A.shape[0]          # one past the last column
        d = _device_system(torch, dev, bad_col, b, base)
        assert _call(gpu_lib, A.shape[0], A.nnz, d, base, stream, its) == pkg.abi.UFE_ERR_INVALID
        d = _device_system(torch, dev, A, b, base)        # ptr[m] says nnz, the call claims fewer
        assert _call(gpu_lib, A.shape[0], A.nnz - 1, d, base, stream, its) == pkg.abi.UFE_ERR_INVALID
        bad_ptr = A.copy()
        bad_ptr.indptr = bad_ptr.indptr.copy()
        bad_ptr.indptr[10], bad_ptr.indptr[11] = bad_ptr.indptr[11], bad_ptr.indptr[10] - 1   # decreasing pair
        d = _device_system(torch, dev, bad_ptr, b, base)
        assert _call(gpu_lib, A.shape[0], A.nnz, d, base, stream, its) == pkg.abi.UFE_ERR_INVALID
    d = _device_system(torch, dev, A, b, 0)
    assert _call(gpu_lib, A.shape[0], A.nnz, d, 0, stream, its) == 0
    x_ref, _ = _reference(gpu_lib, pkg, A, b)
    assert rel_l2(d[4].cpu().numpy(), x_ref) < 1e-8
