"""The allocation-free SpMSpV entry point (gbc_spmspv_select2ndmin_noalloc).

It serves callers that cannot allocate device memory at the point of use
(another component owns the free memory, or cudaMalloc's implicit
synchronisation is not acceptable), so it keeps its working storage in one
fixed device array.  The test drives it through the C ABI with caller-owned
device buffers and checks it against the allocating entry point on two calls
in a row: the second call must not see anything left over from the first.
This file is collected last on purpose (name order)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, A_dev, A, x, xv, torch):
    dx = torch.from_numpy(x).cuda()
    dv = torch.from_numpy(xv).cuda()
    yi = torch.full((A.nrow,), -7, dtype=torch.int32, device="cuda")
    yv = torch.full((A.nrow,), -7, dtype=torch.int64, device="cuda")
    ny = C.c_int32(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.gbc_spmspv_select2ndmin_noalloc(A.nrow, A.ncol, A.nnz, A_dev[0].data_ptr(), A_dev[1].data_ptr(),
                                             dx.data_ptr(), dv.data_ptr(), len(x), yi.data_ptr(), yv.data_ptr(),
                                             C.byref(ny), C.c_void_p(stream))
    return rc, ny.value, yi.cpu().numpy(), yv.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from combblas_gb300 import _lib
    from combblas_gb300 import bfs as B
    from combblas_gb300 import generators as G

    lib = _lib.lib()
    A = G.rmat(16, 8, seed=12, values=None)
    A_dev = (torch.from_numpy(A.colptr).cuda(), torch.from_numpy(A.rowidx).cuda())
    g = B.Graph(A)
    rng = np.random.default_rng(3)
    for nx in (3000, 40):  # a large vector, then a small one: stale entries would show
        x = np.sort(rng.choice(A.ncol, nx, replace=False)).astype(np.int32)
        xv = rng.integers(-10**9, 10**9, nx).astype(np.int64)
        rc, ny, yi, yv = _noalloc(lib, A_dev, A, x, xv, torch)
        assert rc == 0, _lib.lib().gbc_last_error()
        ei, ev = B.SpMXSpV(g, x, xv)
        assert ny == len(ei)
        assert np.array_equal(yi[:ny], ei) and np.array_equal(yv[:ny], ev)


def test_noalloc_allocates_nothing_and_reports_bad_input():
    """After a warm-up call, further calls leave the device's free memory
    unchanged; an out-of-range vector index is reported as GBC_EINVAL (the
    kernel's own bounds check), and the next valid call still gives the right
    answer (every call clears the error flag)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from combblas_gb300 import _lib
    from combblas_gb300 import bfs as B
    from combblas_gb300 import generators as G

    lib = _lib.lib()
    A = G.rmat(12, 8, seed=5, values=None)
    A_dev = (torch.from_numpy(A.colptr).cuda(), torch.from_numpy(A.rowidx).cuda())
    g = B.Graph(A)
    rng = np.random.default_rng(9)
    x = np.sort(rng.choice(A.ncol, 200, replace=False)).astype(np.int32)
    xv = rng.integers(0, 10**6, 200).astype(np.int64)
    dx, dv = torch.from_numpy(x).cuda(), torch.from_numpy(xv).cuda()
    yi = torch.empty(A.nrow, dtype=torch.int32, device="cuda")
    yv = torch.empty(A.nrow, dtype=torch.int64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ny = C.c_int32(-1)

    def call(xp, n):
        return lib.gbc_spmspv_select2ndmin_noalloc(A.nrow, A.ncol, A.nnz, A_dev[0].data_ptr(), A_dev[1].data_ptr(),
                                                   xp, dv.data_ptr(), n, yi.data_ptr(), yv.data_ptr(),
                                                   C.byref(ny), stream)

    assert call(dx.data_ptr(), len(x)) == 0  # warm-up: loads the module on this device
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert call(dx.data_ptr(), len(x)) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    bad = dx.clone()
    bad[7] = A.ncol + 5  # index >= ncol
    torch.cuda.synchronize()
    assert call(bad.data_ptr(), len(x)) == _lib.GBC_OK - 1  # GBC_EINVAL
    assert b"out of range" in lib.gbc_last_error()
    assert call(dx.data_ptr(), len(x)) == 0
    ei, ev = B.SpMXSpV(g, x, xv)
    assert ny.value == len(ei)
    assert np.array_equal(yi.cpu().numpy()[:ny.value], ei) and np.array_equal(yv.cpu().numpy()[:ny.value], ev)


def test_noalloc_rejects_oversized_matrix():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from combblas_gb300 import _lib

    lib = _lib.lib()
    ny = C.c_int32(0)
    rc = lib.gbc_spmspv_select2ndmin_noalloc((1 << 20) + 1, 4, 0, None, None, None, None, 0, None, None,
                                             C.byref(ny), None)
    assert rc == _lib.GBC_OK - 4  # GBC_EOVERFLOW
    assert b"1048576" in lib.gbc_last_error()
