"""The allocation-free dgemv entry point against the regular one.

mgb_dgemv_noalloc serves callers that cannot call cudaMalloc (code inside a
stream capture, plugins whose host framework owns all device memory,
latency-critical paths that must not synchronise on the allocator).  It
keeps its scratch in a fixed device array shared by all calls, so the test
makes two calls in a row for each shape and compares both with mgb_dgemv
through the C ABI, at the 1e-13 relative bar of the dgemv tests.  This file
is collected last so that a failure here does not hide the other results.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _free_bytes():
    # the CUDA runtime libmpla.so is linked against (already loaded)
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("m,n,lda,off", [(4096, 4096, None, 0), (1000, 777, None, 0), (513, 300, 515, 1),
                                         (70000, 20, None, 0)])
def test_noalloc_dgemv_matches_dgemv_twice(gpu, m, n, lda, off):
    rng = np.random.default_rng(m + n)
    lda = lda or m
    buf = np.zeros(off + lda * n)
    A = rng.uniform(-1, 1, (m, n))
    for j in range(n):
        buf[off + j * lda: off + j * lda + m] = A[:, j]
    dA = gpu.DeviceArray.from_numpy(buf)
    a_ptr = dA.ptr + 8 * off
    L = gpu.lib()
    scale = np.abs(A) @ np.ones(n)
    for call in range(2):
        x = rng.uniform(-1, 1, n)
        dx = gpu.DeviceArray.from_numpy(x)
        y_ref, y_na = gpu.DeviceArray(m), gpu.DeviceArray(m)
        gpu.check(L.mgb_dgemv(m, n, a_ptr, lda, dx.ptr, y_ref.ptr, None))
        gpu.synchronize()
        gpu.check(L.mgb_dgemv_noalloc(m, n, a_ptr, lda, dx.ptr, y_na.ptr, None))
        gpu.synchronize()
        got, want = y_na.numpy(), y_ref.numpy()
        assert np.max(np.abs(got - want) / (scale * np.max(np.abs(x)))) <= TOL, (call, m, n)


def test_noalloc_dgemv_allocates_nothing(gpu):
    m = n = 2048
    rng = np.random.default_rng(5)
    dA = gpu.DeviceArray.from_numpy(rng.standard_normal(m * n))
    dx = gpu.DeviceArray.from_numpy(rng.standard_normal(n))
    dy = gpu.DeviceArray(m)
    L = gpu.lib()
    gpu.check(L.mgb_dgemv_noalloc(m, n, dA.ptr, m, dx.ptr, dy.ptr, None))  # first call: set-up
    gpu.synchronize()
    before = _free_bytes()
    for _ in range(3):
        gpu.check(L.mgb_dgemv_noalloc(m, n, dA.ptr, m, dx.ptr, dy.ptr, None))
    gpu.synchronize()
    assert _free_bytes() == before


def test_noalloc_dgemv_rejects_sizes_beyond_its_scratch(gpu):
    L = gpu.lib()
    d = gpu.DeviceArray(16)  # valid pointers; the sizes are rejected before any launch
    # 20000 x ceil(300000/4096) partials exceed the fixed scratch
    st = L.mgb_dgemv_noalloc(20000, 300000, d.ptr, 20000, d.ptr, d.ptr, None)
    assert st == gpu.MGB_ERR_ARG
    assert b"exceeds" in L.mgb_last_error()
    st = L.mgb_dgemv_noalloc(2_000_000, 2, d.ptr, 2_000_000, d.ptr, d.ptr, None)
    assert st == gpu.MGB_ERR_ARG
