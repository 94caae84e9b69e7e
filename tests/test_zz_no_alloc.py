"""The allocation-free dgemv entry point (mgb_dgemv_noalloc).

Some callers of this library may not call cudaMalloc: plugins whose host
framework owns every device allocation, and latency-critical paths that
cannot take the allocator's implicit device synchronisation.  For them
mgb_dgemv_noalloc keeps its scratch in a fixed device array shared by all
calls.  The test makes two calls in a row for each shape (the second call
sees the first call's leftovers in the array) and compares both with the
FP64 oracle and with mgb_dgemv through the C ABI, at the 1e-13 relative bar
of the dgemv tests.  This file is collected last so that a failure here does
not hide the other results.
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
                                         (70000, 20, None, 0), (64, 20000, None, 0)])
def test_noalloc_dgemv_matches_oracle_and_dgemv_twice(gpu, orc, m, n, lda, off):
    rng = np.random.default_rng(m + n)
    lda = lda or m
    buf = np.zeros(off + lda * n)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    for j in range(n):
        buf[off + j * lda: off + j * lda + m] = A[:, j]
    dA = gpu.DeviceArray.from_numpy(buf)
    a_ptr = dA.ptr + 8 * off
    L = gpu.lib()
    for call in range(2):
        x = rng.uniform(-1, 1, n)
        scale = np.abs(A) @ np.abs(x)
        dx = gpu.DeviceArray.from_numpy(x)
        y_ref, y_na = gpu.DeviceArray(m), gpu.DeviceArray(m)
        y_na.upload(np.full(m, np.nan))  # stale output must be overwritten
        gpu.check(L.mgb_dgemv(m, n, a_ptr, lda, dx.ptr, y_ref.ptr, None))
        gpu.synchronize()
        gpu.check(L.mgb_dgemv_noalloc(m, n, a_ptr, lda, dx.ptr, y_na.ptr, None))
        gpu.synchronize()
        got = y_na.numpy()
        want = orc.dgemv(A, x)
        assert np.max(np.abs(got - want) / scale) <= TOL, ("oracle", call, m, n)
        assert np.max(np.abs(got - y_ref.numpy()) / scale) <= TOL, ("mgb_dgemv", call, m, n)


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
    assert b"exceeds" in L.mgb_last_error()
