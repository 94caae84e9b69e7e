"""dgemv / ddot / daxpy on the GPU against the oracle and the reference KAT.

Bar: relative 1e-13 for dgemv (the parity bar of this path), measured against sum_j |A_ij x_j|
so cancellation in a row does not inflate it; the reference's own
known-answer test (test_library.cpp) at 1e-13 instead of its 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def run_dgemv(gpu, A, x, lda=None, offset_elems=0):
    m, n = A.shape
    lda = lda or m
    buf = np.zeros(offset_elems + lda * n)
    for j in range(n):
        buf[offset_elems + j * lda: offset_elems + j * lda + m] = A[:, j]
    dA = gpu.DeviceArray.from_numpy(buf)
    dx = gpu.DeviceArray.from_numpy(x)
    dy = gpu.DeviceArray(m)
    gpu.dgemv(m, n, dA.ptr + 8 * offset_elems, lda, dx.ptr, dy.ptr)
    gpu.synchronize()
    return dy.numpy()


def rel_err(got, want, A, x):
    scale = np.abs(A) @ np.abs(x)
    scale[scale == 0] = 1.0
    return np.max(np.abs(got - want) / scale)


@pytest.mark.parametrize("m,n", [(1, 1), (7, 3), (128, 128), (257, 129), (1000, 1000)])
def test_dgemv_test_library_known_answer(gpu, m, n):
    A = np.arange(m * n, dtype=np.float64).reshape((m, n), order="F")
    x = np.arange(n, dtype=np.float64)
    j = np.arange(n, dtype=np.float64)
    want = m * np.sum(j * j) + np.arange(m) * np.sum(j)
    got = run_dgemv(gpu, A, x)
    nz = want != 0
    assert np.all(np.abs(got[nz] - want[nz]) / np.abs(want[nz]) <= TOL)
    assert np.all(got[~nz] == 0)


@pytest.mark.parametrize("m,n,lda,off", [
    (4096, 4096, None, 0),      # the dense configuration
    (4097, 333, None, 0),       # odd rows: scalar tail of the 128-bit path
    (64, 10000, None, 0),       # few strips, many column splits
    (10000, 3, None, 0),        # fewer columns than one warp chunk
    (513, 700, 515, 0),         # odd lda: 64-bit load path
    (600, 600, 600, 1),         # A not 16-byte aligned: 64-bit load path
    (1, 5000, None, 0),
    (5000, 1, None, 0),
])
def test_dgemv_matches_oracle(gpu, orc, m, n, lda, off):
    rng = np.random.default_rng(m * 31 + n)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    x = rng.uniform(-1, 1, n)
    got = run_dgemv(gpu, A, x, lda=lda, offset_elems=off)
    want = orc.dgemv(A, x)
    assert rel_err(got, want, A, x) <= TOL


@pytest.mark.parametrize("x_out_of_range", [False, True])
def test_dgemv_wide_magnitudes(gpu, orc, x_out_of_range):
    # magnitudes from subnormal to 1e100 with zeros mixed in: the same bar
    rng = np.random.default_rng(11)
    m, n = 1500, 2100
    A = rng.uniform(-1, 1, (m, n)) * 10.0 ** rng.integers(-20, 20, (m, n))
    pick = rng.random((m, n))
    A[pick < 0.05] = 0.0
    A[(pick >= 0.05) & (pick < 0.06)] = 1e-300
    A[(pick >= 0.06) & (pick < 0.07)] = -1e100
    A[(pick >= 0.07) & (pick < 0.075)] = 5e-320  # subnormal
    A = np.asfortranarray(A)
    x = rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-10, 10, n)
    x[::7] = 0.0
    if x_out_of_range:
        x[5] = 3e-200
        x[1900] = 1e80
    got = run_dgemv(gpu, A, x)
    want = orc.dgemv(A, x)
    assert rel_err(got, want, A, x) <= TOL


def test_dgemv_is_bit_reproducible(gpu):
    rng = np.random.default_rng(11)
    A = np.asfortranarray(rng.standard_normal((2048, 3000)))
    x = rng.standard_normal(3000)
    a = run_dgemv(gpu, A, x)
    b = run_dgemv(gpu, A, x)
    assert np.array_equal(a, b)


def test_dgemv_empty_sizes(gpu):
    dy = gpu.DeviceArray.from_numpy(np.full(5, 7.0))
    dA = gpu.DeviceArray(1)
    dx = gpu.DeviceArray(1)
    gpu.dgemv(5, 0, dA.ptr, 5, dx.ptr, dy.ptr)   # n = 0: y = 0
    gpu.synchronize()
    assert np.array_equal(dy.numpy(), np.zeros(5))
    gpu.dgemv(0, 5, dA.ptr, 1, dx.ptr, dy.ptr)   # m = 0: nothing
    with pytest.raises(gpu.MplaError):
        gpu.dgemv(5, 5, dA.ptr, 3, dx.ptr, dy.ptr)  # lda < m


@pytest.mark.parametrize("n", [1, 5, 1000, 65536, 1_000_003])
def test_ddot_daxpy_match_oracle(gpu, orc, n):
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray.from_numpy(y)
    got = gpu.ddot(n, dx.ptr, dy.ptr)
    assert abs(got - orc.ddot(x, y)) <= 1e-13 * float(np.abs(x) @ np.abs(y))
    gpu.daxpy(n, -0.75, dx.ptr, dy.ptr)
    gpu.synchronize()
    # y + a x with one FMA per element: identical to numpy's fma-free value
    # within one rounding
    assert np.allclose(dy.numpy(), y - 0.75 * x, rtol=1e-15, atol=1e-15)
