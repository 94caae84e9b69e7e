"""Matrix-free Gaussian kernel matvecs on the GPU against the oracle.

FP64 kernel: entries within 4 ulp of the oracle's libm exp (the table method
is about 1 ulp; the oracle goes through sqrt then squares, as the reference
does), matvec within 1e-13 relative to sum_j |K_ij x_j|.
Mixed kernels (tensor-core distances and FP32 differences): FP32 arithmetic
and ex2.approx, within 2e-5 relative, bit-reproducible.
"""
import numpy as np
import pytest

from mpla_gb300 import synth

pytestmark = pytest.mark.gpu


def scaled_points(n, dim, ell, seed=0):
    return synth.gauss_points(n, dim, seed) / (np.sqrt(2.0) * ell)


def rel_err(got, want, scale):
    scale = np.where(scale == 0, 1.0, scale)
    return np.max(np.abs(got - want) / scale)


def abs_matvec(op, x):
    """sum_j |K_ij x_j| (K >= 0): the oracle matvec of |x|."""
    return op.matvec(np.abs(x))


@pytest.mark.parametrize("dim", [1, 2, 3, 5])
def test_fp64_entries_within_ulps(gpu, orc, dim):
    pts = scaled_points(300, dim, 0.15, seed=dim)
    dp = gpu.GaussPoints(pts)
    rng = np.random.default_rng(dim)
    i = rng.integers(0, 300, 4000)
    j = rng.integers(0, 300, 4000)
    i[:300] = np.arange(300)
    j[:300] = np.arange(300)   # diagonal
    got = gpu.gauss_entries(dp, i, j, nugget=1e-4)
    op = orc.GaussOp(pts, 1e-4)
    want = np.array([op.entry(a, b) for a, b in zip(i, j)])
    nz = want > 1e-300
    rel = np.abs(got[nz] - want[nz]) / want[nz]
    # exp(-s) is conditioned like s: allow 4 ulp x max(1, s)
    assert np.all(rel <= 4 * 2.2e-16 * np.maximum(1.0, -np.log(want[nz])))


@pytest.mark.parametrize("n,dim,ell", [(1, 2, 0.1), (37, 2, 0.1), (1000, 1, 0.05), (2048, 2, 0.05),
                                       (3001, 3, 0.08), (1500, 6, 0.3)])
def test_fp64_matvec_matches_oracle(gpu, orc, n, dim, ell):
    pts = scaled_points(n, dim, ell, seed=n)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_f64(dp, 1e-4, gpu.NUGGET_DIAGONAL, dx.ptr, dy.ptr)
    gpu.synchronize()
    op = orc.GaussOp(pts, 1e-4)
    assert rel_err(dy.numpy(), op.matvec(x), abs_matvec(op, x)) <= 1e-13


def test_fp64_matvec_rectangular_blocks_with_offsets(gpu, orc):
    n = 2500
    pts = scaled_points(n, 2, 0.07, seed=9)
    x = np.random.default_rng(9).standard_normal(n)
    dp = gpu.GaussPoints(pts)
    op = orc.GaussOp(pts, 1e-3)
    for rows, cols, roff, coff in [(700, 1300, 100, 1200), (1, n, 17, 0), (n, 1, 0, 5), (1000, 1000, 1000, 1000)]:
        dx = gpu.DeviceArray.from_numpy(x[coff:coff + cols])
        dy = gpu.DeviceArray(rows)
        gpu.gauss_matvec_f64(dp, 1e-3, gpu.NUGGET_DIAGONAL, dx.ptr, dy.ptr, rows=rows, cols=cols,
                             row_offset=roff, col_offset=coff)
        gpu.synchronize()
        want = op.matvec(x[coff:coff + cols], rows=rows, cols=cols, roff=roff, coff=coff)
        scale = op.matvec(np.abs(x[coff:coff + cols]), rows=rows, cols=cols, roff=roff, coff=coff)
        assert rel_err(dy.numpy(), want, scale) <= 1e-13, (rows, cols, roff, coff)


def test_fp64_kernel_cu_rule_with_duplicate_points(gpu, orc):
    n = 900
    pts = scaled_points(n, 3, 0.1, seed=5)
    pts[:, 450:] = pts[:, :450]          # every point duplicated
    x = np.random.default_rng(5).standard_normal(n)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_f64(dp, 0.0, gpu.NUGGET_KERNEL_CU, dx.ptr, dy.ptr)
    gpu.synchronize()
    op = orc.GaussOp(pts, 0.0, rule=orc.RULE_KERNEL_CU)
    assert rel_err(dy.numpy(), op.matvec(x), abs_matvec(op, x)) <= 1e-13


def test_fp64_matvec_far_pairs_left_out(gpu, orc):
    # a short length scale: most tile pairs are farther apart than the FP64
    # operator's 2^-80 cut and are not evaluated; the product must still meet
    # the FP64 bar, and its work figure must show the cut
    n, dim, ell = 8192, 2, 0.01
    pts = scaled_points(n, dim, ell, seed=11)
    x = np.random.default_rng(11).standard_normal(n)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_f64(dp, 1e-4, gpu.NUGGET_DIAGONAL, dx.ptr, dy.ptr)
    gpu.synchronize()
    op = orc.GaussOp(pts, 1e-4)
    assert rel_err(dy.numpy(), op.matvec(x), abs_matvec(op, x)) <= 1e-13
    half = (n // 128) * (n // 128 + 1) // 2 * 128 * 128
    assert gpu.gauss_fp64_work(dp) < half // 2


def test_fp64_far_points_underflow_to_zero(gpu):
    pts = np.array([[0.0, 40.0, 1e6], [0.0, 0.0, 0.0]])
    dp = gpu.GaussPoints(pts)
    got = gpu.gauss_entries(dp, np.array([0, 0, 1]), np.array([1, 2, 2]))
    assert got[0] == pytest.approx(np.exp(-1600.0) if np.exp(-1600.0) > 0 else 0.0, abs=1e-300)
    assert got[1] == 0.0 and got[2] == 0.0


@pytest.mark.parametrize("n,dim,ell", [(100, 1, 0.05), (300, 3, 0.1), (4096, 2, 0.05), (5000, 3, 0.08)])
def test_mixed_matvec_close_to_oracle(gpu, orc, mixed_kind, n, dim, ell):
    pts = scaled_points(n, dim, ell, seed=n + 1)
    x = np.random.default_rng(n).standard_normal(n)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_mixed(dp, 1e-4, dx.ptr, dy.ptr)
    op = orc.GaussOp(pts, 1e-4)
    assert rel_err(dy.numpy(), op.matvec(x), abs_matvec(op, x)) <= 2e-5


def test_fp64_matvec_is_bit_reproducible(gpu):
    pts = scaled_points(6000, 2, 0.05, seed=2)
    x = np.random.default_rng(2).standard_normal(6000)
    dp = gpu.GaussPoints(pts)
    dx = gpu.DeviceArray.from_numpy(x)
    outs = []
    for _ in range(2):
        dy = gpu.DeviceArray(6000)
        gpu.gauss_matvec_f64(dp, 1e-4, gpu.NUGGET_DIAGONAL, dx.ptr, dy.ptr)
        gpu.synchronize()
        outs.append(dy.numpy())
    assert np.array_equal(outs[0], outs[1])


def test_mixed_matvec_is_bit_reproducible(gpu, mixed_kind):
    pts = scaled_points(3000, 3, 0.1, seed=3)
    x = np.random.default_rng(3).standard_normal(3000)
    dp = gpu.GaussPoints(pts)
    dx = gpu.DeviceArray.from_numpy(x)
    outs = []
    for _ in range(2):
        dy = gpu.DeviceArray(3000)
        gpu.gauss_matvec_mixed(dp, 1e-4, dx.ptr, dy.ptr)
        gpu.synchronize()
        outs.append(dy.numpy())
    assert np.array_equal(outs[0], outs[1])


def test_mixed_matvec_far_pairs_left_out(gpu, orc):
    # a short length scale: most tile pairs are farther apart than the 2^-40
    # threshold and are not evaluated by the default (FP32-difference)
    # kernel; the product must meet the same bar, and its work figure must
    # show the cut.  (The tensor-core variant evaluates every pair; with
    # tiles spanning ~10 length scales its norm cancellation exceeds the bar
    # here, one of the reasons it is not the default.)
    assert gpu.get_mixed_matvec() == gpu.MIXED_SIMT
    n, dim, ell = 8192, 2, 0.01
    pts = scaled_points(n, dim, ell, seed=9)
    x = np.random.default_rng(9).standard_normal(n)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_mixed(dp, 1e-4, dx.ptr, dy.ptr)
    op = orc.GaussOp(pts, 1e-4)
    assert rel_err(dy.numpy(), op.matvec(x), abs_matvec(op, x)) <= 2e-5
    half = (n // 128) * (n // 128 + 1) // 2 * 128 * 128
    assert gpu.gauss_mixed_work(dp) < half // 2
