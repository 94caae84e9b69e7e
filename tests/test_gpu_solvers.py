"""CG / BiCGSTAB on the GPU against the oracle restatement of mpla.cpp.

Iteration counts: identical within +-1 on well-conditioned systems (the
dense SPD configuration family and kernel systems with a moderate nugget).
On ill-conditioned kernel systems the count of FP64 CG itself moves by a
few percent under a different dot-product order (measured with the oracle:
2924 vs 2998 iterations at n = 1024, d = 2, l = 0.05, nugget 1e-4), so
there the bar is +-3 % and the same final tolerance.
"""
import numpy as np
import pytest

from mpla_gb300 import synth

pytestmark = pytest.mark.gpu


def scaled(n, dim, ell, seed=0):
    return synth.gauss_points(n, dim, seed) / (np.sqrt(2.0) * ell)


@pytest.mark.parametrize("n", [64, 500, 2048])
def test_cg_dense_spd_matches_oracle(gpu, orc, n):
    A, b, x0 = synth.dense_spd(n, seed=1)
    dA, db, dx = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(b), \
        gpu.DeviceArray.from_numpy(x0)
    info = gpu.cg_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=1000, eps=1e-10)
    xo, ko, reso, sto = orc.cg(orc.DenseOp(A), b, x0, iter_max=1000, eps=1e-10)
    assert info.status == 0 and sto == 0
    assert abs(info.iterations - ko) <= 1
    assert info.final_res < 1e-10 and info.true_relres < 1e-9
    assert np.allclose(dx.numpy(), xo, rtol=1e-8, atol=1e-10)


def test_cg_rms_rule_tridiagonal_test_cg_case(gpu, orc):
    """test_cg.cpp: (2,-1) tridiagonal, manufactured b, random x0, RMS stop 1e-10."""
    n = 300
    A = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    rng = np.random.default_rng(1235)
    b = A @ rng.random(n)
    x0 = rng.random(n)
    dA = gpu.DeviceArray.from_numpy(np.asfortranarray(A).ravel(order="F"))
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray.from_numpy(x0)
    info = gpu.cg_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=1000, eps=1e-10, stop_rule=gpu.STOP_RMS)
    xo, ko, reso, sto = orc.cg(orc.DenseOp(A), b, x0, iter_max=1000, eps=1e-10, stop_rule=1)
    assert info.status == 0 and sto == 0
    assert abs(info.iterations - ko) <= 1
    assert np.sqrt(np.mean((A @ dx.numpy() - b) ** 2)) < 1e-9


def test_cg_breakdown_and_cap_statuses(gpu):
    n = 3
    A = np.diag([1.0, -1.0, 2.0])
    dA = gpu.DeviceArray.from_numpy(A.ravel(order="F"))
    db, dx = gpu.DeviceArray.from_numpy(np.ones(3)), gpu.DeviceArray(3)
    dx.zero()
    info = gpu.cg_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=50, eps=1e-12)
    assert info.status == gpu.MGB_ERR_BREAKDOWN
    n = 400
    A = np.diag(np.linspace(1, 1e6, n))
    dA = gpu.DeviceArray.from_numpy(A.ravel(order="F"))
    db, dx = gpu.DeviceArray.from_numpy(np.ones(n)), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.cg_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=5, eps=1e-14)
    assert info.status == gpu.MGB_ERR_NOTCONV and info.iterations == 4


def test_cg_already_converged_x0(gpu):
    n = 50
    A, b, _ = synth.dense_spd(n, seed=2)
    x = np.linalg.solve(A, b)
    dA, db, dx = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(b), \
        gpu.DeviceArray.from_numpy(x)
    info = gpu.cg_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=100, eps=1e-6)
    assert info.status == 0 and info.iterations == 0


@pytest.mark.parametrize("n,dim,ell,nug,band", [
    (1024, 2, 0.02, 1e-2, 1),      # well conditioned: +-1
    (2000, 3, 0.05, 1e-2, 1),
    (1024, 2, 0.05, 1e-4, 0.03),   # the C2 family at small n: +-3 %
    (1500, 3, 0.08, 1e-4, 0.03),   # the C3 family at small n
])
def test_cg_gauss_fp64_matches_oracle(gpu, orc, n, dim, ell, nug, band):
    pts = scaled(n, dim, ell, seed=3)
    b = synth.sincos_rhs(synth.gauss_points(n, dim, 3))
    dp = gpu.GaussPoints(pts)
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.cg_gauss(dp, nug, db.ptr, dx.ptr, iter_max=20000, eps=1e-10)
    op = orc.GaussOp(pts, nug)
    xo, ko, reso, sto = orc.cg(op, b, iter_max=20000, eps=1e-10)
    assert info.status == 0 and sto == 0
    if band >= 1:
        assert abs(info.iterations - ko) <= band
    else:
        assert abs(info.iterations - ko) <= band * ko
    assert orc.true_relres(op, b, dx.numpy()) < 1e-9


@pytest.mark.parametrize("n,dim,ell", [(1024, 2, 0.05), (2000, 3, 0.08), (4096, 2, 0.05)])
def test_cg_gauss_mixed_reaches_fp64_tolerance(gpu, orc, mixed_kind, n, dim, ell):
    pts = scaled(n, dim, ell, seed=4)
    b = synth.sincos_rhs(synth.gauss_points(n, dim, 4))
    dp = gpu.GaussPoints(pts)
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.cg_gauss(dp, 1e-4, db.ptr, dx.ptr, iter_max=100000, eps=1e-10, precision=gpu.PREC_MIXED)
    assert info.status == 0
    op = orc.GaussOp(pts, 1e-4)
    # the error against the FP64 oracle, stated per solve
    assert orc.true_relres(op, b, dx.numpy()) < 1e-10 * 1.01
    assert info.fp64_matvecs >= 2 and info.low_matvecs == info.iterations


def test_bicgstab_dense_matches_oracle(gpu, orc):
    n = 300
    rng = np.random.default_rng(8)
    A = np.asfortranarray(np.eye(n) * 4 + rng.uniform(-1, 1, (n, n)) / np.sqrt(n))
    b = rng.standard_normal(n)
    dA, db, dx = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.bicgstab_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=500, eps=1e-12)
    xo, ko, reso, sto = orc.bicgstab(orc.DenseOp(A), b, iter_max=500, eps=1e-12)
    assert info.status == 0 and sto == 0
    assert abs(info.iterations - ko) <= 1
    assert np.allclose(dx.numpy(), xo, rtol=1e-9, atol=1e-11)


def test_bicgstab_gauss_matches_oracle(gpu, orc):
    n = 800
    pts = scaled(n, 2, 0.03, seed=6)
    b = synth.sincos_rhs(synth.gauss_points(n, 2, 6))
    dp = gpu.GaussPoints(pts)
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.bicgstab_gauss(dp, 1e-2, db.ptr, dx.ptr, iter_max=2000, eps=1e-10)
    op = orc.GaussOp(pts, 1e-2)
    xo, ko, reso, sto = orc.bicgstab(op, b, iter_max=2000, eps=1e-10)
    assert info.status == 0 and sto == 0
    # BiCGSTAB's residual is not monotone; a different dot-product order moves
    # the count more than CG's (the residual histories are compared
    # iteration by iteration in test_gpu_mpla_api.py)
    assert abs(info.iterations - ko) <= max(2, int(0.20 * ko))
    assert orc.true_relres(op, b, dx.numpy()) < 1e-10


def test_cg_gauss_host_entry_point(gpu, orc):
    n = 1500
    pts = scaled(n, 3, 0.08, seed=7)
    b = synth.sincos_rhs(synth.gauss_points(n, 3, 7))
    x, info = gpu.cg_gauss_host(pts, 1e-4, b, precision=gpu.PREC_MIXED)
    assert info.status == 0
    assert orc.true_relres(orc.GaussOp(pts, 1e-4), b, x) < 1e-10 * 1.01


def test_vector_files_roundtrip_with_oracle(gpu, orc, tmp_path):
    x = np.random.default_rng(1).standard_normal(1234)
    dx = gpu.DeviceArray.from_numpy(x)
    p = str(tmp_path / "x.dat")
    gpu.check(gpu.lib().mgb_save_vector(p.encode(), 1234, dx.ptr))
    st, y = orc.load_vector(p, 1234)
    assert st == 0 and np.array_equal(x, y)
    dz = gpu.DeviceArray(1234)
    gpu.check(gpu.lib().mgb_load_vector(p.encode(), 1234, dz.ptr))
    assert np.array_equal(dz.numpy(), x)
    assert gpu.lib().mgb_load_vector(p.encode(), 1000, dz.ptr) == gpu.MGB_ERR_IO
    (tmp_path / "short.dat").write_bytes((1234).to_bytes(4, "little") + b"\0" * 16)
    assert gpu.lib().mgb_load_vector(str(tmp_path / "short.dat").encode(), 1234, dz.ptr) == gpu.MGB_ERR_IO
