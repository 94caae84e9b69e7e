"""This library against the reference MPLA run live on the same GPU.

The reference is compiled from its own sources (oracle/build_ref.py) and
called through its public API (oracle/ref_harness.cu).  Same seeded inputs
on both sides: dgemv to 1e-13 relative, kernel matvecs to 1e-13,
dense CG iteration counts +-1, the Gaussian CG family within 2.5 % (nugget
1e-2) and 3 % (nugget 1e-4), BiCGSTAB within 20 %.
"""
import numpy as np
import pytest

from mpla_gb300 import synth
from oracle import reference as ref

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref.available(), reason="reference MPLA not built on this machine")]


def _rel(got, want, scale):
    scale = np.where(scale == 0, 1.0, scale)
    return float(np.max(np.abs(got - want) / scale))


@pytest.mark.parametrize("n", [1000, 4096])
def test_dgemv_agrees_with_reference(gpu, n):
    rng = np.random.default_rng(n)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    x = rng.uniform(-1, 1, n)
    y_ref, _ = ref.dgemv(A, x)
    dA, dx, dy = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.dgemv(n, n, dA.ptr, n, dx.ptr, dy.ptr)
    gpu.synchronize()
    assert _rel(dy.numpy(), y_ref, np.abs(A) @ np.abs(x)) <= 1e-13


@pytest.mark.parametrize("rule,dim,n", [(0, 2, 3000), (0, 3, 2000), (1, 3, 1500)])
def test_kernel_matvec_agrees_with_reference(gpu, orc, rule, dim, n):
    pts = synth.gauss_points(n, dim, 40 + dim) / (np.sqrt(2) * 0.05)
    if rule == 1:
        pts[:, n // 2:] = pts[:, : n - n // 2]
    x = np.random.default_rng(n).standard_normal(n)
    nugget = 1e-4 if rule == 0 else 0.0
    y_ref = ref.gauss_matvec(pts, nugget, rule, x)
    dp = gpu.GaussPoints(pts)
    dx, dy = gpu.DeviceArray.from_numpy(x), gpu.DeviceArray(n)
    gpu.gauss_matvec_f64(dp, nugget, rule, dx.ptr, dy.ptr)
    gpu.synchronize()
    scale = orc.GaussOp(pts, nugget, rule=rule).matvec(np.abs(x))
    assert _rel(dy.numpy(), y_ref, scale) <= 1e-13


def test_dense_cg_iterations_match_reference(gpu):
    A, b, x0 = synth.dense_spd(1024, seed=7)
    x_ref, mv, _ = ref.solve_dense(A, b, x0, 1000, 1e-10, ref.SOLVER_CG_REL)
    dA, db, dx = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(b), \
        gpu.DeviceArray.from_numpy(x0)
    info = gpu.cg_dense(1024, dA.ptr, db.ptr, dx.ptr, iter_max=1000, eps=1e-10)
    assert info.status == 0
    assert abs(info.iterations - ref.iterations(ref.SOLVER_CG_REL, mv)) <= 1
    assert np.allclose(dx.numpy(), x_ref, rtol=1e-8, atol=1e-10)


# condition numbers 2.3e3 (nugget 1e-2) and 2.3e5 (nugget 1e-4).  The
# count to relres 1e-10 is not a property of the operator alone: at nugget
# 1e-2, numpy FP64 CG on the same system takes 364-369 iterations over
# summation orders of the matvec (caller order, k-d tile order, 128-column
# blocks, this library's slot structure) and over ulp-level perturbations of
# the entries, the reference 368 and this library (k-d tile order, its own
# dot-product tree) 361; at nugget 1e-4 the spread is a few %.
@pytest.mark.parametrize("nugget,band", [(1e-2, 0.025), (1e-4, 0.03)])
def test_gauss_cg_iterations_match_reference(gpu, nugget, band):
    n = 1024
    pts = synth.gauss_points(n, 2, 50) / (np.sqrt(2) * 0.05)
    b = synth.sincos_rhs(synth.gauss_points(n, 2, 50))
    x_ref, mv, _ = ref.solve_gauss(pts, nugget, b, np.zeros(n), 20000, 1e-10, ref.SOLVER_CG_REL)
    k_ref = ref.iterations(ref.SOLVER_CG_REL, mv)
    dp = gpu.GaussPoints(pts)
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.cg_gauss(dp, nugget, db.ptr, dx.ptr, iter_max=20000, eps=1e-10)
    assert info.status == 0
    assert abs(info.iterations - k_ref) <= (band if band >= 1 else band * k_ref)


def test_bicgstab_matches_reference(gpu):
    n = 400
    rng = np.random.default_rng(9)
    A = np.asfortranarray(np.eye(n) * 4 + rng.uniform(-1, 1, (n, n)) / np.sqrt(n))
    b = rng.standard_normal(n)
    x_ref, mv, _ = ref.solve_dense(A, b, np.zeros(n), 500, 1e-12, ref.SOLVER_BICGSTAB)
    dA, db, dx = gpu.DeviceArray.from_numpy(A.ravel(order="F")), gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.bicgstab_dense(n, dA.ptr, db.ptr, dx.ptr, iter_max=500, eps=1e-12)
    k_ref = ref.iterations(ref.SOLVER_BICGSTAB, mv)
    assert info.status == 0
    assert abs(info.iterations - k_ref) <= max(2, int(0.2 * k_ref))
    assert np.allclose(dx.numpy(), x_ref, rtol=1e-8, atol=1e-10)


# The benchmark families at n = 8192: the FP64 CG system of the n = 65536,
# d = 2 configuration (l = 0.05) and the kernel of the n = 131072, d = 3
# mixed configuration (l = 0.08), nugget 1e-4, b = sin(2 pi x1) cos(2 pi x2),
# x0 = 0, relres 1e-10.  The reference runs to convergence (about 4.5 ms per
# iteration on GB300); this library's FP64 count must fall within 3 % of it.
@pytest.mark.parametrize("dim,ell", [(2, 0.05), (3, 0.08)])
def test_gauss_cg_iterations_match_reference_n8192(gpu, dim, ell):
    n = 8192
    prob = synth.gauss_problem(n, dim, ell, 1e-4, seed=0)
    pts, b = prob.scaled(), prob.b
    x_ref, mv, ms = ref.solve_gauss(pts, 1e-4, b, np.zeros(n), 100000, 1e-10, ref.SOLVER_CG_REL)
    k_ref = ref.iterations(ref.SOLVER_CG_REL, mv)
    dp = gpu.GaussPoints(pts)
    db, dx = gpu.DeviceArray.from_numpy(b), gpu.DeviceArray(n)
    dx.zero()
    info = gpu.cg_gauss(dp, 1e-4, db.ptr, dx.ptr, iter_max=100000, eps=1e-10)
    print(f"n={n} d={dim} l={ell}: reference {k_ref} iterations ({ms / 1e3:.1f} s), this library {info.iterations}")
    assert info.status == 0
    assert abs(info.iterations - k_ref) <= 0.03 * k_ref, (info.iterations, k_ref)
