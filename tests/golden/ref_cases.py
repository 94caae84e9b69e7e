"""Seeded inputs of the reference fixtures (tests/golden/ref_golden.npz).

Shared by the generator (make_ref_golden.py, run against the compiled
reference on a GPU) and by the tests that compare the oracle and the library
with the stored reference outputs.
"""
import numpy as np

from mpla_gb300 import synth


def _scaled(n, dim, ell, seed):
    return synth.gauss_points(n, dim, seed) / (np.sqrt(2.0) * ell)


def cases():
    c = {}
    rng = np.random.default_rng(2024)
    A = np.asfortranarray(rng.uniform(-1, 1, (300, 200)))
    c["dgemv_300x200"] = dict(kind="dgemv", A=A, x=rng.uniform(-1, 1, 200))
    A = np.asfortranarray(rng.standard_normal((1024, 1024)))
    c["dgemv_1024"] = dict(kind="dgemv", A=A, x=rng.standard_normal(1024))
    c["gauss_assembler_d2"] = dict(kind="gauss_matvec", pts=_scaled(500, 2, 0.05, 31), nugget=1e-3, rule=0,
                                   x=rng.standard_normal(500))
    c["gauss_assembler_d3"] = dict(kind="gauss_matvec", pts=_scaled(400, 3, 0.1, 32), nugget=1e-4, rule=0,
                                   x=rng.standard_normal(400))
    dup = _scaled(300, 3, 0.1, 33)
    dup[:, 150:] = dup[:, :150]
    c["gauss_kernelcu_dup"] = dict(kind="gauss_matvec", pts=dup, nugget=0.0, rule=1, x=rng.standard_normal(300))
    unit = synth.gauss_points(200, 3, 34)
    c["rhs_assembler"] = dict(kind="gauss_rhs", pts=unit, rule=0)
    c["rhs_kernelcu"] = dict(kind="gauss_rhs", pts=unit, rule=1)
    As, b, x0 = synth.dense_spd(200, seed=35)
    c["cg_dense_rel"] = dict(kind="dense_solve", A=As, b=b, x0=x0, iter_max=1000, eps=1e-10, solver=0)
    T = 2 * np.eye(100) - np.eye(100, k=1) - np.eye(100, k=-1)
    rr = np.random.default_rng(1235)
    c["cg_tridiag_rms"] = dict(kind="dense_solve", A=np.asfortranarray(T), b=T @ rr.random(100), x0=rr.random(100),
                               iter_max=1000, eps=1e-10, solver=1)
    An = np.asfortranarray(np.eye(150) * 4 + rng.uniform(-1, 1, (150, 150)) / np.sqrt(150))
    c["bicgstab_dense"] = dict(kind="dense_solve", A=An, b=rng.standard_normal(150), x0=np.zeros(150),
                               iter_max=500, eps=1e-12, solver=2)
    pts = _scaled(600, 2, 0.03, 36)
    c["cg_gauss_rel"] = dict(kind="gauss_solve", pts=pts, nugget=1e-2,
                             b=synth.sincos_rhs(synth.gauss_points(600, 2, 36)), x0=np.zeros(600),
                             iter_max=5000, eps=1e-10, solver=0)
    return c
