"""The oracle against outputs of the reference MPLA itself.

tests/golden/ref_golden.npz holds what the unmodified reference (compiled
from its sources, run on a GB300 by tests/golden/make_ref_golden.py)
returned for the seeded inputs of tests/golden/ref_cases.py.  This pins the
CPU restatement to the reference: dgemv and the kernel matvecs to 1e-13
relative to sum |a_ij x_j|, the erf right-hand sides to 1e-14 of their
maximum, CG iteration counts to +-1 and the solutions to the solver
tolerance.
"""
from pathlib import Path

import numpy as np
import pytest

from tests.golden.ref_cases import cases

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_golden.npz"
pytestmark = pytest.mark.skipif(not GOLDEN.exists(), reason="reference fixtures not generated yet")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def all_cases():
    return cases()


def _rel(got, want, scale):
    scale = np.where(scale == 0, 1.0, scale)
    return float(np.max(np.abs(got - want) / scale))


def test_dgemv_and_ddot(orc, golden, all_cases):
    for name in ["dgemv_300x200", "dgemv_1024"]:
        c = all_cases[name]
        y = orc.dgemv(c["A"], c["x"])
        assert _rel(y, golden[f"{name}/y"], np.abs(c["A"]) @ np.abs(c["x"])) <= 1e-13
        want = float(golden[f"{name}/ddot"])
        assert abs(orc.ddot(c["x"], c["x"] + 1.0) - want) <= 1e-13 * float(np.abs(c["x"]) @ np.abs(c["x"] + 1))


@pytest.mark.parametrize("name", ["gauss_assembler_d2", "gauss_assembler_d3", "gauss_kernelcu_dup"])
def test_kernel_matvecs(orc, golden, all_cases, name):
    c = all_cases[name]
    op = orc.GaussOp(c["pts"], c["nugget"], rule=c["rule"])
    y = op.matvec(c["x"])
    assert _rel(y, golden[f"{name}/y"], op.matvec(np.abs(c["x"]))) <= 1e-13


@pytest.mark.parametrize("name", ["rhs_assembler", "rhs_kernelcu"])
def test_erf_right_hand_sides(orc, golden, all_cases, name):
    c = all_cases[name]
    b = orc.GaussOp(c["pts"], 0.0).rhs()
    want = golden[f"{name}/b"]
    assert np.max(np.abs(b - want)) <= 1e-14 * np.max(np.abs(want))


@pytest.mark.parametrize("name", ["cg_dense_rel", "cg_tridiag_rms", "bicgstab_dense"])
def test_dense_solvers(orc, golden, all_cases, name):
    c = all_cases[name]
    op = orc.DenseOp(c["A"])
    if c["solver"] == 2:
        x, k, res, st = orc.bicgstab(op, c["b"], c["x0"], iter_max=c["iter_max"], eps=c["eps"])
    else:
        x, k, res, st = orc.cg(op, c["b"], c["x0"], iter_max=c["iter_max"], eps=c["eps"],
                               stop_rule=0 if c["solver"] == 0 else 1)
    assert st == 0
    assert abs(k - int(golden[f"{name}/iterations"])) <= 1
    xr = golden[f"{name}/x"]
    assert np.max(np.abs(x - xr)) <= 1e-7 * max(1.0, np.max(np.abs(xr)))


def test_gauss_cg(orc, golden, all_cases):
    c = all_cases["cg_gauss_rel"]
    op = orc.GaussOp(c["pts"], c["nugget"])
    x, k, res, st = orc.cg(op, c["b"], c["x0"], iter_max=c["iter_max"], eps=c["eps"])
    assert st == 0
    assert abs(k - int(golden["cg_gauss_rel/iterations"])) <= 1
    assert orc.true_relres(op, c["b"], golden["cg_gauss_rel/x"]) < 1e-10 * 1.01
