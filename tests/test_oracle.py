"""The CPU oracle against the reference's own known answers.

The only known-answer test the reference ships for this path is
test_library.cpp:50-74,135-151: A(i,j) = j*m + i (column-major index),
x_j = j, y_j = j + 1; dgemv and ddot must match a host computation to a
relative 1e-12.  Here the expected values are the closed forms
  (A x)_i = m * sum_j j^2 + i * sum_j j,   <x, y> = sum_j j (j + 1),
which are exact in FP64 at these sizes, plus the committed fixture
tests/golden/kat_test_library.npz made by tests/golden/make_kat.py.
"""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def kat_inputs(m, n):
    A = np.arange(m * n, dtype=np.float64).reshape((m, n), order="F")
    x = np.arange(n, dtype=np.float64)
    y = x + 1.0
    return A, x, y


def kat_expected(m, n):
    j = np.arange(n, dtype=np.float64)
    i = np.arange(m, dtype=np.float64)
    Ax = m * np.sum(j * j) + i * np.sum(j)
    xy = float(np.sum(j * (j + 1)))
    return Ax, xy


@pytest.mark.parametrize("m,n", [(1, 1), (3, 5), (64, 64), (100, 37), (1000, 999)])
def test_oracle_dgemv_ddot_known_answer(orc, m, n):
    A, x, y = kat_inputs(m, n)
    Ax, xy = kat_expected(m, n)
    got = orc.dgemv(A, x)
    # integers below 2^53: exact
    assert np.array_equal(got, Ax)
    assert orc.ddot(x, y) == xy


def test_oracle_matches_committed_kat_fixture(orc):
    data = np.load(GOLDEN / "kat_test_library.npz")
    for key in [k for k in data.files if k.startswith("Ax_")]:
        m, n = map(int, key[3:].split("x"))
        A, x, y = kat_inputs(m, n)
        rel = np.abs(orc.dgemv(A, x) - data[key]) / np.abs(data[key]).clip(1e-300)
        assert rel.max() <= 1e-12
        xy = float(data[f"xy_{m}x{n}"])
        assert abs(orc.ddot(x, y) - xy) <= 1e-12 * abs(xy)


def test_oracle_gauss_entries_follow_assembler_definition(orc):
    rng = np.random.default_rng(3)
    pts = rng.random((3, 50)) * 4.0
    op = orc.GaussOp(pts, nugget=1e-4)
    for i, j in [(0, 0), (1, 2), (10, 49), (7, 7)]:
        s = np.sum((pts[:, i] - pts[:, j]) ** 2)
        want = np.exp(-np.sqrt(s) ** 2) + (1e-4 if i == j else 0.0)
        assert op.entry(i, j) == pytest.approx(want, rel=1e-15, abs=0)


def test_oracle_kernelcu_nugget_on_duplicates(orc):
    pts = np.array([[0.0, 0.5, 0.0], [1.0, 0.25, 1.0]])  # points 0 and 2 coincide
    op = orc.GaussOp(pts, nugget=0.0, rule=orc.RULE_KERNEL_CU)
    assert op.entry(0, 0) == 1.0 + 1e-8
    assert op.entry(0, 2) == 1.0 + 1e-8
    assert op.entry(0, 1) == pytest.approx(np.exp(-(0.25 + 0.5625)), rel=1e-15)


def test_oracle_gauss_matvec_blocks(orc):
    rng = np.random.default_rng(4)
    pts = rng.random((2, 120)) * 3
    op = orc.GaussOp(pts, nugget=1e-3)
    x = rng.standard_normal(120)
    K = np.array([[op.entry(i, j) for j in range(120)] for i in range(120)])
    assert np.allclose(op.matvec(x), K @ x, rtol=1e-13, atol=1e-13)
    # off-diagonal block with offsets
    y = op.matvec(x[30:100], rows=40, cols=70, roff=10, coff=30)
    assert np.allclose(y, K[10:50, 30:100] @ x[30:100], rtol=1e-13, atol=1e-13)


def test_oracle_cg_tridiagonal_test_cg_case(orc):
    """test_cg.cpp:57-113: (2,-1) tridiagonal SPD, manufactured b, RMS stop."""
    n = 200
    A = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    rng = np.random.default_rng(1235)
    xs = rng.random(n)
    b = A @ xs
    x, k, res, st = orc.cg(orc.DenseOp(A), b, rng.random(n), iter_max=1000, eps=1e-10, stop_rule=1)
    assert st == 0 and res < 1e-10
    assert np.sqrt(np.mean((A @ x - b) ** 2)) < 1e-9
    assert k <= n + 5


def test_oracle_cg_relative_rule_matches_numpy_solution(orc):
    rng = np.random.default_rng(7)
    n = 60
    M = rng.uniform(-1, 1, (n, n))
    A = M.T @ M / n + np.eye(n)
    b = np.ones(n)
    x, k, res, st = orc.cg(orc.DenseOp(A), b, iter_max=500, eps=1e-12)
    assert st == 0
    assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-9, atol=1e-10)
    assert orc.true_relres(orc.DenseOp(A), b, x) < 1e-11


def test_oracle_cg_breakdown_and_cap(orc):
    A = np.diag([1.0, -1.0, 2.0])
    x, k, res, st = orc.cg(orc.DenseOp(A), np.array([1.0, 1.0, 1.0]), iter_max=50, eps=1e-12)
    assert st == 3  # non-positive curvature
    A = np.diag(np.linspace(1, 1e6, 400))
    x, k, res, st = orc.cg(orc.DenseOp(A), np.ones(400), iter_max=5, eps=1e-14)
    assert st == 2 and k == 4


def test_oracle_bicgstab_nonsymmetric(orc):
    rng = np.random.default_rng(5)
    n = 80
    A = np.eye(n) * 4 + rng.uniform(-1, 1, (n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    x, k, res, st = orc.bicgstab(orc.DenseOp(A), b, iter_max=500, eps=1e-12)
    assert st == 0 and res < 1e-12
    assert np.allclose(A @ x, b, atol=1e-10)


def test_oracle_vector_file_format(orc, tmp_path):
    x = np.linspace(-1, 1, 17)
    p = tmp_path / "v.dat"
    assert orc.save_vector(p, x) == 0
    raw = p.read_bytes()
    assert len(raw) == 4 + 8 * 17 and int.from_bytes(raw[:4], "little", signed=True) == 17
    st, y = orc.load_vector(p, 17)
    assert st == 0 and np.array_equal(x, y)
    assert orc.load_vector(p, 16)[0] == -2


def test_oracle_accurate_residual_is_exact_where_plain_fp64_is_not(orc):
    # Columns come in pairs (a v, -a v) with integer products below 2^52,
    # shuffled apart, plus one column of ones with x = 1 and b = 1: the exact
    # residual is 0.  Double-double residual entries recover it exactly; a
    # plain FP64 residual of the same data carries summation noise.
    rng = np.random.default_rng(5)
    pairs, n = 32, 64
    a = rng.integers(1 << 24, 1 << 26, size=(n, pairs)).astype(np.float64)
    v = rng.integers(1 << 24, 1 << 26, size=pairs).astype(np.float64)
    A = np.zeros((n, 2 * pairs + 1))
    A[:, 0:2 * pairs:2] = a
    A[:, 1:2 * pairs:2] = -a
    A[:, -1] = 1.0
    x = np.concatenate([np.repeat(v, 2), [1.0]])
    perm = rng.permutation(2 * pairs + 1)
    A, x = A[:, perm], x[perm]
    op = orc.DenseOp(np.asfortranarray(np.vstack([A, np.zeros((1, 2 * pairs + 1))])))
    b = np.concatenate([np.ones(n), [0.0]])
    assert orc.true_relres_accurate(op, b, x) == 0.0
    assert orc.true_relres(op, b, x) > 1e-3


def test_halton_library_matches_oracle_restatement(native_lib):
    """mgb_halton (host code) against the oracle's restatement, bit for bit,
    and the first points against the definition (radical inverse in the
    prime bases 2, 3, 5)."""
    import mpla_gb300
    import oracle

    for n, dim, start in [(1000, 3, 0), (257, 16, 9), (4096, 2, 123456)]:
        assert np.array_equal(mpla_gb300.halton(n, dim, start), oracle.halton(n, dim, start))
    first = mpla_gb300.halton(4, 3)
    assert np.allclose(first[0], [1 / 2, 1 / 4, 3 / 4, 1 / 8], rtol=0, atol=1e-15)
    assert np.allclose(first[1], [1 / 3, 2 / 3, 1 / 9, 4 / 9], rtol=0, atol=1e-15)
    assert np.allclose(first[2], [1 / 5, 2 / 5, 3 / 5, 4 / 5], rtol=0, atol=1e-15)
