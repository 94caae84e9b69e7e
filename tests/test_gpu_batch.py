"""The batched multi-system, multi-RHS CG engine.

Every right-hand side of every system reaches the FP64 true relative
residual 1e-10, re-checked by the oracle; FP64 systems follow the oracle's
CG iteration count; a system's result is bitwise the same whether it is
solved alone or inside a batch (its kernels and reduction order do not
depend on the other systems); systems can be added while others run;
admission refuses systems that do not fit in free device memory.

Residuals are re-checked with the oracle's double-double residual
(true_relres_accurate).  On these systems x reaches ~1e4 ||b||, so a plain
FP64 evaluation of ||b - K x|| carries ~1e-10 of summation noise -- the
tolerance itself; the engine's replacement residual is double-double too.
Mixed lanes must certify relres < 1e-10 (the oracle may differ by the
rounding of the FP64 entries, ~1e-11: 1.2e-10 allowed).  FP64 lanes stop on
the recursive residual like the reference's CG (src/mpla.cpp:960-975); their
true residual drifts from it by O(u kappa), so they are held to 1e-8.
"""
import numpy as np
import pytest

from mpla_gb300 import synth

pytestmark = pytest.mark.gpu

EPS = 1e-10
MIXED_ORACLE_TOL = 1.2e-10
FP64_ORACLE_TOL = 1e-8


def make_system(seed, n, dim, ell, nrhs):
    pts = synth.gauss_points(n, dim, seed) / (np.sqrt(2.0) * ell)
    b = np.stack([synth.normal(seed, 500 + k, n) for k in range(nrhs)], axis=1)
    return pts, b


SPECS = [  # seed, n, dim, ell, nrhs, precision (1 = mixed)
    (1, 300, 2, 0.05, 1, 1),
    (2, 1100, 3, 0.08, 3, 1),
    (3, 2000, 2, 0.1, 8, 1),
    (4, 700, 3, 0.2, 5, 1),
    (5, 900, 2, 0.05, 2, 0),
    (6, 512, 3, 0.1, 1, 0),
]


def check_solution(orc, pts, b, x, infos, precision, nugget=1e-4):
    op = orc.GaussOp(pts, nugget)
    for k in range(b.shape[1]):
        assert infos[k].status == 0, infos[k].as_dict()
        assert infos[k].final_res < EPS
        rel = orc.true_relres_accurate(op, b[:, k], x[:, k])
        assert rel < (MIXED_ORACLE_TOL if precision == 1 else FP64_ORACLE_TOL), (k, rel)


def test_batch_solves_every_rhs(gpu, orc):
    batch = gpu.Batch(64)
    systems = {}
    for seed, n, dim, ell, nrhs, prec in SPECS:
        pts, b = make_system(seed, n, dim, ell, nrhs)
        h = batch.add(pts, 1e-4, b, precision=prec, iter_max=100000)
        systems[h] = (pts, b, prec)
    assert batch.run() == 0
    assert sorted(batch.finished()) == sorted(systems)
    for h, (pts, b, prec) in systems.items():
        x, infos = batch.result(h, b.shape[0], b.shape[1])
        check_solution(orc, pts, b, x, infos, prec)
        if prec == 1:
            assert all(i.fp64_matvecs >= 1 and i.true_relres < EPS for i in infos)
    rpt, ms = batch.tuning()
    assert all(r in (0, 1, 2, 4) for r in rpt) and any(r in (1, 2, 4) for r in rpt)
    batch.close()


def test_fp64_batch_iterations_follow_the_oracle(gpu, orc):
    pts, b = make_system(7, 800, 2, 0.03, 2)
    batch = gpu.Batch(4)
    h = batch.add(pts, 1e-2, b, precision=gpu.PREC_FP64, iter_max=20000)
    batch.run()
    x, infos = batch.result(h, 800, 2)
    op = orc.GaussOp(pts, 1e-2)
    for k in range(2):
        _, ko, _, _ = orc.cg(op, b[:, k], iter_max=20000, eps=EPS)
        assert abs(infos[k].iterations - ko) <= max(1, int(0.01 * ko))
    batch.close()


def test_result_is_the_same_alone_and_in_the_mix(gpu):
    pts, b = make_system(8, 1500, 3, 0.08, 3)
    alone = gpu.Batch(4)
    h = alone.add(pts, 1e-4, b)
    alone.run()
    x_alone, i_alone = alone.result(h, 1500, 3)
    alone.close()
    mix = gpu.Batch(32)
    for seed, n, dim, ell, nrhs, prec in SPECS:
        p2, b2 = make_system(seed, n, dim, ell, nrhs)
        mix.add(p2, 1e-4, b2, precision=prec)
    h2 = mix.add(pts, 1e-4, b)
    mix.run()
    x_mix, i_mix = mix.result(h2, 1500, 3)
    mix.close()
    assert np.array_equal(x_alone, x_mix)
    assert [i.iterations for i in i_alone] == [i.iterations for i in i_mix]


def test_continuous_admission_while_running(gpu, orc):
    batch = gpu.Batch(16)
    pts1, b1 = make_system(9, 2500, 2, 0.05, 2)
    h1 = batch.add(pts1, 1e-4, b1)
    active = batch.run(max_steps=200)  # partly solved
    assert active == 1
    pts2, b2 = make_system(10, 600, 3, 0.1, 4)
    h2 = batch.add(pts2, 1e-4, b2)
    assert batch.run() == 0
    for h, pts, b in [(h1, pts1, b1), (h2, pts2, b2)]:
        x, infos = batch.result(h, b.shape[0], b.shape[1])
        check_solution(orc, pts, b, x, infos, 1)
    batch.close()


def test_slots_are_reused_after_release(gpu, orc):
    batch = gpu.Batch(2)
    for rnd in range(3):
        pts, b = make_system(20 + rnd, 400 + 100 * rnd, 2 + rnd % 2, 0.1, 1 + rnd)
        h = batch.add(pts, 1e-4, b, precision=rnd % 2)
        assert batch.run() == 0
        x, infos = batch.result(h, b.shape[0], b.shape[1])
        check_solution(orc, pts, b, x, infos, rnd % 2)
    batch.close()


def test_admission_refuses_when_memory_is_short(gpu):
    pts, b = make_system(11, 256, 2, 0.1, 1)
    batch = gpu.Batch(4)
    with pytest.raises(gpu.MplaError) as e:
        batch.add(pts, 1e-4, b, reserve_bytes=1 << 62)
    assert e.value.status == gpu.MGB_ERR_NOMEM
    with pytest.raises(gpu.MplaError) as e:
        batch.add(pts, 1e-4, np.zeros((256, 9)))
    assert e.value.status == gpu.MGB_ERR_ARG
    batch.close()


def test_batch_edge_cases(gpu, orc):
    batch = gpu.Batch(8)
    # one point: K = 1 + nugget, x = b / (1 + nugget)
    p1 = np.array([[0.3], [0.7]])
    b1 = np.array([[2.0, -1.0]])
    h1 = batch.add(p1, 1e-4, b1, precision=gpu.PREC_MIXED)
    # 129 points (one full tile and one row), 8 right-hand sides, one of them 0
    p2, b2 = make_system(31, 129, 3, 0.1, 8)
    b2[:, 5] = 0.0
    h2 = batch.add(p2, 1e-4, b2, precision=gpu.PREC_MIXED)
    # iteration cap of 1: nothing runs, reported as not converged
    p3, b3 = make_system(32, 200, 2, 0.1, 1)
    h3 = batch.add(p3, 1e-4, b3, precision=gpu.PREC_FP64, iter_max=1)
    assert batch.run() == 0
    x1, i1 = batch.result(h1, 1, 2)
    assert all(i.status == 0 for i in i1)
    assert np.allclose(x1[0], b1[0] / (1.0 + 1e-4), rtol=1e-12)
    x2, i2 = batch.result(h2, 129, 8)
    assert i2[5].status == 0 and i2[5].iterations == 0 and np.all(x2[:, 5] == 0.0)
    b2_nz = [k for k in range(8) if k != 5]
    check_solution(orc, p2, b2[:, b2_nz], x2[:, b2_nz], [i2[k] for k in b2_nz], 1)
    _, i3 = batch.result(h3, 200, 1)
    assert i3[0].status == gpu.MGB_ERR_NOTCONV
    for bad in [dict(points=np.zeros((4, 10)), b=np.ones(10)),       # dim 4
                dict(points=np.zeros((2, 10)), b=np.ones((10, 0)))]:  # no right-hand side
        with pytest.raises(gpu.MplaError) as e:
            batch.add(bad["points"], 1e-4, bad["b"])
        assert e.value.status == gpu.MGB_ERR_ARG
    batch.close()
