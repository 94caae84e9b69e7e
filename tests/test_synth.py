"""The seeded synthetic workloads (mpla_gb300.synth) on the CPU.

Every benchmark and parity input comes from these generators, so they must
give the same values on every machine: the vectorised counter-based stream
is checked against a scalar splitmix64 written out with Python integers, and
the workloads against the shapes and ranges of their configurations.
"""
import numpy as np

from mpla_gb300 import synth

M64 = (1 << 64) - 1


def _mix(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def _stream(seed, stream, count):
    """A sequential splitmix64 generator started at the stream's base."""
    state = _mix((seed ^ ((stream * 0xD1B54A32D192ED03) & M64)) & M64)
    out = []
    for _ in range(count):
        state = (state + 0x9E3779B97F4A7C15) & M64
        out.append(_mix(state))
    return out


def test_counter_stream_equals_sequential_splitmix64():
    for seed, stream in [(0, 0), (0, 10), (1235, 1), (2**63 + 5, 77)]:
        want = _stream(seed, stream, 40)
        got = synth.u64(seed, stream, 40)
        assert [int(v) for v in got] == want
        # any window of the stream is the same values
        assert [int(v) for v in synth.u64(seed, stream, 7, start=20)] == want[20:27]


def test_uniform_takes_the_top_53_bits():
    raw = synth.u64(3, 4, 1000)
    u = synth.uniform(3, 4, 1000)
    assert np.array_equal(u, (raw >> np.uint64(11)).astype(np.float64) / 2.0**53)
    assert u.min() >= 0.0 and u.max() < 1.0


def test_normal_moments():
    z = synth.normal(7, 1, 200000)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert np.all(np.isfinite(z))


def test_gauss_problem_shapes_and_rhs():
    p = synth.gauss_problem(1000, 2, 0.05, 1e-4, seed=0)
    assert p.points.shape == (2, 1000) and p.b.shape == (1000,)
    x1, x2 = p.points
    assert np.array_equal(p.b, np.sin(2 * np.pi * x1) * np.cos(2 * np.pi * x2))
    assert np.allclose(p.scaled(), p.points / (np.sqrt(2.0) * 0.05), rtol=0, atol=0)
    # the same seed gives the same problem
    assert np.array_equal(synth.gauss_problem(1000, 2, 0.05).points, p.points)


def test_batch_spec_follows_its_configuration():
    spec = synth.batch_spec(512)
    assert len(spec.n) == 512
    assert spec.n.min() >= 256 and spec.n.max() <= 16384
    assert set(np.unique(spec.dim)) <= {2, 3}
    assert spec.ell.min() >= 0.03 and spec.ell.max() <= 0.2
    assert spec.nrhs.min() >= 1 and spec.nrhs.max() <= 8
    # log-uniform sizes: about half of the systems below the geometric mean
    assert 0.4 < np.mean(spec.n < np.sqrt(256 * 16384)) < 0.6
    s7 = synth.batch_system(spec, 7)
    assert s7.points.shape == (int(spec.dim[7]), int(spec.n[7]))
    assert s7.b.shape == (int(spec.n[7]), int(spec.nrhs[7]))


def test_dense_spd_is_symmetric_positive_definite():
    A, b, x0 = synth.dense_spd(64, seed=0)
    assert np.allclose(A, A.T, rtol=0, atol=1e-15)
    assert np.linalg.eigvalsh(A).min() >= 1.0 - 1e-12     # M^T M / n + I
    assert np.array_equal(b, np.ones(64)) and np.array_equal(x0, np.zeros(64))
