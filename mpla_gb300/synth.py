"""Seeded synthetic workloads of the GB300 MPLA hot path.

A counter-based splitmix64 stream gives the same bytes on every machine and
in every process: value i of stream (seed, stream_id) is
``mix(base(seed, stream_id) + (i + 1) * GOLDEN)``, i.e. exactly the i-th
output of a sequential splitmix64 generator started at ``base``.  Uniform
doubles take the top 53 bits.

Workloads (the reference publishes no dataset; all inputs are synthetic):
  dense_spd   n x n, A = M^T M / n + I, M_ij ~ U[-1, 1]; b = 1, x0 = 0
  gauss       n points ~ U[0,1]^d, Gaussian kernel of length scale l with a
              nugget, b_i = sin(2 pi x_i1) cos(2 pi x_i2)
  batch       many Gaussian systems of log-uniform size with several
              right-hand sides b ~ N(0, 1)
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_STREAM = np.uint64(0xD1B54A32D192ED03)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _base(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        s = np.array([np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ (np.uint64(stream) * _STREAM)], dtype=np.uint64)
    return _mix(s)[0]


def u64(seed: int, stream: int, count: int, start: int = 0) -> np.ndarray:
    """Raw 64-bit values i = start .. start+count-1 of stream (seed, stream)."""
    i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = _base(seed, stream) + i * GOLDEN
    return _mix(z)


def uniform(seed: int, stream: int, count: int, start: int = 0) -> np.ndarray:
    """Doubles in [0, 1) from the top 53 bits."""
    return (u64(seed, stream, count, start) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, count: int) -> np.ndarray:
    """N(0,1) by Box-Muller on two interleaved uniform streams."""
    u1 = uniform(seed, stream, count)
    u2 = uniform(seed, stream + 0x10000, count)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


# ------------------------------------------------------------------ dense SPD
def dense_matrix_m(n: int, seed: int = 0) -> np.ndarray:
    """M with entries U[-1, 1], column-major order of the stream (Fortran array)."""
    return (2.0 * uniform(seed, 1, n * n) - 1.0).reshape((n, n), order="F")


def dense_spd(n: int, seed: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """A = M^T M / n + I (Fortran order), b = 1, x0 = 0."""
    M = dense_matrix_m(n, seed)
    A = np.asfortranarray(M.T @ M / n + np.eye(n))
    return A, np.ones(n), np.zeros(n)


# ---------------------------------------------------------------- Gaussian
@dataclass
class GaussProblem:
    """Points (structure of arrays, unscaled) and the system parameters."""

    points: np.ndarray   # shape (dim, n), in [0, 1)
    ell: float
    nugget: float
    b: np.ndarray        # shape (n,) or (n, r)

    @property
    def n(self) -> int:
        return self.points.shape[1]

    @property
    def dim(self) -> int:
        return self.points.shape[0]

    def scaled(self) -> np.ndarray:
        """Points scaled by 1/(sqrt(2) l), so that K = exp(-|p_i - p_j|^2)."""
        return np.ascontiguousarray(self.points / (math.sqrt(2.0) * self.ell))


def gauss_points(n: int, dim: int, seed: int = 0, stream0: int = 10) -> np.ndarray:
    return np.stack([uniform(seed, stream0 + d, n) for d in range(dim)])


def sincos_rhs(points: np.ndarray) -> np.ndarray:
    """b_i = sin(2 pi x_i1) cos(2 pi x_i2) (x_i2 = 0 in one dimension)."""
    x1 = points[0]
    x2 = points[1] if points.shape[0] > 1 else np.zeros_like(x1)
    return np.sin(2.0 * np.pi * x1) * np.cos(2.0 * np.pi * x2)


def gauss_problem(n: int, dim: int, ell: float, nugget: float = 1e-4, seed: int = 0) -> GaussProblem:
    pts = gauss_points(n, dim, seed)
    return GaussProblem(points=pts, ell=ell, nugget=nugget, b=sincos_rhs(pts))


# Named configurations of the hot path (sizes as in the benchmark plan).
def config_dense(seed: int = 0):
    return dense_spd(4096, seed)


def config_gauss_fp64(seed: int = 0) -> GaussProblem:
    return gauss_problem(65536, 2, 0.05, 1e-4, seed)


def config_gauss_mixed(seed: int = 0) -> GaussProblem:
    return gauss_problem(131072, 3, 0.08, 1e-4, seed)


@dataclass
class BatchSpec:
    n: np.ndarray      # sizes
    dim: np.ndarray    # 2 or 3
    ell: np.ndarray    # length scales
    nrhs: np.ndarray   # right-hand sides per system


def batch_spec(count: int = 512, n_lo: int = 256, n_hi: int = 16384, rhs_hi: int = 8, seed: int = 0,
               ell_lo: float = 0.03, ell_hi: float = 0.2) -> BatchSpec:
    u = uniform(seed, 100, count)
    n = np.floor(np.exp(np.log(n_lo) + u * (np.log(n_hi) - np.log(n_lo)))).astype(np.int64)
    n = np.clip(n, n_lo, n_hi)
    dim = 2 + (uniform(seed, 101, count) >= 0.5).astype(np.int64)
    ell = ell_lo + (ell_hi - ell_lo) * uniform(seed, 102, count)
    nrhs = 1 + np.floor(uniform(seed, 103, count) * rhs_hi).astype(np.int64)
    nrhs = np.clip(nrhs, 1, rhs_hi)
    return BatchSpec(n=n, dim=dim, ell=ell, nrhs=nrhs)


def batch_system(spec: BatchSpec, k: int, seed: int = 0) -> GaussProblem:
    """System k of a batch: its own point and right-hand-side streams."""
    n, d, r = int(spec.n[k]), int(spec.dim[k]), int(spec.nrhs[k])
    pts = np.stack([uniform(seed, 1000 + 16 * k + j, n) for j in range(d)])
    b = np.stack([normal(seed, 1_000_000 + 16 * k + j, n) for j in range(r)], axis=1)
    return GaussProblem(points=pts, ell=float(spec.ell[k]), nugget=1e-4, b=b)


def serving_requests(rate: float, window: float, seed: int = 0, n_lo: int = 1024, n_hi: int = 32768):
    """Requests of the serving workload: Poisson arrival times at `rate` per
    second over [0, window), n log-uniform in [n_lo, n_hi], d in {2, 3},
    l ~ U[0.03, 0.2], nugget 1e-4, 1-4 N(0,1) right-hand sides, precision
    alternating FP64 (0) / mixed (1).  Returns (arrival, id, scaled points
    dim x n, b n x r, precision) tuples."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > window:
            break
        k = len(out)
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        dim = 2 + int(rng.random() < 0.5)
        ell = float(rng.uniform(0.03, 0.2))
        r = int(rng.integers(1, 5))
        pts = np.stack([uniform(seed, 5000 + 16 * k + j, n) for j in range(dim)]) / (math.sqrt(2.0) * ell)
        b = np.stack([normal(seed, 6_000_000 + 16 * k + j, n) for j in range(r)], axis=1)
        out.append((t, k, pts, b, k % 2))
    return out
