"""CPU oracle of the MPLA hot path — TEST INFRASTRUCTURE, never the product.

ctypes binding of ``mpla_oracle.c`` (an FP64 restatement of the reference
algorithms: dgemv, ddot, the Gaussian kernel entries and matvec, CG with both
stopping rules, BiCGSTAB, the erf right-hand side, the vector file format).
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
it, and only to check results against.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

RULE_DIAGONAL = 0
RULE_KERNEL_CU = 1


class Operator(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("n", C.c_int),
        ("A", C.c_void_p),
        ("lda", C.c_long),
        ("dim", C.c_int),
        ("coords", C.c_void_p),
        ("ld", C.c_long),
        ("nugget", C.c_double),
        ("rule", C.c_int),
    ]


_lib = None


def build() -> Path:
    """Compile the oracle (gcc, OpenMP, no FP contraction)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P, I, D, Lg = C.c_void_p, C.c_int, C.c_double, C.c_long
        L.orc_dgemv.argtypes = [I, I, P, Lg, P, P]
        L.orc_ddot.argtypes = [I, P, P]
        L.orc_ddot.restype = D
        L.orc_gauss_entry_assembler.argtypes = [P, Lg, I, I, I, D]
        L.orc_gauss_entry_assembler.restype = D
        L.orc_gauss_entry_kernelcu.argtypes = [P, Lg, I, I, I]
        L.orc_gauss_entry_kernelcu.restype = D
        L.orc_gauss_matvec.argtypes = [I, I, I, I, I, P, Lg, D, I, P, P]
        L.orc_gauss_rhs.argtypes = [I, I, I, P, Lg, P]
        L.orc_cg.argtypes = [C.POINTER(Operator), P, P, I, D, I, C.POINTER(D), C.POINTER(I), P]
        L.orc_cg.restype = I
        L.orc_bicgstab.argtypes = [C.POINTER(Operator), P, P, I, D, C.POINTER(D), C.POINTER(I), P]
        L.orc_bicgstab.restype = I
        L.orc_true_relres.argtypes = [C.POINTER(Operator), P, P]
        L.orc_true_relres.restype = D
        L.orc_true_relres_accurate.argtypes = [C.POINTER(Operator), P, P]
        L.orc_true_relres_accurate.restype = D
        L.orc_apply.argtypes = [C.POINTER(Operator), P, P]
        L.orc_save_vector.argtypes = [C.c_char_p, I, P]
        L.orc_load_vector.argtypes = [C.c_char_p, I, P]
        _lib = L
    return _lib


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def dgemv(A: np.ndarray, x: np.ndarray) -> np.ndarray:
    """y = A x for a column-major (Fortran-ordered) matrix."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    x = _f64(x)
    y = np.empty(m)
    lib().orc_dgemv(m, n, A.ctypes.data, m, x.ctypes.data, y.ctypes.data)
    return y


def ddot(x, y) -> float:
    x, y = _f64(x), _f64(y)
    return lib().orc_ddot(x.size, x.ctypes.data, y.ctypes.data)


class GaussOp:
    """Gaussian kernel operator on scaled points (structure of arrays)."""

    def __init__(self, scaled_points: np.ndarray, nugget: float, rule: int = RULE_DIAGONAL):
        self.pts = _f64(scaled_points)
        self.dim, self.n = self.pts.shape
        self.nugget = float(nugget)
        self.rule = rule
        self.op = Operator(1, self.n, None, 0, self.dim, self.pts.ctypes.data, self.n, self.nugget, rule)

    def entry(self, i: int, j: int) -> float:
        if self.rule == RULE_KERNEL_CU:
            return lib().orc_gauss_entry_kernelcu(self.pts.ctypes.data, self.n, self.dim, i, j)
        return lib().orc_gauss_entry_assembler(self.pts.ctypes.data, self.n, self.dim, i, j, self.nugget)

    def matvec(self, x, rows=None, cols=None, roff=0, coff=0) -> np.ndarray:
        rows = self.n if rows is None else rows
        cols = self.n if cols is None else cols
        x = _f64(x)
        y = np.empty(rows)
        lib().orc_gauss_matvec(rows, cols, roff, coff, self.dim, self.pts.ctypes.data, self.n, self.nugget,
                               self.rule, x.ctypes.data, y.ctypes.data)
        return y

    def rhs(self) -> np.ndarray:
        b = np.empty(self.n)
        lib().orc_gauss_rhs(self.n, 0, self.dim, self.pts.ctypes.data, self.n, b.ctypes.data)
        return b


class DenseOp:
    def __init__(self, A: np.ndarray):
        self.A = np.asfortranarray(A, dtype=np.float64)
        self.n = self.A.shape[0]
        self.op = Operator(0, self.n, self.A.ctypes.data, self.n, 0, None, 0, 0.0, 0)

    def matvec(self, x) -> np.ndarray:
        return dgemv(self.A, x)


def cg(op, b, x0=None, iter_max=1000, eps=1e-10, stop_rule=0, history=False):
    """Returns (x, iterations, final_res, status[, hist])."""
    b = _f64(b)
    x = np.zeros(op.n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    res, st = C.c_double(), C.c_int()
    hist = np.full(iter_max + 1, np.nan) if history else None
    k = lib().orc_cg(C.byref(op.op), b.ctypes.data, x.ctypes.data, iter_max, eps, stop_rule, C.byref(res),
                     C.byref(st), hist.ctypes.data if history else None)
    out = (x, k, res.value, st.value)
    return out + (hist,) if history else out


def bicgstab(op, b, x0=None, iter_max=1000, eps=1e-10, history=False):
    b = _f64(b)
    x = np.zeros(op.n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    res, st = C.c_double(), C.c_int()
    hist = np.full(iter_max + 1, np.nan) if history else None
    k = lib().orc_bicgstab(C.byref(op.op), b.ctypes.data, x.ctypes.data, iter_max, eps, C.byref(res), C.byref(st),
                           hist.ctypes.data if history else None)
    out = (x, k, res.value, st.value)
    return out + (hist,) if history else out


_PRIMES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53)


def halton(n: int, dim: int, start: int = 0) -> np.ndarray:
    """Halton points (dim x n): coordinate d of point i is the radical inverse
    of start + i + 1 in the d-th prime base, digits least significant first,
    f *= 1/base per digit (the operation order of the library).  The point
    set of generate_quadrature_weights.cpp:107-130, whose GSL generator is
    not available here: this restates the published definition."""
    out = np.empty((dim, n))
    for d in range(dim):
        base = _PRIMES[d]
        inv = 1.0 / base
        k = np.arange(start + 1, start + n + 1, dtype=np.int64)
        f = np.full(n, inv)
        x = np.zeros(n)
        while np.any(k > 0):
            x = x + f * (k % base).astype(np.float64)
            k = k // base
            f = f * inv
        out[d] = x
    return out


def true_relres(op, b, x) -> float:
    b, x = _f64(b), _f64(x)
    return lib().orc_true_relres(C.byref(op.op), b.ctypes.data, x.ctypes.data)


def true_relres_accurate(op, b, x) -> float:
    """||b - A x|| / ||b|| with compensated (double-double) residual entries."""
    b, x = _f64(b), _f64(x)
    return lib().orc_true_relres_accurate(C.byref(op.op), b.ctypes.data, x.ctypes.data)


def save_vector(path: str, x) -> int:
    x = _f64(x)
    return lib().orc_save_vector(str(path).encode(), x.size, x.ctypes.data)


def load_vector(path: str, n: int):
    x = np.empty(n)
    st = lib().orc_load_vector(str(path).encode(), n, x.ctypes.data)
    return st, x
