"""ctypes binding of the compiled reference MPLA (oracle/_ref/libmplaref.so).

TEST INFRASTRUCTURE: the unmodified reference, built from its sources by
oracle/build_ref.py and driven through its public API by ref_harness.cu.
Used to pin the oracle (fixtures in tests/golden/) and, live on a GPU, to
compare the reference with this library; also bench.py's reference arm.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libmplaref.so"

SOLVER_CG_REL = 0   # mpla_generic_conjugate_gradient_with_checkpoint_restart
SOLVER_CG_RMS = 1   # mpla_generic_conjugate_gradient
SOLVER_BICGSTAB = 2

_lib = None


def available() -> bool:
    return LIB_PATH.exists()


def lib(device: int = 0):
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"reference MPLA not built: {LIB_PATH}")
        L = C.CDLL(str(LIB_PATH))
        P, I, D = C.c_void_p, C.c_int, C.c_double
        L.ref_init.argtypes = [I]
        L.ref_dgemv.argtypes = [I, I, P, P, P, I, C.POINTER(D)]
        L.ref_ddot.argtypes = [I, P, P, C.POINTER(D)]
        L.ref_cublas_dgemv.argtypes = [I, P, I, C.POINTER(D)]
        L.ref_solve_dense.argtypes = [I, P, P, P, I, D, I, C.POINTER(I), C.POINTER(D)]
        L.ref_gauss_matvec.argtypes = [I, I, P, D, I, P, P]
        L.ref_gauss_rhs.argtypes = [I, I, P, I, P]
        L.ref_solve_gauss.argtypes = [I, I, P, D, P, P, I, D, I, C.POINTER(I), C.POINTER(D)]
        L.ref_cg_gauss_sample.argtypes = [I, I, P, D, P, I, D, C.POINTER(D), C.POINTER(I)]
        if L.ref_init(device) != 0:
            raise RuntimeError("reference MPLA could not initialise the device")
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def dgemv(A: np.ndarray, x: np.ndarray, reps: int = 0):
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    x = _f(x)
    y = np.empty(m)
    ms = C.c_double()
    assert lib().ref_dgemv(m, n, A.ctypes.data, x.ctypes.data, y.ctypes.data, reps, C.byref(ms)) == 0
    return y, ms.value


def cublas_dgemv_ms(A: np.ndarray, reps: int = 50) -> float:
    """Mean ms of the reference's own cublasDgemv call (mpla.cpp:729) on a
    resident square matrix."""
    A = np.asfortranarray(A, dtype=np.float64)
    ms = C.c_double()
    assert lib().ref_cublas_dgemv(A.shape[0], A.ctypes.data, reps, C.byref(ms)) == 0
    return ms.value


def ddot(x, y) -> float:
    x, y = _f(x), _f(y)
    out = C.c_double()
    assert lib().ref_ddot(x.size, x.ctypes.data, y.ctypes.data, C.byref(out)) == 0
    return out.value


def solve_dense(A, b, x0, iter_max, eps, solver):
    """Returns (x, matvecs, ms); CG iterations = matvecs - 1, BiCGSTAB = (matvecs - 1) / 3."""
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    b = _f(b)
    x = np.array(x0, dtype=np.float64, copy=True)
    mv, ms = C.c_int(), C.c_double()
    assert lib().ref_solve_dense(n, A.ctypes.data, b.ctypes.data, x.ctypes.data, iter_max, eps, solver,
                                 C.byref(mv), C.byref(ms)) == 0
    return x, mv.value, ms.value


def gauss_matvec(pts, nugget, rule, x):
    pts = _f(pts)
    dim, n = pts.shape
    x = _f(x)
    y = np.empty(n)
    assert lib().ref_gauss_matvec(n, dim, pts.ctypes.data, nugget, rule, x.ctypes.data, y.ctypes.data) == 0
    return y


def gauss_rhs(pts, rule):
    pts = _f(pts)
    dim, n = pts.shape
    b = np.empty(n)
    assert lib().ref_gauss_rhs(n, dim, pts.ctypes.data, rule, b.ctypes.data) == 0
    return b


def solve_gauss(pts, nugget, b, x0, iter_max, eps, solver):
    pts = _f(pts)
    dim, n = pts.shape
    b = _f(b)
    x = np.array(x0, dtype=np.float64, copy=True)
    mv, ms = C.c_int(), C.c_double()
    assert lib().ref_solve_gauss(n, dim, pts.ctypes.data, nugget, b.ctypes.data, x.ctypes.data, iter_max, eps,
                                 solver, C.byref(mv), C.byref(ms)) == 0
    return x, mv.value, ms.value


def iterations(solver: int, matvecs: int) -> int:
    """Krylov iterations from the number of core calls (one for r0)."""
    return (matvecs - 1) // 3 if solver == SOLVER_BICGSTAB else matvecs - 1
