"""GB300-native implementation of MPLA's data-parallel hot path.

The native library ``lib/libmpla.so`` (built from ``csrc/`` by ``_build.py``)
exports the drop-in mpla.h C++ API and the C ABI of ``include/mpla_gb300.h``.
This module binds the C ABI with ctypes: device buffers, the dense dgemv /
dot / axpy, the fused Gaussian kernel matvecs and the CG / BiCGSTAB solvers.
There is no CPU fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libmpla.so"

MGB_OK = 0
MGB_ERR_CUDA = 1
MGB_ERR_ARG = 2
MGB_ERR_NOMEM = 3
MGB_ERR_BREAKDOWN = 4
MGB_ERR_NOTCONV = 5
MGB_ERR_NODEV = 6
MGB_ERR_TIMEOUT = 7
MGB_ERR_IO = 8

NUGGET_DIAGONAL = 0
NUGGET_KERNEL_CU = 1
STOP_RELATIVE = 0
STOP_RMS = 1
PREC_FP64 = 0
PREC_MIXED = 1
MIXED_TENSOR = 0
MIXED_SIMT = 1
BATCH_CLASSES = 12  # MGB_BATCH_CLASSES

# Every C-ABI symbol declared in include/mpla_gb300.h (checked by the tests).
C_ABI_SYMBOLS = (
    "mgb_version", "mgb_last_error", "mgb_init", "mgb_shutdown", "mgb_device_sync",
    "mgb_malloc", "mgb_free", "mgb_memcpy_htod", "mgb_memcpy_dtoh", "mgb_memset",
    "mgb_host_alloc", "mgb_host_free",
    "mgb_dgemv", "mgb_dgemv_noalloc", "mgb_ddot", "mgb_daxpy",
    "mgb_gauss_matvec_f64", "mgb_gauss_matvec_mixed", "mgb_gauss_entries_f64",
    "mgb_cg_dense", "mgb_bicgstab_dense", "mgb_cg_gauss", "mgb_bicgstab_gauss", "mgb_cg_gauss_host",
    "mgb_kernel_launches", "mgb_time_gauss_matvec", "mgb_time_dgemv",
    "mgb_save_vector", "mgb_load_vector",
    "mgb_batch_create", "mgb_batch_add", "mgb_batch_run", "mgb_batch_run_async", "mgb_batch_wait", "mgb_batch_ready",
    "mgb_batch_finished", "mgb_batch_result",
    "mgb_batch_tuning", "mgb_batch_destroy",
    "mgb_set_mixed_matvec", "mgb_get_mixed_matvec", "mgb_gauss_mixed_work", "mgb_gauss_fp64_work",
    "mgb_register_generic_device_code", "mgb_unregister_generic_device_code",
    "mgb_halton",
)


class MplaError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class SolveInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("status", C.c_int),
        ("final_res", C.c_double),
        ("true_relres", C.c_double),
        ("fp64_matvecs", C.c_int),
        ("low_matvecs", C.c_int),
        ("seconds", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_SIGS = {
    "mgb_version": (_I, []),
    "mgb_last_error": (C.c_char_p, []),
    "mgb_init": (_I, [_I]),
    "mgb_shutdown": (_I, []),
    "mgb_device_sync": (_I, []),
    "mgb_malloc": (_I, [C.POINTER(_P), C.c_size_t]),
    "mgb_free": (_I, [_P]),
    "mgb_memcpy_htod": (_I, [_P, _P, C.c_size_t]),
    "mgb_memcpy_dtoh": (_I, [_P, _P, C.c_size_t]),
    "mgb_memset": (_I, [_P, _I, C.c_size_t]),
    "mgb_host_alloc": (_I, [C.POINTER(_P), C.c_size_t]),
    "mgb_host_free": (_I, [_P]),
    "mgb_dgemv": (_I, [_I, _I, _P, _I, _P, _P, _P]),
    "mgb_dgemv_noalloc": (_I, [_I, _I, _P, _I, _P, _P, _P]),
    "mgb_ddot": (_I, [_I, _P, _P, C.POINTER(_D), _P]),
    "mgb_daxpy": (_I, [_I, _D, _P, _P, _P]),
    "mgb_gauss_matvec_f64": (_I, [_I, _I, _I, _I, _I, _P, _D, _I, _P, _P, _P]),
    "mgb_gauss_matvec_mixed": (_I, [_I, _I, _P, _D, _P, _P, _P]),
    "mgb_gauss_entries_f64": (_I, [_I, _I, _P, _P, _I, _P, _D, _I, _P, _P]),
    "mgb_cg_dense": (_I, [_I, _P, _I, _P, _P, _I, _D, _I, C.POINTER(SolveInfo), _P]),
    "mgb_bicgstab_dense": (_I, [_I, _P, _I, _P, _P, _I, _D, C.POINTER(SolveInfo), _P]),
    "mgb_cg_gauss": (_I, [_I, _I, _P, _D, _I, _P, _P, _I, _D, _I, _I, C.POINTER(SolveInfo), _P]),
    "mgb_bicgstab_gauss": (_I, [_I, _I, _P, _D, _I, _P, _P, _I, _D, C.POINTER(SolveInfo), _P]),
    "mgb_cg_gauss_host": (_I, [_I, _I, _P, _D, _P, _P, _I, _D, _I, C.POINTER(SolveInfo)]),
    "mgb_kernel_launches": (C.c_longlong, []),
    "mgb_time_gauss_matvec": (_I, [_I, _I, _P, _D, _I, _P, _P, _I, C.POINTER(_D), _P]),
    "mgb_time_dgemv": (_I, [_I, _P, _P, _P, _I, C.POINTER(_D), _P]),
    "mgb_save_vector": (_I, [C.c_char_p, _I, _P]),
    "mgb_register_generic_device_code": (_I, [_P]),
    "mgb_halton": (_I, [_I, _I, C.c_longlong, _P]),
    "mgb_unregister_generic_device_code": (_I, [_P]),
    "mgb_load_vector": (_I, [C.c_char_p, _I, _P]),
    "mgb_batch_create": (_I, [_I, C.POINTER(_P)]),
    "mgb_batch_add": (_I, [_P, _I, _I, _P, _D, _I, _P, _I, _D, _I, C.c_size_t, C.POINTER(_I)]),
    "mgb_batch_run": (_I, [_P, _I, C.POINTER(_I)]),
    "mgb_batch_run_async": (_I, [_P, _I]),
    "mgb_batch_wait": (_I, [_P, C.POINTER(_I)]),
    "mgb_batch_ready": (_I, [_P, C.POINTER(_I)]),
    "mgb_batch_finished": (_I, [_P, _P, _I, C.POINTER(_I)]),
    "mgb_batch_result": (_I, [_P, _I, _P, C.POINTER(SolveInfo), _I]),
    "mgb_batch_tuning": (_I, [_P, _P, _P]),
    "mgb_batch_destroy": (_I, [_P]),
    "mgb_set_mixed_matvec": (_I, [_I]),
    "mgb_get_mixed_matvec": (_I, []),
    "mgb_gauss_mixed_work": (_I, [_I, _I, _P, C.POINTER(C.c_longlong)]),
    "mgb_gauss_fp64_work": (_I, [_I, _I, _P, C.POINTER(C.c_longlong)]),
}


def lib():
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise MplaError(-1, f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> int:
    if status != MGB_OK:
        raise MplaError(status, lib().mgb_last_error().decode(errors="replace"))
    return status


def init(device: int = 0) -> None:
    check(lib().mgb_init(device))


def synchronize() -> None:
    check(lib().mgb_device_sync())


# ------------------------------------------------------------------ buffers
class DeviceArray:
    """A float64/int32 device buffer owned by the library's allocator."""

    def __init__(self, count: int, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        self.count = int(count)
        self.nbytes = self.count * self.dtype.itemsize
        p = C.c_void_p()
        check(lib().mgb_malloc(C.byref(p), max(self.nbytes, 1)))
        self.ptr = p.value

    @classmethod
    def from_numpy(cls, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a.ravel(order="K"))
        d = cls(a.size, a.dtype)
        if a.size:
            check(lib().mgb_memcpy_htod(d.ptr, a.ctypes.data, d.nbytes))
        return d

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype).ravel()
        assert a.size == self.count
        check(lib().mgb_memcpy_htod(self.ptr, a.ctypes.data, self.nbytes))

    def numpy(self) -> np.ndarray:
        out = np.empty(self.count, dtype=self.dtype)
        if self.count:
            check(lib().mgb_memcpy_dtoh(out.ctypes.data, self.ptr, self.nbytes))
        return out

    def zero(self) -> None:
        check(lib().mgb_memset(self.ptr, 0, self.nbytes))

    def free(self) -> None:
        if self.ptr:
            lib().mgb_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _coord_array(coords) -> C.Array:
    """Host array of device pointers, one per dimension."""
    ptrs = [c.ptr if isinstance(c, DeviceArray) else int(c) for c in coords]
    return (C.c_void_p * len(ptrs))(*ptrs)


class GaussPoints:
    """Device-resident structure-of-arrays points (already scaled)."""

    def __init__(self, scaled_points: np.ndarray):
        pts = np.ascontiguousarray(scaled_points, dtype=np.float64)
        self.dim, self.n = pts.shape
        self.buf = DeviceArray.from_numpy(pts)
        self._arr = (C.c_void_p * self.dim)(*[self.buf.ptr + 8 * self.n * d for d in range(self.dim)])

    @property
    def coords(self):
        return self._arr


# ------------------------------------------------------------------- BLAS
def _s(stream):
    return None if stream is None else C.c_void_p(int(stream))


def dgemv(m, n, A_ptr, lda, x_ptr, y_ptr, stream=None) -> None:
    check(lib().mgb_dgemv(m, n, A_ptr, lda, x_ptr, y_ptr, _s(stream)))


def ddot(n, x_ptr, y_ptr, stream=None) -> float:
    r = C.c_double()
    check(lib().mgb_ddot(n, x_ptr, y_ptr, C.byref(r), _s(stream)))
    return r.value


def daxpy(n, alpha, x_ptr, y_ptr, stream=None) -> None:
    check(lib().mgb_daxpy(n, float(alpha), x_ptr, y_ptr, _s(stream)))


def gauss_matvec_f64(pts: GaussPoints, nugget, rule, x_ptr, y_ptr, rows=None, cols=None, row_offset=0,
                     col_offset=0, stream=None) -> None:
    rows = pts.n if rows is None else rows
    cols = pts.n if cols is None else cols
    check(lib().mgb_gauss_matvec_f64(rows, cols, row_offset, col_offset, pts.dim, pts.coords, float(nugget),
                                     rule, x_ptr, y_ptr, _s(stream)))


def gauss_matvec_mixed(pts: GaussPoints, nugget, x_ptr, y_ptr, stream=None) -> None:
    check(lib().mgb_gauss_matvec_mixed(pts.n, pts.dim, pts.coords, float(nugget), x_ptr, y_ptr, _s(stream)))


def gauss_entries(pts: GaussPoints, i: np.ndarray, j: np.ndarray, nugget=0.0, rule=NUGGET_DIAGONAL) -> np.ndarray:
    di = DeviceArray.from_numpy(np.asarray(i, dtype=np.int32))
    dj = DeviceArray.from_numpy(np.asarray(j, dtype=np.int32))
    out = DeviceArray(len(di.numpy()))
    check(lib().mgb_gauss_entries_f64(pts.n, di.count, di.ptr, dj.ptr, pts.dim, pts.coords, float(nugget), rule,
                                      out.ptr, None))
    return out.numpy()


def set_mixed_matvec(kind: int) -> None:
    """Kernel of the mixed-precision matvec (MIXED_TENSOR or MIXED_SIMT) for
    matvecs and solvers set up afterwards."""
    check(lib().mgb_set_mixed_matvec(int(kind)))


def gauss_mixed_work(pts: GaussPoints) -> int:
    """Kernel entries one mixed matvec of this system evaluates."""
    out = C.c_longlong()
    check(lib().mgb_gauss_mixed_work(pts.n, pts.dim, pts.coords, C.byref(out)))
    return out.value


def gauss_fp64_work(pts: GaussPoints) -> int:
    """Kernel entries one FP64 matvec of this system evaluates."""
    out = C.c_longlong()
    check(lib().mgb_gauss_fp64_work(pts.n, pts.dim, pts.coords, C.byref(out)))
    return out.value


def get_mixed_matvec() -> int:
    return int(lib().mgb_get_mixed_matvec())


def halton(n: int, dim: int, start: int = 0) -> np.ndarray:
    """Halton points (dim x n) of the quadrature-weight application: host
    code of the library, no device needed."""
    out = np.empty((dim, n))
    check(lib().mgb_halton(n, dim, start, out.ctypes.data))
    return out


def kernel_launches() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().mgb_kernel_launches())


def time_gauss_matvec(pts: GaussPoints, nugget, precision, x_ptr, y_ptr, reps=10, stream=None) -> float:
    """Mean milliseconds per launch of the Gaussian matvec kernel (CUDA events)."""
    ms = C.c_double()
    check(lib().mgb_time_gauss_matvec(pts.n, pts.dim, pts.coords, float(nugget), precision, x_ptr, y_ptr, reps,
                                      C.byref(ms), _s(stream)))
    return ms.value


def time_dgemv(n, A_ptr, x_ptr, y_ptr, reps=10, stream=None) -> float:
    ms = C.c_double()
    check(lib().mgb_time_dgemv(n, A_ptr, x_ptr, y_ptr, reps, C.byref(ms), _s(stream)))
    return ms.value


# ---------------------------------------------------------------- solvers
def _solve(status: int, info: SolveInfo, allow_notconv: bool) -> SolveInfo:
    if status == MGB_ERR_NOTCONV and allow_notconv:
        return info
    if status == MGB_ERR_BREAKDOWN and allow_notconv:
        return info
    check(status)
    return info


def cg_dense(n, A_ptr, b_ptr, x_ptr, iter_max=1000, eps=1e-10, stop_rule=STOP_RELATIVE, lda=None, stream=None,
             allow_notconv=True) -> SolveInfo:
    info = SolveInfo()
    st = lib().mgb_cg_dense(n, A_ptr, lda or n, b_ptr, x_ptr, iter_max, eps, stop_rule, C.byref(info), _s(stream))
    return _solve(st, info, allow_notconv)


def bicgstab_dense(n, A_ptr, b_ptr, x_ptr, iter_max=1000, eps=1e-10, lda=None, stream=None,
                   allow_notconv=True) -> SolveInfo:
    info = SolveInfo()
    st = lib().mgb_bicgstab_dense(n, A_ptr, lda or n, b_ptr, x_ptr, iter_max, eps, C.byref(info), _s(stream))
    return _solve(st, info, allow_notconv)


def cg_gauss(pts: GaussPoints, nugget, b_ptr, x_ptr, iter_max=100000, eps=1e-10, stop_rule=STOP_RELATIVE,
             precision=PREC_FP64, rule=NUGGET_DIAGONAL, stream=None, allow_notconv=True) -> SolveInfo:
    info = SolveInfo()
    st = lib().mgb_cg_gauss(pts.n, pts.dim, pts.coords, float(nugget), rule, b_ptr, x_ptr, iter_max, eps, stop_rule,
                            precision, C.byref(info), _s(stream))
    return _solve(st, info, allow_notconv)


def bicgstab_gauss(pts: GaussPoints, nugget, b_ptr, x_ptr, iter_max=100000, eps=1e-10, rule=NUGGET_DIAGONAL,
                   stream=None, allow_notconv=True) -> SolveInfo:
    info = SolveInfo()
    st = lib().mgb_bicgstab_gauss(pts.n, pts.dim, pts.coords, float(nugget), rule, b_ptr, x_ptr, iter_max, eps,
                                  C.byref(info), _s(stream))
    return _solve(st, info, allow_notconv)


def cg_gauss_host(scaled_points: np.ndarray, nugget: float, b: np.ndarray, x0: np.ndarray | None = None,
                  iter_max=100000, eps=1e-10, precision=PREC_MIXED, allow_notconv=True):
    """End-to-end solve from host buffers (points, b, x0 in host memory)."""
    pts = np.ascontiguousarray(scaled_points, dtype=np.float64)
    dim, n = pts.shape
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    info = SolveInfo()
    st = lib().mgb_cg_gauss_host(n, dim, pts.ctypes.data, float(nugget), b.ctypes.data, x.ctypes.data, iter_max,
                                 eps, precision, C.byref(info))
    _solve(st, info, allow_notconv)
    return x, info


# ---------------------------------------------------------------- batching
class Batch:
    """Many independent Gaussian kernel systems (1..8 right-hand sides each)
    advanced together on the device; see ``mgb_batch_*`` in mpla_gb300.h."""

    def __init__(self, max_systems: int = 512):
        h = _P()
        check(lib().mgb_batch_create(int(max_systems), C.byref(h)))
        self._h = h
        self.max_systems = int(max_systems)

    def add(self, scaled_points: np.ndarray, nugget: float, b: np.ndarray, precision: int = PREC_MIXED,
            eps: float = 1e-10, iter_max: int = 200000, reserve_bytes: int = 0) -> int:
        """Admit one system; ``scaled_points`` is dim x n (K_ij = exp(-|x_i-x_j|^2)),
        ``b`` is n or n x nrhs.  Raises MplaError(MGB_ERR_NOMEM) when refused."""
        pts = np.ascontiguousarray(scaled_points, dtype=np.float64)
        dim, n = pts.shape
        bb = np.asarray(b, dtype=np.float64)
        if bb.ndim == 1:
            bb = bb[:, None]
        if bb.shape[0] != n:
            raise ValueError("b must have one row per point")
        bcol = np.asfortranarray(bb)
        out = _I()
        check(lib().mgb_batch_add(self._h, n, dim, pts.ctypes.data, float(nugget), bb.shape[1], bcol.ctypes.data,
                                  int(precision), float(eps), int(iter_max), int(reserve_bytes), C.byref(out)))
        return out.value

    def run(self, max_steps: int = 1 << 30) -> int:
        """Advance every system by up to ``max_steps`` iterations; returns the
        number of systems still running."""
        act = _I()
        check(lib().mgb_batch_run(self._h, int(min(max_steps, 2**31 - 1)), C.byref(act)))
        return act.value

    def run_async(self, max_steps: int) -> None:
        """Enqueue up to ``max_steps`` iterations on the batch's own stream."""
        check(lib().mgb_batch_run_async(self._h, int(min(max_steps, 2**31 - 1))))

    def wait(self) -> int:
        """Wait for the enqueued iterations; returns the systems still running."""
        act = _I()
        check(lib().mgb_batch_wait(self._h, C.byref(act)))
        return act.value

    def ready(self) -> bool:
        """True when the iterations enqueued by run_async have finished."""
        r = _I()
        check(lib().mgb_batch_ready(self._h, C.byref(r)))
        return bool(r.value)

    def finished(self) -> list[int]:
        buf = (_I * self.max_systems)()
        cnt = _I()
        check(lib().mgb_batch_finished(self._h, buf, self.max_systems, C.byref(cnt)))
        return [buf[i] for i in range(cnt.value)]

    def result(self, handle: int, n: int, nrhs: int, release: bool = True):
        """x (n x nrhs) and a SolveInfo per right-hand side.  A right-hand side
        that did not converge is reported in its SolveInfo, not raised."""
        x = np.zeros((nrhs, n))
        infos = (SolveInfo * nrhs)()
        st = lib().mgb_batch_result(self._h, int(handle), x.ctypes.data, infos, int(bool(release)))
        if st not in (MGB_OK, MGB_ERR_NOTCONV, MGB_ERR_BREAKDOWN):
            check(st)
        return x.T.copy(), list(infos)

    def tuning(self):
        """Per class (dim 2|3 x R 1|2|3|4|6|8): FP32 matvec rows per thread
        chosen by the autotuner, and the timed ms of the 1/2/4 variants."""
        rpt = (_I * BATCH_CLASSES)()
        ms = (C.c_float * (3 * BATCH_CLASSES))()
        check(lib().mgb_batch_tuning(self._h, rpt, ms))
        return list(rpt), [list(ms[3 * c:3 * c + 3]) for c in range(BATCH_CLASSES)]

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().mgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
