"""A user-defined system_assembler subclass through the generic adapter.

MPLA's plugin seam is a user subclass of system_assembler whose virtual
get_matrix_entry the generic cores call per entry (src/system_assembler.h:6-12,
src/generic_system_adapter.cu:7-23, 83-137), device-linked with the adapter
(src/Makefile:96-114).  tests/native/user_assembler.cu defines a
non-Gaussian one -- an inverse multiquadric with a diagonal shift,
K_ij = 1/sqrt(0.25 + |p_i - p_j|^2) + 5 delta_ij (condition number near 240,
where an FP64 CG count is stable to +-1 under last-bit perturbations of K;
with a shift of 0.5 the oracle's own count moves by 4 under 2e-16 relative
perturbations) -- and is built with -rdc
against lib/mpla_generic_device.o and libmpla.so, as a user would.  Checked
against FP64 references built here: the matvec through both generic cores at
1e-13 relative to sum_j |K_ij x_j|, the right-hand side exactly, and CG
through mpla_generic_conjugate_gradient_with_checkpoint_restart with the
streamed generic core against the oracle's CG on the same matrix (iteration
count +-1).
"""
import os
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mpla_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def imq_matrix(pts):
    dim, n = pts.shape
    sq = np.full((n, n), 0.25)
    for d in range(dim):
        diff = pts[d][:, None] - pts[d][None, :]
        sq = sq + diff * diff
    return 1.0 / np.sqrt(sq) + 5.0 * np.eye(n)


@pytest.fixture(scope="module")
def program(gpu, tmp_path_factory):
    import mpla_gb300
    from mpla_gb300 import _build

    if not _build.DEVICE_OBJ.exists():
        _build.build()
    out = tmp_path_factory.mktemp("user_assembler") / "user_assembler"
    libdir = mpla_gb300.LIB_PATH.parent
    nvcc = shutil.which("nvcc") or str(CUDA_HOME / "bin" / "nvcc")
    cmd = [nvcc, *_build.ARCH, "-std=c++17", "-rdc=true", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "native" / "user_assembler.cu"), str(_build.DEVICE_OBJ),
           "-L", str(libdir), "-Xlinker", "-rpath", "-Xlinker", str(libdir), "-lmpla", "-lcublas", "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return out


def run(program, mode, workdir, n, dim):
    res = subprocess.run([str(program), mode, str(workdir), str(n), str(dim)], capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "RESULT ok 1" in res.stdout
    return res.stdout


@pytest.mark.parametrize("n,dim", [(3000, 2), (1000, 3), (129, 1)])
def test_user_assembler_matvec_and_rhs(program, tmp_path, n, dim):
    pts = synth.gauss_points(n, dim, 70 + dim) * 4.0
    x = np.random.default_rng(n).standard_normal(n)
    pts.astype(np.float64).tofile(tmp_path / "pts.bin")
    x.tofile(tmp_path / "x.in.bin")
    run(program, "matvec", tmp_path, n, dim)
    K = imq_matrix(pts)
    want = K @ x
    scale = np.abs(K) @ np.abs(x)
    for name in ("y.bin", "y2.bin"):
        got = np.fromfile(tmp_path / name)
        assert np.max(np.abs(got - want) / scale) <= 1e-13, name
    assert np.array_equal(np.fromfile(tmp_path / "rhs.bin"), 1.0 + pts[0])


def test_user_assembler_cg_matches_oracle(program, orc, tmp_path):
    n, dim = 2000, 2
    pts = synth.gauss_points(n, dim, 77) * 4.0
    b = synth.normal(77, 1, n)
    pts.tofile(tmp_path / "pts.bin")
    b.tofile(tmp_path / "b.bin")
    out = run(program, "cg", tmp_path, n, dim)
    m = re.search(r"stopped after (\d+) iterations", out)
    assert m, out
    k = int(m.group(1))
    K = imq_matrix(pts)
    x_orc, k_orc, _, st = orc.cg(orc.DenseOp(K), b, np.zeros(n), iter_max=5000, eps=1e-10)
    assert st == 0
    assert abs(k - k_orc) <= 1, (k, k_orc)
    x = np.fromfile(tmp_path / "x.bin")
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) < 1.01e-10
    assert np.max(np.abs(x - x_orc)) <= 1e-8 * np.max(np.abs(x_orc))
