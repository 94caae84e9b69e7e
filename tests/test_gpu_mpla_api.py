"""The drop-in mpla.h API, driven by a C++ program written like MPLA's own
test and benchmark programs (tests/native/mpla_drivers.cpp), compared with
the oracle."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mpla_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


@pytest.fixture(scope="module")
def driver(gpu, tmp_path_factory):
    import mpla_gb300

    out = tmp_path_factory.mktemp("native") / "mpla_drivers"
    cxx = shutil.which("g++") or "g++"
    libdir = mpla_gb300.LIB_PATH.parent
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(CUDA_HOME / "include"),
           str(ROOT / "tests" / "native" / "mpla_drivers.cpp"), "-o", str(out),
           "-L", str(libdir), f"-Wl,-rpath,{libdir}", "-lmpla",
           "-L", str(CUDA_HOME / "lib64"), f"-Wl,-rpath,{CUDA_HOME / 'lib64'}", "-lcudart", "-lcublas"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def run(driver, *args, cwd=None):
    res = subprocess.run([str(driver), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    vals = {}
    for line in res.stdout.splitlines():
        if line.startswith("RESULT "):
            _, k, v = line.split()
            vals[k] = float(v)
    return vals, res.stdout


@pytest.mark.parametrize("m,n", [(1, 1), (100, 37), (1000, 1000)])
def test_known_answer_through_mpla_h(driver, m, n):
    vals, _ = run(driver, "kat", m, n)
    assert vals["ok"] == 1
    for v in range(3):
        assert vals[f"dgemv_relerr_{v}"] <= 1e-13
    assert vals["ddot_relerr"] <= 1e-13


def test_tridiagonal_cg_user_core_and_library_core(driver):
    vals, out = run(driver, "cg_tridiag", 300)
    assert vals["ok"] == 1
    # mpla_generic_conjugate_gradient prints "%d: %e" every 10 iterations
    assert "10: " in out


def test_checkpoint_files_and_restart(driver, tmp_path):
    vals, out = run(driver, "cg_checkpoint", 200, 0, cwd=tmp_path)
    assert vals["ok"] == 1
    assert "Checkpointing..." in out and "MPLA CG stopped after" in out
    for name in ["x.dat", "r.dat", "d.dat", "z.dat"]:
        raw = (tmp_path / name).read_bytes()
        assert len(raw) == 4 + 8 * 200 and int.from_bytes(raw[:4], "little") == 200
    # restart from the files written by the first run
    vals, out = run(driver, "cg_checkpoint", 200, 1, cwd=tmp_path)
    assert vals["ok"] == 1


def write_points(path, pts):
    with open(path, "wb") as f:
        f.write(np.int32(pts.shape[1]).tobytes() + np.int32(pts.shape[0]).tobytes())
        f.write(np.ascontiguousarray(pts, dtype=np.float64).tobytes())


@pytest.mark.parametrize("which", [1, 2])
def test_assembler_plugin_cg_and_bicgstab_match_oracle(driver, orc, tmp_path, which):
    n, nug = 1200, 1e-2
    # points scaled by 1/(sqrt(2) 0.3) stay near the unit cube, so the erf
    # right-hand side (the kernel's integral over [0,1]^3) is not negligible
    pts = synth.gauss_points(n, 3, 21) / (np.sqrt(2) * 0.3)
    write_points(tmp_path / "p.bin", pts)
    vals, out = run(driver, "kernel", tmp_path / "p.bin", "-", tmp_path / "out.bin", which, nug)
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    x, b = raw[:n], raw[n:]
    op = orc.GaussOp(pts, nug)
    # get_rhs_entry: CUDA's erf against glibc's, a difference of two erfs
    want = op.rhs()
    assert np.max(np.abs(b - want)) <= 1e-14 * np.max(np.abs(want))
    assert orc.true_relres(op, b, x) < 1e-10
    assert "MPLA CG stopped after" in out
    # the printed residual history follows the oracle's iteration by iteration
    printed = {}
    for line in out.splitlines():
        if line.startswith("Iteration: "):
            k, r = line.split("\t")
            printed[int(k.split()[1])] = float(r.split(":")[1])
    if which == 2:
        _, ko, _, _, hist = orc.bicgstab(op, b, iter_max=5000, eps=1e-10, history=True)
    else:
        _, ko, _, _, hist = orc.cg(op, b, iter_max=20000, eps=1e-10, history=True)
    # six printed digits; BiCGSTAB amplifies last-bit differences of the
    # matvec within a few iterations, CG much later
    last, tol = (6, 5e-6) if which == 2 else (12, 2e-6)
    early = [k for k in sorted(printed) if k <= last]
    assert early, out[:500]
    for k in early:
        assert printed[k] == pytest.approx(hist[k], rel=tol), k


def test_kernel_descriptor_core_matches_oracle(driver, orc, tmp_path):
    n = 900
    pts = synth.gauss_points(n, 2, 22) / (np.sqrt(2) * 0.01)   # short length scale: well conditioned
    write_points(tmp_path / "p.bin", pts)
    b = synth.sincos_rhs(synth.gauss_points(n, 2, 22))
    b.tofile(tmp_path / "b.bin")
    vals, out = run(driver, "kernel", tmp_path / "p.bin", tmp_path / "b.bin", tmp_path / "out.bin", 0, 0.0)
    x = np.fromfile(tmp_path / "out.bin", dtype=np.float64)[:n]
    op = orc.GaussOp(pts, 0.0, rule=orc.RULE_KERNEL_CU)
    assert orc.true_relres(op, b, x) < 1e-10
