"""Rounding of the tensor cores' FP32 accumulation (tcgen05.mma, BF16).

The mixed-precision Gaussian matvec does not form its squared distances on
the tensor cores, and this test records why.  tests/native/tc_accumulation.cu
runs one 128 x 128 x 32 tcgen05.mma on operands whose row sums have exact
values; all products are exact in FP32, so the differences are the
accumulation's rounding.  Measured on GB300: sums are truncated toward zero
(1 + 0.75 ulp gives 1, -1 - 0.75 ulp gives -1, 3 + 0.75 ulp(3) gives 3), and
terms are aligned to the largest one before adding (2^30 + 1 - 2^30 gives 0).
A squared distance -s = 2 u.v - |u|^2 - |v|^2 summed this way carries an
error of up to an ulp of its largest term, of one sign, the same for every
entry of a tile pair whose terms have similar magnitudes: a coherent
perturbation of the FP32 operator of ~1e-7 relative, which at a 1e-4 nugget
is enough to make the mixed CG stagnate (the FP32-difference kernel's
rounding is to nearest and uncorrelated between entries).
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def test_tcgen05_fp32_accumulation_truncates(gpu, tmp_path):
    from mpla_gb300 import _build

    exe = tmp_path / "tc_accumulation"
    nvcc = shutil.which("nvcc") or str(CUDA_HOME / "bin" / "nvcc")
    res = subprocess.run([nvcc, *_build.ARCH, "-std=c++17", "-O2", "-I", str(ROOT / "mpla_gb300" / "csrc"),
                          str(ROOT / "tests" / "native" / "tc_accumulation.cu"), "-o", str(exe)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and "cuda=no error err=0" in res.stdout, res.stdout + res.stderr
    got = {}
    for line in res.stdout.splitlines():
        if line.startswith("CASE "):
            _, c, g, e = line.split()
            got[int(c)] = (float(g), float(e))
    u23 = 2.0 ** -23
    assert got[0] == (1.0, 1.0 + 0.75 * u23)            # round to nearest would give 1 + 2^-23
    assert got[5] == (-1.0, -1.0 - 0.75 * u23)          # toward zero for negative sums too
    assert got[8] == (3.0, 3.0 + 0.75 * 2.0 ** -22)
    assert got[2] == (0.0, 1.0)                         # 1 is lost against 2^30 - 2^30
    assert got[3][0] < got[3][1]                        # sixteen quarter-ulps: truncated
