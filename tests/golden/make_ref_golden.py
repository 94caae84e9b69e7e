"""Writes ref_golden.npz: outputs of the reference MPLA itself on small seeded
inputs, used to pin the oracle (tests/test_oracle_vs_reference.py).

Runs on a machine with a GPU, after oracle/build_ref.py has built the
reference (oracle/_ref/libmplaref.so):

    python tests/golden/make_ref_golden.py [output.npz]

Inputs are regenerated from the seeds by mpla_gb300.synth, so only the
reference's outputs are stored.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mpla_gb300 import synth  # noqa: E402
from oracle import reference as ref  # noqa: E402
from tests.golden.ref_cases import cases  # noqa: E402


def main(out_path: str):
    out = {}
    for name, case in cases().items():
        kind = case["kind"]
        if kind == "dgemv":
            y, _ = ref.dgemv(case["A"], case["x"])
            out[f"{name}/y"] = y
            out[f"{name}/ddot"] = np.array(ref.ddot(case["x"], case["x"] + 1.0))
        elif kind == "gauss_matvec":
            out[f"{name}/y"] = ref.gauss_matvec(case["pts"], case["nugget"], case["rule"], case["x"])
        elif kind == "gauss_rhs":
            out[f"{name}/b"] = ref.gauss_rhs(case["pts"], case["rule"])
        elif kind == "dense_solve":
            x, mv, _ = ref.solve_dense(case["A"], case["b"], case["x0"], case["iter_max"], case["eps"],
                                       case["solver"])
            out[f"{name}/x"] = x
            out[f"{name}/iterations"] = np.array(ref.iterations(case["solver"], mv))
        elif kind == "gauss_solve":
            x, mv, _ = ref.solve_gauss(case["pts"], case["nugget"], case["b"], case["x0"], case["iter_max"],
                                       case["eps"], case["solver"])
            out[f"{name}/x"] = x
            out[f"{name}/iterations"] = np.array(ref.iterations(case["solver"], mv))
        print(name, "done", flush=True)
    np.savez_compressed(out_path, **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).resolve().parent / "ref_golden.npz"))
