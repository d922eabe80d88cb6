"""Generate the full-size fixtures ``large_*.npz`` by running the reference
AMReX CPU MLMG (``oracle/_ref/<machine>/ref_driver``, built from the reference sources
by ``oracle/ref/Makefile``) on the seeded inputs of ``cases.LARGE_CASES``.

    make -C oracle/ref -j8
    python tests/golden/make_large_golden.py [name-prefix ...]

A full phi at 256^3 is 134 MB, so each fixture keeps the reference's
iteration count, per-iteration bottom BiCGStab counts, residual history,
max|phi|, sum(phi), sum(phi^2) and phi at 4096 seeded cells
(``cases.large_sample_index``), about 100 KB.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden import cases  # noqa: E402
from tests.golden.make_golden import DRIVER, run_case  # noqa: E402


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref -j8")
    only = sys.argv[1:]
    for name, case in cases.LARGE_CASES.items():
        if only and not any(name.startswith(p) for p in only):
            continue
        out = run_case(case["mode"], case)
        phi = out["phi"]
        idx = cases.large_sample_index(phi.size)
        payload = {"case": np.array(repr(case)), "result": np.array(out["result"]),
                   "phi_stats": np.array([np.abs(phi).max(), phi.sum(), (phi * phi).sum()]),
                   "phi_sample": phi[idx]}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
        print("wrote", name, out["result"].splitlines()[3])


if __name__ == "__main__":
    main()
