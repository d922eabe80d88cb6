"""Generate the golden fixtures in this folder by running the reference AMReX
CPU MLMG (built from the reference sources by ``oracle/ref/Makefile`` into
``oracle/_ref/<machine>/ref_driver``) on seeded synthetic inputs.

    make -C oracle/ref -j8          # needs the reference source tree
    python tests/golden/make_golden.py [name-prefix ...]

Each fixture is a ``.npz`` holding the case description (as the text of the
driver's case file), the inputs that are not regenerated from seeds, and the
reference's outputs.  The parity tests rebuild the same inputs from the same
seeds with ``amrex_gb300.synth`` and compare against these outputs.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from amrex_gb300 import synth  # noqa: E402
from tests.golden import cases  # noqa: E402

from oracle import reference  # noqa: E402

DRIVER = reference.driver_path()


def run_case(mode, case):
    with tempfile.TemporaryDirectory() as d:
        files = cases.write_inputs(case, d)
        with open(os.path.join(d, "case.txt"), "w") as f:
            f.write(cases.case_text(case, files))
        env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "8"))
        subprocess.run([DRIVER, mode, d], check=True, env=env, stdout=subprocess.DEVNULL)
        out = {}
        res = os.path.join(d, "result.txt")
        if os.path.exists(res):
            out["result"] = open(res).read()
        for name in ("phi.bin", "out.bin", "fb_out.bin", "fx.bin", "fy.bin", "fz.bin", "gx.bin", "gy.bin", "gz.bin",
                     "res.bin", "phi_fabs.bin"):
            p = os.path.join(d, name)
            if os.path.exists(p):
                out[name[:-4]] = np.fromfile(p, dtype=np.float64)
        p = os.path.join(d, "hier.txt")
        if os.path.exists(p):
            out["hier"] = open(p).read()
        return out


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref -j8")
    only = sys.argv[1:]          # optional name prefixes to regenerate
    for name, case in cases.CASES.items():
        if only and not any(name.startswith(p) for p in only):
            continue
        mode = case["mode"]
        out = run_case(mode, case)
        payload = {"case": np.array(repr(case))}
        if "result" in out:
            payload["result"] = np.array(out["result"])
        if "hier" in out:
            payload["hier"] = np.array(out["hier"])
        for k in ("phi", "out", "fb_out", "fx", "fy", "fz", "gx", "gy", "gz", "res", "phi_fabs"):
            if k in out:
                payload[k] = out[k]
        if mode == "fb":
            payload["fb_in"] = cases.fb_input(case)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
        print("wrote", name)


if __name__ == "__main__":
    main()
