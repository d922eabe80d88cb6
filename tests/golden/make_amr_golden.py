"""Generate the AMR golden fixtures in this folder with the reference AMReX
(oracle/_ref/<machine>/ref_driver, built by oracle/ref/Makefile):

* ``amrgrids_<name>.npz``: the grids AmrMesh::MakeNewGrids makes when every
  level tags the cells where |RHS| exceeds the 90th (or the case's
  ``tag_pct``-th) percentile of |RHS| on that level (blocking factor 8, max_grid_size, n_error_buf 1, grid_eff 0.7);
* ``amrresid_<name>.npz`` (cases with ``resid``): MLMG::compResidual of the
  case's initial guess over every AMR level (solution residuals with the
  coarse/fine boundary values, reflux, average-down), packed per level;
* ``amrsolve_<name>.npz``: the reference's composite multi-level MLPoisson
  (or MLABecLaplacian) solve on those grids -- phi on every level's boxes (for the configuration-
  size case only per-level statistics and phi at seeded sample cells),
  residual history and bottom iteration counts.

    python tests/golden/make_amr_golden.py [name-prefix ...]
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
from tests.golden import amr_cases  # noqa: E402

from oracle import reference  # noqa: E402

DRIVER = reference.driver_path()


def _run(mode, d, lines):
    with open(os.path.join(d, "case.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "8"))
    subprocess.run([DRIVER, mode, d], check=True, env=env, stdout=subprocess.DEVNULL)


def make(name, case):
    n, nlev = case["n"], case["nlev"]
    with tempfile.TemporaryDirectory() as d:
        rhs = [amr_cases.level_rhs(case, lev) for lev in range(nlev)]
        for lev in range(nlev):
            rhs[lev].astype(np.float64).tofile(os.path.join(d, f"rhs_l{lev}.bin"))
            sb = amr_cases.level_solbc(case, lev)
            if sb is not None:
                sb.astype(np.float64).tofile(os.path.join(d, f"solbc_l{lev}.bin"))
            co = amr_cases.level_abec(case, lev)
            if co is not None:
                for key, arr in zip(("a", "bx", "by", "bz"), co[2:]):
                    arr.astype(np.float64).tofile(os.path.join(d, f"{key}_l{lev}.bin"))
        thresh = [float(np.percentile(np.abs(r), case.get("tag_pct", 90))) for r in rhs]
        per = case.get("periodic", (0, 0, 0))
        bc = " ".join("200" if p else "101" for p in per)   # LinOpBCType: Periodic 200, Dirichlet 101
        base = [f"n {n} {n} {n}", f"nlev {nlev}", f"max_grid_size {case['max_grid_size']}",
                f"blocking_factor {case.get('blocking_factor', 8)}", "n_error_buf 1", "grid_eff 0.7",
                "thresh " + " ".join(repr(t) for t in thresh),
                "periodic " + " ".join(str(int(p)) for p in per), f"lobc {bc}", f"hibc {bc}"]
        _run("amrgrids", d, base)
        grids = amr_cases.parse_grids(open(os.path.join(d, "grids.txt")).read())
        np.savez_compressed(os.path.join(HERE, f"amrgrids_{name}.npz"), case=np.array(repr(case)),
                            grids=np.array(open(os.path.join(d, "grids.txt")).read()))
        print("wrote amrgrids", name, [len(g) for g in grids])
        summary = case.get("solve") == "summary"
        lines = base + [f"tol_rel {case.get('tol_rel', 1e-10)}", "tol_abs 0.0",
                        f"agg_grid_size {case.get('agg_grid_size', 32)}",
                        f"con_grid_size {case.get('con_grid_size', 32)}",
                        f"max_fmg_iter {case.get('max_fmg_iter', 0)}"]
        if case.get("abec"):
            lines += ["op abec", f"alpha {case['abec'][0]!r}", f"beta {case['abec'][1]!r}"]
        for lev, g in enumerate(grids):
            lines.append(f"boxes_l{lev} " + " ".join(str(v) for b in g for v in b))
        if case.get("resid"):
            # MLMG::compResidual of the initial guess over every AMR level
            _run("amrresid", d, lines)
            payload = {"case": np.array(repr(case)), "grids": np.array(open(os.path.join(d, "grids.txt")).read())}
            for lev, g in enumerate(grids):
                m = n << lev
                res = np.fromfile(os.path.join(d, f"res_l{lev}.bin"), dtype=np.float64).reshape(m, m, m)
                payload[f"res_l{lev}"] = amr_cases.pack_boxes(res, g)
            np.savez_compressed(os.path.join(HERE, f"amrresid_{name}.npz"), **payload)
            print("wrote amrresid", name)
        if not case.get("solve", True):
            return
        _run("amrsolve", d, lines)
        payload = {"case": np.array(repr(case)), "grids": np.array(open(os.path.join(d, "grids.txt")).read()),
                   "result": np.array(open(os.path.join(d, "result.txt")).read())}
        for lev, g in enumerate(grids):
            m = n << lev
            phi = np.fromfile(os.path.join(d, f"phi_l{lev}.bin"), dtype=np.float64).reshape(m, m, m)
            flat = amr_cases.pack_boxes(phi, g)
            if summary:
                # too large to store: the level's max|phi|, sum and sum of
                # squares, and phi at seeded sample cells of its boxes
                idx = amr_cases.sample_index(flat.size, lev)
                payload[f"phi_l{lev}_stats"] = np.array([np.abs(flat).max(), flat.sum(), (flat * flat).sum()])
                payload[f"phi_l{lev}_sample"] = flat[idx]
            else:
                payload[f"phi_l{lev}"] = flat
        np.savez_compressed(os.path.join(HERE, f"amrsolve_{name}.npz"), **payload)
        print("wrote amrsolve", name)


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref -j8")
    only = sys.argv[1:]
    for name, case in amr_cases.CASES.items():
        if only and not any(name.startswith(p) for p in only):
            continue
        make(name, case)


if __name__ == "__main__":
    main()
