"""A fixed solve for profilers (ncu launch lists and single-kernel captures).

    python -m amrex_gb300.profile_case --n 256 --mode mixed --solves 1 [--graph] [--fused] [--opt name=value]
    python -m amrex_gb300.profile_case --amr tests/golden/amrgrids_c2.npz --mode mixed --graph

Builds the benchmark workload (variable-coefficient MLABecLaplacian, log-normal
b with contrast 1e3, Gaussian-blob RHS, max_grid_size 64) at n^3 and runs
`--solves` solves to 1e-10 in the given precision mode.  With --amr, the
composite MLPoisson over the AMR grids stored in that file (base n and RHS
seed from the file) instead.
"""
from __future__ import annotations

import argparse
import time

import ast

import numpy as np

import amrex_gb300 as ag
from amrex_gb300 import synth, workloads


def run_amr(args):
    z = np.load(args.amr)
    case = ast.literal_eval(str(z["case"]))
    grids = []
    for line in str(z["grids"]).strip().splitlines():
        p = line.split()
        if p[0] == "level":
            grids.append([])
        else:
            grids[-1].append(tuple(int(v) for v in p))
    P = workloads.amr_problem(case["n"], grids, case["rhs_seed"], precision={"fp64": 0, "mixed": 1}[args.mode],
                              graph=args.graph, fused=args.fused)
    m = P["mlmg"]
    for kv in args.opt:
        k, v = kv.split("=")
        m.setOption(k, float(v))
    for s in range(args.solves):
        for x in P["sols"]:
            x.setVal(0.0)
        t = time.perf_counter()
        r = m.solve(P["sols"], P["rhss"], 1e-10, 0.0)
        print(f"solve {s}: {m.getNumIters()} iters, resid {r:.3e}, device {m.solveTimeMs():.2f} ms, "
              f"wall {(time.perf_counter() - t) * 1e3:.2f} ms")
    print("kernel launches:", ag.kernel_launches())
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--mgs", type=int, default=64)
    ap.add_argument("--mode", default="mixed")
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--fused", action="store_true")
    ap.add_argument("--opt", action="append", default=[], help="engine option name=value (repeatable)")
    ap.add_argument("--amr", default=None, help="AMR grids file (amrgrids_*.npz): composite MLPoisson solve")
    args = ap.parse_args()
    if args.amr:
        return run_amr(args)
    n = args.n
    rhs_h = synth.gaussian_rhs(n, 1001)
    bx, by, bz = synth.lognormal_bcoef(n, 2001, sigma_cells=5.0, max_ratio=1e3)
    domain = ag.Box((0, 0, 0), (n - 1, n - 1, n - 1))
    ba = ag.BoxArray(domain).maxSize(args.mgs)
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain)
    sol = ag.MultiFab(ba, dm, 1, 1)
    rhs = ag.MultiFab(ba, dm, 1, 0)
    rhs.set_global(rhs_h)
    op = ag.MLABecLaplacian(geom, ba, dm)
    op.setDomainBC((101,) * 3, (101,) * 3)
    op.setScalars(1.0, 1.0)
    op.setACoeffs(0, 1.0)
    faces = []
    for d, arr in enumerate((bx, by, bz)):
        f = ag.MultiFab(ba, dm, 1, 0, nodal_dir=d)
        f.set_global(arr)
        faces.append(f)
    op.setBCoeffs(0, faces)
    m = ag.MLMG(op)
    m.setPrecision(args.mode)
    m.setGraph(args.graph)
    m.setFusedSmoother(args.fused)
    for kv in args.opt:
        k, v = kv.split("=")
        m.setOption(k, float(v))
    m.setTimeKernels(True)
    for s in range(args.solves):
        sol.setVal(0.0)
        t = time.perf_counter()
        r = m.solve(sol, rhs, 1e-10, 0.0)
        print(f"solve {s}: {m.getNumIters()} iters, resid {r:.3e}, device {m.solveTimeMs():.2f} ms, "
              f"wall {(time.perf_counter() - t) * 1e3:.2f} ms")
        if s == 0:
            m.smootherStats(reset=True)
    ms, n_l, nbytes = m.smootherStats(reset=True)
    if n_l:
        print(f"finest-level smoother: {n_l} launches, {ms / n_l * 1e3:.1f} us each, "
              f"{nbytes / (ms / n_l * 1e-3) / 1e9:.0f} GB/s algorithmic")
    print("kernel launches:", ag.kernel_launches())
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
