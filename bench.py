#!/usr/bin/env python
"""Benchmark: MLMG time to a 1e-10 relative residual on the 256^3
variable-coefficient MLABecLaplacian (alpha = a = beta = 1, face b =
exp(kappa g) of a smoothed Gaussian random field with max/min contrast 1e3,
Gaussian-blob RHS, homogeneous Dirichlet, max_grid_size 64), mixed precision
(FP32 V-cycles inside FP64 refinement, CUDA-graph replay) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one full solve from a zero initial guess.  Inputs (256^3 FP64
arrays of 134 MB, larger than the 129 MB L2) stay resident in HBM for the
device-timed `value`; `e2e` repeats the step through the C ABI with host
buffers (RHS upload and solution download inside the timed region).  Under
torchrun every rank solves its own replica (no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
MGS = 64
RHS_SEED, B_SEED = 1001, 2001
TOL_REL = 1e-10
# the reference's own solve of this workload (iterations, residual history,
# phi statistics and samples), generated by tests/golden/make_large_golden.py
REF_FIXTURE = "large_c1_256"
METRIC = "MLMG time-to-1e-10 residual, 256^3 variable-coefficient ABecLaplacian, mixed FP32/FP64"


def workload_config():
    """The workload both arms time (the implementation is described by each
    line's own keys)."""
    return {"workload": f"MLABecLaplacian {N}^3, max_grid_size {MGS} ({(N // MGS) ** 3} boxes), log-normal b "
                        f"(contrast 1e3, 5-cell Gaussian field), Gaussian-blob RHS, Dirichlet, tol_rel 1e-10",
            "n": N, "max_grid_size": MGS, "rhs_seed": RHS_SEED, "b_seed": B_SEED,
            "agg_grid_size": 32, "con_grid_size": 32,
            "l2": "inputs larger than L2 (134 MB FP64 arrays vs 129 MB L2), no flush"}


def make_inputs():
    from amrex_gb300 import synth
    rhs = synth.gaussian_rhs(N, RHS_SEED)
    bx, by, bz = synth.lognormal_bcoef(N, B_SEED, sigma_cells=5.0, max_ratio=1e3)
    return rhs, (bx, by, bz)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier_max(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="mlmg_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or self.path is None or not os.path.exists(self.path):
            return None
        rows = []
        with open(self.path) as f:
            lines = f.readlines()
        os.unlink(self.path)
        for line in lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                try:
                    rows.append((float(p[1]), float(p[2]), p[5], p[6], p[7], p[8]))
                except ValueError:
                    pass
        if not rows:
            return None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[2:]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch(mode):
    """dram bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json), scaled to this workload; None if absent."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(mode)
    if not e:
        return None
    return float(e["bytes_per_cell"]) * N ** 3


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def reference_fixture():
    from tests.golden import load
    try:
        return load.load(REF_FIXTURE)
    except FileNotFoundError:
        return None


def reference_solves(nsolve, threads):
    """Full MLMG::solve calls of the reference's own CPU MLMG (built from its
    sources by oracle/reference.py) on this workload: one process, the MG
    hierarchy set up by the first call, ``nsolve`` solves from a zero initial
    guess.  Returns the MLMG "Solve" timer of each call in ms (the first one
    includes the setup), the run's iteration count, or None with the reason
    when the reference cannot be built here."""
    import re
    import tempfile
    from oracle import reference
    from tests.golden import cases
    t0 = time.perf_counter()
    exe = reference.driver()
    build_s = time.perf_counter() - t0
    if exe is None:
        return None, reference.driver.reason
    case = dict(cases.LARGE_CASES[REF_FIXTURE], repeat=nsolve, verbose=1)
    with tempfile.TemporaryDirectory() as d:
        files = cases.write_inputs(case, d)
        with open(os.path.join(d, "case.txt"), "w") as f:
            f.write(cases.case_text(case, files))
        out = reference.run("solve", d, threads=threads, capture=True).stdout
        from tests.golden import load
        res = load.parse_result(open(os.path.join(d, "result.txt")).read())
    timers = [float(v) * 1e3 for v in re.findall(r"MLMG: Timers: Solve = ([0-9.eE+-]+)", out)]
    if len(timers) != nsolve:        # no timer lines: the harness's wall clock around solve()
        timers = [v * 1e3 for v in res["solve_seconds"]]
    return {"solve_ms": timers, "niters": res["niters"], "threads": res["threads"], "build_s": build_s,
            "final_resid_rel": res["final_resid"] / max(res["rhs_norm"], res["init_resid"])}, ""


def port_solve(rhs, bcoef, threads):
    """The C restatement of the reference MLMG (oracle) on the host cores:
    one full FP64 solve of this workload, setup excluded (ms)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle
    from tests.golden import cases
    c = cases._c(mode="solve", op="abec", n=(N, N, N), max_grid_size=MGS)
    arrays = {"sol": np.zeros((N + 2,) * 3), "rhs": rhs, "a": np.ones((N,) * 3),
              "bx": bcoef[0], "by": bcoef[1], "bz": bcoef[2]}
    _, info = oracle.solve(c, arrays)
    return info["iter_seconds"] * 1e3, info["niters"]


def cpu_baseline(rhs, bcoef):
    """One full solve of this workload by the reference's own CPU MLMG on all
    host cores (its "Solve" timer, setup excluded); the oracle port when the
    reference cannot be built here."""
    cores = os.cpu_count() or 1
    r, why = reference_solves(2, cores)
    if r is not None:
        return {"value": r["solve_ms"][1], "unit": "ms", "cores": r["threads"], "kind": "reference",
                "cpu_model": cpu_model(), "iters": r["niters"],
                "sample": f"one full {N}^3 FP64 MLMG::solve to 1e-10 ({r['niters']} V-cycles; MLMG Solve timer, "
                          f"setup excluded: a first solve built the hierarchy), OpenMP on {r['threads']} threads"}
    ms, iters = port_solve(rhs, bcoef, cores)
    return {"value": ms, "unit": "ms", "cores": cores, "kind": "port", "cpu_model": cpu_model(), "iters": iters,
            "sample": f"one full {N}^3 FP64 solve to 1e-10 by the C restatement of the reference ({iters} "
                      f"V-cycles, setup excluded), OpenMP on {cores} threads; the reference itself: {why}"}


def run_reference(args, ws, rank):
    """The reference arm: full solves of the reference's own CPU MLMG on the
    host cores, rank 0 only (the other ranks return at once)."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    r, why = reference_solves(args.warmup + args.steps, cores)
    extra = {}
    if r is not None:
        timed = r["solve_ms"][args.warmup:]
        steady = r["solve_ms"][1:] or r["solve_ms"]
        extra = {"setup_ms": r["solve_ms"][0] - statistics.median(steady), "iters": r["niters"],
                 "final_resid_rel": r["final_resid_rel"], "build_s": r["build_s"], "solve_ms_all": r["solve_ms"]}
        kind = "reference"
        sample = (f"{args.steps} full {N}^3 FP64 MLMG::solve calls to 1e-10 after {args.warmup} warm-up calls "
                  f"(the first builds the MG hierarchy), MLMG Solve timer, OpenMP on {r['threads']} threads")
        threads = r["threads"]
        if not args.no_one_thread:
            one, _ = reference_solves(2, 1)
            if one is not None:
                extra["one_thread_ms"] = one["solve_ms"][1]
    else:
        rhs, bcoef = make_inputs()
        timed = [port_solve(rhs, bcoef, cores)[0] for _ in range(args.warmup + args.steps)][args.warmup:]
        kind, threads = "port", cores
        sample = (f"{args.steps} full {N}^3 FP64 solves by the C restatement of the reference (setup excluded), "
                  f"OpenMP on {cores} threads; the reference itself: {why}")
    v = statistics.median(timed)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(timed), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(),
            "implementation": "the reference's CPU MLMG (FP64, OpenMP) compiled from its sources with g++ -O2",
            "cpu_baseline": {"value": v, "unit": "ms", "cores": threads, "kind": kind, "cpu_model": cpu_model(),
                             "sample": sample},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(extra)
    print(json.dumps(line), flush=True)


def reference_parity(phi64, fp64_iters, phim):
    """The GPU's FP64 and mixed solutions against the reference's own solve
    of this workload (iteration count, phi statistics and 4096 seeded
    samples; tests/test_gpu_large.py asserts the same)."""
    g = reference_fixture()
    if g is None:
        return None
    from tests.golden import cases
    mx = float(g["phi_stats"][0])
    idx = cases.large_sample_index(phi64.size)

    def diff(phi):
        return float(np.abs(phi.ravel()[idx] - g["phi_sample"]).max() / mx)
    return {"reference_iters": g["result"]["niters"], "fp64_iters": fp64_iters,
            "phi_rel_diff_fp64_vs_reference_samples": diff(phi64),
            "phi_rel_diff_mixed_vs_reference_samples": diff(phim)}


def bench_c0(stream, reps=5):
    """The 64^3 constant-coefficient MLPoisson (max_grid_size 32, 8 boxes,
    Gaussian-blob RHS seed 1000, Dirichlet), FP64 and mixed (graph, fused
    sweeps), device time per solve from a zero initial guess."""
    import torch
    import amrex_gb300 as ag
    n = 64
    from amrex_gb300 import synth
    domain = ag.Box((0, 0, 0), (n - 1, n - 1, n - 1))
    ba = ag.BoxArray(domain).maxSize(32)
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain)
    sol = ag.MultiFab(ba, dm, 1, 1)
    rhs = ag.MultiFab(ba, dm, 1, 0)
    rhs.set_global(synth.gaussian_rhs(n, 1000))
    op = ag.MLPoisson(geom, ba, dm)
    op.setDomainBC((101,) * 3, (101,) * 3)
    op.setLevelBC(0, None)
    out = {"workload": "MLPoisson 64^3, max_grid_size 32 (8 boxes), Gaussian-blob RHS (seed 1000), Dirichlet, "
                       "tol_rel 1e-10"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for prec in ("fp64", "mixed"):
        m = ag.MLMG(op)
        m.setPrecision(prec)
        m.setGraph(True)
        m.setFusedSmoother(prec == "mixed")
        for _ in range(2):
            sol.setVal(0.0)
            m.solve(sol, rhs, TOL_REL, 0.0)
        e0.record(stream)
        for _ in range(reps):
            sol.setVal(0.0)
            m.solve(sol, rhs, TOL_REL, 0.0)
        e1.record(stream)
        e1.synchronize()
        out[f"{prec}_ms"] = e0.elapsed_time(e1) / reps
        out[f"{prec}_iters"] = m.getNumIters()
    return out


def _tuned_options(chosen):
    """engine options of an autotuner choice (the report's last line)"""
    march = "columns" in chosen
    opts = [("march_sweep", 1 if march else 0)]
    if march:
        opts.append(("march_tz", int(chosen.rsplit(" ", 1)[-1])))
    if "one block" in chosen:
        opts += [("coarse_block", 1), ("coarse_cells", 512 if "8^3" in chosen else 4096)]
    else:
        opts.append(("coarse_block", 0))
    opts.append(("fused_tma", 0 if "cp.async" in chosen else 1))
    return opts


def bench_batch(stream, nsolve=64):
    """The batch of independent solves of uneven sizes (cube edges from
    {32, 48, ..., 128}, max_grid_size 32, per-solve seeded b and RHS), mixed
    precision in one batched call, against the same solves run one after
    another through plain FP64 MLMG.  Device time on the library stream."""
    import torch
    import amrex_gb300 as ag
    from amrex_gb300 import workloads
    specs = workloads.batch_specs(nsolve, 4000)
    probs = [workloads.abec_problem(s.n, 32, s.rhs_seed, s.b_seed) for s in specs]
    cells = sum(s.n ** 3 for s in specs)

    def make_mixed():
        out = []
        for p in probs:
            m = ag.MLMG(p["op"])
            m.setPrecision("mixed")
            m.setGraph(True)
            m.setFusedSmoother(True)
            out.append(m)
        return out

    sols, rhss = [p["sol"] for p in probs], [p["rhs"] for p in probs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # two candidate settings for the batch, each on its own solvers (a batch
    # engine is built once for its settings; the batch runs with the settings
    # of its first solver): the autotuner's pick on the largest solve, and the
    # default tiled TMA sweep; one timed batched call each keeps the faster
    big = max(range(nsolve), key=lambda q: specs[q].n)
    tuned = make_mixed()
    _, tune_report = tuned[big].autotune(sols[big], rhss[big], vcycles=4)
    chosen = tune_report.strip().splitlines()[-1].replace("chosen: ", "")
    tuned[0].setFusedSmoother(not chosen.startswith("colour passes"))
    for name, val in _tuned_options(chosen):
        tuned[0].setOption(name, val)
    cands = [(chosen, tuned), ("fused sweep, 32x8x8 tiles, TMA staging (default)", make_mixed())]

    def run_batch(ms):
        for x in sols:
            x.setVal(0.0)
        return ag.solve_batched(ms, sols, rhss, TOL_REL, 0.0)

    trial = []
    for label, ms in cands:
        run_batch(ms)
        e0.record(stream)
        run_batch(ms)
        e1.record(stream)
        e1.synchronize()
        trial.append((e0.elapsed_time(e1), label, ms))
    _, chosen, mixed = min(trial, key=lambda t: t[0])
    del cands, tuned, trial

    def batched():
        return run_batch(mixed)

    batched()
    reps = 3
    e0.record(stream)
    for _ in range(reps):
        st = batched()
    e1.record(stream)
    e1.synchronize()
    batch_ms = e0.elapsed_time(e1) / reps
    iters_b = [m.getNumIters() for m in mixed]
    phib = [x.get_global((s.n,) * 3) for x, s in zip(sols, specs)]
    fp64 = []
    for p in probs:
        m = ag.MLMG(p["op"])
        m.setPrecision("fp64")
        fp64.append(m)

    def sequential():
        for m, x, b in zip(fp64, sols, rhss):
            x.setVal(0.0)
            m.solve(x, b, TOL_REL, 0.0)

    sequential()
    e0.record(stream)
    sequential()
    e1.record(stream)
    e1.synchronize()
    seq_ms = e0.elapsed_time(e1)
    err = max(float(np.abs(a - x.get_global((s.n,) * 3)).max() / np.abs(x.get_global((s.n,) * 3)).max())
              for a, x, s in zip(phib, sols, specs))
    return {"workload": f"{nsolve} independent MLABecLaplacian solves, cube edges uniform in {{32,48,...,128}} "
                        f"(seed 4000), max_grid_size 32, per-solve seeds 4001..{4000 + nsolve}, tol_rel 1e-10",
            "nsolve": nsolve, "cells": cells, "edges": [s.n for s in specs],
            "batched_mixed_ms": batch_ms, "solves_per_s": nsolve / (batch_ms * 1e-3),
            "sequential_fp64_ms": seq_ms, "sequential_fp64_solves_per_s": nsolve / (seq_ms * 1e-3),
            "speedup": seq_ms / batch_ms, "all_converged": all(v == 0 for v in st),
            "iters_mixed": [min(iters_b), max(iters_b)],
            "iters_fp64": [min(m.getNumIters() for m in fp64), max(m.getNumIters() for m in fp64)],
            "phi_rel_diff_vs_fp64_max": err, "settings": chosen}


def bench_adjoint(stream, n=128):
    """Adjoint gradients dJ/db (all faces) and dJ/df of J = 0.5 |phi - phi_t|^2
    over the central (n/2)^3 for the n^3 variable-coefficient ABecLaplacian:
    one mlmg_adjoint_grad call (transposed solve to 1e-10 plus the fused
    face-gradient contraction), FP64 and mixed, device time."""
    import torch
    import amrex_gb300 as ag
    from amrex_gb300 import workloads
    p = workloads.abec_problem(n, 64, 1003, 2003)
    out = {"workload": f"adjoint of MLABecLaplacian {n}^3 (log-normal b, contrast 1e3), J over the central "
                       f"{n // 2}^3, tol_rel 1e-10"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for prec in ("fp64", "mixed"):
        m = ag.MLMG(p["op"])
        m.setPrecision(prec)
        m.setGraph(prec == "mixed")
        m.setFusedSmoother(prec == "mixed")
        p["sol"].setVal(0.0)
        m.solve(p["sol"], p["rhs"], TOL_REL, 0.0)
        phi = p["sol"].get_global((n, n, n))
        tgt, region = workloads.adjoint_objective(n, float(phi.std()))
        g = np.zeros_like(phi)
        g[region] = phi[region] - tgt[region]
        gm = ag.MultiFab(p["ba"], p["dm"], 1, 0)
        gm.set_global(g)
        lam = ag.MultiFab(p["ba"], p["dm"], 1, 0)
        gb = [ag.MultiFab(p["ba"], p["dm"], 1, 0, nodal_dir=d) for d in range(3)]
        m.adjointGrad(p["sol"], gm, TOL_REL, 0.0, lam, gb)
        reps = 3
        e0.record(stream)
        for _ in range(reps):
            m.adjointGrad(p["sol"], gm, TOL_REL, 0.0, lam, gb)
        e1.record(stream)
        e1.synchronize()
        out[f"{prec}_ms"] = e0.elapsed_time(e1) / reps
        out[f"{prec}_iters"] = m.getNumIters()
    return out


def bench_amr(stream, reps=3):
    """The 3-level AMR composite MLPoisson (base 128^3, refinement ratio 2,
    AmrMesh grids tagged where |RHS| exceeds its 90th percentile, blocking
    factor 8, max_grid_size 64), FP64 and mixed, CUDA-graph iterations,
    device time per solve from a zero initial guess."""
    import torch
    import amrex_gb300 as ag
    from amrex_gb300 import workloads
    from tests.golden import amr_cases
    g = amr_cases.load("amrgrids", "c2")
    grids, case = g["grids"], g["case"]
    P = workloads.amr_problem(case["n"], grids, case["rhs_seed"], precision=0, graph=True)
    cells = [sum((b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in lv) for lv in grids]
    out = {"workload": f"3-level AMR composite MLPoisson, base {case['n']}^3, ratio 2, blocking factor 8, "
                       f"max_grid_size {case['max_grid_size']}, levels tagged where |RHS| > p90 (seed "
                       f"{case['rhs_seed']}), Dirichlet, tol_rel 1e-10",
           "boxes": [len(lv) for lv in grids], "cells": cells}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phis = {}
    for prec in ("fp64", "mixed"):
        m = P["mlmg"] if prec == "fp64" else ag.MLMG(P["op"])
        m.setPrecision(prec)
        m.setGraph(True)
        m.setFusedSmoother(prec == "mixed")      # fused sweeps on level 0's V-cycle and the fine levels

        def step():
            for x in P["sols"]:
                x.setVal(0.0)
            return m.solve(P["sols"], P["rhss"], TOL_REL, 0.0)

        step()
        ag.kernel_launches(reset=True)
        dev = 0.0
        e0.record(stream)
        for _ in range(reps):
            resid = step()
            dev += m.solveTimeMs()
        e1.record(stream)
        e1.synchronize()
        out[f"{prec}_ms"] = e0.elapsed_time(e1) / reps
        # the solve's own device time: its iterations, without the transfers
        # between the MultiFabs and the level fields and the zero fill
        out[f"{prec}_solve_device_ms"] = dev / reps
        out[f"{prec}_iters"] = m.getNumIters()
        out[f"{prec}_final_resid_rel"] = resid / m.getInitRHS()
        out[f"{prec}_launches_per_solve"] = ag.kernel_launches() // reps
        phis[prec] = [np.concatenate([x.get_fab(i)[1:-1, 1:-1, 1:-1].ravel() for i in range(len(lv))])
                      for x, lv in zip(P["sols"], grids)]
    out["speedup_mixed_vs_fp64"] = out["fp64_ms"] / out["mixed_ms"]
    out["phi_rel_diff_mixed_vs_fp64"] = max(float(np.abs(a - b).max() / np.abs(b).max())
                                            for a, b in zip(phis["mixed"], phis["fp64"]))
    try:
        ref = amr_cases.load("amrsolve", "c2")
        out["reference_fp64_iters"] = ref["result"]["niters"]
        out["phi_rel_diff_fp64_vs_reference_samples"] = max(
            float(np.abs(phis["fp64"][lv][amr_cases.sample_index(phis["fp64"][lv].size, lv)]
                         - ref[f"phi_l{lv}_sample"]).max() / ref[f"phi_l{lv}_stats"][0]) for lv in range(len(grids)))
    except FileNotFoundError:
        pass
    return out


def run_gb300(args, ws, rank, local):
    import torch
    import amrex_gb300 as ag
    from amrex_gb300 import capi

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    rhs_h, bcoef_h = make_inputs()
    domain = ag.Box((0, 0, 0), (N - 1, N - 1, N - 1))
    ba = ag.BoxArray(domain).maxSize(MGS)
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain)
    sol = ag.MultiFab(ba, dm, 1, 1)
    rhs = ag.MultiFab(ba, dm, 1, 0)
    rhs.set_global(rhs_h)
    op = ag.MLABecLaplacian(geom, ba, dm)
    op.setDomainBC((101,) * 3, (101,) * 3)
    op.setLevelBC(0, None)
    op.setScalars(1.0, 1.0)
    op.setACoeffs(0, 1.0)
    faces = []
    for d in range(3):
        f = ag.MultiFab(ba, dm, 1, 0, nodal_dir=d)
        f.set_global(bcoef_h[d])
        faces.append(f)
    op.setBCoeffs(0, faces)
    mixed = ag.MLMG(op)
    mixed.setPrecision("mixed")
    mixed.setGraph(True)
    mixed.setFusedSmoother(True)
    fp64 = ag.MLMG(op)
    fp64.setPrecision("fp64")
    fp64.setTimeKernels(True)

    stream = torch.cuda.ExternalStream(capi.lib().mlmg_stream())

    def step(m):
        sol.setVal(0.0)
        m.solve(sol, rhs, TOL_REL, 0.0)

    # --- plain FP64 GPU MLMG (the comparator), also the phi reference
    for _ in range(2):
        step(fp64)
    fp64.smootherStats(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nfp = max(2, min(args.steps, 5))
    barrier(ws)
    e0.record(stream)
    for _ in range(nfp):
        step(fp64)
    e1.record(stream)
    e1.synchronize()
    fp64_ms = e0.elapsed_time(e1) / nfp
    fp64_iters = fp64.getNumIters()
    fp64_sm = fp64.smootherStats(reset=True)
    phi64 = sol.get_global((N, N, N))
    # the same FP64 solve with each iteration replayed as a CUDA graph (no
    # launch overhead in the comparison)
    fp64g = ag.MLMG(op)
    fp64g.setPrecision("fp64")
    fp64g.setGraph(True)
    for _ in range(2):
        step(fp64g)
    e0.record(stream)
    for _ in range(nfp):
        step(fp64g)
    e1.record(stream)
    e1.synchronize()
    fp64_graph_ms = e0.elapsed_time(e1) / nfp
    del fp64g

    # --- mixed + graph: the headline
    for _ in range(args.warmup):
        step(mixed)
    ag.kernel_launches(reset=True)
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step(mixed)
        e1.record(stream)
        e1.synchronize()
    launches = ag.kernel_launches()
    ms = e0.elapsed_time(e1) / args.steps
    ms = barrier_max(ms, ws)
    iters = mixed.getNumIters()
    phim = sol.get_global((N, N, N))
    # the dominant kernels' live launch times, from a separate run with CUDA
    # events around the finest-level sweeps and the FP64 outer residual (the
    # events sit between the graph's kernels, so the headline run has none)
    mixed.setTimeKernels(True)
    step(mixed)
    mixed.smootherStats(reset=True)
    mixed.residualStats(reset=True)
    for _ in range(max(2, min(args.steps, 5))):
        step(mixed)
    sm_ms, sm_n, sm_bytes = mixed.smootherStats(reset=True)
    r_ms, r_n, r_bytes, r_flops = mixed.residualStats(reset=True)
    mixed.setTimeKernels(False)
    rel_diff = float(np.abs(phim - phi64).max() / np.abs(phi64).max())
    ref = reference_parity(phi64, fp64_iters, phim)

    # --- end to end through the C ABI with host buffers (pinned, as a host
    # code would keep its input and output arrays)
    import torch as _t
    rhs_pin = _t.empty((N, N, N), dtype=_t.float64, pin_memory=True).numpy()
    rhs_pin[...] = rhs_h
    sol_h = _t.zeros((N, N, N), dtype=_t.float64, pin_memory=True).numpy()
    rhs.set_global(rhs_pin)                 # warm the transfer path once
    sol.get_global((N, N, N), out=sol_h)
    ne2e = max(2, min(args.steps, 5))
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(ne2e):
        rhs.set_global(rhs_pin)             # host -> device
        sol.setVal(0.0)
        mixed.solve(sol, rhs, TOL_REL, 0.0)
        sol.get_global((N, N, N), out=sol_h)  # device -> host
    e2e_ms = (time.perf_counter() - t0) * 1e3 / ne2e
    e2e_ms = barrier_max(e2e_ms, ws)

    # FP64 roofline of the outer residual: this GPU's FMA rate, measured by
    # the library's register-resident FMA kernel
    fp64_peak = ag.fp64_fma_rate()
    r_avg = r_ms / max(r_n, 1)
    outer = {"kernel": "k_residual_s<double,float>: the FP64 outer residual r = f - A phi (stencil form, 7 FMAs "
                       "per cell; FP32 copy of r and per-solve max-norm on the integer pipe)",
             "bound": "fp64", "avg_launch_ms": r_avg, "launches_timed": r_n,
             "flops_per_launch": r_flops, "bytes_per_launch": r_bytes,
             "achieved_tflops": r_flops / (r_avg * 1e-3) / 1e12 if r_n else None,
             "fp64_peak_tflops": fp64_peak, "fp64_peak_kind": "measured in-run (FMA chains, mlmg_fp64_fma_rate)",
             "achieved_gbs": r_bytes / (r_avg * 1e-3) / 1e9 if r_n else None}
    outer["fp64_frac"] = outer["achieved_tflops"] / fp64_peak if r_n and fp64_peak > 0 else None

    peak, peak_kind = peaks()
    outer["hbm_frac"] = outer["achieved_gbs"] / peak if r_n else None
    avg_launch_ms = sm_ms / max(sm_n, 1)
    achieved = sm_bytes / (avg_launch_ms * 1e-3) / 1e9 if sm_n else None
    traffic = traffic_per_launch("mixed")
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 V-cycle / f64 residual", "data": "synthetic (seeded generators, no dataset)",
        "config": workload_config(),
        "implementation": {"precision": "FP32 V-cycles (fused two-colour sweeps) in FP64 iterative refinement",
                           "cuda_graph": True, "fp64_comparator": "the same engine in FP64 throughout, eager "
                           "launches (fp64_ms) and graph-replayed iterations (fp64_graph_ms)"},
        "iters": iters, "fp64_ms": fp64_ms, "fp64_graph_ms": fp64_graph_ms, "fp64_iters": fp64_iters,
        "speedup_vs_fp64": fp64_ms / ms, "speedup_vs_fp64_graph": fp64_graph_ms / ms,
        "phi_rel_diff_vs_fp64": rel_diff, "reference_parity": ref,
        "roofline": {"kernel": "finest-level fused two-colour Gauss-Seidel sweep (FP32, k_sweep_fused2, TMA staging)",
                     "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": traffic, "bytes_per_launch": sm_bytes, "avg_launch_ms": avg_launch_ms,
                     "launches_timed": sm_n,
                     "fp64_smoother": {"avg_launch_ms": fp64_sm[0] / max(fp64_sm[1], 1),
                                       "achieved": (fp64_sm[2] / (fp64_sm[0] / max(fp64_sm[1], 1) * 1e-3) / 1e9)
                                       if fp64_sm[1] else None},
                     "outer_residual": outer},
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(rhs_h.nbytes),
                "d2h_bytes_per_step": int(sol_h.nbytes)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if not args.no_batch:
        line["c0"] = bench_c0(stream)
        line["batch"] = bench_batch(stream)
        line["adjoint"] = bench_adjoint(stream)
        line["amr"] = bench_amr(stream)
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(rhs_h, bcoef_h)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-one-thread", action="store_true", help="reference arm: skip the 1-thread solve")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
