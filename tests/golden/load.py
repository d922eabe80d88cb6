"""Loading helpers for the golden fixtures in this folder."""
from __future__ import annotations

import ast
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["case"] = ast.literal_eval(str(out["case"]))
    if "result" in out:
        out["result"] = parse_result(str(out["result"]))
    if "hier" in out:
        out["hier"] = parse_hier(str(out["hier"]))
    return out


def parse_result(text):
    r = {}
    for line in text.strip().splitlines():
        parts = line.split()
        if not parts:
            continue
        key, vals = parts[0], parts[1:]
        if key in ("history", "solve_seconds", "final_resid", "init_resid", "rhs_norm"):
            r[key] = [float(v) for v in vals] if key in ("history", "solve_seconds") else float(vals[0])
        else:
            r[key] = [int(v) for v in vals] if key == "cg_iters" else int(vals[0])
    return r


def parse_hier(text):
    levels = []
    for line in text.strip().splitlines():
        parts = line.split()
        if parts[0] == "level":
            levels.append([])
        else:
            levels[-1].append(tuple(int(v) for v in parts))
    return levels


def names(prefix):
    return sorted(f[:-4] for f in os.listdir(HERE) if f.startswith(prefix) and f.endswith(".npz"))
