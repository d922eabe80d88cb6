"""Compile tests/cpp/facade_solve.cpp against include/mlmg_gb300.H and the
in-tree library (g++; used by tests/test_cpp_facade.py)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build(out_dir):
    libdir = os.path.join(ROOT, "amrex_gb300")
    exe = os.path.join(out_dir, "facade_solve")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "facade_solve.cpp"), "-o", exe, "-L", libdir, "-lamrex_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return exe, r.stderr
