"""The reference AMReX CPU MLMG, compiled from its own sources (checker and
CPU baseline only).

TEST INFRASTRUCTURE ONLY: used by the fixture generators under
``tests/golden/``, by ``__graft_entry__.build()`` and by the CPU-baseline and
reference legs of ``bench.py`` -- never by the library itself.

* ``source_dir()``: the reference source tree -- ``$AMREX_REFERENCE``, else
  the read-only checkout at /root/reference, else the copy of its MLMG sources
  in ``baseline/_ref/amrex`` (git-ignored) that ``copy_sources`` makes so that
  a machine without the checkout can still build the reference.
* ``driver(build=True)``: ``oracle/_ref/<machine>/ref_driver`` (the harness
  ``oracle/ref/ref_driver.cpp`` linked with the reference's Src/Base,
  Src/Boundary, Src/AmrCore and Src/LinearSolvers/MLMG, one build directory
  per CPU architecture), built by ``oracle/ref/Makefile`` with g++ when it is
  missing.
* ``run(mode, case_dir, threads)``: run the driver on a case directory.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CHECKOUT = "/root/reference"
COPY = os.path.join(ROOT, "baseline", "_ref", "amrex")
# the parts of the reference tree oracle/ref/Makefile compiles or includes
COPY_DIRS = ("Src/Base", "Src/Boundary", "Src/AmrCore", "Src/LinearSolvers/MLMG")
COPY_FILES_GLOB_DIR = "Src/LinearSolvers"


def source_dir():
    for d in (os.environ.get("AMREX_REFERENCE"), CHECKOUT, COPY):
        if d and os.path.isfile(os.path.join(d, "Src", "LinearSolvers", "MLMG", "AMReX_MLMG.cpp")):
            return d
    return None


def copy_sources(src=None, dst=COPY):
    """Copy the reference sources the Makefile needs into ``dst`` (skipped
    when the copy is already there)."""
    src = src or source_dir()
    if src is None or os.path.abspath(src) == os.path.abspath(dst):
        return dst if src else None
    stamp = os.path.join(dst, ".complete")
    if os.path.exists(stamp):
        return dst
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    for d in COPY_DIRS:
        shutil.copytree(os.path.join(src, d), os.path.join(dst, d))
    top = os.path.join(src, COPY_FILES_GLOB_DIR)
    for f in os.listdir(top):
        if f.endswith(".H"):
            shutil.copy2(os.path.join(top, f), os.path.join(dst, COPY_FILES_GLOB_DIR, f))
    open(stamp, "w").close()
    return dst


def out_dir():
    return os.path.join(HERE, "_ref", platform.machine() or "host")


def driver_path():
    return os.path.join(out_dir(), "ref_driver")


def driver(build=True, jobs=None, timeout=900):
    """Path of the reference driver for this machine, building it when it is
    missing; None (with the reason in ``driver.reason``) when it cannot be
    built."""
    exe = driver_path()
    if os.path.exists(exe) or not build:
        driver.reason = "" if os.path.exists(exe) else "not built"
        return exe if os.path.exists(exe) else None
    src = source_dir()
    if src is None:
        driver.reason = "no reference source tree (set AMREX_REFERENCE)"
        return None
    jobs = jobs or os.cpu_count() or 8
    r = subprocess.run(["make", "-C", os.path.join(HERE, "ref"), f"-j{jobs}", f"REF={src}", f"OUT={out_dir()}"],
                       stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True, timeout=timeout)
    if r.returncode != 0 or not os.path.exists(exe):
        driver.reason = "reference build failed: " + (r.stderr.strip().splitlines() or ["?"])[-1][:200]
        return None
    driver.reason = ""
    return exe


driver.reason = ""


def run(mode, case_dir, threads=None, capture=False):
    exe = driver()
    if exe is None:
        raise RuntimeError(driver.reason)
    env = dict(os.environ)
    if threads is not None:
        env["OMP_NUM_THREADS"] = str(threads)
    return subprocess.run([exe, mode, case_dir], check=True, env=env, text=True,
                          stdout=subprocess.PIPE if capture else subprocess.DEVNULL)
