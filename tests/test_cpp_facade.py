"""The C++ facade (include/mlmg_gb300.H): a program written against the
reference's C++ API names and signatures compiles against it and, on a GPU,
solves the 64^3 MLPoisson configuration to the reference's answer."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from amrex_gb300 import build as libbuild
from tests.cpp import build_example
from tests.golden import cases, load


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    libbuild.build()
    path, warnings = build_example.build(str(tmp_path_factory.mktemp("cpp")))
    return path, warnings


def test_facade_example_compiles_cleanly(exe):
    path, warnings = exe
    assert os.path.exists(path)
    assert "warning" not in warnings, warnings


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [0, 1])
def test_facade_solve_matches_reference(exe, tmp_path, mixed):
    g = load.load("solve_poisson_c0")
    c = g["case"]
    n = c["n"][0]
    rhs = cases.inputs(c)["rhs"]
    rf, pf = tmp_path / "rhs.bin", tmp_path / "phi.bin"
    np.ascontiguousarray(rhs, dtype=np.float64).tofile(rf)
    r = subprocess.run([exe[0], str(n), str(c["max_grid_size"]), str(rf), str(pf), str(mixed)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    phi = np.fromfile(pf, dtype=np.float64).reshape(n, n, n)
    ref = g["phi"].reshape(phi.shape)
    assert np.abs(phi - ref).max() <= (1e-10 if not mixed else 1e-8) * np.abs(ref).max()
    iters = int(r.stdout.split()[1])
    assert iters == g["result"]["niters"] or mixed
