"""The library's symbolic analysis (turbomodal_gb300/csrc/sym.cpp, run on the host by
tests/native/symbolic_dump.cpp) against the oracle's restatement of SimplicialLDLT::analyzePattern
(src/hermitian_lanczos.cpp:20; Eigen's AMD in its cs_amd form, elimination tree, column counts):
bit-exact on the harmonic operator K_k - sigma M_k and on the 2n Lancaster operator of the
Coriolis QEP.  The GPU tests check the same through tmg_symbolic; this runs without a GPU."""

import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import ROOT
from test_solve_schedule import lancaster_pattern, operator_pattern

CSRC = os.path.join(ROOT, "turbomodal_gb300", "csrc")


@pytest.fixture(scope="module")
def dumper(tmp_path_factory):
    d = tmp_path_factory.mktemp("sym")
    exe = str(d / "symbolic_dump")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "native", "symbolic_dump.cpp"),
                    os.path.join(CSRC, "sym.cpp"), "-o", exe], check=True)
    return exe, d


@pytest.mark.parametrize("case", ["config0", "bladed", "config0_lancaster"])
def test_symbolic_bit_exact_on_host(dumper, oracle, case):
    from turbomodal_gb300.meshgen import config_mesh, sector_mesh

    exe, d = dumper
    mesh = config_mesh(0) if case.startswith("config0") else sector_mesh(
        12, 8, 3, seed=4, blade=dict(ns=10, nc=4, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))
    pat = str(d / f"{case}.pat")
    (lancaster_pattern if case.endswith("lancaster") else operator_pattern)(oracle, mesh, 3000.0, pat)
    out = str(d / f"{case}.sym")
    subprocess.run([exe, pat, out], check=True)
    raw = np.fromfile(out, np.int32)
    with open(pat, "rb") as f:
        n, nnz = np.fromfile(f, np.int64, 2)
        p = np.fromfile(f, np.int64, n + 1)
        i = np.fromfile(f, np.int32, nnz)
    perm, parent, cc = raw[:n], raw[n:2 * n], raw[2 * n:3 * n]
    P = sp.csc_matrix((np.ones(nnz), i, p), shape=(n, n))
    op, opar, occ = oracle.ldl_symbolic(P)
    assert np.array_equal(perm, op)
    assert np.array_equal(parent, opar)
    assert np.array_equal(cc, occ)
