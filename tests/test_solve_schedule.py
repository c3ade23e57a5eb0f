"""The triangular-solve schedule on the host: the library's supernodal analysis and solve plan
(turbomodal_gb300/csrc/sym.cpp) replayed with the device kernels' index arithmetic
(tests/native/solve_schedule_check.cpp: the warp-per-subtree kernels, then the level kernels)
must stay inside every panel, front vector and solution vector, solve every supernode exactly
once per direction and reproduce a plain supernodal solve to roundoff (1e-12 relative), and every
column's fill must lie inside its supernode's front, for fundamental and for relaxed supernodes
(amalgamation by analyze(relax > 0), one of the autotuner's shapes), on the harmonic operator
and on the 2n Lancaster operator of the Coriolis QEP."""

import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import ROOT

CSRC = os.path.join(ROOT, "turbomodal_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    d = tmp_path_factory.mktemp("sched")
    exe = str(d / "solve_schedule_check")
    cmd = ["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "native", "solve_schedule_check.cpp"),
           os.path.join(CSRC, "sym.cpp"), "-o", exe]
    subprocess.run(cmd, check=True)
    return exe, d


def operator_pattern(oracle, mesh, rpm, path):
    from turbomodal_gb300.meshgen import TITANIUM

    om = oracle.OracleModel(mesh, TITANIUM)
    om.prepare(rpm)
    K, M = om.matrix("Kk", k=1), om.matrix("Mk", k=1)
    P = sp.tril(sp.csc_matrix((abs(K) + abs(M)) > 0, dtype=float)).tocsc()
    P.sort_indices()
    with open(path, "wb") as f:
        np.array([P.shape[0], P.nnz], np.int64).tofile(f)
        P.indptr.astype(np.int64).tofile(f)
        P.indices.astype(np.int32).tofile(f)


def lancaster_pattern(oracle, mesh, rpm, path):
    """Lower triangle of the Coriolis QEP operator L1 - sigma L2 = [[D - sigma M, K], [K, -sigma K]]
    of harmonic 1 (src/modal_solver.cpp:151-198)."""
    from turbomodal_gb300.meshgen import TITANIUM

    om = oracle.OracleModel(mesh, TITANIUM)
    om.prepare(rpm, True)
    K, M, G = (abs(om.matrix(x, k=1)) for x in ("Kk", "Mk", "Gk"))
    A = sp.bmat([[M + G, K], [K, K]])
    P = sp.tril(sp.csc_matrix(A > 0, dtype=float)).tocsc()
    P.sort_indices()
    with open(path, "wb") as f:
        np.array([P.shape[0], P.nnz], np.int64).tofile(f)
        P.indptr.astype(np.int64).tofile(f)
        P.indices.astype(np.int32).tofile(f)


@pytest.mark.parametrize("relax", [0.0, 0.2])
@pytest.mark.parametrize("case", ["config0", "bladed", "config0_lancaster"])
def test_solve_schedule_matches_plain_solve(checker, oracle, case, relax):
    from turbomodal_gb300.meshgen import config_mesh, sector_mesh

    exe, d = checker
    mesh = config_mesh(0) if case.startswith("config0") else sector_mesh(
        12, 8, 3, seed=4, blade=dict(ns=10, nc=4, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))
    pat = str(d / f"{case}.pat")
    if not os.path.exists(pat):
        if case.endswith("lancaster"):
            lancaster_pattern(oracle, mesh, 3000.0, pat)
        else:
            operator_pattern(oracle, mesh, 3000.0, pat)
    out = subprocess.run([exe, pat, str(relax), "0"], check=True, capture_output=True, text=True).stdout
    vals = dict(kv.split("=") for kv in out.split())
    assert int(vals["bounds_errors"]) == 0
    assert int(vals["struct_errors"]) == 0
    assert float(vals["max_rel_err"]) <= 1e-12
    assert int(vals["launches"]) > 0
    # most fronts of these sectors are narrow leaves: the subtree kernels carry them
    assert int(vals["subtrees"]) > 0 and 2 * int(vals["subtree_fronts"]) > int(vals["supernodes"])
