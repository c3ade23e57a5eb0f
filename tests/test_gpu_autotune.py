"""Supernode-shape autotuner (TMG_OPT_AUTOTUNE) on the device.

The tuner times candidate shapes (relaxed amalgamation, front width caps, the tensor-core row
threshold) on the first batch of a new complex operator pattern and keeps the fastest.  The
shapes change only how the factorisation is blocked: the refined results must equal an untuned
solver's within 1e-9 relative (both precisions), the report must list every trial with exactly
one chosen, and a second context on the same design must take the cached choice without trials.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_autotuned_solve_matches_untuned(precision):
    from turbomodal_gb300.meshgen import TITANIUM, scaled_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = scaled_mesh(20000, 36, seed=7)
    base = CyclicSymmetrySolver(m, TITANIUM, precision=precision)
    tuned = CyclicSymmetrySolver(m, TITANIUM, precision=precision)
    tuned.set_option("autotune", 1)
    ks = [1, 4, 17]
    a = {r.harmonic_index: r for r in base.solve_at_rpm(5000.0, 8, ks)}
    b = {r.harmonic_index: r for r in tuned.solve_at_rpm(5000.0, 8, ks)}
    rep = tuned.tuning_report()
    assert len(rep) >= 4 and sum(r["chosen"] for r in rep) == 1
    assert all(r["factor_ms"] > 0 and r["solve_ms"] > 0 and r["l_entries"] > 0 for r in rep)
    for k in ks:
        np.testing.assert_allclose(b[k].frequencies, a[k].frequencies, rtol=1e-9)
    again = CyclicSymmetrySolver(m, TITANIUM, precision=precision)
    again.set_option("autotune", 1)
    c = {r.harmonic_index: r for r in again.solve_rpm_sweep([5000.0], 8, ks)[0]}
    assert again.tuning_report() == []      # the cached choice, no trials
    for k in ks:
        np.testing.assert_allclose(c[k].frequencies, a[k].frequencies, rtol=1e-9)
