"""GPU: the C1 configuration end to end -- sigma_min sweep of the unit circle
(DLP Kress, N = 512 at k = 42, 200 k in [40, 42]) and refine_minima.

* sigma_min(A(k)) against the oracle's FP64 SVD values (tests/golden/c1_sweep.json,
  made by tests/golden/make_golden.py c1) at all 200 k: 2e-12 relative
  (measured 8.3e-13; the smallest sigma_min is 5e-4, whose LAPACK value itself
  carries eps * sigma_max / sigma_min ~ 1e-12 of relative rounding);
* the minima the sweep detects (get_eigenvalues, threshold 200) are the
  oracle's 17 (of the 19 J_m zeros in the range, one sits at the range edge
  and two are 0.007 apart, inside one 0.01 grid step);
* refine_minima's roots are zeros of J_m (40-digit mpmath values,
  tests/golden/circle_eigs.json) to 2e-8, the resolution of the minimum of
  lambda_min(A^H A).
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


def test_c1_sweep_and_refine(qb):
    g = json.loads((GOLD / "c1_sweep.json").read_text())
    ks, so = np.array(g["ks"]), np.array(g["sigma"])
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(g["pts_scaling_factor"], b)
    sig = qb.k_sweep(sol, b, ks)
    assert np.all(np.abs(sig - so) <= 2e-12 * so)
    mins = qb.get_eigenvalues(ks, sig)
    assert len(mins) == 17
    assert np.allclose(mins, qb.get_eigenvalues(ks, so))
    kr, tr, hist = qb.refine_minima(sol, b, ks, sig)
    zeros = np.array([r["k"] for r in json.loads((GOLD / "circle_eigs.json").read_text())["ranges"]["40_42"]])
    assert len(kr) == 17
    for k in kr:
        assert np.min(np.abs(zeros - k)) < 2e-8, k
    assert np.all(tr < 1e-6)
