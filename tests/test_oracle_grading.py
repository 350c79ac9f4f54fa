"""Corner grading (kress_grading_global_multi_corner.jl:53-146) on the CPU.

* the graded map is monotone with positive Jacobian, and the graded
  quadrature integrates the perimeter;
* the graded DLP (oracle) on a 1 x 0.7 rectangle (four corners) gives the
  exact Dirichlet eigenvalues pi sqrt(m^2 + (n/0.7)^2) to 1e-9 at N = 200
  (the reference's own solver test checks rectangles to 1e-3, solvertests.jl:39-49).
"""
import math

import numpy as np

from oracle import assembly as OA, beyn as OB


def test_graded_map_properties(qb):
    sig, t, jac, jac2, w = qb.multi_kress_graded_nodes_data(96, [0.0, 1.0, 3.0], q=4.0)
    assert np.all(np.diff(sig) > 0) and np.all(jac > 0)
    order = np.argsort(t)
    assert np.all(np.diff(t[order]) > 0)
    b = qb.make_full_ellipse_mushroom()
    sol = qb.DLP_kress_global_corners(1.0, b, kressq=4)
    pts, sol = qb.points_with_n(sol, b, 300, 20.0)
    perim = sum(c.length for c in b.components[0])
    assert abs(np.sum(pts.ws * np.hypot(*pts.tangent.T)) - perim) < 1e-6


def test_graded_rectangle_eigenvalues(qb):
    b = qb.make_rectangle(1.0, 0.7)
    sol = qb.DLP_kress_global_corners(1.0, b, kressq=4)
    pts, sol = qb.points_with_n(sol, b, 200, 10.0)
    k0, R = 10.0 + 0j, 0.5
    lam, *_ = OB.solve_beyn(lambda zj: [OA.dlp_fredholm(pts, z) for z in zj], pts.n, k0, R, nq=32, r=16,
                            svd_tol=1e-12, rng=np.random.default_rng(1))
    lam = np.sort(lam[(np.abs(lam - k0) < R) & (np.abs(lam.imag) < 1e-6)].real)
    ex = np.sort([math.pi * math.hypot(m, n / 0.7) for m in range(1, 9) for n in range(1, 9)
                  if abs(math.pi * math.hypot(m, n / 0.7) - 10.0) < R])
    assert len(lam) == len(ex) > 0
    assert np.max(np.abs(lam - ex) / ex) < 1e-9
