"""GPU: the Chebyshev panel autotuner (chebyshev_params,
chebyshev_optimal_panelization.jl:221-307).

* from a coarse start the panel counts grow until every interpolated H0, H1,
  J0, J1 is within tol (absolute) of the direct device values at the sampled
  radii;
* the tuned panels reproduce the directly evaluated operator to about the
  interpolation tolerance (1e-10 absolute on the special functions gives
  1e-9 relative on the entries here);
* a tolerance that max_iter cannot reach returns the best effort (ETIMEOUT
  with strict=True).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_grows_until_tol_and_matches_direct(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 400, 25.0)
    ws = qb.Workspace(sol, pts)
    zj, _ = qb.contour(25.0 + 0j, 0.4, 8)
    nh, Mh, nj, Mj, err = qb.chebyshev_params(sol, pts, zj, ws=ws, npanels_h_init=200, M_h_init=5,
                                              npanels_j_init=100, M_j_init=5, tol=1e-10, sampling_points=20000)
    assert nh > 200 and nj > 100
    assert np.all(err < 1e-10)
    cheb = qb.assemble(ws, zj[:2], cheb=(nh, Mh, nj, Mj))
    direct = qb.assemble(ws, zj[:2])
    for c, d in zip(cheb, direct):
        assert np.max(np.abs(c - d)) / np.max(np.abs(d)) < 1e-9


def test_autotune_best_effort(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 300, 20.0)
    ws = qb.Workspace(sol, pts)
    zj = np.array([20.0 + 0.1j])
    nh, Mh, nj, Mj, err = qb.chebyshev_params(sol, pts, zj, ws=ws, npanels_h_init=50, M_h_init=3,
                                              npanels_j_init=50, M_j_init=3, tol=1e-15, max_iter=2)
    assert nh == 75 and nj == 75  # one growth step of 1.5x, then max_iter
    with pytest.raises(qb._lib.QBGError):
        qb.chebyshev_params(sol, pts, zj, ws=ws, npanels_h_init=50, M_h_init=3, npanels_j_init=50, M_j_init=3,
                            tol=1e-15, max_iter=2, strict=True)


def test_min_cost_choice_meets_tol(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 400, 25.0)
    ws = qb.Workspace(sol, pts)
    zj, _ = qb.contour(25.0 + 0j, 0.4, 8)
    nh, Mh, nj, Mj, err, cost = qb.chebyshev_params_min_cost(sol, pts, zj, ws=ws, tol=1e-10, degrees=(5, 9, 13),
                                                             sampling_points=20000)
    assert Mh in (5, 9, 13) and np.all(err < 1e-10) and cost > 0
    cheb = qb.assemble(ws, zj[:1], cheb=(nh, Mh, nj, Mj))[0]
    direct = qb.assemble(ws, zj[:1])[0]
    assert np.max(np.abs(cheb - direct)) / np.max(np.abs(direct)) < 1e-9
