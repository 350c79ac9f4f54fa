"""Oracle checks for the symmetry-reduced DLP and the CFIE k-derivatives (CPU).

* orbit maps (symmetry.jl:214-319) against the node coordinates of the full
  stadium: every orbit member is the reflected copy of its representative;
* host orbit maps equal the oracle's;
* CFIE dA/dk, d2A/dk2 (cfie_kress.jl:619-757) against central differences of
  A(k) on one smooth component (the off-component double-layer derivative
  keeps the reference's sign and is not differenced here);
* the four parity sectors of the reduced stadium DLP partition the spectrum
  of the full operator (the image kernels are regular trapezoid terms, so the
  sector eigenvalues agree with the full ones to the quadrature error, ~1e-8).
"""
import numpy as np
import pytest

from oracle import assembly as OA, beyn as OB


def _stadium(qb, n, k, sym):
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, b, symmetry=sym)
    pts, sol = qb.points_with_n(sol, b, n, k)
    return b, sol, pts


@pytest.mark.parametrize("sym,osym", [("XY", ("xy", -1, 1)), ("X", ("x", -1)), ("Y", ("y", 1)), ("R", ("rot", 4, 1))])
def test_orbits_host_equal_oracle(qb, sym, osym):
    s = {"XY": qb.XYReflection(-1, 1), "X": qb.XReflection(-1), "Y": qb.YReflection(1),
         "R": qb.Rotation(4, 1)}[sym]
    N = 48
    f, full, sc = qb.periodic_symmetry_index_orbits(N, s)
    of, ofull, osc = OA.periodic_symmetry_index_orbits(N, osym)
    assert np.array_equal(f, of) and np.array_equal(full, ofull) and np.allclose(sc, osc)
    with pytest.raises(ValueError):
        qb.periodic_symmetry_index_orbits(N + 2, qb.XYReflection(1, 1))


def test_orbits_are_reflections_of_stadium_nodes(qb):
    _, sol, pts = _stadium(qb, 256, 20.0, qb.XYReflection(-1, -1))
    assert pts.n % 4 == 0
    f, full, _ = qb.periodic_symmetry_index_orbits(pts.n, sol.symmetry)
    X = pts.xy
    assert np.allclose(X[full[:, 1]], X[full[:, 0]] * [-1, 1], atol=1e-13)
    assert np.allclose(X[full[:, 2]], X[full[:, 0]] * [1, -1], atol=1e-13)
    assert np.allclose(X[full[:, 3]], -X[full[:, 0]], atol=1e-13)


def test_cfie_derivatives_match_differences(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 120, 10.0)
    k, h = 10.3, 1e-4
    A, A1, A2 = OA.cfie_matrix_derivs(pts, k)
    Ap, A0, Am = (OA.cfie_matrix(pts, k + d) for d in (h, 0.0, -h))
    assert np.array_equal(A, A0)
    assert np.abs(A1 - (Ap - Am) / (2 * h)).max() / np.abs(A1).max() < 1e-7
    assert np.abs(A2 - (Ap - 2 * A0 + Am) / h ** 2).max() / np.abs(A2).max() < 1e-5


def test_reduced_sectors_partition_full_spectrum(qb):
    _, sol, pts = _stadium(qb, 160, 8.0, qb.XYReflection(-1, -1))
    N = pts.n
    k0, R, nq = 8.0 + 0j, 0.5, 16
    sel = lambda l: np.sort_complex(l[(np.abs(l - k0) < R) & (np.abs(l.imag) < 1e-3)])
    lf, *_ = OB.solve_beyn(lambda zj: [OA.dlp_fredholm(pts, z) for z in zj], N, k0, R, nq=nq, r=32,
                           svd_tol=1e-12, rng=np.random.default_rng(1))
    lf = sel(lf)
    total = 0
    for px in (1, -1):
        for py in (1, -1):
            orb = qb.periodic_symmetry_index_orbits(N, qb.XYReflection(px, py))
            lr, *_ = OB.solve_beyn(lambda zj: [OA.dlp_fredholm_reduced(pts, z, orb) for z in zj], len(orb[0]), k0,
                                   R, nq=nq, r=16, svd_tol=1e-12, rng=np.random.default_rng(1))
            lr = sel(lr)
            total += len(lr)
            for l in lr:
                assert np.min(np.abs(lf - l)) / abs(l) < 1e-6
    assert total == len(lf) > 0
