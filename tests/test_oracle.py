"""CPU tests of the oracle against known answers and golden vectors.

The reference (Julia) cannot run on either machine, so the oracle is pinned by
(a) circle Dirichlet eigenvalues = zeros of J_m (example_circle_eigval_convergence.jl:15
uses the same check), (b) mpmath values of H0/H1/J0/J1 stored in
tests/golden/bessel_mpmath.json, (c) the closed form of the Kress weights.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest
from scipy import special as sp

from oracle import assembly as OA, beyn as OB
from qbgpu import geometry as G, solvers as S

GOLD = Path(__file__).parent / "golden"


def test_kress_column_closed_form():
    for N in (8, 9, 64, 65, 128):
        c = OA.kress_R_column(N)
        m = np.arange(N)
        if N % 2 == 0:
            n = N // 2
            ref = -(4 * math.pi / N) * sum(np.cos(2 * math.pi * p * m / N) / p for p in range(1, n)) \
                  - (4 * math.pi / N ** 2) * (-1.0) ** m
        else:
            n = (N - 1) // 2
            ref = -(4 * math.pi / N) * sum(np.cos(2 * math.pi * p * m / N) / p for p in range(1, n + 1))
        assert np.max(np.abs(c - ref)) < 1e-13


def test_golden_bessel_pins_scipy():
    """Oracle special functions (SciPy/AMOS) agree with mpmath golden values."""
    g = json.loads((GOLD / "bessel_mpmath.json").read_text())
    for row in g["values"]:
        z = complex(*row["z"])
        ref = [complex(*v) for v in row["j0j1y0y1"]]
        got = [sp.jv(0, z), sp.jv(1, z), sp.yv(0, z), sp.yv(1, z)]
        scale = max(abs(v) for v in ref)
        assert max(abs(a - b) for a, b in zip(got, ref)) <= 5e-15 * max(scale, 1.0)


def test_node_count_rule():
    assert G.node_count(42.0, 2 * math.pi, 12.2) == 512
    assert G.node_count(1.0, 1.0, 1.0, min_pts=21) == 22  # rounded up to even
    assert G.node_count(100.0, 2 * math.pi, 1.0, needed=4) % 4 == 0


def test_geometry_star_and_stadium():
    star = G.make_star()
    p = G.points_single_curve(star.components[0][0], 256)
    # trapezoid of |gamma'| over sigma equals the length
    L = np.sum(np.hypot(p.tangent[:, 0], p.tangent[:, 1])) * (2 * math.pi / 256)
    assert abs(L - star.length) < 1e-12
    # area by the shoelace formula on the parametrisation (spectrally accurate)
    area = 0.5 * np.sum(p.xy[:, 0] * p.tangent[:, 1] - p.xy[:, 1] * p.tangent[:, 0]) * (2 * math.pi / 256)
    assert abs(area - star.area) < 1e-12
    st = G.make_full_stadium(1.0, 1.0)
    assert abs(st.length - (4.0 + 2 * math.pi)) < 1e-14
    assert G._component_corners(st.components[0]) == []
    q = G.points_smooth_composite(st.components[0], 400)
    sp_ = np.hypot(q.tangent[:, 0], q.tangent[:, 1])
    assert np.allclose(sp_, st.length / (2 * math.pi), rtol=1e-13)  # arc-length parametrised


def test_cfie_hole_orientation():
    b = G.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))
    pts = S.evaluate_points(S.CFIE_kress(10.0, b), b, 20.0)
    assert len(pts) == 2
    # hole reversed: clockwise -> negative signed area
    p = pts[1]
    area = 0.5 * np.sum(p.xy[:, 0] * p.tangent[:, 1] - p.xy[:, 1] * p.tangent[:, 0]) * (2 * math.pi / p.n)
    assert area < 0


def test_oracle_circle_dirichlet_eigenvalue():
    """sigma_min(I - D) vanishes at a zero of J_m and not between zeros."""
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.DLP_kress(10.0, b), b, 20.0)
    z = sp.jn_zeros(3, 3)  # 6.38, 9.76, 13.015
    k = float(z[2])
    s_at = OB.sigma_min(OA.dlp_fredholm(pts, k))
    s_off = OB.sigma_min(OA.dlp_fredholm(pts, k + 0.05))
    assert s_at < 1e-11
    assert s_off > 1e-4


def test_oracle_cfie_matches_dlp_eigenvalue():
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.CFIE_kress(10.0, b), b, 20.0)
    k = float(sp.jn_zeros(2, 3)[2])
    assert OB.sigma_min(OA.cfie_matrix(pts, k)) < 1e-11


def test_oracle_dlp_derivative_fd():
    b = G.make_star()
    pts = S.evaluate_points(S.DLP_kress(10.0, b), b, 15.0)
    k, h = 15.0, 1e-4
    F, F1, F2 = OA.dlp_fredholm(pts, k, derivs=True)
    Fp = OA.dlp_fredholm(pts, k + h)
    Fm = OA.dlp_fredholm(pts, k - h)
    assert np.max(np.abs((Fp - Fm) / (2 * h) - F1)) < 1e-6
    assert np.max(np.abs((Fp - 2 * F + Fm) / h ** 2 - F2)) < 1e-3


def test_oracle_beyn_circle():
    """Beyn on the unit circle finds the J_m zeros inside the disk."""
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.DLP_kress(12.0, b), b, 15.0)
    k0, R = 15.0, 0.4
    lam, Uk, Y, info = OB.solve_beyn(lambda zj: [OA.dlp_fredholm(pts, z) for z in zj], pts.n, k0, R, nq=32, r=24,
                                     svd_tol=1e-12, rng=np.random.default_rng(2))
    ex = sorted(x for m in range(0, 30) for x in sp.jn_zeros(m, 10) if abs(x - k0) < R - 0.02)
    got = sorted(l.real for l in lam if abs(l - k0) < R - 0.02 and abs(l.imag) < 1e-6)
    # degenerate (m, -m) pairs appear twice in the Beyn spectrum
    exd = sorted(ex + [x for m in range(1, 30) for x in sp.jn_zeros(m, 10) if abs(x - k0) < R - 0.02])
    assert len(got) == len(exd)
    assert np.max(np.abs(np.array(got) - np.array(exd))) < 1e-9


def test_oracle_chebyshev_route_matches_direct():
    """The panel route (reference defaults) reproduces the direct operator to ~1e-12."""
    from oracle import chebyshev as OC
    b = G.make_star()
    pts = S.evaluate_points(S.CFIE_kress(8.0, b), b, 40.0)
    k = 40.0 + 0.3j
    A_d = OA.cfie_matrix(pts, k)
    A_c = OC.cfie_matrix(pts, k)
    assert np.max(np.abs(A_c - A_d)) < 1e-11
    p = S.evaluate_points(S.DLP_kress(8.0, b), b, 40.0)
    F_d = OA.dlp_fredholm(p, k)
    F_c = OC.dlp_fredholm(p, k)
    assert np.max(np.abs(F_c - F_d)) < 1e-11
