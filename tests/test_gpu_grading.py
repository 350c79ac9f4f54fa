"""GPU parity on corner-graded boundaries (DLP_kress_global_corners and
CFIE_kress_global_corners with kressq = 4): device entries equal the
oracle's (1e-12, rectangle and half-ellipse mushroom), and the mixed Beyn
eigenvalues of the rectangle (direct Hankel values) equal
pi sqrt(m^2 + (n/0.7)^2) to 1e-9."""
import math

import numpy as np
import pytest

from oracle import assembly as OA

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("geom", ["rectangle", "mushroom"])
def test_graded_dlp_and_cfie_entries(qb, geom):
    b = qb.make_rectangle(1.0, 0.7) if geom == "rectangle" else qb.make_full_ellipse_mushroom()
    for cls in (qb.DLP_kress_global_corners, qb.CFIE_kress_global_corners):
        sol = cls(1.0, b, kressq=4)
        pts, sol = qb.points_with_n(sol, b, 240, 15.0)
        ws = qb.Workspace(sol, pts)
        z = 15.2 + 0.1j
        got = qb.assemble(ws, [z])[0]
        if sol.kind == "dlp":
            ref = OA.dlp_fredholm(pts, z)
        else:
            ref = OA.cfie_matrix(qb.solvers.as_list(pts), z)
        assert _rel(got, ref) < 1e-12
        gd = qb.construct_matrices(sol, pts, ws, 15.3, derivs=True)
        rd = OA.assemble(sol.kind, pts, 15.3, derivs=True)
        for g, r in zip(gd, rd):
            assert _rel(g, r) < 1e-12


def test_graded_rectangle_beyn(qb):
    b = qb.make_rectangle(1.0, 0.7)
    sol = qb.DLP_kress_global_corners(1.0, b, kressq=4)
    pts, sol = qb.points_with_n(sol, b, 240, 10.0)
    ws = qb.Workspace(sol, pts)
    k0, R = 10.0 + 0j, 0.5
    # direct Hankel values: the reference's default uniform panels (15000 on [0.95 r_min, r_max]) cannot
    # resolve H0, H1 at the tiny pair distances next to graded corners (5e-9 here)
    lam = qb.solve(sol, pts, k0, R, nq=32, r=16, svd_tol=1e-12, rng=np.random.default_rng(1), ws=ws, mixed=True,
                   use_chebyshev=False)
    lam = np.sort(lam[(np.abs(lam - k0) < R) & (np.abs(lam.imag) < 1e-6)].real)
    ex = np.sort([math.pi * math.hypot(m, n / 0.7) for m in range(1, 9) for n in range(1, 9)
                  if abs(math.pi * math.hypot(m, n / 0.7) - 10.0) < R])
    assert len(lam) == len(ex) > 0
    assert np.max(np.abs(lam - ex) / ex) < 1e-9
