"""GPU parity: CFIE with Alpert quadrature through the C ABI against the
oracle (cfie_alpert.jl). Entries 1e-12 relative to the max-norm (real k with
k-derivatives, complex k, one component and a hole); mixed hi = fl32 of the
FP64 entry; Beyn eigenvalues on the unit disk equal the zeros of J_m (1e-9).
"""
import numpy as np
import pytest
from scipy import special as sp

from oracle import alpert as OAL

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _case(qb, hole, order=12, n=240, k=15.0):
    b = qb.make_circle_with_hole() if hole else qb.make_star(0.2, 5)
    sol = qb.CFIE_alpert(1.0, b, alpert_order=order)
    pts, sol = qb.points_with_n(sol, b, n, k)
    ws = qb.Workspace(sol, pts)
    curves = [c[0] for c in b.components]
    from qbgpu.alpert import ALPERT_LOG_RULES
    return sol, pts, ws, curves, ALPERT_LOG_RULES[order]


@pytest.mark.parametrize("hole,order", [(False, 12), (True, 8), (False, 16)])
def test_alpert_real_k_with_derivatives(qb, hole, order):
    sol, pts, ws, curves, rule = _case(qb, hole, order)
    k = 15.3
    got = qb.construct_matrices(sol, pts, ws, k, derivs=True)
    ref = OAL.cfie_alpert_matrix(curves, pts, k, rule, order, derivs=True)
    for g, r in zip(got, ref):
        assert _rel(g, r) < 1e-12


def test_alpert_complex_k_and_mixed(qb):
    sol, pts, ws, curves, rule = _case(qb, True, 12)
    ks = [15.1 + 0.2j, 14.8 - 0.1j]
    got = qb.assemble(ws, ks)
    for z, g in zip(ks, got):
        assert _rel(g, OAL.cfie_alpert_matrix(curves, pts, z, rule, 12)) < 1e-12
    hi = qb.assemble(ws, ks, mixed=True)
    for g, h in zip(got, hi):
        assert np.array_equal(h, g.astype(np.complex64))


def test_alpert_beyn_unit_disk(qb):
    b = qb.make_circle(1.0)
    sol = qb.CFIE_alpert(1.0, b, alpert_order=12)
    pts, sol = qb.points_with_n(sol, b, 160, 12.0)
    ws = qb.Workspace(sol, pts)
    k0, R = 11.8 + 0j, 0.4
    lam = qb.solve(sol, pts, k0, R, nq=32, r=24, svd_tol=1e-10, rng=np.random.default_rng(2), ws=ws, mixed=True)
    lam = np.sort(lam[(np.abs(lam - k0) < R) & (np.abs(lam.imag) < 1e-6)].real)
    ref = []
    for m in range(0, 30):
        z = sp.jn_zeros(m, 10)
        z = z[np.abs(z - k0.real) < R]
        ref += list(z) * (1 if m == 0 else 2)
    ref = np.sort(ref)
    assert len(lam) == len(ref) > 0
    assert np.max(np.abs(lam - ref) / ref) < 1e-9


def test_alpert_through_chebyshev_panels(qb):
    """The Alpert route through Chebyshev panels
    (chebyshev_euclidian_helmholtz_cfie_alpert.jl:533-1253: H0, H1 from the
    panels on the grid pairs and the correction nodes, direct values below
    r_min): panels tuned to 1e-13 reproduce the oracle's direct entries to
    1e-11 (A) and 1e-10 (A', A''); the complex64 form rounds those FP64
    values."""
    import math
    sol, pts, ws, curves, rule = _case(qb, True, 12)
    ks = [15.1 + 0.2j, 14.8 - 0.1j]
    zref = 15.0 + 0.5 * np.exp(2j * math.pi * np.arange(8) / 8)
    cheb = qb.chebyshev_params(sol, pts, zref, ws=ws, tol=1e-13)[:4]
    got = qb.assemble(ws, ks, cheb=cheb)
    for z, g in zip(ks, got):
        assert _rel(g, OAL.cfie_alpert_matrix(curves, pts, z, rule, 12)) < 1e-11
    gd = qb.assemble(ws, [15.2], cheb=cheb, deriv=True)
    for g, r in zip(gd, OAL.cfie_alpert_matrix(curves, pts, 15.2, rule, 12, derivs=True)):
        assert _rel(g, r) < 1e-10
    hi = qb.assemble(ws, ks, mixed=True, cheb=cheb)
    for g, h in zip(got, hi):
        assert np.array_equal(h, g.astype(np.complex64))
