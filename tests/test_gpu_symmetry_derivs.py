"""GPU parity: symmetry-reduced DLP (direct and Chebyshev routes, FP64 and
mixed) and CFIE k-derivatives, through the C ABI, against the oracle.

Tolerances: FP64 entries 1e-12 relative to the matrix max-norm (direct) and
1e-11 (Chebyshev: the same panels on both sides, differences come from the
device Bessel values at the Lobatto nodes, ~1e-15); mixed hi = fl32 of the
FP64 value; reduced Beyn eigenvalues: plain vs oracle 1e-11, mixed vs plain
1e-10.
"""
import numpy as np
import pytest

from oracle import assembly as OA, beyn as OB, chebyshev as OC

pytestmark = pytest.mark.gpu
PARAMS = (2000, 6, 800, 6)


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _stadium(qb, n, k, sym):
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, b, symmetry=sym)
    pts, sol = qb.points_with_n(sol, b, n, k)
    return sol, pts, qb.Workspace(sol, pts)


@pytest.mark.parametrize("sym", [(-1, -1), (1, -1)])
def test_reduced_dlp_direct_real_k_with_derivs(qb, sym):
    sol, pts, ws = _stadium(qb, 320, 20.0, qb.XYReflection(*sym))
    orb = qb.periodic_symmetry_index_orbits(pts.n, sol.symmetry)
    assert ws.dim == pts.n // 4
    k = 20.37
    F, F1, F2 = qb.construct_matrices(sol, pts, ws, k, derivs=True)
    R, R1, R2 = OA.dlp_fredholm_reduced(pts, k, orb, derivs=True)
    assert _rel(F, R) < 1e-12
    assert _rel(F1, R1) < 1e-12
    assert _rel(F2, R2) < 1e-12


def test_reduced_dlp_rotation_direct(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.DLP_kress(1.0, b, symmetry=qb.Rotation(5, 2))
    pts, sol = qb.points_with_n(sol, b, 300, 20.0)
    ws = qb.Workspace(sol, pts)
    orb = qb.periodic_symmetry_index_orbits(pts.n, sol.symmetry)
    F = qb.construct_matrices(sol, pts, ws, 19.1)
    assert _rel(F, OA.dlp_fredholm_reduced(pts, 19.1, orb)) < 1e-12


def test_reduced_dlp_chebyshev_complex_k(qb):
    sol, pts, ws = _stadium(qb, 320, 20.0, qb.XYReflection(-1, -1))
    orb = qb.periodic_symmetry_index_orbits(pts.n, sol.symmetry)
    ks = [20.1 + 0.3j, 19.7 - 0.2j]
    got = qb.assemble(ws, ks, cheb=PARAMS)
    for z, g in zip(ks, got):
        assert _rel(g, OC.dlp_fredholm_reduced(pts, z, orb, PARAMS)) < 1e-11
    gotd = qb.assemble(ws, ks[:1], deriv=True, cheb=PARAMS)
    ref = OC.dlp_fredholm_reduced(pts, ks[0], orb, PARAMS, derivs=True)
    for g, r in zip(gotd, ref):
        assert _rel(g, r) < 1e-11
    # mixed: hi word is the FP64 value rounded once
    hi = qb.assemble(ws, ks[:1], mixed=True, cheb=PARAMS)[0]
    assert np.array_equal(hi, got[0].astype(np.complex64))


def test_reduced_beyn_plain_vs_oracle_and_mixed(qb):
    sol, pts, ws = _stadium(qb, 400, 25.0, qb.XYReflection(-1, -1))
    orb = qb.periodic_symmetry_index_orbits(pts.n, sol.symmetry)
    k0, R, nq, r = 25.0 + 0j, 0.4, 24, 24
    sel = lambda l: np.sort_complex(l[(np.abs(l - k0) < R) & (np.abs(l.imag) < 1e-3)])
    lam = sel(qb.solve(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(2), ws=ws,
                       use_chebyshev=False))
    lo, *_ = OB.solve_beyn(lambda zj: [OA.dlp_fredholm_reduced(pts, z, orb) for z in zj], ws.dim, k0, R, nq=nq,
                           r=r, svd_tol=1e-12, rng=np.random.default_rng(2))
    lo = sel(lo)
    assert len(lam) == len(lo) > 0
    assert np.max(np.abs(lam - lo) / np.abs(lo)) < 1e-11
    lm = sel(qb.solve(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(2), ws=ws,
                      mixed=True))
    assert len(lm) == len(lam)
    assert np.max(np.abs(lm - lam) / np.abs(lam)) < 1e-10


@pytest.mark.parametrize("hole", [False, True])
def test_cfie_derivatives_direct_real_k(qb, hole):
    b = qb.make_circle_with_hole() if hole else qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 240, 15.0)
    ws = qb.Workspace(sol, pts)
    k = 15.2
    got = qb.construct_matrices(sol, pts, ws, k, derivs=True)
    ref = OA.cfie_matrix_derivs(qb.solvers.as_list(pts), k)
    for g, r in zip(got, ref):
        assert _rel(g, r) < 1e-12


def test_cfie_derivatives_chebyshev_complex_k(qb):
    b = qb.make_circle_with_hole()
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 240, 15.0)
    ws = qb.Workspace(sol, pts)
    z = 15.1 + 0.25j
    got = qb.assemble(ws, [z], deriv=True, cheb=PARAMS)
    ref = OC.cfie_matrix_derivs(qb.solvers.as_list(pts), z, PARAMS)
    for g, r in zip(got, ref):
        assert _rel(g, r) < 1e-11
