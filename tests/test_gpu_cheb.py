"""GPU parity of the Chebyshev-panel route (device-built tables) against the
oracle's restatement of the reference's panels (same panel breaks, degree,
DCT-I fit and Clenshaw evaluation, SciPy/AMOS node values).

Tolerance: 1e-12 relative to the matrix max-norm between the device and the
oracle panel routes (both interpolate the same node values); 1e-11 absolute
between the panel route and the direct operator; Beyn eigenvalues of the
panel route vs the oracle's direct route: 1e-11 relative.
"""
import numpy as np
import pytest

from oracle import assembly as OA, beyn as OB, chebyshev as OC

pytestmark = pytest.mark.gpu


def _relerr(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("params", [(15000, 5, 3000, 5), (4000, 7, 1000, 6)])
def test_cfie_cheb_vs_oracle_panels(qb, params):
    for b in (qb.make_star(), qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))):
        sol = qb.CFIE_kress(8.0, b)
        pts = qb.evaluate_points(sol, b, 40.0)
        ws = qb.Workspace(sol, pts)
        ks = [40.0 + 0.4j, 39.8 - 0.2j, 40.1 + 0.0j]
        got = qb.assemble(ws, ks, cheb=params)
        for g_, k in zip(got, ks):
            ref = OC.cfie_matrix(pts, k, params)
            assert _relerr(g_, ref) < 1e-12
            assert np.max(np.abs(g_ - OA.cfie_matrix(pts, k))) < 1e-11


def test_dlp_cheb_vs_oracle_panels_and_derivs(qb):
    b = qb.make_star()
    sol = qb.DLP_kress(8.0, b)
    pts = qb.evaluate_points(sol, b, 40.0)
    ws = qb.Workspace(sol, pts)
    ks = [40.0 + 0.3j, 40.2]
    got = qb.assemble(ws, ks, cheb=True)
    for g_, k in zip(got, ks):
        assert _relerr(g_, OC.dlp_fredholm(pts, k)) < 1e-12
    F, F1, F2 = qb.assemble(ws, [40.2], deriv=True, cheb=True)
    R, R1, R2 = OC.dlp_fredholm(pts, 40.2, derivs=True)
    assert _relerr(F, R) < 1e-12 and _relerr(F1, R1) < 1e-12 and _relerr(F2, R2) < 1e-11


def test_mixed_cheb_split_words(qb):
    """The mixed form stores hi + lo; hi alone is the FP64 value rounded once."""
    b = qb.make_star()
    sol = qb.CFIE_kress(8.0, b)
    pts = qb.evaluate_points(sol, b, 40.0)
    ws = qb.Workspace(sol, pts)
    k = 40.0 + 0.4j
    hi = qb.assemble(ws, [k], mixed="mixed", cheb=True)[0]
    ref = qb.assemble(ws, [k], cheb=True)[0]
    assert hi.dtype == np.complex64
    assert np.array_equal(hi, ref.astype(np.complex64))


def test_beyn_cheb_eigenvalues(qb):
    b = qb.make_star()
    sol = qb.CFIE_kress(9.0, b)
    pts = qb.evaluate_points(sol, b, 30.0)
    ws = qb.Workspace(sol, pts)
    N = ws.dim
    k0, R, nq, r = 30.0 + 0j, 0.3, 24, 16
    sel = lambda l: np.sort_complex(l[(np.abs(l - k0) < R) & (np.abs(l.imag) < 1e-6)])
    lo, _, _, _ = OB.solve_beyn(lambda zj: [OA.cfie_matrix(pts, z) for z in zj], N, k0, R, nq=nq, r=r,
                                svd_tol=1e-12, rng=np.random.default_rng(7))
    o = sel(lo)
    for form in ("fp64", "mixed"):
        lam, _, _, info = qb.solve_vect(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(7),
                                        ws=ws, mixed=form, use_chebyshev=True)
        a = sel(lam)
        assert len(a) == len(o) > 0
        assert np.max(np.abs(a - o) / np.abs(o)) < 1e-11


@pytest.mark.parametrize("form", ["cfie", "dlp"])
def test_cheb_tables_at_high_k_vs_direct(qb, form):
    """Device-built tables at high k: with 60000 H panels of degree 7 at
    k ~ 150 interpolation adds < 1e-15, so the Chebyshev assembly equals the
    direct-evaluation assembly to the Bessel functions' own accuracy (bound
    5e-14; measured 1.8e-15 - 5.1e-15). With the reference's default panels
    the two differ by the panels' interpolation error near r_min, 2.8e-12
    for this CFIE case."""
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b) if form == "cfie" else qb.DLP_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 1024, 150.0)
    ws = qb.Workspace(sol, pts)
    ks = [150.0 + 0.3j, 149.6 - 0.2j, 150.2 + 0.0j]
    cheb = qb.assemble(ws, ks, cheb=(60000, 7, 12000, 7))
    direct = qb.assemble(ws, ks)
    for c, d in zip(cheb, direct):
        rel = np.max(np.abs(c - d)) / np.max(np.abs(d))
        print(f"{form} cheb vs direct {rel:.3e}")
        assert rel < 5e-14
