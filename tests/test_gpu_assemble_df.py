"""GPU: Chebyshev-panel assembly of the mixed form on double-float (FP32 pair)
arithmetic. Full operators (no symmetry) run on the J/E tables
(k_cheb_build_je / k_assemble_je_df: J0, J1 and the entire parts of Y0, Y1 on
1.5x the J panels, the logarithm and the pole of the Hankel functions applied
per pair) and are checked against the FP64 direct assembly (no tables); the
symmetry-reduced DLP runs on the H and J tables of the FP64 route and is
checked against the FP64 Chebyshev assembly of the same tables.

hi + lo must carry the FP64 value: |hi + lo - A64| <= 1e-13 max|A64| overall
and <= 1e-12 |A64| elementwise where |A64| >= 1e-3 max|A64| (measured at most
3e-13 on full operators, 4.1e-13 on the reflected stadium, whose reduced
entries sum the pair and its orbit images). The double-float
sums carry ~2^-48 of the sum of |terms| (FP64: 2^-53), so small entries that
are cancelling sums (cross-component pairs, near zeros of J0, J1) keep an
absolute, not a relative, error bound (1.6e-12 relative measured at
|A64| ~ 1e-6 max on the holed disk); hi alone is A64 rounded to complex64
(|hi - A64| <= 2^-23 |A64| + 1e-13 max|A64|). CFIE (all four series, the
cross-component pairs of a holed domain) and DLP (J1, H1 only), complex
wavenumbers, and a low wavenumber whose near pairs take the direct FP64
route (|k| r < 0.2)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(qb, ws, ks, ref_direct=False):
    # the J/E tables and the FP64 route's H and J tables interpolate
    # differently, so full operators are held against the FP64 direct
    # evaluation (no tables); the reduced ones share the FP64 route's tables
    ref = qb.assemble(ws, ks) if ref_direct else qb.assemble(ws, ks, cheb=True)
    out = qb.assemble(ws, ks, mixed=True, cheb=True, split_lo=True)
    nk = len(ks)
    for q in range(nk):
        a = ref[q]
        hi, lo = out[q], out[nk + q]
        v = hi.astype(np.complex128) + lo.astype(np.complex128)
        scale = np.max(np.abs(a))
        err = np.abs(v - a)
        assert np.max(err) <= 1e-13 * scale, (q, np.max(err) / scale)
        big = np.abs(a) >= 1e-3 * scale
        small = (np.abs(a) >= 1e-6 * scale) & ~big
        print(f"k={ks[q]}: max err/max|A| {np.max(err) / scale:.2e}, big entries rel {np.max(err[big] / np.abs(a[big])):.2e}"
              f", small entries rel {np.max(err[small] / np.abs(a[small])) if small.any() else 0.0:.2e}")
        assert np.max(err[big] / np.abs(a[big])) <= 1e-12, (q, np.max(err[big] / np.abs(a[big])))
        assert np.all(np.abs(hi.astype(np.complex128) - a) <= 2.0 ** -23 * np.abs(a) + 1e-13 * scale)


@pytest.mark.parametrize("ks", [[25.0 + 0.3j, 24.7 - 0.2j], [2.0 + 0.1j]])
def test_df_assembly_cfie_star(qb, ks):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 400, 25.0)
    _check(qb, qb.Workspace(sol, pts), ks, ref_direct=True)


def test_df_assembly_cfie_holed(qb):
    b = qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 500, 20.0)
    _check(qb, qb.Workspace(sol, pts), [20.0 + 0.2j, 19.5 + 0.0j], ref_direct=True)


def test_df_assembly_dlp_stadium(qb):
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 600, 30.0)
    _check(qb, qb.Workspace(sol, pts), [30.0 + 0.25j, 29.6 - 0.1j], ref_direct=True)


def test_df_assembly_je_high_k(qb):
    """The bench's regime: CFIE star at k ~ 200 (|k| r from 0.6 to 500, the
    series branch of the table builder below |k r| = 4 and the asymptotic one
    above), panels tuned to 1e-13 (chebyshev_params_min_cost), against the
    FP64 direct assembly (no tables): |hi + lo - A| <= 2e-13 max|A|."""
    import math
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 1024, 200.0)
    ws = qb.Workspace(sol, pts)
    ks = [200.0 + 0.4j, 199.6 - 0.3j]
    zref = 200.0 + 0.5 * np.exp(2j * math.pi * np.arange(8) / 8)
    cheb = tuple(int(x) for x in qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=1e-13)[:4])
    ref = qb.assemble(ws, ks)
    out = qb.assemble(ws, ks, mixed=True, cheb=cheb, split_lo=True)
    for q in range(len(ks)):
        a = ref[q]
        v = out[q].astype(np.complex128) + out[len(ks) + q].astype(np.complex128)
        scale = np.max(np.abs(a))
        err = np.max(np.abs(v - a)) / scale
        print(f"k={ks[q]} panels {cheb}: max err/max|A| {err:.2e}")
        assert err <= 2e-13, (q, err)


def _reduced(qb, b, sym, n, k, corners=True):
    sol = (qb.DLP_kress_global_corners if corners else qb.DLP_kress)(1.0, b, symmetry=sym)
    pts, sol = qb.points_with_n(sol, b, n, k)
    return qb.Workspace(sol, pts)


@pytest.mark.parametrize("sym", ["xy", "x"])
def test_df_assembly_reduced_stadium(qb, sym):
    """Symmetry-reduced DLP (main pair plus orbit images) in double-float:
    XY reflection (three images) and a single reflection (one image)."""
    s = qb.XYReflection(-1, 1) if sym == "xy" else qb.XReflection(-1)
    ws = _reduced(qb, qb.make_full_stadium(1.0, 1.0), s, 640, 30.0)
    _check(qb, ws, [30.0 + 0.2j, 29.7 - 0.15j])


@pytest.mark.parametrize("n_rot,m", [(4, 1), (5, 2)])
def test_df_assembly_reduced_rotation(qb, n_rot, m):
    """Rotation sectors with complex orbit scales: C4 (three images, double-float
    route) and C5 (orbits of five nodes, FP64 route of the same launcher)."""
    ws = _reduced(qb, qb.make_star(0.2, n_rot), qb.Rotation(n_rot, m), 600, 25.0, corners=False)
    _check(qb, ws, [25.0 + 0.2j, 24.6 + 0.05j])
