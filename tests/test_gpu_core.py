"""GPU parity tests: device kernels through the C ABI against the FP64 oracle.

Tolerances: FP64 assembly entries 1e-12 relative to the matrix max-norm
(special functions agree with AMOS to ~1e-15, the geometry is identical);
mixed assembly 2e-6; Beyn moments with the same probe block 1e-10 relative;
eigenvalues: plain FP64 vs oracle 1e-12 relative, mixed vs plain 1e-10
relative (the project's accuracy target).
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest
from scipy import special as sp

from oracle import assembly as OA, beyn as OB

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


def _relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_bessel_device_vs_mpmath(qb):
    g = json.loads((GOLD / "bessel_mpmath.json").read_text())
    z = np.array([complex(*r["z"]) for r in g["values"]])
    ref = np.array([[complex(*v) for v in r["j0j1y0y1"]] for r in g["values"]])
    got = qb.bessel01(z)
    err = np.abs(got - ref).max(axis=1) / np.maximum(np.abs(ref).max(axis=1), 1.0)
    assert err.max() < 2e-14, (z[np.argmax(err)], err.max())
    big = np.abs(z) >= 12.0
    got32 = qb.bessel01(z[big], f32=True)
    err32 = np.abs(got32 - ref[big]).max(axis=1) / np.abs(ref[big]).max(axis=1)
    assert err32.max() < 3e-6


@pytest.mark.parametrize("deriv", [False, True])
def test_dlp_real_k_vs_oracle(qb, deriv):
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(10.0, b)
    pts = qb.evaluate_points(sol, b, 30.0)
    ws = qb.Workspace(sol, pts)
    for k in (29.3, 30.0):
        got = qb.assemble(ws, [k], deriv=deriv)
        ref = OA.dlp_fredholm(pts, k, derivs=deriv)
        ref = ref if deriv else (ref,)
        for g_, r_ in zip(got, ref):
            assert _relerr(g_, r_) < 1e-12


def test_dlp_star_complex_k_vs_oracle(qb):
    b = qb.make_star()
    sol = qb.DLP_kress(8.0, b)
    pts = qb.evaluate_points(sol, b, 40.0)
    ws = qb.Workspace(sol, pts)
    ks = [40.0 + 0.4j, 39.7 - 0.3j]
    got = qb.assemble(ws, ks)
    for g_, k in zip(got, ks):
        assert _relerr(g_, OA.dlp_fredholm(pts, k)) < 1e-12


def test_cfie_complex_k_vs_oracle(qb):
    for b in (qb.make_star(), qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))):
        sol = qb.CFIE_kress(8.0, b)
        pts = qb.evaluate_points(sol, b, 30.0)
        ws = qb.Workspace(sol, pts)
        ks = [30.0 + 0.5j, 30.2 - 0.1j, 29.9 + 0.0j]
        got = qb.assemble(ws, ks)
        for g_, k in zip(got, ks):
            assert _relerr(g_, OA.cfie_matrix(pts, k)) < 1e-12


def test_mixed_assembly_vs_oracle(qb):
    b = qb.make_star()
    sol = qb.CFIE_kress(8.0, b)
    pts = qb.evaluate_points(sol, b, 60.0)
    ws = qb.Workspace(sol, pts)
    ks = [60.0 + 0.5j, 60.3 - 0.2j]
    got = qb.assemble(ws, ks, mixed="mixed")   # FP64 values rounded once to complex64
    got32 = qb.assemble(ws, ks, mixed="fp32")  # FP32 kernel values
    for g_, g32, k in zip(got, got32, ks):
        ref = OA.cfie_matrix(pts, k)
        assert g_.dtype == np.complex64 and g32.dtype == np.complex64
        assert _relerr(g_.astype(np.complex128), ref) < 1.2e-7
        assert _relerr(g32.astype(np.complex128), ref) < 2e-6


def test_sigma_min_vs_oracle_and_bessel_zero(qb):
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(10.0, b)
    pts = qb.evaluate_points(sol, b, 20.0)
    ws = qb.Workspace(sol, pts)
    z = float(sp.jn_zeros(3, 3)[2])
    ks = np.array([z - 0.05, z, z + 0.05])
    sig = qb.sigma_min(ws, ks)
    ref = np.array([OB.sigma_min(OA.dlp_fredholm(pts, k)) for k in ks])
    assert np.allclose(sig[[0, 2]], ref[[0, 2]], rtol=1e-10)
    assert sig[1] < 1e-11


def _beyn_case(qb, mixed):
    b = qb.make_star()
    sol = qb.CFIE_kress(9.0, b)
    pts = qb.evaluate_points(sol, b, 30.0)
    ws = qb.Workspace(sol, pts)
    return b, sol, pts, ws


def test_beyn_moments_fp64_vs_oracle(qb):
    b, sol, pts, ws = _beyn_case(qb, False)
    N = ws.dim
    k0, R, nq, r = 30.0 + 0j, 0.3, 16, 12
    V = qb.probe_matrix(N, r, np.random.default_rng(5))
    bh = qb.BeynHandle(ws, k0, R, nq, use_chebyshev=False)
    A0, A1 = bh.moments(V)
    zj, wj = OB.contour(k0, R, nq)
    Ts = [OA.cfie_matrix(pts, z) for z in zj]
    R0, R1, _ = OB.moments(Ts, zj, wj, V)
    assert _relerr(A0, R0) < 1e-10
    assert _relerr(A1, R1) < 1e-10
    # second call with a wider block reuses the factors (r -> 2r regrowth)
    V2 = qb.probe_matrix(N, 2 * r, np.random.default_rng(6))
    A0b, _ = bh.moments(V2)
    R0b, _, _ = OB.moments(Ts, zj, wj, V2)
    assert _relerr(A0b, R0b) < 1e-10


def test_beyn_eigenvalues_plain_vs_oracle_and_mixed(qb):
    b, sol, pts, ws = _beyn_case(qb, False)
    N = ws.dim
    k0, R, nq, r = 30.0 + 0j, 0.3, 24, 16
    lam, Uk, Y, info = qb.solve_vect(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(7),
                                     ws=ws, use_chebyshev=False)
    lo, _, _, _ = OB.solve_beyn(lambda zj: [OA.cfie_matrix(pts, z) for z in zj], N, k0, R, nq=nq, r=r,
                                svd_tol=1e-12, rng=np.random.default_rng(7))
    sel = lambda l: np.sort_complex(l[(np.abs(l - k0) < R) & (np.abs(l.imag) < 1e-6)])
    a, o = sel(lam), sel(lo)
    assert len(a) == len(o) and len(a) > 0
    assert np.max(np.abs(a - o) / np.abs(o)) < 1e-12
    lm, _, _, infom = qb.solve_vect(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(7),
                                    ws=ws, mixed=True, use_chebyshev=False)
    m = sel(lm)
    assert len(m) == len(a)
    assert np.max(np.abs(m - a) / np.abs(a)) < 1e-10
    assert infom["stats"][0]["refine_sweeps"] >= 1
    # FP32 form: operator rounded to FP32, so the error is bounded by that rounding, not by 1e-10
    lf, _, _, _ = qb.solve_vect(sol, pts, k0, R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(7),
                                ws=ws, mixed="fp32")
    f = sel(lf)
    assert len(f) == len(a)
    assert np.max(np.abs(f - a) / np.abs(a)) < 1e-7


def test_sigma_min_star_cfie_vs_oracle(qb):
    """sigma_min of a CFIE operator without symmetry (a generic spectrum) at
    several k: inverse iteration agrees with the oracle's full SVD to 1e-10."""
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 300, 15.0)
    ws = qb.Workspace(sol, pts)
    ks = np.linspace(14.6, 15.4, 5)
    sig = qb.sigma_min(ws, ks)
    ref = np.array([OB.sigma_min(OA.cfie_matrix(pts, k)) for k in ks])
    assert np.allclose(sig, ref, rtol=1e-10, atol=0.0)
