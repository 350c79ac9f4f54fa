"""CPU tests of the oracle's EBIM eigen step (oracle/ebim.py).

* the corrected k converges to a circle Dirichlet eigenvalue (a zero of J_0)
  at third order in the distance of the trial k (the expansion is second
  order), in both conventions;
* SciPy's left eigenvectors of the pencil satisfy u^H A = lambda u^H A', the
  property solve_full!'s correction relies on;
* on the circle with a hole (CFIE) the conventions differ: solve_krylov!'s u
  is the eigenvector of (A^{-1} A')^H, not a left vector of the pencil, and its
  |Re(k_c) - k| < dk rule drops a root that solve_full! keeps.
"""
import numpy as np
import scipy.linalg as sla
from scipy import special as sp

from oracle import assembly as OA, ebim as OE
from qbgpu import geometry as G, solvers as S


def test_oracle_ebim_circle_third_order():
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.DLP_kress(10.0, b), b, 16.0)
    z0 = float(sp.jn_zeros(0, 5)[4])
    for d in (0.002, 0.005, 0.01):
        kt = z0 + d
        A, dA, ddA = OA.dlp_fredholm(pts, kt, derivs=True)
        for kc, tens in (OE.solve_full(A, dA, ddA, kt, 0.05), OE.solve_krylov(A, dA, ddA, kt, 0.05, nev=5)):
            assert len(kc) == 1
            assert abs(kc[0] - z0) < 3.0 * d ** 3
            assert abs(tens[0] - d) < 3.0 * d ** 3


def test_oracle_ebim_left_vectors_and_conventions():
    hb = G.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))
    pts = S.evaluate_points(S.CFIE_kress(10.0, hb), hb, 12.0)
    k, dk = 12.3, 0.15
    A, dA, ddA = OA.cfie_matrix_derivs(pts, k)
    lam, VL, VR = sla.eig(A, dA, left=True, right=True)
    for i in np.nonzero(np.abs(lam) < 0.2)[0]:
        u = VL[:, i]
        assert np.linalg.norm(u.conj() @ A - lam[i] * (u.conj() @ dA)) < 1e-12 * np.linalg.norm(A) * np.linalg.norm(u)
    kf, _ = OE.solve_full(A, dA, ddA, k, dk)
    kk, _ = OE.solve_krylov(A, dA, ddA, k, dk, nev=6)
    assert len(kf) == 4 and len(kk) == 3
    # the root at 12.139 has |Re(k_c) - k| > dk: kept by solve_full only
    assert np.min(np.abs(kf - 12.139)) < 1e-3 and np.min(np.abs(kk - 12.139)) > 0.05
    # shared roots differ at the level of the two second-order terms
    d = [np.min(np.abs(kf - x)) for x in kk]
    assert max(d) > 1e-7 and max(d) < 1e-2


def test_oracle_newton_refine_circle():
    """newton_refine_svd! converges to a zero of J_m from a sweep-grid guess;
    the tension sqrt(lambda_min(A^H A)) bottoms out near sqrt(eps) |A|."""
    from oracle import sweep as OS
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.DLP_kress(10.0, b), b, 16.0)
    z = float(sp.jn_zeros(3, 3)[2])  # 13.0152
    k, t = OS.newton_refine_svd(lambda kk: OA.dlp_fredholm(pts, kk, derivs=True), z + 2e-3, z - 0.01, z + 0.01)
    assert abs(k - z) < 1e-8
    assert t < 1e-7


def test_oracle_boundary_density_circle():
    """On the circle at the simple eigenvalue j_{0,5} (a zero of J_0), the
    adjoint Fredholm matrix is singular and its null vector, the boundary
    normal derivative of the J_0 mode, is constant along the boundary."""
    from oracle import sweep as OS
    b = G.make_circle(1.0)
    pts = S.evaluate_points(S.DLP_kress(10.0, b), b, 16.0)
    z = float(sp.jn_zeros(0, 5)[4])
    sig, u = OS.smallest_nullvec(OS.adjoint_fredholm(OA.dlp_fredholm(pts, z), pts.ds))
    assert sig < 1e-10
    assert np.max(np.abs(np.abs(u) - np.abs(u).mean())) < 1e-8 * np.abs(u).mean()
    sig2, _ = OS.smallest_nullvec(OS.adjoint_fredholm(OA.dlp_fredholm(pts, z + 0.05), pts.ds))
    assert sig2 > 1e-4


def test_ebim_merge_and_windows():
    """Host logic of compute_spectrum_ebim (ebim.jl:1158-1268): the window grid
    and Weyl nev, and overlap_and_merge_ebim! (ebim.jl:1059-1107) keeping the
    lower-tension copy of a root found by two windows."""
    from qbgpu import ebim as QE
    b = G.make_circle(1.0)
    ks, dks, nevs = QE.ebim_windows(b, 14.0, 15.0)
    assert ks[0] == 14.0 and ks[-1] < 15.0 and ks[-1] + dks[-1] >= 15.0
    assert all(abs(d - 0.05 * k ** (-1 / 3)) < 1e-15 for k, d in zip(ks, dks))
    assert nevs[0] == int(np.ceil((np.pi * 14.0 / (2 * np.pi) - 2 * np.pi / (4 * np.pi)) * dks[0])) + 10
    kl, tl, cl = [], [], []
    QE.overlap_and_merge_ebim(kl, tl, [14.7959518, 14.9309177], [3e-3, 2e-2], cl, 14.78, 14.80)
    QE.overlap_and_merge_ebim(kl, tl, [14.7959517, 14.8212687], [1e-3, 4e-3], cl, 14.80, 14.82)
    assert len(kl) == 3
    assert abs(kl[0] - 14.7959517) < 1e-12 and tl[0] == 1e-3  # the lower tension wins
    assert cl == [True, False, False]
