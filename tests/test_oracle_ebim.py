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


def test_refine_minima_host_logic(monkeypatch):
    """refine_minima (sweepmethods.jl:471-565) orchestration with the device
    Newton step faked: window = max(3 dk_grid, 1e-3) shrinking by 3 per level,
    pts_scaling_factor x (1, 1.5, 2), each level starting from the previous k,
    and the stop_k_tol early exit."""
    from qbgpu import sweep as SW
    calls = []

    class FakeWS:
        def __init__(self, solver, pts):
            self.factor = solver.pts_scaling_factor

        def close(self):
            pass

    def fake_newton(ws, k0, a, b, maxiter, tol):
        calls.append((ws.factor, k0, a, b))
        return k0 + 1e-4 / ws.factor, 1e-9  # moves less at finer levels

    monkeypatch.setattr(SW, "Workspace", FakeWS)
    monkeypatch.setattr(SW, "evaluate_points", lambda s, b, k: None)
    monkeypatch.setattr(SW, "newton_refine_svd", fake_newton)
    b = G.make_circle(1.0)
    sol = S.DLP_kress(10.0, b)
    ks = np.linspace(13.0, 13.04, 9)              # grid step 0.005
    tens = np.abs(ks - 13.0152) + 1e-6           # one minimum
    kr, tr, hist = SW.refine_minima(sol, b, ks, tens, threshold=1.0)
    assert len(kr) == 1 and len(hist[0]) == 3
    assert [c[0] for c in calls] == [10.0, 15.0, 20.0]
    w = [c[3] - c[1] for c in calls]
    assert abs(w[0] - 0.015) < 1e-12 and abs(w[1] - 0.005) < 1e-12 and abs(w[2] - 0.015 / 9) < 1e-12
    assert calls[1][1] == hist[0][0]["k"] and calls[2][1] == hist[0][1]["k"]
    assert kr[0] == hist[0][2]["k"]
    calls.clear()
    kr, tr, hist = SW.refine_minima(sol, b, ks, tens, threshold=1.0, stop_k_tol=1e-4)
    assert len(hist[0]) == 2  # |k2 - k1| = 1e-4 / 15 <= stop_k_tol ends the ladder at level 2


def test_compute_spectrum_ebim_host_logic(monkeypatch):
    """compute_spectrum_ebim orchestration with the device step faked: one
    discretisation per segment (the first built at ks[0], later ones at their
    last k, reused while k_next <= k_first / 0.95), the Weyl nev per window,
    the merge and the final [k1, k2] filter."""
    from qbgpu import ebim as QE
    built, solved = [], []

    class FakeWS:
        def __init__(self, solver, pts):
            built.append(pts)

        def close(self):
            pass

    def fake_solve(ws, k, dk, nev, full, return_imag_part):
        solved.append((k, dk, nev))
        return np.array([14.0 + 0.5 * round((k - 14.0) / 0.5)]), np.array([abs(k - 14.0)])

    monkeypatch.setattr(QE, "Workspace", FakeWS)
    monkeypatch.setattr(QE, "solve", fake_solve)
    import qbgpu.solvers as QS
    monkeypatch.setattr(QS, "evaluate_points", lambda s, b, k: k)
    b = G.make_circle(1.0)
    ks, dks, nevs = QE.ebim_windows(b, 13.0, 15.0)
    out, tens = QE.compute_spectrum_ebim(S.DLP_kress(10.0, b), b, 13.0, 15.0)
    assert [s[2] for s in solved] == nevs and [s[0] for s in solved] == ks
    # segments: the first discretised at ks[0] (pts0), later ones at their last window's k
    plan = QE.segment_plan(ks, 0.95)
    assert built == [kd for _, _, kd in plan]
    assert built[0] == ks[0] and built[-1] == ks[-1]
    # roots 13.0, 13.5, 14.0, 14.5, 15.0 merged to one copy each, the best (lowest tension) kept
    assert list(out) == [13.0, 13.5, 14.0, 14.5, 15.0]
    assert tens[2] == min(abs(k - 14.0) for k in ks)


def test_ebim_segment_plan_follows_reference_rule():
    """segment_plan against a literal restatement of ebim.jl:1195-1226 in
    1-based indices: seg_last grows while ks[seg_last+1] <= ks[seg_first] /
    seg_reuse_frac; pts = seg_first == 1 ? pts0 (built at ks[1]) :
    evaluate_points(ks[seg_last])."""
    from qbgpu import ebim as QE
    b = G.make_circle(1.0)
    for k1, k2, frac in ((13.0, 15.0, 0.95), (40.0, 44.0, 0.99), (5.0, 9.0, 0.8)):
        ks, _, _ = QE.ebim_windows(b, k1, k2)
        ref = []
        seg_first = 1
        while seg_first <= len(ks):
            seg_last = seg_first
            while seg_last < len(ks) and ks[seg_last + 1 - 1] <= ks[seg_first - 1] / frac:
                seg_last += 1
            ref.append((seg_first - 1, seg_last - 1, ks[0] if seg_first == 1 else ks[seg_last - 1]))
            seg_first = seg_last + 1
        assert QE.segment_plan(ks, frac) == ref
        assert len(ref) >= 2
