"""GPU: Beyn moments reduced on the device (qbg_beyn_moments_qr). With
A0 = Q R the thin QR of the kept moment columns and C = Q^H A1:
R is upper triangular, R^H R = A0^H A0 and R^H C = A0^H A1 (to 1e-12 of
|A0|^2, |A0||A1|), for one call and for columns appended by a second call
(the r -> 2r regrowth); a wrong column count is rejected before any work;
eigenvalues from the reduced moments equal those from the full basis (1e-12
relative) with and without rank saturation, in FP64 and in the mixed form."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _star(qb, n_nodes=400, k=25.0):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, n_nodes, k)
    return sol, pts, qb.Workspace(sol, pts)


@pytest.mark.parametrize("mixed", [False, True])
def test_qr_reduction_matches_moments(qb, mixed):
    sol, pts, ws = _star(qb)
    rng = np.random.default_rng(4)
    V1 = qb.probe_matrix(ws.dim, 12, rng)
    V2 = qb.probe_matrix(ws.dim, 12, rng)
    bh = qb.BeynHandle(ws, 25.0 + 0.05j, 0.4, 16, mixed=mixed)
    try:
        A0a, A1a = bh.moments(V1)
        A0b, A1b = bh.moments(V2)
        R1, C1 = bh.moments_qr(V1)
        R2, C2 = bh.moments_qr(V2, append=True)
    finally:
        bh.close()
    for (Rm, Cm, A0, A1) in ((R1, C1, A0a, A1a), (R2, C2, np.hstack([A0a, A0b]), np.hstack([A1a, A1b]))):
        assert np.array_equal(Rm, np.triu(Rm))
        s0 = np.linalg.norm(A0) ** 2
        s01 = np.linalg.norm(A0) * np.linalg.norm(A1)
        assert np.max(np.abs(Rm.conj().T @ Rm - A0.conj().T @ A0)) < 1e-12 * s0
        assert np.max(np.abs(Rm.conj().T @ Cm - A0.conj().T @ A1)) < 1e-12 * s01


def test_qr_rejects_wrong_column_count(qb):
    from qbgpu import _lib
    sol, pts, ws = _star(qb, 200, 15.0)
    bh = qb.BeynHandle(ws, 15.0, 0.3, 8, mixed=False)
    try:
        V = np.asfortranarray(qb.probe_matrix(ws.dim, 4, np.random.default_rng(1)))
        Rm = np.empty((5, 5), np.complex128)
        st = _lib.BeynStats()
        rc = _lib.load().qbg_beyn_moments_qr(bh._h, _lib.vptr(V), 4, 0, 5, _lib.vptr(Rm), _lib.vptr(Rm),
                                             C.byref(st))
        assert rc == _lib.QBG_EINVAL
        assert "m = 5" in _lib.last_error()
    finally:
        bh.close()


@pytest.mark.parametrize("mixed,r", [(False, 8), (True, 8), (True, 24)])
def test_solve_reduced_equals_full_basis(qb, mixed, r):
    sol, pts, ws = _star(qb)
    kw = dict(nq=24, r=r, svd_tol=1e-12, mixed=mixed, ws=ws)
    lam_r, info_r = qb.solve(sol, pts, 25.0 + 0j, 0.5, rng=np.random.default_rng(7), return_info=True, **kw)
    B, Uk, info_f = qb.construct_B_matrix(sol, pts, ws.dim, 25.0 + 0j, 0.5, rng=np.random.default_rng(7),
                                          return_info=True, basis=True, **{k: v for k, v in kw.items()
                                                                           if k != "ws"}, ws=ws)
    lam_f = np.linalg.eigvals(B)
    assert info_r["rk"] == info_f["rk"] and info_r["r"] == info_f["r"]
    sel = lambda l: np.sort_complex(l[(np.abs(l - 25.0) < 0.5) & (np.abs(l.imag) < 1e-6)])
    a, f = sel(lam_r), sel(lam_f)
    assert len(a) == len(f) > 0
    assert np.max(np.abs(a - f) / np.abs(f)) < 1e-12


def test_beyn_B_entry_matches_host_path(qb):
    """qbg_beyn_B (construct_B_matrix in one library call: device QR of A0,
    host one-sided Jacobi SVD of R, the absolute rank test, one regrowth with
    the appended block) against construct_B_matrix on the same probes, whose
    SVD runs in LAPACK on the full A0: same rank and final column count,
    eigenvalues of B inside the contour to 5e-11 relative (measured 4.7e-12
    and 1.1e-11 with different summation orders of the FP64 products, at
    svd_tol 1e-12, where the kept singular values reach 1e-12; all of them to
    1e-9), the same singular values to 1e-12 of
    the largest, and U_k spanning the same space (principal-angle cosines
    within 1e-8 of one, the median within 1e-13)."""
    import numpy as np
    b = qb.make_star()
    sol = qb.CFIE_kress(9.0, b)
    pts = qb.evaluate_points(sol, b, 30.0)
    ws = qb.Workspace(sol, pts)
    N = ws.dim
    k0, R, nq, r = 30.0 + 0j, 0.3, 24, 8
    for svd_tol in (1e-12, 1e-3):
        rng = np.random.default_rng(11)
        V1 = qb.probe_matrix(N, r, rng)
        V2 = qb.probe_matrix(N, r, rng)
        bh = qb.BeynHandle(ws, k0, R, nq)
        B, Uk, info = bh.B_matrix(V1, V2, svd_tol=svd_tol)
        bh.close()
        Bh, Ukh, infoh = qb.construct_B_matrix(sol, pts, N, k0, R, nq=nq, r=r, svd_tol=svd_tol,
                                               rng=np.random.default_rng(11), ws=ws, return_info=True)
        assert info["rk"] == infoh["rk"] > 0 and info["r"] == infoh["r"]
        assert np.max(np.abs(info["S"] - infoh["S"])) <= 1e-12 * infoh["S"][0]
        lam, lamh = np.linalg.eigvals(B), np.linalg.eigvals(Bh)
        rel = np.array([np.min(np.abs(lamh - x)) / abs(x) for x in lam])
        inside = np.abs(lam - k0) < R
        assert inside.any()
        # the eigenvalues inside the contour are the well-conditioned ones; the
        # spurious ones outside it carry the conditioning of the truncated A0
        assert rel[inside].max() < 5e-11, (svd_tol, rel[inside].max())
        assert rel.max() < 1e-9, (svd_tol, rel.max())
        # cosines of the principal angles; the directions whose singular values
        # sit near svd_tol are fixed only to eps * S[0] / S[rk-1] (1.5e-10
        # measured at svd_tol 1e-12), the rest to rounding
        s = np.linalg.svd(Uk.conj().T @ Ukh, compute_uv=False)
        assert np.all(np.abs(s - 1.0) < 1e-8)
        assert np.median(np.abs(s - 1.0)) < 1e-13
