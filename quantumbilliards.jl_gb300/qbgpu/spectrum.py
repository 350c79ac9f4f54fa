"""Beyn spectrum driver (mirrors beyn.jl): Weyl window planning
(plan_weyl_windows, :141-160, with the area-term estimates of :65-134),
disks from windows (:167-173), the residual filters
(residual_and_norm_select :557-593, imag_k_check_EXPERIMENTAL :623-721) and
compute_spectrum_beyn (:778-921).

The device does the N^2 and N^3 work: all disks' contour nodes in one batch
(batched=True), T(lambda) at the candidates and T(lambda) phi with its norms
(qbg_candidate_residuals). The host keeps the small dense steps.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .beyn import BeynHandle, _B_from_moments, probe_matrix
from .operators import DEFAULT_CHEB, Workspace, _ks_array, chebyshev_params
from .solvers import evaluate_points
from .symmetry import Reflection, Rotation


# --------------------------------------------------------------------------
# Weyl windows (area term only, as the reference's planner)
# --------------------------------------------------------------------------
def _area(billiard, fundamental: bool, symmetry=None) -> float:
    A = float(billiard.area)
    if fundamental and symmetry is not None:
        if isinstance(symmetry, Rotation):
            A /= symmetry.n
        elif isinstance(symmetry, Reflection):
            A /= 4.0 if symmetry.axis == "origin" else 2.0
    return A


def delta_weyl(A: float, k: float, dk: float) -> float:
    return A * ((k + dk) ** 2 - k ** 2) / (4 * math.pi)


def initial_step_from_dos(A, k, m, min_step=1e-6):
    rho = max(A * k / (2 * math.pi), 1e-12)
    return max(m / rho, min_step)


def grow_upper_bound(A, k, m, dk0, remaining, max_grows=60):
    dk = min(remaining, max(dk0, np.finfo(float).eps * max(k, 1.0)))
    for _ in range(max_grows):
        if delta_weyl(A, k, dk) >= m - np.finfo(float).eps:
            return dk, True
        if dk >= 0.999999 * remaining:
            return remaining, False
        dk = min(remaining, 2 * dk)
    return dk, delta_weyl(A, k, dk) >= m


def bisect_for_delta_k(A, k, m, lo, hi, tol_levels=0.1, maxit=50):
    nlo = delta_weyl(A, k, lo)
    if abs(nlo - m) <= tol_levels:
        return lo
    nhi = delta_weyl(A, k, hi)
    if abs(nhi - m) <= tol_levels:
        return hi
    for _ in range(maxit):
        mid = 0.5 * (lo + hi)
        nm = delta_weyl(A, k, mid)
        if abs(nm - m) <= tol_levels:
            return mid
        if nm < m:
            lo = mid
        else:
            hi = mid
        if hi - lo <= max(1e-12, 1e-9 * max(1.0, k)):
            return 0.5 * (lo + hi)
    return 0.5 * (lo + hi)


def plan_weyl_windows(billiard, k1, k2, m=10, Rmax=1.0, fundamental=True, tol_levels=0.1, maxit=50, symmetry=None):
    """Windows [kL, kR] covering [k1, k2], each holding about m levels by the
    Weyl area estimate and at most 2 Rmax long (beyn.jl:141-160)."""
    A = _area(billiard, fundamental, symmetry)
    iv = []
    k = float(k1)
    eps = np.finfo(float).eps
    while k < k2 - eps:
        rem_raw = k2 - k
        rem = 2.0 * Rmax if rem_raw > 2 * Rmax else rem_raw
        if delta_weyl(A, k, rem) <= m + tol_levels and rem == rem_raw:
            iv.append((k, float(k2)))
            break
        dk0 = initial_step_from_dos(A, k, m)
        hi, ok = grow_upper_bound(A, k, m, dk0, rem)
        if not ok:
            iv.append((k, k + hi))
            k += hi
            continue
        dk = bisect_for_delta_k(A, k, m, 0.0, hi, tol_levels, maxit)
        kR = min(k + dk, k + rem)
        iv.append((k, kR))
        k = kR
    return iv


def beyn_disks_from_windows(iv):
    """Centre = window midpoint, radius = half the length (beyn.jl:167-173)."""
    k0 = np.array([complex(0.5 * (a + b)) for a, b in iv], dtype=np.complex128)
    R = np.array([0.5 * (b - a) for a, b in iv])
    return k0, R


# --------------------------------------------------------------------------
# residual filters
# --------------------------------------------------------------------------
def candidate_residuals(ws: Workspace, lambdas, Phi, cheb=None) -> np.ndarray:
    """Rows (||T phi||_2, ||T phi||_1, opnorm(T,1), ||phi||_1, ||phi||_2) per candidate."""
    lam = _ks_array(lambdas)
    Phi = np.asfortranarray(Phi, dtype=np.complex128)
    out = np.empty((len(lam), 5))
    prm = None
    if cheb is not None and cheb is not False:
        prm = C.byref(L.ChebParams(*(DEFAULT_CHEB if cheb is True else cheb)))
    L.check(L.load().qbg_candidate_residuals(ws.handle, L.dptr(lam.view(np.float64)), len(lam), L.vptr(Phi), prm,
                                             L.dptr(out)))
    return out


def residual_and_norm_select(ws: Workspace, lam, Uk, Y, k0, R, res_tol, matnorm="one", epss=1e-15,
                             auto_discard_spurious=True, cheb=True):
    """beyn.jl:557-593: keep candidates inside the disk with ||T(lambda) phi|| < res_tol.
    Returns (idx, Phi_kept, tens, tensN)."""
    lam = np.asarray(lam)
    inside = np.nonzero(np.abs(lam - k0) <= R)[0]
    N = Uk.shape[0]
    if len(inside) == 0:
        return inside, np.zeros((N, 0), complex), np.zeros(0), np.zeros(0)
    if matnorm != "one":
        raise NotImplementedError("matnorm=:one is the driver's setting (beyn.jl:882)")
    Phi = Uk @ Y[:, inside]
    o = candidate_residuals(ws, lam[inside], Phi, cheb)
    tens = o[:, 0]
    tensN = o[:, 1] / (o[:, 2] * (o[:, 3] + epss) + epss)
    keep = np.ones(len(inside), bool) if not auto_discard_spurious else tens < res_tol
    return inside[keep], Phi[:, keep], tens[keep], tensN[keep]


def imag_k_check(ws_list, lams, Uks, Ys, k0s, Rs, res_tol, pad=20, group_size=100, cheb=True):
    """imag_k_check_EXPERIMENTAL (beyn.jl:623-721): check candidates in order of
    decreasing |Im lambda|, group by group, dropping those with
    ||T(lambda) phi|| >= res_tol, until `pad` checked candidates in a row pass."""
    cands = []
    inside = []
    for i, lam in enumerate(lams):
        idx = np.nonzero(np.abs(lam - k0s[i]) <= Rs[i])[0]
        inside.append(idx)
        for j in idx:
            cands.append((i, int(j), abs(lam[j].imag), lam[j].real))
    cands.sort(key=lambda c: -c[2])
    drop = set()
    res = {}
    streak = 0
    pos = 0
    stop = False
    while pos < len(cands) and not stop:
        group = cands[pos:pos + group_size]
        for iw in sorted({c[0] for c in group}):
            sub = [c for c in group if c[0] == iw]
            Phi = np.column_stack([Uks[iw] @ Ys[iw][:, j] for _, j, _, _ in sub])
            o = candidate_residuals(ws_list[iw], [lams[iw][j] for _, j, _, _ in sub], Phi, cheb)
            for c, r in zip(sub, o[:, 0]):
                res[(c[0], c[1])] = r
        for c in group:
            r = res[(c[0], c[1])]
            if r >= res_tol:
                drop.add((c[0], c[1]))
                streak = 0
            else:
                streak += 1
                if streak >= pad:
                    stop = True
                    break
        pos += len(group)
    keep, resid = [], []
    for i, idx in enumerate(inside):
        kk = [j for j in idx if (i, int(j)) not in drop]
        keep.append(np.array(kk, dtype=int))
        resid.append(np.array([res.get((i, int(j)), np.nan) for j in kk]))
    return keep, resid


# --------------------------------------------------------------------------
# driver
# --------------------------------------------------------------------------
def compute_spectrum_beyn(solver, billiard, k1, k2, m=50, Rmax=0.5, nq=48, r=None, svd_tol=1e-12, res_tol=1e-9,
                          auto_discard_spurious=True, use_chebyshev=True, cheb=DEFAULT_CHEB, cheb_tol=1e-13,
                          max_iter=20, sampling_points=50000, mixed=True, batched=True, use_imag_check=True,
                          return_imag_part=False, rng=None):
    """compute_spectrum_beyn (beyn.jl:778-921). Returns
    (ks, tens, us, pts, tensN) over all windows.

    batched=True discretises once at the largest k of the interval and runs
    every disk's contour nodes in one device batch (a finer grid than the
    reference's per-disk discretisation, same for all disks); batched=False
    discretises per disk at real(k0) as the reference does."""
    r = r if r is not None else m + 15
    rng = rng if rng is not None else np.random.default_rng(0)
    fundamental = getattr(solver, "symmetry", None) is not None
    iv = plan_weyl_windows(billiard, k1, k2, m=m, Rmax=Rmax, fundamental=fundamental,
                           symmetry=getattr(solver, "symmetry", None))
    if len(iv) >= 2:  # merge a degenerate last window (beyn.jl:782-794)
        (kL2, kR2), (kL3, kR3) = iv[-2], iv[-1]
        if kR3 - kL3 <= max(100 * np.finfo(float).eps * k2, 1e-9 * max(k2, 1.0)):
            if kR3 - kL2 <= 2 * Rmax + 10 * np.finfo(float).eps * k2:
                iv[-2] = (kL2, kR3)
            iv.pop()
    k0, R = beyn_disks_from_windows(iv)
    if len(k0) == 0:
        return [], [], [], [], []
    if batched:
        kref = float(np.max(k0.real + R))
        pts_one = evaluate_points(solver, billiard, kref)
        ws_one = Workspace(solver, pts_one)
        all_pts = [pts_one] * len(k0)
        all_ws = [ws_one] * len(k0)
    else:
        all_pts = [evaluate_points(solver, billiard, float(z.real)) for z in k0]
        all_ws = [Workspace(solver, p) for p in all_pts]
    if use_chebyshev:
        imax = int(np.argmax(k0.real + R))
        th = 2 * math.pi * np.arange(nq) / nq
        zref = k0[imax] + R[imax] * np.exp(1j * th)
        cheb = chebyshev_params(solver, all_pts[imax], zref, ws=all_ws[imax], npanels_h_init=cheb[0], M_h_init=cheb[1],
                                npanels_j_init=cheb[2], M_j_init=cheb[3], tol=cheb_tol,
                                sampling_points=sampling_points, max_iter=max_iter)[:4]
    lams, Uks, Ys = [], [], []
    if batched:
        N = all_ws[0].dim
        bh = BeynHandle(all_ws[0], k0, R, nq, mixed, use_chebyshev=use_chebyshev, cheb=cheb if use_chebyshev else None)
        try:
            V = probe_matrix(N, r, rng)
            A0s, A1s = bh.moments(V)
            S = [np.linalg.svd(a, compute_uv=False) for a in A0s]
            grow = [int(np.count_nonzero(s >= svd_tol)) == r and 2 * r < N for s in S]
            if any(grow):
                A0n, A1n = bh.moments(probe_matrix(N, r, rng))
        finally:
            bh.close()
        for d in range(len(k0)):
            A0, A1 = A0s[d], A1s[d]
            if grow[d]:
                A0, A1 = np.hstack([A0, A0n[d]]), np.hstack([A1, A1n[d]])
            B, Uk, rk, _ = _B_from_moments(A0, A1, svd_tol)
            lam, Y = (np.linalg.eig(B) if rk else (np.zeros(0, complex), np.zeros((0, 0), complex)))
            lams.append(lam), Uks.append(Uk), Ys.append(Y)
    else:
        from .beyn import solve_vect
        for d in range(len(k0)):
            lam, Uk, Y, _ = solve_vect(solver, all_pts[d], k0[d], R[d], nq=nq, r=r, svd_tol=svd_tol, rng=rng,
                                       mixed=mixed, ws=all_ws[d], use_chebyshev=use_chebyshev,
                                       cheb=cheb if use_chebyshev else None)
            lams.append(lam), Uks.append(Uk), Ys.append(Y)
    cheb_res = cheb if use_chebyshev else None
    ks, tens, us, pts_out, tensN = [], [], [], [], []
    if use_imag_check:
        keep, resid = imag_k_check(all_ws, lams, Uks, Ys, k0, R, res_tol, cheb=cheb_res)
        for d in range(len(k0)):
            for jj, j in enumerate(keep[d]):
                lam = lams[d][j]
                ks.append(lam if return_imag_part else lam.real)
                tens.append(abs(lam.imag))
                tensN.append(resid[d][jj])
                us.append(Uks[d] @ Ys[d][:, j])
                pts_out.append(all_pts[d])
    else:
        for d in range(len(k0)):
            if len(lams[d]) == 0:
                continue
            idx, Phi, t, tn = residual_and_norm_select(all_ws[d], lams[d], Uks[d], Ys[d], k0[d], R[d], res_tol,
                                                       auto_discard_spurious=auto_discard_spurious, cheb=cheb_res)
            for jj, j in enumerate(idx):
                lam = lams[d][j]
                ks.append(lam if return_imag_part else lam.real)
                tens.append(t[jj])
                tensN.append(tn[jj])
                us.append(Phi[:, jj])
                pts_out.append(all_pts[d])
    return ks, tens, us, pts_out, tensN
