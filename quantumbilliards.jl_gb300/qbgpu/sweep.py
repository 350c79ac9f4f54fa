"""sigma_min sweep (mirrors sweepmethods.jl:51-60, 132-217).

``k_sweep`` discretises once at max(ks) (sweepmethods.jl:52), builds the
workspace, and returns sigma_min(A(k)) for every k, computed on the device by
FP64 LU and block inverse iteration (the reference: LAPACK.gesvd!('N','N',A)[end],
macros.jl:159-161). ``get_eigenvalues`` is the reference's peak search on the
second difference of log10(sigma) (sweepmethods.jl:193-217).
``newton_refine_svd`` (sweepmethods.jl:307-368) runs on the device
(qbg_newton_refine); ``refine_minima`` (sweepmethods.jl:471-565) drives it over
the minima with the reference's discretisation levels and shrinking windows.
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from . import _lib as L
from .operators import Workspace, sigma_min
from .solvers import evaluate_points


def k_sweep(solver, billiard, ks, ws: Workspace = None, pts=None):
    ks = np.asarray(ks, dtype=np.float64)
    if ws is None:
        pts = pts if pts is not None else evaluate_points(solver, billiard, float(ks.max()))
        ws = Workspace(solver, pts)
    return sigma_min(ws, ks)


def get_eigenvalues(ks, tens, threshold=200.0):
    ks = np.asarray(ks, dtype=np.float64)
    y = np.log10(np.abs(np.asarray(tens, dtype=np.float64)))
    g1 = np.diff(y) / np.diff(ks)
    x1 = 0.5 * (ks[:-1] + ks[1:])
    g2 = np.diff(g1) / np.diff(x1)
    x2 = 0.5 * (x1[:-1] + x1[1:])
    out = [x2[i] for i in range(1, len(g2) - 1) if g2[i] > g2[i - 1] and g2[i] > g2[i + 1] and g2[i] > threshold]
    return np.array(out)


def newton_refine_svd(ws: Workspace, k0, a=0.0, b=np.inf, maxiter=8, tol=1e-12, return_iters=False):
    """newton_refine_svd! (sweepmethods.jl:307-368) on the workspace's
    discretisation: returns (k, tension) [, Newton steps]."""
    lib = L.load()
    k, t, it = C.c_double(), C.c_double(), C.c_int32()
    L.check(lib.qbg_newton_refine(ws.handle, float(k0), float(a), float(b), int(maxiter), float(tol), C.byref(k),
                                  C.byref(t), C.byref(it)))
    return (k.value, t.value, it.value) if return_iters else (k.value, t.value)


def refine_minima(solver, billiard, ks, tens, threshold=200.0, pts_refinement_factors=(1.0, 1.5, 2.0),
                  dim_refinement_factors=(1.0, 1.1, 1.25), window_shrink=3.0, stop_k_tol=0.0, stop_t_tol=0.0,
                  initial_refinement_interval=1e-3, newton_max_iter=8, newton_tol=1e-12):
    """refine_minima (sweepmethods.jl:471-565) for the boundary-integral
    solvers: every minimum of the sweep (get_eigenvalues, or the single k) is
    refined by newton_refine_svd at the discretisation levels
    pts_scaling_factor * pts_refinement_factors[l] inside a window of
    max(3 dk_grid, initial_refinement_interval) that shrinks by window_shrink
    per level; a level stops the ladder early when stop_k_tol / stop_t_tol are
    met. dim_refinement_factors belong to the basis methods and are unused.
    Returns (k, tension, histories)."""
    ks = np.asarray(ks, dtype=np.float64)
    tens = np.asarray(tens, dtype=np.float64)
    if len(ks) != len(tens) or len(pts_refinement_factors) != len(dim_refinement_factors):
        raise ValueError("ks and tens, and the two factor lists, must have equal lengths")
    ks_approx = ks.copy() if len(ks) == 1 else get_eigenvalues(ks, tens, threshold)
    sols, trefs, hists = [], [], []
    for kcur in ks_approx:
        idx0 = int(np.argmin(np.abs(ks - kcur)))
        dk_grid = initial_refinement_interval
        if len(ks) > 1:
            d = np.abs(ks - ks[idx0])
            d = d[d > 0]
            if len(d):
                dk_grid = float(d.min())
        window = max(3 * dk_grid, initial_refinement_interval)
        hist = []
        kprev = tprev = float("nan")
        for lev, pf in enumerate(pts_refinement_factors, start=1):
            s = copy.copy(solver)
            s.pts_scaling_factor = pf * solver.pts_scaling_factor
            ws = Workspace(s, evaluate_points(s, billiard, kcur))
            try:
                knew, tnew = newton_refine_svd(ws, kcur, kcur - window, kcur + window, newton_max_iter, newton_tol)
            finally:
                ws.close()
            hist.append(dict(level=lev, pts_factor=pf, k=knew, tension=tnew, window=window))
            if lev > 1:
                kconv = stop_k_tol > 0 and abs(knew - kprev) <= stop_k_tol
                tconv = stop_t_tol > 0 and abs(tnew - tprev) <= stop_t_tol
                if kconv or tconv:
                    kcur, tprev = knew, tnew
                    break
            kprev, tprev, kcur = knew, tnew, knew
            window /= window_shrink
        sols.append(kcur)
        trefs.append(tprev)
        hists.append(hist)
    return np.array(sols), np.array(trefs), hists
