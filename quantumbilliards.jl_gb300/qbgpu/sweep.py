"""sigma_min sweep (mirrors sweepmethods.jl:51-60, 132-217).

``k_sweep`` discretises once at max(ks) (sweepmethods.jl:52), builds the
workspace, and returns sigma_min(A(k)) for every k; the SVD is cuSOLVER's
gesvd on the device (the reference: LAPACK.gesvd!('N','N',A)[end],
macros.jl:159-161). ``get_eigenvalues`` is the reference's peak search on the
second difference of log10(sigma) (sweepmethods.jl:193-217).
"""
from __future__ import annotations

import numpy as np

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
