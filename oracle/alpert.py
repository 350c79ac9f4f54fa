"""FP64 restatement of the CFIE-Alpert assembly (test infrastructure only).

Follows cfie_alpert.jl: kernel terms _dlp_terms/_slp_terms :233-287, Lagrange
stencils :371-431, the periodic cache :724-789, the periodic self block
:947-1013 with derivatives :1014-1087, and the off-component blocks
:1261-1350. The rule constants (Alpert 1999, log-singular end correction) are
read from the product's table; tests/test_oracle_alpert.py pins them by the
convergence order of the corrected trapezoid rule on known log integrals.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special as sp

from . import assembly as OA

TWO_PI = 2.0 * math.pi


def _lagrange(xi, nodes):
    w = np.ones(len(nodes))
    for j, xj in enumerate(nodes):
        for l, xl in enumerate(nodes):
            if l != j:
                w[j] *= (xi - xl) / (xj - xl)
    return w


def _stencil(xi, ninterp):
    j0 = math.floor(xi - ninterp / 2.0 + 1.0)
    offs = np.arange(j0, j0 + ninterp)
    return offs, _lagrange(xi, offs.astype(float))


def _terms(k, r, inn, s, w, derivs):
    """(value, d/dk, d2/dk2) of d + ik s (cfie_alpert.jl:233-287)."""
    h0, h1 = sp.hankel1(0, k * r), sp.hankel1(1, k * r)
    d0 = w * (0.5j * k * inn * h1 / r)
    s0 = w * (0.5j * h0 * s)
    v0 = d0 + 1j * k * s0
    if not derivs:
        return v0, None, None
    d1 = w * (0.5j * inn * k * h0)
    d2 = w * (0.5j * inn * (h0 - k * r * h1))
    s1 = w * (-0.5j * r * h1 * s)
    s2 = w * (0.5j * r * (h1 - k * r * h0) * s / k)
    return v0, d1 + 1j * s0 + 1j * k * s1, d2 + 2j * s1 + 1j * k * s2


def cfie_alpert_matrix(curves, pts, k, rule, order, derivs=False):
    """A (and A', A'') for closed components ``curves`` with nodes ``pts``
    (holes reversed as the solver does); rule = (a, x[], w[])."""
    a, rx, rw = rule
    offs = OA.component_offsets(pts)
    Nt = offs[-1]
    A = np.zeros((Nt, Nt), complex)
    A1 = np.zeros_like(A) if derivs else None
    A2 = np.zeros_like(A) if derivs else None
    ninterp = order + 3
    for ci, (crv, p) in enumerate(zip(curves, pts)):
        N = p.n
        o = offs[ci]
        h = p.ws[0]
        X, Y = p.xy[:, 0], p.xy[:, 1]
        dX, dY = p.tangent[:, 0], p.tangent[:, 1]
        spd = np.hypot(dX, dY)
        DX = X[:, None] - X[None, :]
        DY = Y[:, None] - Y[None, :]
        R = np.hypot(DX, DY)
        np.fill_diagonal(R, 1.0)
        inn = dY[None, :] * DX - dX[None, :] * DY
        i = np.arange(N)
        d = np.abs(i[:, None] - i[None, :])
        d = np.minimum(d, N - d)
        band = d < a  # includes the diagonal
        v0, v1, v2 = _terms(k, R, inn, spd[None, :], h, derivs)
        blk = np.where(band, 0.0, -v0)
        blk[np.arange(N), np.arange(N)] = 1.0
        sl = slice(o, o + N)
        A[sl, sl] = blk
        if derivs:
            A1[sl, sl] = np.where(band, 0.0, -v1)
            A2[sl, sl] = np.where(band, 0.0, -v2)
        # orientation of the stored parameter order (cfie_alpert.jl:458-471)
        dd = math.fmod(p.ts[1] - p.ts[0] + math.pi, TWO_PI)
        sg = 1 if (dd + (TWO_PI if dd < 0 else 0.0)) - math.pi >= 0 else -1
        u = p.ts / TWO_PI
        for pp in range(len(rx)):
            fac = h * rw[pp]
            for sgn in (1, -1):
                xi = sgn * rx[pp]
                st, wt = _stencil(xi, ninterp)
                us = np.mod(u + sg * xi / N, 1.0)
                q = crv.curve(us)
                t = sg * crv.tangent(us) / TWO_PI
                dx, dy = X - q[:, 0], Y - q[:, 1]
                r2 = dx * dx + dy * dy
                ok = np.isfinite(r2) & (r2 > np.finfo(float).eps ** 2)
                r = np.sqrt(np.where(ok, r2, 1.0))
                innc = t[:, 1] * dx - t[:, 0] * dy
                c0, c1, c2 = _terms(k, r, innc, np.hypot(t[:, 0], t[:, 1]), fac, derivs)
                for m in range(ninterp):
                    cols = o + np.mod(i + st[m], N)
                    rows = o + i
                    A[rows[ok], cols[ok]] -= (c0 * wt[m])[ok]
                    if derivs:
                        A1[rows[ok], cols[ok]] -= (c1 * wt[m])[ok]
                        A2[rows[ok], cols[ok]] -= (c2 * wt[m])[ok]
    for ca, pa in enumerate(pts):
        for cb, pb in enumerate(pts):
            if ca == cb:
                continue
            dx = pa.xy[:, 0][:, None] - pb.xy[:, 0][None, :]
            dy = pa.xy[:, 1][:, None] - pb.xy[:, 1][None, :]
            r = np.hypot(dx, dy)
            innb = pb.tangent[:, 1][None, :] * dx - pb.tangent[:, 0][None, :] * dy
            sb = np.hypot(pb.tangent[:, 0], pb.tangent[:, 1])[None, :]
            v0, v1, v2 = _terms(k, r, innb, sb, pb.ws[None, :], derivs)
            sa, sbl = slice(offs[ca], offs[ca + 1]), slice(offs[cb], offs[cb + 1])
            A[sa, sbl] = -v0
            if derivs:
                A1[sa, sbl] = -v1
                A2[sa, sbl] = -v2
    return (A, A1, A2) if derivs else A
