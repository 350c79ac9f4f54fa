"""FP64 restatement of the reference's Chebyshev-panel route (test only).

* _chebfit! (DCT-I on Chebyshev-Lobatto nodes, c_0 halved)   chebyshev_core.jl:67-80
* _breaks_uniform, _find_panel_uniform                        chebyshev_core.jl:95-103,
                                                              chebyshev_bessels.jl:574-580
* plan_h / plan_j (H over [rmin, rmax], J over [0, rmax])     chebyshev_bessels.jl:461-528
* Clenshaw evaluation                                         chebyshev_core.jl:114-345
* CFIE evaluator cutoffs (|z| < 0.2 -> direct Hankel)          chebyshev_bessels.jl:1190-1207
* DLP evaluator (panels everywhere above rmin)                chebyshev_bessels.jl:1051-1096
* block caches: rmin = 0.95 min r, rmax = 1.05 max r          chebyshev_euclidian_helmholtz_cfie_kress.jl:396-456
The node values come from SciPy's AMOS wrappers, as the reference's come from AMOS.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special as sp

from . import assembly as OA


def breaks(lo, hi, npan):
    h = (hi - lo) / npan
    b = lo + np.arange(npan + 1) * h
    b[-1] = hi
    return b


def fit(vals):
    """vals (..., M+1) at t_j = cos(pi j / M) -> Chebyshev coefficients (..., M+1)."""
    M = vals.shape[-1] - 1
    j = np.arange(M + 1)
    C = np.cos(np.pi * np.outer(j, j) / M)  # [m, j]
    w = np.ones(M + 1)
    w[0] = w[-1] = 0.5
    c = (2.0 / M) * np.einsum("...j,mj->...m", vals * w, C)
    c[..., 0] *= 0.5
    return c


def clenshaw(c, t):
    """c (n, M+1) per point, t (n,) -> values (n,)."""
    M = c.shape[-1] - 1
    b1 = np.zeros(t.shape, complex)
    b2 = np.zeros(t.shape, complex)
    u = 2 * t
    for m in range(M, 0, -1):
        b0 = u * b1 - b2 + c[:, m]
        b2, b1 = b1, b0
    return t * b1 - b2 + c[:, 0]


class Plan:
    def __init__(self, k, lo, hi, npan, M, fn):
        self.k, self.lo, self.hi, self.npan, self.M = k, lo, hi, npan, M
        self.dr = (hi - lo) / npan
        self.invdr = 1.0 / self.dr
        b = breaks(lo, hi, npan)
        tn = np.cos(np.pi * np.arange(M + 1) / M)
        a, bb = b[:-1, None], b[1:, None]
        r = ((bb + a) + (bb - a) * tn[None, :]) / 2
        self.a, self.b = b[:-1], b[1:]
        self.c = fit(fn(k * r))

    def locate(self, r):
        p = np.floor((r - self.lo) * self.invdr).astype(np.int64)
        p = np.clip(p, 0, self.npan - 1)
        a, b = self.a[p], self.b[p]
        return p, (2 * r - (b + a)) / (b - a)

    def __call__(self, r):
        p, t = self.locate(r)
        return clenshaw(self.c[p], t)


def r_range(pts):
    xy = np.concatenate([p.xy for p in pts])
    d = np.hypot(xy[:, None, 0] - xy[None, :, 0], xy[:, None, 1] - xy[None, :, 1])
    d = d[d > np.finfo(float).eps]
    return 0.95 * d.min(), 1.05 * d.max()


def _jfun(k, nu):
    if np.imag(k) == 0:
        return lambda z: np.real(sp.jv(nu, z)).astype(complex)
    return lambda z: sp.jv(nu, z)


def funcs(k, r, rmin, rmax, params, small_cut):
    nh, Mh, nj, Mj = params
    h0p = Plan(k, rmin, rmax, nh, Mh, lambda z: sp.hankel1(0, z))
    h1p = Plan(k, rmin, rmax, nh, Mh, lambda z: sp.hankel1(1, z))
    j0p = Plan(k, 0.0, rmax, nj, Mj, _jfun(k, 0))
    j1p = Plan(k, 0.0, rmax, nj, Mj, _jfun(k, 1))
    shape = r.shape
    rr = r.ravel()
    h0, h1 = h0p(rr), h1p(rr)
    direct = (rr < rmin) | (abs(k) * rr < small_cut)
    if np.any(direct):
        h0[direct] = sp.hankel1(0, k * rr[direct])
        h1[direct] = sp.hankel1(1, k * rr[direct])
    return (h0.reshape(shape), h1.reshape(shape), j0p(rr).reshape(shape), j1p(rr).reshape(shape))


def cfie_matrix(pts, k, params=(15000, 5, 3000, 5)):
    pts = pts if isinstance(pts, list) else [pts]
    rmin, rmax = r_range(pts)
    same, off = {}, {}
    for a, p in enumerate(pts):
        R = OA.geom_cache(p)["R"]
        same[a] = funcs(k, R, rmin, rmax, params, 0.2)
    for a, pa in enumerate(pts):
        for b, pb in enumerate(pts):
            if a != b:
                R = np.hypot(pa.xy[:, 0][:, None] - pb.xy[:, 0][None, :], pa.xy[:, 1][:, None] - pb.xy[:, 1][None, :])
                h0, h1, _, _ = funcs(k, R, rmin, rmax, params, 0.2)
                off[(a, b)] = (h0, h1)
    return OA.cfie_matrix(pts, k, funcs_same=same, funcs_off=off)


def dlp_fredholm(p, k, params=(15000, 5, 3000, 5), derivs=False):
    rmin, rmax = r_range([p])
    R = OA.geom_cache(p)["R"]
    return OA.dlp_fredholm(p, k, derivs=derivs, funcs=funcs(k, R, rmin, rmax, params, 0.0))


def cfie_matrix_derivs(pts, k, params=(15000, 5, 3000, 5)):
    """(A, A', A'') with interpolated H0, H1, J0, J1
    (chebyshev_euclidian_helmholtz_cfie_kress.jl:881-1060)."""
    pts = pts if isinstance(pts, list) else [pts]
    rmin, rmax = r_range(pts)
    same, off = {}, {}
    for a, p in enumerate(pts):
        same[a] = funcs(k, OA.geom_cache(p)["R"], rmin, rmax, params, 0.2)
    for a, pa in enumerate(pts):
        for b, pb in enumerate(pts):
            if a != b:
                R = np.hypot(pa.xy[:, 0][:, None] - pb.xy[:, 0][None, :], pa.xy[:, 1][:, None] - pb.xy[:, 1][None, :])
                h0, h1, _, _ = funcs(k, R, rmin, rmax, params, 0.2)
                off[(a, b)] = (h0, h1)
    return OA.cfie_matrix_derivs(pts, k, funcs_same=same, funcs_off=off)


def dlp_fredholm_reduced(p, k, orbits, params=(15000, 5, 3000, 5), derivs=False):
    """Symmetry-reduced DLP with the H/J panels for the Kress-split entries and
    the H panels for the image kernels
    (chebyshev_euclidian_helmholtz_dlp_kress.jl:771-847, 953-1054)."""
    rmin, rmax = r_range([p])
    nh, Mh, _, _ = params
    h0p = Plan(k, rmin, rmax, nh, Mh, lambda z: sp.hankel1(0, z))
    h1p = Plan(k, rmin, rmax, nh, Mh, lambda z: sp.hankel1(1, z))

    def image_h(r):
        rr = r.ravel()
        h0, h1 = h0p(rr), h1p(rr)
        d = rr < rmin
        if np.any(d):
            h0[d] = sp.hankel1(0, k * rr[d])
            h1[d] = sp.hankel1(1, k * rr[d])
        return h0.reshape(r.shape), h1.reshape(r.shape)

    R = OA.geom_cache(p)["R"]
    return OA.dlp_fredholm_reduced(p, k, orbits, derivs=derivs, funcs=funcs(k, R, rmin, rmax, params, 0.0),
                                   image_h=image_h)
