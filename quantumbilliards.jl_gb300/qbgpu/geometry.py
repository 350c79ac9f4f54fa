"""Boundary discretisation on the host (O(N) work, FP64).

This module restates the reference's curve primitives and the periodic Kress
node construction that feed the device kernels:

* curves: ``CircleSegment`` (src/billiards/geometry/circlesegment.jl:16-33,
  175-183, 197-260), ``LineSegment`` (linesegment.jl:139-260) and
  ``PolarSegment`` (polarsegment.jl:98-160; the reference differentiates the
  radial function with ForwardDiff, here the caller supplies the analytic
  first and second derivatives);
* billiards: unit circle (circle.jl:69-75), full stadium (stadium.jl:23-37,
  52-63), circle with circular holes, and the smooth star
  r(theta) = 1 + eps*cos(n*theta) built as a PolarSegment;
* ``BoundaryPointsCFIE`` (boundarypoints.jl:487-503) and the node builders
  ``_evaluate_points`` for DLP_kress (dlp_kress.jl:359-386), the smooth
  composite path of the global-corner solvers (dlp_kress.jl:422-454,
  cfie.jl:682-747, boundarypoints.jl:727-772) and CFIE_kress (cfie.jl:535-560,
  822-834, orientation reversal of holes cfie.jl:458-470).

Node count rule (dlp_kress.jl:362-373): N = max(min_pts, round(k*L*b/2pi)),
rounded up to a multiple of 2 (smooth Kress), of lcm(2, n) for a rotation of
order n and of 4 for a reflection symmetry. ``round`` ties to even in both the
reference and Python.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

TWO_PI = 2.0 * math.pi


# --------------------------------------------------------------------------
# curves, parameter u in [0, 1]
# --------------------------------------------------------------------------
class CircleSegment:
    """Arc R*(cos(a*u+s), sin(a*u+s)) + centre; circlesegment.jl:16-18, 61-66."""

    def __init__(self, R, arc_angle, shift_angle, x0, y0, orientation=1):
        self.radius = float(R)
        self.arc_angle = float(arc_angle)
        self.shift_angle = float(shift_angle)
        self.center = (float(x0), float(y0))
        self.orientation = int(orientation)
        self.length = abs(self.radius * self.arc_angle)

    def curve(self, u):
        u = np.asarray(u, dtype=np.float64)
        th = self.arc_angle * u + self.shift_angle
        return np.stack([self.radius * np.cos(th) + self.center[0],
                         self.radius * np.sin(th) + self.center[1]], axis=-1)

    def tangent(self, u):
        u = np.asarray(u, dtype=np.float64)
        th = self.arc_angle * u + self.shift_angle
        R, a = self.radius, self.arc_angle
        return self.orientation * np.stack([-R * a * np.sin(th), R * a * np.cos(th)], axis=-1)

    def tangent_2(self, u):
        u = np.asarray(u, dtype=np.float64)
        th = self.arc_angle * u + self.shift_angle
        R, aa = self.radius, self.arc_angle ** 2
        return np.stack([-R * aa * np.cos(th), -R * aa * np.sin(th)], axis=-1)

    def arc_length(self, u):
        return self.length * np.asarray(u, dtype=np.float64)


class LineSegment:
    """Straight segment pt0 -> pt1; linesegment.jl:139-260."""

    def __init__(self, pt0, pt1, orientation=1):
        self.pt0 = np.asarray(pt0, dtype=np.float64)
        self.pt1 = np.asarray(pt1, dtype=np.float64)
        self.orientation = int(orientation)
        self.length = float(np.hypot(*(self.pt1 - self.pt0)))

    def curve(self, u):
        u = np.asarray(u, dtype=np.float64)[..., None]
        return self.pt0 + u * (self.pt1 - self.pt0)

    def tangent(self, u):
        u = np.asarray(u, dtype=np.float64)
        v = self.orientation * (self.pt1 - self.pt0)
        return np.broadcast_to(v, u.shape + (2,)).copy()

    def tangent_2(self, u):
        u = np.asarray(u, dtype=np.float64)
        return np.zeros(u.shape + (2,))

    def arc_length(self, u):
        return self.length * np.asarray(u, dtype=np.float64)


class PolarSegment:
    """Closed curve gamma(u) = rho(2*pi*u) * (cos 2*pi*u, sin 2*pi*u).

    The reference builds the same object from a closure with ForwardDiff
    tangents (polarsegment.jl:60-64, 132-160); here rho, rho' and rho'' are
    given analytically so the derivatives are exact to rounding.
    """

    def __init__(self, rho: Callable, drho: Callable, ddrho: Callable, nquad: int = 4096):
        self.rho, self.drho, self.ddrho = rho, drho, ddrho
        # closed-curve length by the periodic trapezoid rule (spectrally exact
        # for a smooth periodic integrand); the reference integrates with QuadGK.
        u = (np.arange(nquad) + 0.5) / nquad
        self.length = float(np.mean(np.hypot(*self.tangent(u).T)))

    def _parts(self, u):
        u = np.asarray(u, dtype=np.float64)
        th = TWO_PI * u
        return th, self.rho(th), self.drho(th), self.ddrho(th)

    def curve(self, u):
        th, r, _, _ = self._parts(u)
        return np.stack([r * np.cos(th), r * np.sin(th)], axis=-1)

    def tangent(self, u):
        th, r, dr, _ = self._parts(u)
        c, s = np.cos(th), np.sin(th)
        return TWO_PI * np.stack([dr * c - r * s, dr * s + r * c], axis=-1)

    def tangent_2(self, u):
        th, r, dr, ddr = self._parts(u)
        c, s = np.cos(th), np.sin(th)
        return TWO_PI ** 2 * np.stack([ddr * c - 2 * dr * s - r * c,
                                       ddr * s + 2 * dr * c - r * s], axis=-1)

    def arc_length(self, u):
        u = np.atleast_1d(np.asarray(u, dtype=np.float64))
        out = np.empty_like(u)
        for n, uu in enumerate(u):
            m = max(64, int(2048 * uu))
            if uu <= 0:
                out[n] = 0.0
                continue
            x, w = np.polynomial.legendre.leggauss(64)
            # composite Gauss-Legendre on [0, uu]
            edges = np.linspace(0.0, uu, max(2, m // 64 + 1))
            acc = 0.0
            for a, b in zip(edges[:-1], edges[1:]):
                t = 0.5 * (b - a) * x + 0.5 * (b + a)
                acc += 0.5 * (b - a) * np.sum(w * np.hypot(*self.tangent(t).T))
            out[n] = acc
        return out


class EllipseArc:
    """gamma(u) = c + (a cos th, b sin th), th = th0 + (th1 - th0) u: the
    elliptic cap of the mushroom billiards (ellipse_mushroom.jl; the reference
    writes it as a PolarSegment of a parametric closure)."""

    def __init__(self, a, b, th0, th1, cx=0.0, cy=0.0, nquad=2048):
        self.a, self.b, self.th0, self.th1, self.c = float(a), float(b), float(th0), float(th1), (cx, cy)
        self.length = float(self.arc_length(1.0)[0])

    def _th(self, u):
        u = np.asarray(u, dtype=np.float64)
        return self.th0 + (self.th1 - self.th0) * u, self.th1 - self.th0

    def curve(self, u):
        th, _ = self._th(u)
        return np.stack([self.c[0] + self.a * np.cos(th), self.c[1] + self.b * np.sin(th)], axis=-1)

    def tangent(self, u):
        th, d = self._th(u)
        return d * np.stack([-self.a * np.sin(th), self.b * np.cos(th)], axis=-1)

    def tangent_2(self, u):
        th, d = self._th(u)
        return d * d * np.stack([-self.a * np.cos(th), -self.b * np.sin(th)], axis=-1)

    def arc_length(self, u):
        u = np.atleast_1d(np.asarray(u, dtype=np.float64))
        x, w = np.polynomial.legendre.leggauss(64)
        out = np.empty_like(u)
        for n, uu in enumerate(u):
            edges = np.linspace(0.0, uu, 17)
            acc = 0.0
            for lo, hi in zip(edges[:-1], edges[1:]):
                t = 0.5 * (hi - lo) * x + 0.5 * (hi + lo)
                acc += 0.5 * (hi - lo) * np.sum(w * np.hypot(*self.tangent(t).T))
            out[n] = acc
        return out


# --------------------------------------------------------------------------
# billiards
# --------------------------------------------------------------------------
@dataclass
class Billiard:
    """full_boundary: list of components; each component is a list of curves."""
    name: str
    components: List[List[object]]
    area: float
    symmetry_axes: Sequence[str] = ()

    @property
    def length(self) -> float:
        return float(sum(c.length for comp in self.components for c in comp))

    @property
    def outer_length(self) -> float:
        return float(sum(c.length for c in self.components[0]))


def make_circle(radius: float = 1.0) -> Billiard:
    """circle.jl:69-75: one CircleSegment of arc 2*pi starting at angle 0."""
    return Billiard("circle", [[CircleSegment(radius, TWO_PI, 0.0, 0.0, 0.0)]], math.pi * radius ** 2,
                    ("x", "y"))


def make_star(eps: float = 0.2, n: int = 5) -> Billiard:
    """Smooth star r(theta) = 1 + eps*cos(n*theta) as a PolarSegment."""
    rho = lambda th: 1.0 + eps * np.cos(n * th)
    drho = lambda th: -eps * n * np.sin(n * th)
    ddrho = lambda th: -eps * n * n * np.cos(n * th)
    area = math.pi * (1.0 + 0.5 * eps * eps)
    return Billiard(f"star{n}_{eps}", [[PolarSegment(rho, drho, ddrho)]], area, ("x",))


def make_full_stadium(half_width: float = 1.0, radius: float = 1.0) -> Billiard:
    """Five-piece counter-clockwise stadium of stadium.jl:23-37."""
    hw, r = float(half_width), float(radius)
    p2, p3 = (hw, r), (-hw, r)
    p5, p6 = (-hw, -r), (hw, -r)
    arc1 = CircleSegment(r, math.pi / 2, 0.0, hw, 0.0)
    line1 = LineSegment(p2, p3)
    arc2 = CircleSegment(r, math.pi, math.pi / 2, -hw, 0.0)
    line2 = LineSegment(p5, p6)
    arc3 = CircleSegment(r, math.pi / 2, 3 * math.pi / 2, hw, 0.0)
    area = 4.0 * hw * r + math.pi * r * r
    return Billiard("stadium", [[arc1, line1, arc2, line2, arc3]], area, ("x", "y"))


def make_rectangle(width: float = 1.0, height: float = 1.0) -> Billiard:
    """make_full_rectangle (rectangle.jl:72-95): the rectangle centred at the
    origin as eight counter-clockwise line segments starting at the middle of
    the right side (four true corners, four straight joins); Dirichlet
    eigenvalues k^2 = pi^2 (m^2/w^2 + n^2/h^2)."""
    hw, hh = 0.5 * float(width), 0.5 * float(height)
    pts = [(hw, 0.0), (hw, hh), (0.0, hh), (-hw, hh), (-hw, 0.0), (-hw, -hh), (0.0, -hh), (hw, -hh)]
    segs = [LineSegment(pts[j], pts[(j + 1) % 8]) for j in range(8)]
    return Billiard("rectangle", [segs], float(width) * float(height), ())


def make_full_ellipse_mushroom(stem_width=0.6, stem_height=1.0, cap_height=0.8, cap_width=1.2) -> Billiard:
    """make_full_ellipse_mushroom (ellipse_mushroom.jl): rectangular stem of
    width stem_width and height stem_height under a half-ellipse cap of
    semi-axes cap_width, cap_height; segments stem bottom, stem right, right
    connector, cap, left connector, stem left, all shifted by (stem_width/2, 0)
    as there. Six true corners."""
    w2, hs, a, b = 0.5 * stem_width, stem_height, cap_width, cap_height
    ox = w2
    P = lambda x, y: (x + ox, y)
    segs = [LineSegment(P(-w2, -hs), P(w2, -hs)), LineSegment(P(w2, -hs), P(w2, 0.0)),
            LineSegment(P(w2, 0.0), P(a, 0.0)), EllipseArc(a, b, 0.0, math.pi, ox, 0.0),
            LineSegment(P(-a, 0.0), P(-w2, 0.0)), LineSegment(P(-w2, 0.0), P(-w2, -hs))]
    area = stem_width * stem_height + 0.5 * math.pi * a * b
    return Billiard("ellipse_mushroom", [segs], area, ())


def make_circle_with_hole(R: float = 1.0, hole=(0.3, 0.1, 0.2)) -> Billiard:
    """Outer circle R plus one circular hole (cx, cy, rh); the hole is traversed
    counter-clockwise here and reversed by the CFIE node builder
    (cfie.jl:822-834, 458-470)."""
    cx, cy, rh = hole
    outer = CircleSegment(R, TWO_PI, 0.0, 0.0, 0.0)
    inner = CircleSegment(rh, TWO_PI, 0.0, cx, cy)
    return Billiard("circle_hole", [[outer], [inner]], math.pi * (R * R - rh * rh))


# --------------------------------------------------------------------------
# boundary points
# --------------------------------------------------------------------------
@dataclass
class BoundaryPointsCFIE:
    """Mirror of boundarypoints.jl:487-503 (SoA, FP64)."""
    xy: np.ndarray          # (N, 2)
    tangent: np.ndarray     # (N, 2) d gamma / d sigma
    tangent_2: np.ndarray   # (N, 2)
    ts: np.ndarray          # computational parameter sigma (N,)
    tphys: np.ndarray
    ws: np.ndarray          # quadrature weights (N,)
    ws_der: np.ndarray
    ds: np.ndarray
    compid: int = 1
    is_periodic: bool = True

    @property
    def n(self) -> int:
        return int(self.xy.shape[0])


def s_mid(N: int) -> np.ndarray:
    """cfie.jl:424: sigma_j = 2*pi*(j - 1/2)/N, j = 1..N."""
    return TWO_PI * (np.arange(1, N + 1, dtype=np.float64) - 0.5) / N


def node_count(k: float, L: float, b: float, min_pts: int = 20, needed: int = 2) -> int:
    """dlp_kress.jl:362-373."""
    N = max(int(min_pts), int(round(k * L * b / TWO_PI)))
    rem = N % needed
    if rem:
        N += needed - rem
    return N


def _needed(symmetry, base=2):
    from .symmetry import needed_multiple
    return needed_multiple(symmetry, base)


def points_single_curve(crv, N: int, compid: int = 1) -> BoundaryPointsCFIE:
    """_evaluate_points(::DLP_kress / ::CFIE_kress, crv, ...) for a given N."""
    ts = s_mid(N)
    u = ts / TWO_PI
    xy = crv.curve(u)
    t1 = crv.tangent(u) / TWO_PI
    t2 = crv.tangent_2(u) / TWO_PI ** 2
    ss = crv.arc_length(u)
    ds = np.append(np.diff(ss), crv.length + ss[0] - ss[-1])
    ws = np.full(N, TWO_PI / N)
    return BoundaryPointsCFIE(xy, t1, t2, ts, ts.copy(), ws, np.ones(N), ds, compid, True)


def _composite_eval(comp, t: float):
    """_eval_composite_geom_global_t (boundarypoints.jl:727-772)."""
    lens = np.array([c.length for c in comp])
    cum = np.concatenate([[0.0], np.cumsum(lens)])
    Ltot = cum[-1]
    s = (t / TWO_PI) * Ltot
    if s >= Ltot:
        j, u = 0, 0.0
    else:
        j = int(np.searchsorted(cum, s, side="right")) - 1
        j = min(max(j, 0), len(comp) - 1)
        while j < len(comp) - 1 and s >= cum[j + 1]:
            j += 1
        u = 0.0 if lens[j] == 0 else (s - cum[j]) / lens[j]
        u = min(max(u, 0.0), 1.0)
    crv = comp[j]
    du_dt = 0.0 if lens[j] == 0 else Ltot / (TWO_PI * lens[j])
    return crv.curve(u), crv.tangent(u) * du_dt, crv.tangent_2(u) * du_dt ** 2


def points_smooth_composite(comp, N: int, compid: int = 1) -> BoundaryPointsCFIE:
    """_evaluate_points_smooth_composite (dlp_kress.jl:422-454)."""
    ts = s_mid(N)
    h = TWO_PI / N
    xy = np.empty((N, 2)); t1 = np.empty((N, 2)); t2 = np.empty((N, 2))
    for i, t in enumerate(ts):
        q, gt, gtt = _composite_eval(comp, t)
        xy[i], t1[i], t2[i] = q, gt, gtt
    ds = np.hypot(t1[:, 0], t1[:, 1]) * h
    return BoundaryPointsCFIE(xy, t1, t2, ts, ts.copy(), np.full(N, h), np.ones(N), ds, compid, True)


def _smoothstep(u, q):
    u = np.clip(u, 0.0, 1.0)
    a, b = u ** q, (1.0 - u) ** q
    return a / (a + b)


def _smoothstep_1(u, q):
    u = np.clip(u, np.finfo(float).eps, 1.0 - np.finfo(float).eps)
    a, b = u ** q, (1.0 - u) ** q
    return q * u ** (q - 1) * (1.0 - u) ** (q - 1) / (a + b) ** 2


def _smoothstep_2(u, q):
    u = np.clip(u, np.finfo(float).eps, 1.0 - np.finfo(float).eps)
    d = u ** q + (1.0 - u) ** q
    dp = q * (u ** (q - 1) - (1.0 - u) ** (q - 1))
    return _smoothstep_1(u, q) * ((q - 1) / u - (q - 1) / (1.0 - u) - 2.0 * dp / d)


def multi_kress_graded_nodes_data(N: int, corners, q: float = 3.0, minsep_tol: float = 1e-12):
    """kress_grading_global_multi_corner.jl:53-146: uniform sigma_j = h (j - 1/2)
    mapped by t = left + L v((sigma - left)/L) between consecutive corners with
    the Kress smoothstep v(u) = u^q / (u^q + (1-u)^q). Returns (sigma, t, dt/dsigma,
    d2t/dsigma2, weights h dt/dsigma); q shrinks by 0.9 while mapped nodes are
    closer than minsep_tol."""
    h = TWO_PI / N
    sig = np.sort(np.mod(0.5 * h + h * np.arange(N), TWO_PI))
    cs = sorted({float(np.mod(c, TWO_PI)) for c in corners})
    cu = []
    for c in cs:
        if not cu or abs(c - cu[-1]) > math.sqrt(np.finfo(float).eps):
            cu.append(c)
    if not cu:
        return sig, sig.copy(), np.ones(N), np.zeros(N), np.full(N, h)
    cu = np.array(cu)
    qq = float(q)
    if qq <= 1.0:
        raise ValueError("Require q > 1.")
    while qq > 1.0:
        if len(cu) == 1:
            left = np.full(N, cu[0]) - np.where(sig < cu[0], TWO_PI, 0.0)
            right = left + TWO_PI
        else:
            j = np.searchsorted(cu, sig, side="right") - 1
            left = np.where(j < 0, cu[-1] - TWO_PI, cu[np.clip(j, 0, len(cu) - 1)])
            right = np.where(j < 0, cu[0], np.where(j >= len(cu) - 1, cu[0] + TWO_PI, cu[np.clip(j + 1, 0, len(cu) - 1)]))
        Lw = right - left
        u = (sig - left) / Lw
        tmap = np.mod(left + Lw * _smoothstep(u, qq), TWO_PI)
        jac = _smoothstep_1(u, qq)
        jac2 = _smoothstep_2(u, qq) / Lw
        ts = np.sort(tmap)
        gaps = np.diff(np.concatenate([ts, [ts[0] + TWO_PI]]))
        if gaps.min() >= minsep_tol:
            return sig, tmap, jac, jac2, h * jac
        qq = max(1.0, 0.9 * qq)
    raise ValueError("Kress grading is impossible: q reached 1 with nodes closer than minsep_tol")


def points_graded_composite(comp, N: int, corners, q: float, compid: int = 1,
                            minsep_tol: float = 1e-12) -> BoundaryPointsCFIE:
    """_evaluate_points(::DLP_kress_global_corners, comp) with corners
    (dlp_kress.jl:505-540): nodes at t(sigma_j), gamma' = gamma_t jac,
    gamma'' = gamma_tt jac^2 + gamma_t jac2, weights h, sigma for the Kress log term."""
    sig, tmap, jac, jac2, _ = multi_kress_graded_nodes_data(N, corners, q, minsep_tol)
    h = TWO_PI / N
    xy = np.empty((N, 2)); t1 = np.empty((N, 2)); t2 = np.empty((N, 2))
    for i in range(N):
        qpt, gt, gtt = _composite_eval(comp, tmap[i])
        xy[i] = qpt
        t1[i] = np.asarray(gt) * jac[i]
        t2[i] = np.asarray(gtt) * jac[i] ** 2 + np.asarray(gt) * jac2[i]
    ds = np.hypot(t1[:, 0], t1[:, 1]) * h
    return BoundaryPointsCFIE(xy, t1, t2, sig, tmap, np.full(N, h), jac, ds, compid, True)


def reverse_orientation(p: BoundaryPointsCFIE) -> BoundaryPointsCFIE:
    """_reverse_component_orientation (cfie.jl:458-470)."""
    return BoundaryPointsCFIE(p.xy[::-1].copy(), (-p.tangent)[::-1].copy(), p.tangent_2[::-1].copy(),
                              p.ts[::-1].copy(), p.tphys[::-1].copy(), p.ws[::-1].copy(),
                              p.ws_der[::-1].copy(), p.ds[::-1].copy(), p.compid, p.is_periodic)


def _component_corners(comp, angle_tol=1e-8):
    """_component_corner_locations (boundarypoints.jl:609-650)."""
    def unit(v):
        v = np.asarray(v, dtype=np.float64)
        return v / np.hypot(*v)

    def is_corner(a, b):
        tl, tr = unit(a.tangent(1.0)), unit(b.tangent(0.0))
        cr = tl[0] * tr[1] - tl[1] * tr[0]
        dt = min(max(tl[0] * tr[0] + tl[1] * tr[1], -1.0), 1.0)
        return math.atan2(abs(cr), dt) > angle_tol

    lens = np.array([c.length for c in comp])
    cum = np.concatenate([[0.0], np.cumsum(lens)])
    out = []
    if len(comp) > 1 and is_corner(comp[-1], comp[0]):
        out.append(0.0)
    for j in range(len(comp) - 1):
        if is_corner(comp[j], comp[j + 1]):
            out.append(TWO_PI * cum[j + 1] / cum[-1])
    return out
