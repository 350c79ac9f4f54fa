"""Boundary nodes of the Kress/Alpert solvers, restated for the oracle (test
infrastructure only; nothing here imports the product).

Curves (parameter u in [0, 1]):
* circle arcs          circlesegment.jl:16-33, 61-66, 134-266 (tangent and
                       second tangent both carry the orientation sign)
* line segments        linesegment.jl:139-260
* polar segments       polarsegment.jl:60-64, 98-160, 202-258: the reference
                       differentiates its closure with ForwardDiff and
                       integrates the arc length with QuadGK; here the closure
                       is a SymPy expression differentiated symbolically and
                       the arc length comes from scipy.integrate.quad

Billiards: unit circle (circle.jl:69-75), full stadium (stadium.jl:23-37),
circle with circular holes (circle_with_circle_holes.jl:43-55), full
elliptic-cap mushroom (ellipse_mushroom.jl:69-95), full rectangle
(rectangle.jl:72-95) and the smooth star r(theta) = 1 + eps cos(n theta) as a
polar segment of the closure t -> r(2 pi t) (cos 2 pi t, sin 2 pi t).

Node builders:
* N = max(min_pts, round(k L b / 2 pi)), rounded up to the needed multiple
  (dlp_kress.jl:362-373, cfie.jl:535-545, cfie.jl:946-957)
* smooth single curve, sigma_j = 2 pi (j - 1/2) / N (dlp_kress.jl:359-386,
  cfie.jl:533-560)
* smooth composite through the global parameter t (dlp_kress.jl:422-454,
  boundarypoints.jl:727-772)
* corner detection (boundarypoints.jl:609-650) and Kress grading
  (kress_grading_global_multi_corner.jl:40-146, dlp_kress.jl:505-540)
* CFIE components with holes orientation-reversed (cfie.jl:458-470, 822-834)
* the Alpert periodic grid (cfie.jl:946-972)
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import sympy as sy
from scipy import integrate

TWO_PI = 2.0 * math.pi


# --------------------------------------------------------------------------
# curves
# --------------------------------------------------------------------------
class Arc:
    """origin + centre + R (cos(a u + s), sin(a u + s))."""

    def __init__(self, R, arc, shift, cx, cy, origin=(0.0, 0.0), orientation=1):
        self.R, self.a, self.s = float(R), float(arc), float(shift)
        self.c = np.array([cx + origin[0], cy + origin[1]], dtype=np.float64)
        self.o = float(orientation)
        self.length = abs(self.R * self.a)

    def curve(self, u):
        th = self.a * np.asarray(u, dtype=np.float64) + self.s
        return np.stack([self.c[0] + self.R * np.cos(th), self.c[1] + self.R * np.sin(th)], axis=-1)

    def tangent(self, u):
        th = self.a * np.asarray(u, dtype=np.float64) + self.s
        f = self.o * self.R * self.a
        return np.stack([-f * np.sin(th), f * np.cos(th)], axis=-1)

    def tangent_2(self, u):
        th = self.a * np.asarray(u, dtype=np.float64) + self.s
        f = self.o * self.R * self.a * self.a
        return np.stack([-f * np.cos(th), -f * np.sin(th)], axis=-1)

    def arc_length(self, u):
        return self.length * np.asarray(u, dtype=np.float64)


class Line:
    """origin + p0 + u (p1 - p0)."""

    def __init__(self, p0, p1, origin=(0.0, 0.0), orientation=1):
        o = np.asarray(origin, dtype=np.float64)
        self.p0 = np.asarray(p0, dtype=np.float64) + o
        self.p1 = np.asarray(p1, dtype=np.float64) + o
        self.o = float(orientation)
        d = self.p1 - self.p0
        self.length = float(math.sqrt(d[0] * d[0] + d[1] * d[1]))

    def curve(self, u):
        u = np.asarray(u, dtype=np.float64)
        return self.p0 + u[..., None] * (self.p1 - self.p0)

    def tangent(self, u):
        u = np.asarray(u, dtype=np.float64)
        return np.zeros(u.shape + (2,)) + self.o * (self.p1 - self.p0)

    def tangent_2(self, u):
        return np.zeros(np.shape(u) + (2,))

    def arc_length(self, u):
        return self.length * np.asarray(u, dtype=np.float64)


class Polar:
    """A closure t -> (x(t), y(t)) given as SymPy expressions in ``t``; its
    derivatives are taken symbolically (exact, like ForwardDiff) and its arc
    length by adaptive quadrature."""

    def __init__(self, x_expr, y_expr, t, origin=(0.0, 0.0)):
        self.origin = np.asarray(origin, dtype=np.float64)
        dx, dy = sy.diff(x_expr, t), sy.diff(y_expr, t)
        ddx, ddy = sy.diff(dx, t), sy.diff(dy, t)
        self._f = [sy.lambdify(t, e, "numpy") for e in (x_expr, y_expr, dx, dy, ddx, ddy)]
        self.length = self._quad(0.0, 1.0)

    def _ev(self, i, u):
        u = np.asarray(u, dtype=np.float64)
        return np.broadcast_to(np.asarray(self._f[i](u), dtype=np.float64), u.shape)

    def curve(self, u):
        return np.stack([self._ev(0, u) + self.origin[0], self._ev(1, u) + self.origin[1]], axis=-1)

    def tangent(self, u):
        return np.stack([self._ev(2, u), self._ev(3, u)], axis=-1)

    def tangent_2(self, u):
        return np.stack([self._ev(4, u), self._ev(5, u)], axis=-1)

    def _speed(self, u):
        return math.hypot(float(self._f[2](u)), float(self._f[3](u)))

    def _quad(self, a, b):
        with warnings.catch_warnings():
            # short gaps reach the rounding floor before epsrel; that is the answer
            warnings.simplefilter("ignore", integrate.IntegrationWarning)
            v, _ = integrate.quad(self._speed, a, b, epsabs=1e-15, epsrel=1e-14, limit=400)
        return v

    def arc_length(self, u):
        """Arc length from 0 to each u: quadrature over the gaps between
        consecutive sorted parameters, accumulated."""
        u = np.atleast_1d(np.asarray(u, dtype=np.float64))
        order = np.argsort(u)
        out = np.empty_like(u)
        acc, prev = 0.0, 0.0
        for i in order:
            acc += self._quad(prev, u[i]) if u[i] > prev else 0.0
            prev = max(prev, u[i])
            out[i] = acc
        return out


# --------------------------------------------------------------------------
# billiards
# --------------------------------------------------------------------------
@dataclass
class Billiard:
    name: str
    components: List[list]
    area: float

    @property
    def outer_length(self) -> float:
        return float(sum(c.length for c in self.components[0]))


def circle(R=1.0):
    return Billiard("circle", [[Arc(R, TWO_PI, 0.0, 0.0, 0.0)]], math.pi * R * R)


def star(eps=0.2, n=5):
    t = sy.Symbol("t", real=True)
    th = 2 * sy.pi * t
    r = 1 + eps * sy.cos(n * th)
    return Billiard("star", [[Polar(r * sy.cos(th), r * sy.sin(th), t)]], math.pi * (1 + eps * eps / 2))


def full_stadium(half_width=1.0, radius=1.0):
    w, r = float(half_width), float(radius)
    segs = [Arc(r, math.pi / 2, 0.0, w, 0.0), Line((w, r), (-w, r)), Arc(r, math.pi, math.pi / 2, -w, 0.0),
            Line((-w, -r), (w, -r)), Arc(r, math.pi / 2, 3 * math.pi / 2, w, 0.0)]
    return Billiard("stadium", [segs], 4 * w * r + math.pi * r * r)


def circle_with_holes(R=1.0, holes=((0.3, 0.1, 0.2),)):
    comps = [[Arc(R, TWO_PI, 0.0, 0.0, 0.0)]]
    area = math.pi * R * R
    for (x, y, rh) in holes:
        comps.append([Arc(rh, TWO_PI, 0.0, 0.0, 0.0, origin=(x, y))])
        area -= math.pi * rh * rh
    return Billiard("circle_holes", comps, area)


def full_ellipse_mushroom(stem_width=0.6, stem_height=1.0, cap_height=0.8, cap_width=1.2):
    t = sy.Symbol("t", real=True)
    o = (stem_width / 2, 0.0)
    w2, h = stem_width / 2, stem_height
    cap = Polar(cap_width * sy.cos(sy.pi * t), cap_height * sy.sin(sy.pi * t), t, origin=o)
    segs = [Line((-w2, -h), (w2, -h), o), Line((w2, -h), (w2, 0.0), o), Line((w2, 0.0), (cap_width, 0.0), o),
            cap, Line((-cap_width, 0.0), (-w2, 0.0), o), Line((-w2, 0.0), (-w2, -h), o)]
    return Billiard("ellipse_mushroom", [segs], stem_width * stem_height + 0.5 * math.pi * cap_width * cap_height)


def full_rectangle(width=1.0, height=1.0):
    a, b = width / 2, height / 2
    p = [(a, 0.0), (a, b), (0.0, b), (-a, b), (-a, 0.0), (-a, -b), (0.0, -b), (a, -b)]
    return Billiard("rectangle", [[Line(p[i], p[(i + 1) % 8]) for i in range(8)]], width * height)


# --------------------------------------------------------------------------
# node sets
# --------------------------------------------------------------------------
@dataclass
class Nodes:
    """The fields of BoundaryPointsCFIE (boundarypoints.jl:487-503) the oracle uses."""
    xy: np.ndarray
    tangent: np.ndarray
    tangent_2: np.ndarray
    ts: np.ndarray
    tphys: np.ndarray
    ws: np.ndarray
    ws_der: np.ndarray
    ds: np.ndarray
    compid: int = 1

    @property
    def n(self) -> int:
        return int(self.xy.shape[0])


def needed_multiple(symmetry, base):
    """symmetry: None, ("x"|"y"|"xy", ...) reflections, ("rot", n, m) rotations."""
    if symmetry is None:
        return base
    if symmetry[0] == "rot":
        return base * int(symmetry[1]) // math.gcd(base, int(symmetry[1]))
    return base * 4 // math.gcd(base, 4)


def node_count(k, L, b, min_pts=20, needed=2):
    N = max(int(min_pts), int(round(k * L * b / TWO_PI)))
    if N % needed:
        N += needed - N % needed
    return N


def _sigma(N):
    return TWO_PI * (np.arange(1, N + 1) - 0.5) / N


def nodes_smooth_curve(crv, N, compid=1):
    ts = _sigma(N)
    u = ts / TWO_PI
    ss = crv.arc_length(u)
    ds = np.empty(N)
    ds[:-1] = ss[1:] - ss[:-1]
    ds[-1] = crv.length + ss[0] - ss[-1]
    return Nodes(crv.curve(u), crv.tangent(u) / TWO_PI, crv.tangent_2(u) / TWO_PI ** 2, ts, ts.copy(),
                 np.full(N, TWO_PI / N), np.ones(N), ds, compid)


def _lengths(comp):
    lens = [c.length for c in comp]
    cum = [0.0]
    for x in lens:
        cum.append(cum[-1] + x)
    return lens, cum, cum[-1]


def _composite_at(comp, t):
    """Point, d/dt and d2/dt2 of a composite component at the global t."""
    lens, cum, Lt = _lengths(comp)
    s = t / TWO_PI * Lt
    if s >= Lt:
        j, u = 0, 0.0
    else:
        j = 0
        for q in range(len(comp)):
            if cum[q] <= s:
                j = q
        j = min(max(j, 0), len(comp) - 1)
        while j < len(comp) - 1 and s >= cum[j + 1]:
            j += 1
        u = 0.0 if lens[j] == 0 else min(max((s - cum[j]) / lens[j], 0.0), 1.0)
    c = comp[j]
    f = 0.0 if lens[j] == 0 else Lt / (TWO_PI * lens[j])
    return c.curve(u), c.tangent(u) * f, c.tangent_2(u) * f * f


def nodes_smooth_composite(comp, N, compid=1):
    ts = _sigma(N)
    h = TWO_PI / N
    xy, t1, t2 = (np.empty((N, 2)) for _ in range(3))
    for i, t in enumerate(ts):
        xy[i], t1[i], t2[i] = _composite_at(comp, t)
    ds = np.hypot(t1[:, 0], t1[:, 1]) * h
    return Nodes(xy, t1, t2, ts, ts.copy(), np.full(N, h), np.ones(N), ds, compid)


def corner_locations(comp, angle_tol=1e-8):
    def unit(v):
        v = np.asarray(v, dtype=np.float64)
        return v / math.hypot(v[0], v[1])

    def corner(left, right):
        a, b = unit(left.tangent(1.0)), unit(right.tangent(0.0))
        cr = a[0] * b[1] - a[1] * b[0]
        dt = min(max(a[0] * b[0] + a[1] * b[1], -1.0), 1.0)
        return math.atan2(abs(cr), dt) > angle_tol

    _, cum, Lt = _lengths(comp)
    out = [0.0] if corner(comp[-1], comp[0]) else []
    for j in range(len(comp) - 1):
        if corner(comp[j], comp[j + 1]):
            out.append(TWO_PI * cum[j + 1] / Lt)
    return out


def _wrap(x):
    y = math.fmod(x, TWO_PI)
    return y + TWO_PI if y < 0 else y


def _step(u, q):
    u = min(max(u, 0.0), 1.0)
    a, b = u ** q, (1 - u) ** q
    return a / (a + b)


def _step_1(u, q):
    e = np.finfo(float).eps
    u = min(max(u, e), 1 - e)
    a, b = u ** q, (1 - u) ** q
    return q * u ** (q - 1) * (1 - u) ** (q - 1) / (a + b) ** 2


def _step_2(u, q):
    e = np.finfo(float).eps
    u = min(max(u, e), 1 - e)
    d = u ** q + (1 - u) ** q
    dp = q * (u ** (q - 1) - (1 - u) ** (q - 1))
    return _step_1(u, q) * ((q - 1) / u - (q - 1) / (1 - u) - 2 * dp / d)


def graded_nodes_data(N, corners, q=3.0, minsep_tol=1e-12):
    """(sigma, t(sigma), t', t'', h t') of the Kress multi-corner grading."""
    h = TWO_PI / N
    sig = np.sort(np.array([_wrap(h / 2 + j * h) for j in range(N)]))
    cs = sorted(_wrap(float(c)) for c in corners)
    cu = []
    for c in cs:
        if not cu or abs(c - cu[-1]) > math.sqrt(np.finfo(float).eps):
            cu.append(c)
    if not cu:
        return sig, sig.copy(), np.ones(N), np.zeros(N), np.full(N, h)
    q = float(q)
    if q <= 1:
        raise ValueError("Require q>1.")
    m = len(cu)
    while q > 1:
        tm, j1, j2 = np.empty(N), np.empty(N), np.empty(N)
        for i, x in enumerate(sig):
            if m == 1:
                lo, hi = cu[0], cu[0] + TWO_PI
            else:
                j = sum(1 for c in cu if c <= x)  # searchsortedlast, 1-based
                if j == 0:
                    lo, hi = cu[-1] - TWO_PI, cu[0]
                elif j == m:
                    lo, hi = cu[-1], cu[0] + TWO_PI
                else:
                    lo, hi = cu[j - 1], cu[j]
            Lw = hi - lo
            u = (x - lo) / Lw
            tm[i] = _wrap(lo + Lw * _step(u, q))
            j1[i] = _step_1(u, q)
            j2[i] = _step_2(u, q) / Lw
        st = np.sort(tm)
        gaps = np.append(np.diff(st), st[0] + TWO_PI - st[-1])
        if gaps.min() >= minsep_tol:
            return sig, tm, j1, j2, h * j1
        q = max(1.0, 0.9 * q)
    raise ValueError("Kress grading is impossible")


def nodes_graded_composite(comp, N, corners, q, compid=1, minsep_tol=1e-12):
    sig, tm, j1, j2, _ = graded_nodes_data(N, corners, q, minsep_tol)
    h = TWO_PI / N
    xy, t1, t2 = (np.empty((N, 2)) for _ in range(3))
    for i in range(N):
        p, gt, gtt = _composite_at(comp, tm[i])
        xy[i] = p
        t1[i] = gt * j1[i]
        t2[i] = gtt * j1[i] ** 2 + gt * j2[i]
    ds = np.hypot(t1[:, 0], t1[:, 1]) * h
    return Nodes(xy, t1, t2, sig, tm, np.full(N, h), j1, ds, compid)


def reversed_nodes(p: Nodes) -> Nodes:
    return Nodes(p.xy[::-1].copy(), -p.tangent[::-1], p.tangent_2[::-1].copy(), p.ts[::-1].copy(),
                 p.tphys[::-1].copy(), p.ws[::-1].copy(), p.ws_der[::-1].copy(), p.ds[::-1].copy(), p.compid)


def evaluate_points(kind, billiard, k, b, min_pts=20, symmetry=None, kressq=4.0, corners_ok=True):
    """kind: "dlp_kress", "dlp_kress_global_corners", "cfie_kress",
    "cfie_kress_global_corners" or "cfie_alpert". DLP kinds return one node
    set, CFIE kinds a list (holes reversed)."""
    out = []
    for idx, comp in enumerate(billiard.components, start=1):
        L = sum(c.length for c in comp)
        if kind == "cfie_alpert":
            if len(comp) != 1:
                raise ValueError("the periodic Alpert grid takes single closed curves")
            p = nodes_smooth_curve(comp[0], node_count(k, L, b, min_pts, needed_multiple(symmetry, 1)), idx)
        elif kind in ("dlp_kress", "cfie_kress"):
            if len(comp) != 1:
                raise ValueError("Kress requires each boundary component to be a single smooth closed curve")
            p = nodes_smooth_curve(comp[0], node_count(k, L, b, min_pts, needed_multiple(symmetry, 2)), idx)
        else:
            cor = corner_locations(comp)
            if cor:
                N = node_count(k, L, b, min_pts, needed_multiple(symmetry, 1))
                p = nodes_graded_composite(comp, N, cor, kressq, idx)
            else:
                N = node_count(k, L, b, min_pts, needed_multiple(symmetry, 2))
                p = nodes_smooth_composite(comp, N, idx)
        out.append(p if idx == 1 else reversed_nodes(p))
    if kind.startswith("dlp"):
        if len(out) != 1:
            raise ValueError("the DLP solvers take one boundary component")
        return out[0]
    return out


def points_with_n(kind, billiard, n_outer, k_ref, **kw):
    """Nodes with the outer component forced to n_outer nodes: b chosen so
    that k_ref L b / 2 pi = n_outer. Returns (nodes, b)."""
    b = TWO_PI * n_outer / (k_ref * billiard.outer_length)
    return evaluate_points(kind, billiard, k_ref, b, **kw), b
