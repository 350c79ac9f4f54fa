"""The product's boundary nodes against the oracle's own restatement of
evaluate_points (oracle/geometry.py, which shares no code with the product):
smooth single curves (DLP_kress, CFIE_kress, CFIE_alpert), smooth composites
(the stadium, with and without its XY reflection), Kress-graded composites
(rectangle, elliptic-cap mushroom) and CFIE holes (reversed orientation), at
the configurations the benchmarks run (star N = 2048, reduced stadium
N = 4096) and at small sizes. Positions, tangents, parameters and weights
agree to 1e-14 of their scale. The arc-length steps ds are differences of
cumulative arc lengths (QuadGK in the reference, adaptive Gauss-Kronrod here,
composite Gauss-Legendre in the product), so they agree to 1e-14 of the
component's length, the rounding of those differences."""
import numpy as np
import pytest

from oracle import geometry as OG


def _as_list(p):
    return p if isinstance(p, list) else [p]


def _compare(prod, orac, ds_tol=1e-14):
    prod, orac = _as_list(prod), _as_list(orac)
    assert len(prod) == len(orac)
    for a, b in zip(prod, orac):
        assert a.n == b.n
        for f in ("xy", "tangent", "tangent_2", "ts", "tphys", "ws", "ws_der"):
            x, y = np.asarray(getattr(a, f)), np.asarray(getattr(b, f))
            scale = max(1.0, float(np.max(np.abs(y))))
            assert np.max(np.abs(x - y)) <= 1e-14 * scale, (f, np.max(np.abs(x - y)))
        assert np.max(np.abs(a.ds - b.ds)) <= ds_tol * np.sum(np.abs(b.ds)), ("ds", np.max(np.abs(a.ds - b.ds)))


CASES = [
    # (product billiard, oracle billiard, product solver, oracle kind, symmetry, N, k_ref)
    ("circle", "dlp", None, 512, 42.0),
    ("star", "dlp", None, 300, 30.0),
    ("star", "cfie", None, 2048, 200.0),
    ("star", "alpert", None, 301, 30.0),
    ("stadium", "dlp_gc", None, 400, 20.0),
    ("stadium", "dlp_gc", "xy", 4096, 300.5),
    ("stadium", "cfie_gc", None, 640, 40.0),
    ("hole", "cfie", None, 300, 30.0),
    ("hole", "alpert", None, 300, 30.0),
    ("rectangle", "dlp_gc", None, 200, 10.0),
    ("mushroom", "dlp_gc", None, 300, 20.0),
    ("mushroom", "cfie_gc", None, 240, 15.0),
]


def _product(qb, geom, kind, sym, N, k):
    b = {"circle": lambda: qb.make_circle(1.0), "star": lambda: qb.make_star(0.2, 5),
         "stadium": lambda: qb.make_full_stadium(1.0, 1.0), "hole": lambda: qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2)),
         "rectangle": lambda: qb.make_rectangle(1.0, 0.7), "mushroom": lambda: qb.make_full_ellipse_mushroom()}[geom]()
    cls = {"dlp": qb.DLP_kress, "cfie": qb.CFIE_kress, "alpert": qb.CFIE_alpert, "dlp_gc": qb.DLP_kress_global_corners,
           "cfie_gc": qb.CFIE_kress_global_corners}[kind]
    s = qb.symmetry.XYReflection(-1, -1) if sym == "xy" else None
    sol = cls(1.0, b, symmetry=s, kressq=4)
    pts, _ = qb.points_with_n(sol, b, N, k)
    return pts


def _oracle(geom, kind, sym, N, k):
    b = {"circle": lambda: OG.circle(1.0), "star": lambda: OG.star(0.2, 5), "stadium": lambda: OG.full_stadium(1.0, 1.0),
         "hole": lambda: OG.circle_with_holes(1.0, ((0.3, 0.1, 0.2),)), "rectangle": lambda: OG.full_rectangle(1.0, 0.7),
         "mushroom": lambda: OG.full_ellipse_mushroom()}[geom]()
    kk = {"dlp": "dlp_kress", "cfie": "cfie_kress", "alpert": "cfie_alpert", "dlp_gc": "dlp_kress_global_corners",
          "cfie_gc": "cfie_kress_global_corners"}[kind]
    pts, _ = OG.points_with_n(kk, b, N, k, symmetry=("xy", -1, -1) if sym == "xy" else None, kressq=4.0)
    return pts


@pytest.mark.parametrize("geom,kind,sym,N,k", CASES)
def test_product_nodes_equal_oracle_nodes(qb, geom, kind, sym, N, k):
    _compare(_product(qb, geom, kind, sym, N, k), _oracle(geom, kind, sym, N, k))


def test_oracle_node_rules():
    """N rule and multiples: even N for smooth Kress, multiples of 4 under a
    reflection, of n under a rotation, none for graded corners and the
    periodic Alpert grid; graded nodes cluster at the corners."""
    assert OG.node_count(42.0, 2 * np.pi, 12.2) == 512
    assert OG.node_count(10.0, 1.0, 1.0, min_pts=20) == 20
    assert OG.needed_multiple(None, 2) == 2 and OG.needed_multiple(("xy", -1, -1), 2) == 4
    assert OG.needed_multiple(("rot", 5, 0), 2) == 10 and OG.needed_multiple(None, 1) == 1
    p = OG.evaluate_points("dlp_kress_global_corners", OG.full_rectangle(1.0, 0.7), 10.0, 3.3)
    assert p.n == OG.node_count(10.0, 3.4, 3.3, needed=1)
    d = np.hypot(*np.diff(p.xy, axis=0).T)
    corner = np.min(np.hypot(p.xy[:, 0] - 0.5, p.xy[:, 1] - 0.35))
    assert corner < 0.2 * np.median(d)
