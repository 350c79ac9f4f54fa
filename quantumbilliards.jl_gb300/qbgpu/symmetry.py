"""Boundary symmetries and the orbit maps of the symmetry-reduced DLP
(mirrors symmetry.jl: XReflection/YReflection/XYReflection :97-130, Rotation,
periodic_symmetry_index_orbits :214-261, _build_periodic_orbit_maps :300-319).

Node indices are 0-based here. On a cyclic discretisation with nodes at
t_j = 2 pi (j + 1/2)/N that starts on the positive x axis (as the stadium and
the polar curves do), reflections and rotations act on indices:
  x -> -x : q -> N/2 - 1 - q,  y -> -y : q -> N - 1 - q,  rotation by pi : q -> q + N/2,
  rotation by 2 pi l/n : q -> q + l N/n   (all mod N).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Tuple

import numpy as np


@dataclass(frozen=True)
class Reflection:
    """axis: "y_axis" (x -> -x), "x_axis" (y -> -y) or "origin" (both);
    parity: the wavefunction's parity per reflection (+1 / -1)."""
    axis: str
    parity: Tuple[int, ...]


@dataclass(frozen=True)
class Rotation:
    """C_n rotation with angular-momentum sector m: chi_l = exp(2 pi i m l / n)."""
    n: int
    m: int = 0


def XReflection(parity: int) -> Reflection:
    return Reflection("y_axis", (int(parity),))


def YReflection(parity: int) -> Reflection:
    return Reflection("x_axis", (int(parity),))


def XYReflection(parity_x: int, parity_y: int) -> Reflection:
    return Reflection("origin", (int(parity_x), int(parity_y)))


def needed_multiple(symmetry, base: int = 2) -> int:
    """Node-count divisibility (dlp_kress.jl:362-370): even N, times the
    rotation order, or a multiple of 4 for any reflection."""
    if symmetry is None:
        return base
    if isinstance(symmetry, Rotation):
        return math.lcm(base, int(symmetry.n))
    return math.lcm(base, 4)


def periodic_symmetry_index_orbits(N: int, sym):
    """(fund, fund_to_full [m x norb], fund_to_scale [m x norb]), 0-based.

    fund[b] is the representative of orbit b; fund_to_full[b] lists the full
    indices of the orbit with their phase u(g(q)) = chi u(q) in fund_to_scale."""
    if isinstance(sym, Reflection):
        if sym.axis in ("y_axis", "x_axis"):
            if N % 2:
                raise ValueError("a reflection needs an even node count")
            m = N // 2
            p = complex(sym.parity[0])
            qs = [[q, (N - 1 - q) % N] for q in range(m)]
            ss = [[1.0, p]] * m
        elif sym.axis == "origin":
            if N % 4:
                raise ValueError("the XY reflection needs a node count divisible by 4")
            m = N // 4
            px, py = complex(sym.parity[0]), complex(sym.parity[1])
            qs = [[q, (N // 2 - 1 - q) % N, (N - 1 - q) % N, (q + N // 2) % N] for q in range(m)]
            ss = [[1.0, px, py, px * py]] * m
        else:
            raise ValueError(f"unsupported reflection axis {sym.axis}")
    elif isinstance(sym, Rotation):
        n = int(sym.n)
        if N % n:
            raise ValueError("the rotation order must divide the node count")
        m = N // n
        chi = [complex(math.cos(2 * math.pi * sym.m * l / n), math.sin(2 * math.pi * sym.m * l / n))
               for l in range(n)]
        qs = [[(q + l * (N // n)) % N for l in range(n)] for q in range(m)]
        ss = [chi] * m
    else:
        raise TypeError("symmetry must be a Reflection or a Rotation")
    full = np.asarray(qs, dtype=np.int64)
    scale = np.asarray(ss, dtype=np.complex128)
    count = np.bincount(full.ravel(), minlength=N)
    if full.max() >= N or not np.all(count == 1):
        raise ValueError("periodic symmetry orbits do not partition the nodes")
    return np.arange(m, dtype=np.int64), full, scale


def _match(targets, xy, tol):
    """Index of the node of xy at each target position (within tol)."""
    from scipy.spatial import cKDTree
    d, idx = cKDTree(xy).query(targets)
    if np.any(d > tol):
        raise ValueError("the symmetry does not map the boundary nodes onto each other "
                         f"(largest mismatch {float(d.max()):.3e})")
    return idx.astype(np.int64)


def geometric_orbits(xy, sym, tol=1e-10):
    """Orbits of the global nodes of a CFIE workspace (build_cfie_kress_workspace,
    cfie_kress.jl:264-289 with build_symmetry_maps / apply_symmetry_orbit_from_maps,
    symmetry.jl:746-800): every group element maps each node to the node at
    its image position; the nodes are visited in global order and each
    unvisited node opens an orbit [g, images...] with scales [1, characters...].
    Returns (fund, fund_to_full [m x norb], fund_to_scale [m x norb]), 0-based."""
    xy = np.asarray(xy, dtype=np.float64)
    x, y = xy[:, 0], xy[:, 1]
    if isinstance(sym, Reflection):
        if sym.axis == "y_axis":
            maps = [_match(np.stack([-x, y], 1), xy, tol)]
            sc = [1.0, float(sym.parity[0])]
        elif sym.axis == "x_axis":
            maps = [_match(np.stack([x, -y], 1), xy, tol)]
            sc = [1.0, float(sym.parity[0])]
        elif sym.axis == "origin":
            px, py = float(sym.parity[0]), float(sym.parity[1])
            maps = [_match(np.stack([-x, y], 1), xy, tol), _match(np.stack([x, -y], 1), xy, tol),
                    _match(np.stack([-x, -y], 1), xy, tol)]
            sc = [1.0, px, py, px * py]
        else:
            raise ValueError(f"unsupported reflection axis {sym.axis}")
        scales = np.asarray(sc, dtype=np.complex128)
    elif isinstance(sym, Rotation):
        n = int(sym.n)
        maps = []
        for l in range(1, n):
            c, s = math.cos(2 * math.pi * l / n), math.sin(2 * math.pi * l / n)
            maps.append(_match(np.stack([c * x - s * y, s * x + c * y], 1), xy, max(tol, 1e-8)))
        scales = np.asarray([complex(math.cos(2 * math.pi * sym.m * l / n), math.sin(2 * math.pi * sym.m * l / n))
                             for l in range(n)], dtype=np.complex128)
    else:
        raise TypeError("symmetry must be a Reflection or a Rotation")
    N = len(xy)
    visited = np.zeros(N, dtype=bool)
    fund, full = [], []
    for g in range(N):
        if visited[g]:
            continue
        orb = [g] + [int(mp[g]) for mp in maps]
        fund.append(g)
        full.append(orb)
        visited[orb] = True
    full = np.asarray(full, dtype=np.int64)
    return (np.asarray(fund, dtype=np.int64), full,
            np.broadcast_to(scales, full.shape).astype(np.complex128))


def reduction(solver, pts):
    """Orbit maps for a solver with a symmetry, or None (the reduced workspace
    is used exactly when the solver has a symmetry, dlp_kress.jl:234,
    cfie_kress.jl:264-289). DLP: the periodic index orbits of the one
    component (symmetry.jl:214-261). CFIE: the geometric orbits of all the
    global nodes (geometric_orbits)."""
    if getattr(solver, "symmetry", None) is None:
        return None
    sym = solver.symmetry
    plist = pts if isinstance(pts, list) else [pts]
    if solver.kind == "dlp":
        return periodic_symmetry_index_orbits(plist[0].n, sym)
    return geometric_orbits(np.concatenate([np.asarray(p.xy) for p in plist]), sym)
