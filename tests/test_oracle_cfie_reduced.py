"""Symmetry-reduced CFIE on the CPU (cfie_kress.jl:264-289, 512-617): the
geometric orbits of the global nodes (symmetry.jl:746-800) and the orbit sum
of full Kress-split entries (oracle/assembly.cfie_reduced) make the reduction
exact, so the eigenvalues of the operator's parity sectors together are the
full operator's (stadium, XY reflection; circle with a centred hole, X
reflection), to rounding."""
import numpy as np
import numpy.linalg as la
import pytest

from oracle import assembly as OA


def _sectors(qb, b, cls, syms, N, k):
    ev = []
    for sym in syms:
        s = cls(1.0, b, symmetry=sym)
        p, s = qb.points_with_n(s, b, N, k)
        orb = qb.symmetry.reduction(s, p)
        assert len(orb[0]) * orb[1].shape[1] == sum(x.n for x in qb.solvers.as_list(p))
        ev.extend(la.eigvals(OA.cfie_reduced(qb.solvers.as_list(p), k, orb)))
    return np.array(ev)


def _max_mismatch(a, b):
    return max(np.min(np.abs(a - x)) for x in b)


def test_stadium_xy_sectors_partition_the_spectrum(qb):
    b = qb.make_full_stadium(1.0, 1.0)
    p, _ = qb.points_with_n(qb.CFIE_kress_global_corners(1.0, b), b, 80, 5.0)
    full = la.eigvals(OA.cfie_matrix(qb.solvers.as_list(p), 5.0 + 0.1j))
    syms = [qb.XYReflection(px, py) for px in (-1, 1) for py in (-1, 1)]
    s = []
    for sym in syms:
        sol = qb.CFIE_kress_global_corners(1.0, b, symmetry=sym)
        pp, sol = qb.points_with_n(sol, b, 80, 5.0)
        s.extend(la.eigvals(OA.cfie_reduced(qb.solvers.as_list(pp), 5.0 + 0.1j, qb.symmetry.reduction(sol, pp))))
    s = np.array(s)
    assert len(s) == len(full)
    assert _max_mismatch(full, s) < 1e-12 and _max_mismatch(s, full) < 1e-12


def test_hole_x_reflection_sectors_and_orbits(qb):
    hb = qb.make_circle_with_hole(1.0, (0.0, 0.0, 0.3))
    p, _ = qb.points_with_n(qb.CFIE_kress(1.0, hb), hb, 120, 8.0)
    full = la.eigvals(OA.cfie_matrix(qb.solvers.as_list(p), 8.0))
    s = _sectors(qb, hb, qb.CFIE_kress, [qb.XReflection(-1), qb.XReflection(1)], 120, 8.0)
    assert len(s) == len(full)
    assert _max_mismatch(full, s) < 1e-12
    sol = qb.CFIE_kress(1.0, hb, symmetry=qb.XReflection(-1))
    pp, sol = qb.points_with_n(sol, hb, 120, 8.0)
    fund, orb, sc = qb.symmetry.reduction(sol, pp)
    xy = np.concatenate([x.xy for x in pp])
    assert np.allclose(xy[orb[:, 1]], xy[orb[:, 0]] * [-1.0, 1.0], atol=1e-12)  # x -> -x images
    assert np.all(sc[:, 1] == -1.0) and np.array_equal(fund, orb[:, 0])


def test_asymmetric_hole_is_refused(qb):
    hb = qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2))
    sol = qb.CFIE_kress(1.0, hb, symmetry=qb.XReflection(1))
    p, sol = qb.points_with_n(sol, hb, 120, 8.0)
    with pytest.raises(ValueError):
        qb.symmetry.reduction(sol, p)
