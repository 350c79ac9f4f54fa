"""Symmetry-reduced CFIE on the device (cfie_kress.jl:512-617, derivatives
:758-892, Chebyshev route chebyshev_euclidian_helmholtz_cfie_kress.jl:698-825)
against the oracle's restatement (oracle/assembly.cfie_reduced: the orbit sum
of full Kress-split entries):

* the desymmetrised stadium (CFIE_kress_global_corners, XY reflection, every
  parity sector) and the circle with a centred hole (CFIE_kress, X reflection):
  direct FP64 values at real k with A', A'' and at complex k, 1e-12 of the
  max-norm; through Chebyshev panels tuned to 1e-13, 1e-11; the complex64
  hi + lo values within 1e-13 of the FP64 ones;
* because every orbit member keeps its Kress split, the reduction is exact:
  the Beyn eigenvalues of the four parity sectors of the stadium together are
  the full operator's, to 1e-10.
"""
import math

import numpy as np
import pytest

from oracle import assembly as OA

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _stadium(qb, px, py, n=400, k=20.0):
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.CFIE_kress_global_corners(1.0, b, symmetry=qb.XYReflection(px, py))
    pts, sol = qb.points_with_n(sol, b, n, k)
    return b, sol, pts


@pytest.mark.parametrize("px,py", [(-1, -1), (1, -1), (-1, 1), (1, 1)])
def test_reduced_cfie_stadium_direct(qb, px, py):
    b, sol, pts = _stadium(qb, px, py)
    ws = qb.Workspace(sol, pts)
    orb = qb.symmetry.reduction(sol, pts)
    assert ws.dim == len(orb[0]) == 100
    plist = qb.solvers.as_list(pts)
    got = qb.construct_matrices(sol, pts, ws, 20.3, derivs=True)
    ref = OA.cfie_reduced(plist, 20.3, orb, derivs=True)
    for g, r in zip(got, ref):
        assert _rel(g, r) < 1e-12
    z = 20.1 + 0.3j
    assert _rel(qb.assemble(ws, [z])[0], OA.cfie_reduced(plist, z, orb)) < 1e-12
    ws.close()


def test_reduced_cfie_hole_and_chebyshev(qb):
    hb = qb.make_circle_with_hole(1.0, (0.0, 0.0, 0.3))
    sol = qb.CFIE_kress(1.0, hb, symmetry=qb.XReflection(-1))
    pts, sol = qb.points_with_n(sol, hb, 240, 15.0)
    ws = qb.Workspace(sol, pts)
    orb = qb.symmetry.reduction(sol, pts)
    plist = qb.solvers.as_list(pts)
    assert ws.dim == len(orb[0]) == sum(p.n for p in plist) // 2
    z = 15.2 + 0.2j
    ref = OA.cfie_reduced(plist, z, orb)
    assert _rel(qb.assemble(ws, [z])[0], ref) < 1e-12
    got = qb.construct_matrices(sol, pts, ws, 15.0, derivs=True)
    for g, r in zip(got, OA.cfie_reduced(plist, 15.0, orb, derivs=True)):
        assert _rel(g, r) < 1e-12
    zref = 15.0 + 0.5 * np.exp(2j * math.pi * np.arange(8) / 8)
    cheb = qb.chebyshev_params(sol, pts, zref, ws=ws, tol=1e-13)[:4]
    gc = qb.assemble(ws, [z], cheb=cheb)[0]
    assert _rel(gc, ref) < 1e-11
    gd = qb.assemble(ws, [z], cheb=cheb, deriv=True)
    rd = OA.cfie_reduced(plist, z, orb, derivs=True)
    for g, r in zip(gd, rd):
        assert _rel(g, r) < 1e-10
    hi, lo = qb.assemble(ws, [z], mixed=True, cheb=cheb, split_lo=True)
    assert np.max(np.abs(hi.astype(np.complex128) + lo - gc)) < 1e-13 * np.max(np.abs(gc))
    ws.close()


def test_reduced_cfie_sectors_partition_full_spectrum(qb):
    k0, R = 10.0 + 0j, 0.4
    lam_s = []
    for px in (-1, 1):
        for py in (-1, 1):
            b, sol, pts = _stadium(qb, px, py, 240, 10.0)
            lam = qb.solve(sol, pts, k0, R, nq=32, r=16, svd_tol=1e-12, rng=np.random.default_rng(3),
                           use_chebyshev=False)
            lam_s.extend(lam[(np.abs(lam - k0) < R) & (np.abs(lam.imag) < 1e-3)])
    b = qb.make_full_stadium(1.0, 1.0)
    full = qb.CFIE_kress_global_corners(1.0, b)
    pts, full = qb.points_with_n(full, b, 240, 10.0)
    lam = qb.solve(full, pts, k0, R, nq=32, r=40, svd_tol=1e-12, rng=np.random.default_rng(3), use_chebyshev=False)
    # 240 nodes leave imaginary parts of 1e-7..1e-5 (the discretisation error);
    # the oracle's Beyn on its reduced matrices gives the same nine values
    lam_f = np.sort_complex(lam[(np.abs(lam - k0) < R) & (np.abs(lam.imag) < 1e-3)])
    lam_s = np.sort_complex(np.array(lam_s))
    assert len(lam_s) == len(lam_f) == 9
    assert np.max(np.abs(lam_s - lam_f) / np.abs(lam_f)) < 1e-10
