"""GPU: solve_pipelined (a sequence of disks; the next disk's handle built on
a second thread while the current disk solves, each disk's host QR of the
moments, SVDs and eig(B) on a worker thread) against `solve` with the same
probe generator, disk by disk, and against itself with one disk in flight
(overlap=False, identical to 1e-12): three disks
of the CFIE star (one whose rank saturates and regrows, one that does not),
mixed and FP64 forms, and r >= N/2 (no regrowth block).

With the moments reduced on the device (host_qr=False) the computation is
`solve`'s: every eigenvalue of B agrees to 1e-12 and the ranks are equal.
With the host QR (LAPACK zgeqrf / zunmqr, the default) R differs from the
device QR's by rounding, and eigenvalues of B carried by singular values
near svd_tol move by ~eps |A0| / sigma: the eigenvalues inside 0.9 R (the
ones the method computes) agree to 1e-10 relative, each with the nearest of
the other set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _star(qb, n_nodes=400, k=25.0):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, n_nodes, k)
    return sol, pts, qb.Workspace(sol, pts)


def _same(a, b):
    a, b = np.sort_complex(np.asarray(a)), np.sort_complex(np.asarray(b))
    assert len(a) == len(b)
    if len(a):
        assert np.max(np.abs(a - b)) <= 1e-12 * max(1.0, np.max(np.abs(b)))


def _inside_match(a, b, k0, R):
    a, b = np.asarray(a), np.asarray(b)
    for x, y in ((a, b), (b, a)):
        sel = x[np.abs(x - k0) < 0.9 * R]
        for v in sel:
            assert len(y) and np.min(np.abs(y - v)) <= 1e-10 * abs(v), (v, np.min(np.abs(y - v)))
    return int(np.count_nonzero(np.abs(b - k0) < 0.9 * R))


@pytest.mark.parametrize("mixed", [True, False])
def test_pipelined_matches_solve(qb, mixed):
    sol, pts, ws = _star(qb)
    k0s = [25.0 + 0.05j, 24.2 + 0.0j, 25.6 - 0.02j]
    kw = dict(nq=16, r=12, svd_tol=1e-12, mixed=mixed, ws=ws)
    rngs = lambda: [np.random.default_rng(10 + d) for d in range(3)]
    lams_d, info_d = qb.solve_pipelined(sol, pts, k0s, 0.4, rngs=rngs(), return_info=True, host_qr=False, **kw)
    lams_h = qb.solve_pipelined(sol, pts, k0s, 0.4, rngs=rngs(), **kw)
    lams_1 = qb.solve_pipelined(sol, pts, k0s, 0.4, rngs=rngs(), host_qr=False, overlap=False, **kw)
    assert len(lams_d) == 3 and len(info_d["rk"]) == 3
    for a, b in zip(lams_1, lams_d):  # one disk or two in flight: the same computation
        _same(a, b)
    inside = 0
    for d, k0 in enumerate(k0s):
        ref, rinfo = qb.solve(sol, pts, k0, 0.4, rng=np.random.default_rng(10 + d), return_info=True, **kw)
        _same(lams_d[d], ref)
        assert info_d["r"][d] == rinfo["r"] and info_d["rk"][d] == rinfo["rk"]
        inside += _inside_match(lams_h[d], ref, k0, 0.4)
    assert inside > 0


def test_pipelined_without_regrowth_block(qb):
    sol, pts, ws = _star(qb, 60, 8.0)
    kw = dict(nq=12, r=40, svd_tol=1e-10, mixed=True, ws=ws)  # 2r >= N: no regrowth block
    ref = qb.solve(sol, pts, 8.0 + 0.02j, 0.5, rng=np.random.default_rng(3), **kw)
    lams_d = qb.solve_pipelined(sol, pts, [8.0 + 0.02j], 0.5, rngs=[np.random.default_rng(3)], host_qr=False, **kw)
    _same(lams_d[0], ref)
    lams_h = qb.solve_pipelined(sol, pts, [8.0 + 0.02j], 0.5, rngs=[np.random.default_rng(3)], **kw)
    _inside_match(lams_h[0], ref, 8.0 + 0.02j, 0.5)
