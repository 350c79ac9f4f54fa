"""GPU: solve_pipelined (a sequence of disks, each disk's host SVDs and
eig(B) on a worker thread while the device runs the next disk) returns, disk
by disk, the eigenvalues of `solve` with the same probe generator: three
disks of the CFIE star (one whose rank saturates and regrows, one that does
not), mixed and FP64 forms, to 1e-12 relative; with r >= N/2 (no regrowth
block) as well."""
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


@pytest.mark.parametrize("mixed", [True, False])
def test_pipelined_matches_solve(qb, mixed):
    sol, pts, ws = _star(qb)
    k0s = [25.0 + 0.05j, 24.2 + 0.0j, 25.6 - 0.02j]
    kw = dict(nq=16, r=12, svd_tol=1e-12, mixed=mixed, ws=ws)
    lams, info = qb.solve_pipelined(sol, pts, k0s, 0.4, rngs=[np.random.default_rng(10 + d) for d in range(3)],
                                    return_info=True, **kw)
    assert len(lams) == 3 and len(info["rk"]) == 3
    for d, k0 in enumerate(k0s):
        ref, rinfo = qb.solve(sol, pts, k0, 0.4, rng=np.random.default_rng(10 + d), return_info=True, **kw)
        _same(lams[d], ref)
        assert info["r"][d] == rinfo["r"] and info["rk"][d] == rinfo["rk"]


def test_pipelined_without_regrowth_block(qb):
    sol, pts, ws = _star(qb, 60, 8.0)
    kw = dict(nq=12, r=40, svd_tol=1e-10, mixed=True, ws=ws)  # 2r >= N: no regrowth block
    lams = qb.solve_pipelined(sol, pts, [8.0 + 0.02j], 0.5, rngs=[np.random.default_rng(3)], **kw)
    ref = qb.solve(sol, pts, 8.0 + 0.02j, 0.5, rng=np.random.default_rng(3), **kw)
    _same(lams[0], ref)
