"""GPU: the library's caching device allocator. A second Beyn handle of the
same shape is served entirely from cached blocks (no new driver allocation)
and gives bit-identical moments; releasing the cache empties it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pool_reuses_blocks_and_releases(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 400, 25.0)
    ws = qb.Workspace(sol, pts)
    V = qb.probe_matrix(ws.dim, 16, np.random.default_rng(2))
    out, delta = [], []
    for _ in range(2):
        s0 = qb.pool_stats()
        bh = qb.BeynHandle(ws, 25.0, 0.4, 16, mixed=True)
        out.append(bh.moments(V))
        bh.close()
        s1 = qb.pool_stats()
        delta.append((s1["hits"] - s0["hits"], s1["misses"] - s0["misses"]))
    assert delta[1][0] > 0 and delta[1][1] == 0, delta
    for a, r in zip(out[0], out[1]):
        assert np.array_equal(a, r)
    assert qb.pool_stats()["cached_bytes"] > 0
    qb.release_cached_memory()
    st = qb.pool_stats()
    assert st["cached_bytes"] == 0 and st["live_bytes"] > 0  # the workspace's geometry stays
