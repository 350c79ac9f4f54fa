"""GPU: the request server (qbg_serve_*).

* alone versus in the mix: every request of a seeded mixed stream gives the
  same result when it runs alone (one worker, no merging) and when it runs
  among the others (four workers, Beyn requests merged into device batches):
  FP64 Beyn moments, EBIM matrices and sweep values to 1e-13; mixed Beyn
  moments to 1e-10 (the refinement stops on the batch's largest residual);
* Beyn requests queued behind a running sweep on one geometry, with the same
  nq, L and precision, are merged into one device batch and give their
  results when alone;
* with max_sweeps = 1 the sweeps run one after another while EBIM requests
  submitted behind them pass them;
* a request larger than the HBM budget is refused at submission (QBG_EBUDGET).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _stream(qb):
    rng = np.random.default_rng(4)
    star = qb.make_star(0.2, 5)
    s1 = qb.CFIE_kress(1.0, star)
    p1, s1 = qb.points_with_n(s1, star, 320, 20.0)
    hole = qb.make_circle_with_hole()
    s2 = qb.CFIE_kress(1.0, hole)
    p2, s2 = qb.points_with_n(s2, hole, 256, 20.0)
    ws = [qb.Workspace(s1, p1), qb.Workspace(s2, p2)]
    reqs = []
    for q in range(10):
        g = int(rng.integers(0, 2))
        kind = ["beyn", "beyn", "beyn", "ebim", "sweep"][int(rng.integers(0, 5))]
        k = float(rng.uniform(18.0, 22.0))
        if kind == "beyn":
            reqs.append(("beyn", g, k, bool(rng.integers(0, 2)), qb.probe_matrix(ws[g].dim, 12, rng)))
        elif kind == "ebim":
            reqs.append(("ebim", g, k, None, None))
        else:
            reqs.append(("sweep", g, k, None, np.linspace(k, k + 0.2, 4)))
    return ws, reqs


def _submit(srv, ws, r):
    kind, g, k, mixed, extra = r
    if kind == "beyn":
        return srv.submit_beyn(ws[g], k, 0.4, 12, extra, mixed=mixed)
    if kind == "ebim":
        return srv.submit_ebim(ws[g], k)
    return srv.submit_sweep(ws[g], extra)


def _key(res, kind):
    if kind == "beyn":
        return [res["A0"], res["A1"]]
    if kind == "ebim":
        return [res["A"], res["dA"], res["ddA"]]
    return [res["sig"]]


def test_alone_versus_in_the_mix(qb):
    ws, reqs = _stream(qb)
    alone = []
    with qb.Server(workers=1, max_batch=1) as srv:
        for r in reqs:
            alone.append(srv.wait(_submit(srv, ws, r)))
    with qb.Server(workers=4, max_batch=8) as srv:
        handles = [_submit(srv, ws, r) for r in reqs]
        mix = [srv.wait(h) for h in handles]
    for r, a, m in zip(reqs, alone, mix):
        tol = 1e-10 if (r[0] == "beyn" and r[3]) else 1e-13
        for x, y in zip(_key(m, r[0]), _key(a, r[0])):
            assert _rel(x, y) < tol, (r[0], r[3])


def test_queued_beyn_requests_merge(qb):
    ws, _ = _stream(qb)
    rng = np.random.default_rng(7)
    reqs = [("beyn", 0, 20.0 + 0.3 * q, q < 3, qb.probe_matrix(ws[0].dim, 12, rng)) for q in range(4)]
    with qb.Server(workers=1, max_batch=1) as srv:
        alone = [srv.wait(_submit(srv, ws, r)) for r in reqs]
    with qb.Server(workers=1, max_batch=8) as srv:
        blocker = srv.submit_sweep(ws[1], np.linspace(20.0, 21.5, 16))  # holds the only worker
        handles = [_submit(srv, ws, r) for r in reqs]
        merged = [srv.wait(h) for h in handles]
        srv.wait(blocker)
    assert [m["batched"] for m in merged] == [3, 3, 3, 1]
    for r, a, m in zip(reqs, alone, merged):
        tol = 1e-10 if r[3] else 1e-13
        for x, y in zip(_key(m, r[0]), _key(a, r[0])):
            assert _rel(x, y) < tol, r[3]


def test_budget_refusal(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 512, 20.0)
    ws = qb.Workspace(sol, pts)
    with qb.Server(hbm_budget=64 << 20, workers=1) as srv:
        with pytest.raises(qb._lib.QBGError) as e:
            srv.submit_beyn(ws, 20.0, 0.4, 48, qb.probe_matrix(ws.dim, 16, np.random.default_rng(0)))
        assert e.value.status == qb._lib.QBG_EBUDGET


def test_sweeps_run_one_at_a_time(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 320, 20.0)
    ws = qb.Workspace(sol, pts)
    ks = np.linspace(20.0, 20.3, 4)
    with qb.Server(workers=4, max_sweeps=1) as srv:
        hs = [srv.submit_sweep(ws, ks + 0.5 * q) for q in range(3)]
        he = [srv.submit_ebim(ws, 20.0 + 0.1 * q) for q in range(2)]
        rs = [srv.wait(h) for h in hs]
        re = [srv.wait(h) for h in he]
    iv = sorted((h.t_submit * 1e3 + r["queue_ms"], h.t_submit * 1e3 + r["queue_ms"] + r["run_ms"]) for h, r in zip(hs, rs))
    for (s0, e0), (s1, e1) in zip(iv, iv[1:]):
        assert s1 >= e0 - 1.0  # the next sweep starts when the previous one has ended
    second_start = iv[1][0]
    for h, r in zip(he, re):
        assert h.t_submit * 1e3 + r["queue_ms"] < second_start
    for q, r in enumerate(rs):
        assert np.all(np.isfinite(r["sig"])) and np.all(r["sig"] > 0)
