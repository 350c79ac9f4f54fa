"""Served mixed request stream: Poisson arrivals of Beyn / EBIM / sweep
requests on mixed geometries and sizes through the request server, with
p50/p99 latency (arrival -> result on the host) and throughput.

    python serve_workload.py --requests 2000 --rate 20 --nmin 1024 --nmax 8192

Seeded synthetic stream: geometry uniform over {unit circle with an
off-centre hole of radius 0.2 (CFIE), full stadium (DLP, smooth composite),
half-ellipse-cap mushroom (DLP, corner-graded, kressq = 4), star
r = 1 + 0.2 cos 5 theta (CFIE)}; N log-uniform in [nmin, nmax] (rounded
to the node-count rule); k uniform in [kmin, kmax]; by default 60% Beyn disks
(radius 0.5, 32..64 contour nodes, L probes, mixed form), 30% EBIM (A, A',
A'' at one k), 10% sigma_min sweeps (nk wavenumbers), set by --mix. Discretisations are built and
uploaded before the clock starts; the clock covers submission, the device
work, the copies back and the host part of a Beyn request (SVD, eigvals).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE / "quantumbilliards.jl_gb300"))

import numpy as np  # noqa: E402


def make_stream(qb, args):
    rng = np.random.default_rng(args.seed)
    geoms = [("hole", qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2)), qb.CFIE_kress),
             ("stadium", qb.make_full_stadium(1.0, 1.0), qb.DLP_kress_global_corners),
             ("mushroom", qb.make_full_ellipse_mushroom(), qb.DLP_kress_global_corners),
             ("star", qb.make_star(0.2, 5), qb.CFIE_kress)]
    reqs = []
    t = 0.0
    for q in range(args.requests):
        t += rng.exponential(1.0 / args.rate)
        gname, bil, cls = geoms[int(rng.integers(0, len(geoms)))]
        n = int(round(math.exp(rng.uniform(math.log(args.nmin), math.log(args.nmax)))))
        k = float(rng.uniform(args.kmin, args.kmax))
        u = rng.uniform()
        kind = "beyn" if u < args.mix[0] else ("ebim" if u < args.mix[0] + args.mix[1] else "sweep")
        sol = cls(1.0, bil)
        pts, sol = qb.points_with_n(sol, bil, n, k)
        ws = qb.Workspace(sol, pts)
        r = dict(t=t, kind=kind, geom=gname, n=ws.dim, k=k, ws=ws)
        if kind == "beyn":
            r["nq"] = int(rng.integers(32, 65))
            r["V"] = qb.probe_matrix(ws.dim, args.L, rng)
        elif kind == "sweep":
            r["ks"] = k + 0.01 * np.arange(args.nk)
        reqs.append(r)
    return reqs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=60)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--nmin", type=int, default=1024)
    ap.add_argument("--nmax", type=int, default=3072)
    ap.add_argument("--kmin", type=float, default=50.0)
    ap.add_argument("--kmax", type=float, default=800.0)
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--nk", type=int, default=64)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--max-batch", type=int, default=8)
    ap.add_argument("--max-sweeps", type=int, default=1)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--mix", default="0.6,0.3,0.1", help="fractions of Beyn, EBIM and sweep requests")
    a = ap.parse_args(argv)
    a.mix = [float(x) for x in a.mix.split(",")]
    import build_qbgpu
    build_qbgpu.build()
    import qbgpu as qb
    reqs = make_stream(qb, a)
    lat = {}
    info = {}
    lock = threading.Lock()
    with qb.Server(hbm_budget=int(a.budget_gb * 2 ** 30), workers=a.workers, max_batch=a.max_batch,
                   max_sweeps=a.max_sweeps) as srv, \
            ThreadPoolExecutor(max_workers=64) as pool:
        t0 = time.perf_counter()

        def finish(i, h, t_arr):
            res = srv.wait(h)
            done = time.perf_counter()
            nl = 0
            if reqs[i]["kind"] == "beyn":
                lam = res["lam"]
                nl = int(np.count_nonzero((np.abs(lam - reqs[i]["k"]) < 0.5) & (np.abs(lam.imag) < 1e-3)))
            with lock:
                lat[i] = (done - t_arr) * 1e3
                info[i] = dict(batched=res["batched"], queue_ms=res["queue_ms"], run_ms=res["run_ms"], eig=nl,
                               lag_ms=(h.t_submit - t_arr) * 1e3, wait_ms=(done - h.t_submit) * 1e3)

        futs = []
        for i, r in enumerate(reqs):
            now = time.perf_counter() - t0
            if r["t"] > now:
                time.sleep(r["t"] - now)
            t_arr = t0 + r["t"]
            if r["kind"] == "beyn":
                h = srv.submit_beyn(r["ws"], r["k"], 0.5, r["nq"], r["V"], mixed=True)
            elif r["kind"] == "ebim":
                h = srv.submit_ebim(r["ws"], r["k"])
            else:
                h = srv.submit_sweep(r["ws"], r["ks"])
            futs.append(pool.submit(finish, i, h, t_arr))
        for f in futs:
            f.result()
        wall = time.perf_counter() - t0
    L = np.array([lat[i] for i in range(len(reqs))])
    per = {}
    for kind in ("beyn", "ebim", "sweep"):
        idx = [i for i in range(len(reqs)) if reqs[i]["kind"] == kind]
        v = np.array([lat[i] for i in idx])
        if len(v):
            qv = np.array([info[i]["queue_ms"] for i in idx])
            rv = np.array([info[i]["run_ms"] for i in idx])
            lv = np.array([info[i]["lag_ms"] for i in idx])
            hv = np.array([info[i]["wait_ms"] - info[i]["queue_ms"] - info[i]["run_ms"] for i in idx])
            per[kind] = dict(count=int(len(v)), p50_ms=float(np.percentile(v, 50)), p99_ms=float(np.percentile(v, 99)),
                             submit_lag_p50_ms=float(np.percentile(lv, 50)), queue_p50_ms=float(np.percentile(qv, 50)),
                             run_p50_ms=float(np.percentile(rv, 50)), host_p50_ms=float(np.percentile(hv, 50)))
    eig = sum(info[i]["eig"] for i in info)
    out = dict(requests=len(reqs), rate_per_s=a.rate, wall_s=wall, p50_ms=float(np.percentile(L, 50)),
               p99_ms=float(np.percentile(L, 99)), mean_ms=float(L.mean()), throughput_req_per_s=len(reqs) / wall,
               eigenvalues=eig, eigenvalues_per_s=eig / wall, per_kind=per,
               beyn_batched_max=max([info[i]["batched"] for i in info] + [1]),
               beyn_in_batches=int(sum(1 for i in info if info[i]["batched"] > 1)),
               config=dict(nmin=a.nmin, nmax=a.nmax, kmin=a.kmin, kmax=a.kmax, L=a.L, nk=a.nk,
                           budget_gb=a.budget_gb, workers=a.workers, max_batch=a.max_batch, max_sweeps=a.max_sweeps,
                           seed=a.seed, mix=a.mix))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
