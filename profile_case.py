"""Run one named workload once, for profilers (ncu) and quick checks.

    python profile_case.py beyn --nq 8 --form mixed
    python profile_case.py assemble --nq 8
    python profile_case.py disks --n 4096 --ndisk 32 --nq 48 --L 96
    python profile_case.py large --n 16384 --nq 48 --L 128 --chunk 8
    python profile_case.py newton

Cases use the bench workload (CFIE Kress, star r = 1 + 0.2 cos 5 theta,
N = 2048, k0 = 200, R = 0.5, L = 64) with an adjustable number of contour nodes
so that a capture stays small (a few GB on the device at most).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE / "quantumbilliards.jl_gb300"))

import numpy as np  # noqa: E402


def star_case(qb, n_nodes=2048, k0=200.0, kind="cfie"):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b) if kind == "cfie" else qb.DLP_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, n_nodes, k0)
    return b, sol, pts


def disks_case(qb, a):
    """Batched Beyn on the desymmetrised stadium: DLP_kress_global_corners with
    XYReflection(-1, -1), N full nodes (m = N/4), ndisk disks of radius 0.5
    centred at 300.5 + d, nq nodes each, L probes, panels tuned to 1e-12."""
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, b, symmetry=qb.XYReflection(-1, -1))
    k0s = 300.5 + np.arange(a.ndisk)
    pts, sol = qb.points_with_n(sol, b, a.n, float(k0s[-1] + 0.5))
    ws = qb.Workspace(sol, pts)
    t0 = time.perf_counter()
    zref = k0s[-1] + 0.5 * np.exp(2j * math.pi * np.arange(a.nq) / a.nq)
    if a.tune == "reference":
        cheb = qb.chebyshev_params(sol, pts, zref, ws=ws, tol=1e-12, sampling_points=50000)[:4]
    else:
        # the main entry plus norb - 1 image terms per reduced entry, tables for every node of every disk
        cheb = qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=1e-12, entries=float(ws.dim) ** 2 * a.ndisk
                                            * a.nq, terms_per_entry=4.0, tables_per_call=a.ndisk * a.nq)[:4]
    t1 = time.perf_counter()
    # the first batch allocates every buffer from the driver (cold); later
    # batches of the same shape reuse the library's cached blocks (warm)
    times = []
    for _ in range(max(1, a.repeat)):
        ts = time.perf_counter()
        lams, info = qb.solve_disks(sol, pts, k0s, 0.5, nq=a.nq, r=a.L, svd_tol=1e-10, rng=np.random.default_rng(3),
                                    mixed=a.form, ws=ws, return_info=True, cheb=cheb)
        times.append(time.perf_counter() - ts)
    n_in = sum(int(np.count_nonzero((np.abs(l - k) < 0.5) & (np.abs(l.imag) < 1e-3))) for l, k in zip(lams, k0s))
    st = info["stats"]
    warm = min(times[1:]) if len(times) > 1 else times[0]
    print(json.dumps(dict(case="disks", N=pts.n, m=ws.dim, ndisk=a.ndisk, nq=a.nq, operators=a.ndisk * a.nq, L=a.L,
                          form=a.form, cheb=list(map(int, cheb)), autotune_s=t1 - t0, solve_s_cold=times[0],
                          solve_s_warm=warm, eigenvalues=n_in, eigenvalues_per_s_warm=n_in / warm,
                          eigenvalues_per_s_cold=n_in / times[0], rk=info["rk"],
                          ms_assemble=st[0]["ms_assemble"], ms_factor=st[0]["ms_factor"],
                          ms_solve=[s["ms_solve"] for s in st], refine=[s["refine_history"] for s in st],
                          host_ms=info.get("host_ms"))))


def large_case(qb, a):
    """CFIE_kress_global_corners on the full stadium at N = a.n, k0 = 1500:
    A, A', A'' in complex128 at k0 (EBIM), then one Beyn moments call with
    nq nodes streamed a.chunk at a time and L probes."""
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.CFIE_kress_global_corners(1.0, b)
    pts, sol = qb.points_with_n(sol, b, a.n, 1500.0)
    ws = qb.Workspace(sol, pts)
    t0 = time.perf_counter()
    mats = qb.assemble(ws, [1500.0 + 0j], deriv=True, cheb=True)
    t1 = time.perf_counter()
    del mats
    bh = qb.BeynHandle(ws, 1500.0, 0.5, a.nq, mixed=a.form, node_chunk=a.chunk)
    V = qb.probe_matrix(ws.dim, a.L, np.random.default_rng(5))
    t2 = time.perf_counter()
    A0, A1 = bh.moments(V)
    t3 = time.perf_counter()
    st = bh.last_stats
    bh.close()
    S = np.linalg.svd(A0, compute_uv=False)
    print(json.dumps(dict(case="large", N=ws.dim, ebim_assembly_s=t1 - t0, moments_s=t3 - t2, nq=a.nq, L=a.L,
                          chunk=a.chunk, form=a.form, rank_1e10=int(np.count_nonzero(S >= 1e-10)),
                          ms_assemble=st["ms_assemble"], ms_factor=st["ms_factor"], ms_solve=st["ms_solve"],
                          refine=st["refine_history"], ms_residual=st["ms_residual"])))


def sweep_case(qb):
    """The sigma_min sweep of the unit circle (DLP Kress, pts_scaling_factor
    12.2: N = 512 at k = 42) over 200 k in [40, 42], then refine_minima."""
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(12.2, b)
    ks = np.linspace(40.0, 42.0, 200)
    qb.k_sweep(sol, b, ks[:4])  # warm-up
    t0 = time.perf_counter()
    sig = qb.k_sweep(sol, b, ks)
    t1 = time.perf_counter()
    kr, tr, hist = qb.refine_minima(sol, b, ks, sig)
    t2 = time.perf_counter()
    print(json.dumps(dict(case="sweep", N=512, nk=len(ks), sweep_s=t1 - t0, refine_s=t2 - t1, minima=len(kr),
                          refined=[round(float(k), 10) for k in kr])))


def newton_case(qb):
    """One newton_refine_svd call (two Newton steps) on the unit circle, DLP
    Kress with pts_scaling_factor 12.2 discretised at k = 40.06 (N = 490),
    window [40.0574, 40.0594], twice (the second call warm)."""
    from qbgpu import sweep
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(12.2, b)
    ws = qb.Workspace(sol, qb.evaluate_points(sol, b, 40.06))
    for _ in range(2):
        t0 = time.perf_counter()
        k, t, it = sweep.newton_refine_svd(ws, 40.0584, 40.0574, 40.0594, 8, 1e-12, return_iters=True)
        print(json.dumps(dict(case="newton", N=ws.dim, k=k, tension=t, iters=it, ms=(time.perf_counter() - t0) * 1e3)))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["beyn", "assemble", "disks", "large", "ebim", "sweep", "newton"])
    ap.add_argument("--ndisk", type=int, default=32)
    ap.add_argument("--repeat", type=int, default=1, help="disks: batches run back to back (first cold, rest warm)")
    ap.add_argument("--chunk", type=int, default=8)
    ap.add_argument("--tune", default="min_cost", choices=["min_cost", "reference"])
    ap.add_argument("--nq", type=int, default=8)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--form", default="mixed", choices=["fp64", "mixed", "fp32"])
    ap.add_argument("--direct", action="store_true", help="direct Hankel evaluation instead of Chebyshev panels")
    ap.add_argument("--cheb-tol", type=float, default=0.0,
                    help="beyn / assemble: panels by chebyshev_params_min_cost at this tolerance (the bench's "
                         "1e-13) instead of the reference's defaults")
    ap.add_argument("--cheb-panels", default="",
                    help="beyn / assemble: explicit panels n_h,M_h,n_j,M_j (no tuning launches; the bench's "
                         "C2 tuning gives 7695,9,863,9)")
    ap.add_argument("--dk", type=float, default=0.05, help="ebim: window half-width")
    ap.add_argument("--nev", type=int, default=5, help="ebim: eigenvalues of the block iteration")
    ap.add_argument("--full", action="store_true", help="ebim: solve_full! convention (every root in the box)")
    ap.add_argument("--gemm-engine", type=int, default=1, choices=[0, 1, 2],
                    help="complex64 GEMM engine of the FP32 LU and solves (qbg_set_gemm_engine)")
    a = ap.parse_args(argv)
    import build_qbgpu
    build_qbgpu.build()
    import qbgpu as qb
    qb.set_gemm_engine(a.gemm_engine)
    if a.case == "sweep":
        return sweep_case(qb)
    if a.case == "newton":
        return newton_case(qb)
    if a.case == "disks":
        return disks_case(qb, a)
    if a.case == "large":
        return large_case(qb, a)
    b, sol, pts = star_case(qb, a.n)
    ws = qb.Workspace(sol, pts)
    cheb = None
    if a.cheb_panels and a.case in ("beyn", "assemble"):
        cheb = tuple(int(x) for x in a.cheb_panels.split(","))
    elif a.cheb_tol > 0 and a.case in ("beyn", "assemble"):
        zref = 200.0 + 0.5 * np.exp(2j * math.pi * np.arange(a.nq) / a.nq)
        cheb = tuple(int(x) for x in qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=a.cheb_tol)[:4])
        print("panels", cheb)
    t0 = time.perf_counter()
    if a.case == "ebim":
        k_ebim, reps = 200.0, 3
        if a.n >= 8192:  # CFIE on the full stadium at k0 = 1500, the large-N EBIM configuration
            ws.close()
            bs = qb.make_full_stadium(1.0, 1.0)
            sol = qb.CFIE_kress_global_corners(1.0, bs)
            pts, sol = qb.points_with_n(sol, bs, a.n, 1500.0)
            ws = qb.Workspace(sol, pts)
            k_ebim, reps = 1500.0, 1
        for rep in range(reps):
            t1 = time.perf_counter()
            kc, tens, info = qb.ebim.solve(ws, k_ebim, a.dk, nev=a.nev, full=a.full, return_info=True)
            print("ebim", "full" if a.full else "krylov", "N", ws.dim, "roots", np.round(kc, 6).tolist(),
                  "tens", np.round(tens, 6).tolist(), info, "ms %.1f" % ((time.perf_counter() - t1) * 1e3), flush=True)
    elif a.case == "beyn":
        lam, info = qb.solve(sol, pts, 200.0 + 0j, 0.5, nq=a.nq, r=a.L, svd_tol=1e-12, rng=np.random.default_rng(1),
                             mixed=a.form, ws=ws, return_info=True, use_chebyshev=not a.direct, cheb=cheb)
        print("beyn", a.form, "eigenvalues", len(lam), "stats", info["stats"][0])
    else:
        zj = 200.0 + 0.5 * np.exp(2j * math.pi * np.arange(a.nq) / a.nq)
        out = qb.assemble(ws, zj, mixed=a.form, cheb=None if a.direct else (cheb if cheb else True),
                          split_lo=a.form == "mixed")
        print("assembled", len(out), out[0].shape)
    print("wall ms", (time.perf_counter() - t0) * 1e3)


if __name__ == "__main__":
    main()
