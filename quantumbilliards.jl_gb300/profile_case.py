"""Run one named workload once, for profilers (ncu) and quick checks.

    python quantumbilliards.jl_gb300/profile_case.py beyn --nq 8 --form mixed
    python quantumbilliards.jl_gb300/profile_case.py assemble --nq 8

Cases use the bench workload (CFIE Kress, star r = 1 + 0.2 cos 5 theta,
N = 2048, k0 = 200, R = 0.5, L = 64) with an adjustable number of contour nodes
so that a capture stays small (a few GB on the device at most).
"""
from __future__ import annotations

import argparse
import math
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import numpy as np  # noqa: E402


def star_case(qb, n_nodes=2048, k0=200.0, kind="cfie"):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b) if kind == "cfie" else qb.DLP_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, n_nodes, k0)
    return b, sol, pts


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["beyn", "assemble"])
    ap.add_argument("--nq", type=int, default=8)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--form", default="mixed", choices=["fp64", "mixed", "fp32"])
    ap.add_argument("--direct", action="store_true", help="direct Hankel evaluation instead of Chebyshev panels")
    a = ap.parse_args(argv)
    import build_qbgpu
    build_qbgpu.build()
    import qbgpu as qb
    b, sol, pts = star_case(qb, a.n)
    ws = qb.Workspace(sol, pts)
    t0 = time.perf_counter()
    if a.case == "beyn":
        lam, info = qb.solve(sol, pts, 200.0 + 0j, 0.5, nq=a.nq, r=a.L, svd_tol=1e-12, rng=np.random.default_rng(1),
                             mixed=a.form, ws=ws, return_info=True, use_chebyshev=not a.direct)
        print("beyn", a.form, "eigenvalues", len(lam), "stats", info["stats"][0])
    else:
        zj = 200.0 + 0.5 * np.exp(2j * math.pi * np.arange(a.nq) / a.nq)
        out = qb.assemble(ws, zj, mixed=a.form, cheb=None if a.direct else True)
        print("assembled", len(out), out[0].shape)
    print("wall ms", (time.perf_counter() - t0) * 1e3)


if __name__ == "__main__":
    main()
