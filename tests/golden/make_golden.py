"""Regenerate the golden vectors in this folder (run from the repo root).

bessel_mpmath.json: J0, J1, Y0, Y1 at complex z computed by mpmath with 40
significant digits, covering the ranges the assembly kernels meet
(|z| from 1e-4 to 6e3, |Im z| <= 3). These pin both the oracle (SciPy/AMOS)
and the device special functions.

circle_eigs.json: Dirichlet eigenvalues of the unit circle (zeros of J_m)
in [40, 42] and [14.6, 15.4], the known answers of the sigma_min sweep and the
Beyn disk on the circle.

c1_sweep.json (``python tests/golden/make_golden.py c1``, about 80 s): the
oracle's sigma_min sweep of the unit circle, DLP Kress with
pts_scaling_factor 12.2 (N = 512 at k = 42), 200 k in [40, 42] -- the smallest
singular value of the FP64 Fredholm matrix at each k.

c2_beyn.json (``... c2``, a few minutes on 8 cores): the oracle's Beyn disk
of the star r = 1 + 0.2 cos 5 theta, CFIE Kress, N = 2048 (b chosen at
k = 200), k0 = 200, R = 0.5, 48 nodes, 64 probes drawn from PCG64 seed 2 and
extended by a second draw of 64 when the rank saturates, svd_tol 1e-12; direct
AMOS kernel values. All eigenvalues of B, the rank and the singular values.

c2_beyn_fresh.json (``... c2fresh``): the same disk with the reference's own
regrowth, a fresh N x 2r block drawn after the first r columns (beyn.jl:291-309);
it checks the host-core restatement of the reference's path (oracle/cpu.py).
The rank saturates at 2r on this disk, so eigenvalues near the contour depend
on the probe block at the 1e-9 level: each fixture matches one probe policy.

c3_beyn.json (``... c3``): one disk of the desymmetrised stadium, DLP Kress
global corners on the full stadium (half width 1, radius 1) with the XY
reflection of parities (-1, -1), N = 4096 (b chosen at k = 332), m = 1024
reduced unknowns, k0 = 300.5, R = 0.5, 48 nodes, 96 probes from PCG64 seed 3
(extended by 96 when the rank saturates), svd_tol 1e-10; direct AMOS values.

Everything here is computed by the oracle alone (oracle/geometry.py builds the
nodes); nothing imports the product.
"""
import json
import sys
from pathlib import Path

import mpmath as mp
import numpy as np
from scipy import special as sp

mp.mp.dps = 40
HERE = Path(__file__).resolve().parent


def bessel_rows():
    rng = np.random.default_rng(20261203)
    zs = [complex(x, 0.0) for x in (1e-4, 1e-3, 0.199, 0.2, 1.0, 5.0, 11.9, 12.0, 15.99, 16.0, 16.01, 20.0, 40.0,
                                     200.0, 1000.0, 6000.0)]
    for _ in range(64):
        az = 10 ** rng.uniform(-4, np.log10(6000))
        y = rng.uniform(-1, 1) * min(3.0, 0.5 * az)
        x = np.sqrt(max(az * az - y * y, 1e-12))
        zs.append(complex(x, y))
    rows = []
    for z in zs:
        zz = mp.mpc(z.real, z.imag)
        vals = [mp.besselj(0, zz), mp.besselj(1, zz), mp.bessely(0, zz), mp.bessely(1, zz)]
        rows.append({"z": [z.real, z.imag], "j0j1y0y1": [[float(v.real), float(v.imag)] for v in vals]})
    return rows


def circle_eigs(lo, hi):
    out = []
    for m in range(0, 80):
        for x in sp.jn_zeros(m, 40):
            if lo <= x <= hi:
                out.append({"m": m, "k": float(mp.besseljzero(m, int(np.argmin(abs(sp.jn_zeros(m, 40) - x))) + 1))})
    return sorted(out, key=lambda r: r["k"])


def _oracle_path():
    root = HERE.parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))


def c1_sweep():
    _oracle_path()
    from oracle import assembly as OA, beyn as OB, geometry as OG
    ks = np.linspace(40.0, 42.0, 200)
    pts = OG.evaluate_points("dlp_kress", OG.circle(1.0), float(ks.max()), 12.2)
    sig = [float(OB.sigma_min(OA.dlp_fredholm(pts, k))) for k in ks]
    return {"N": int(pts.n), "pts_scaling_factor": 12.2, "ks": ks.tolist(), "sigma": sig}


def _disk_record(res, cfg):
    lam = res["lam"]
    return dict(cfg, rk=int(res["rk"]), r_used=int(res["r"]), eigenvalues=[[float(x.real), float(x.imag)] for x in lam],
                singular_values=[float(x) for x in res["S"]])


def c2_beyn(workers=8, regrow="extend"):
    _oracle_path()
    import os
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import beyn as OB, geometry as OG
    pts, b = OG.points_with_n("cfie_kress", OG.star(0.2, 5), 2048, 200.0)
    cfg = dict(workload="beyn_cfie_kress_star_N2048_k0_200_R0.5_nq48_L64", N=int(pts[0].n), pts_scaling_factor=b,
               k0=200.0, R=0.5, nq=48, L=64, seed=2, regrow=regrow, svd_tol=1e-12, kernel="direct AMOS")
    res = OB.beyn_disk(("cfie", pts), pts[0].n, 200.0 + 0j, 0.5, 48, 64, 1e-12, 2, regrow, workers)
    return _disk_record(res, cfg)


def c3_beyn(workers=8):
    _oracle_path()
    import os
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import assembly as OA, beyn as OB, geometry as OG
    sym = ("xy", -1, -1)
    p, b = OG.points_with_n("dlp_kress_global_corners", OG.full_stadium(1.0, 1.0), 4096, 332.0, symmetry=sym)
    orb = OA.periodic_symmetry_index_orbits(p.n, sym)
    m = len(orb[0])
    cfg = dict(workload="beyn_dlp_reduced_stadium_N4096_m1024_k0_300.5_R0.5_nq48_L96", N=int(p.n), m=m,
               pts_scaling_factor=b, k0=300.5, R=0.5, nq=48, L=96, seed=3, regrow="extend", svd_tol=1e-10,
               symmetry="XYReflection(-1, -1)", kernel="direct AMOS")
    res = OB.beyn_disk(("dlp_reduced", p, orb), m, 300.5 + 0j, 0.5, 48, 96, 1e-10, 3, "extend", workers)
    return _disk_record(res, cfg)


if __name__ == "__main__" and sys.argv[1:2] in (["c1"], ["c2"], ["c2fresh"], ["c3"]):
    which = sys.argv[1]
    fn = {"c1": c1_sweep, "c2": c2_beyn, "c2fresh": lambda: c2_beyn(regrow="fresh"), "c3": c3_beyn}[which]
    out = {"c1": "c1_sweep.json", "c2": "c2_beyn.json", "c2fresh": "c2_beyn_fresh.json", "c3": "c3_beyn.json"}[which]
    (HERE / out).write_text(json.dumps(fn()))
    print("written", out)
elif __name__ == "__main__":
    (HERE / "bessel_mpmath.json").write_text(json.dumps({"dps": 40, "values": bessel_rows()}, indent=1))
    (HERE / "circle_eigs.json").write_text(json.dumps({"ranges": {"40_42": circle_eigs(40.0, 42.0),
                                                                  "14.6_15.4": circle_eigs(14.6, 15.4)}},
                                                      indent=1))
    print("written")
