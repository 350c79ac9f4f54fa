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


def c1_sweep():
    root = HERE.parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "quantumbilliards.jl_gb300"))
    from oracle import assembly as OA, beyn as OB
    from qbgpu import geometry as G, solvers as S
    b = G.make_circle(1.0)
    sol = S.DLP_kress(12.2, b)
    ks = np.linspace(40.0, 42.0, 200)
    pts = S.evaluate_points(sol, b, float(ks.max()))
    sig = [float(OB.sigma_min(OA.dlp_fredholm(pts, k))) for k in ks]
    return {"N": int(pts.n), "pts_scaling_factor": 12.2, "ks": ks.tolist(), "sigma": sig}


if __name__ == "__main__" and sys.argv[1:] == ["c1"]:
    (HERE / "c1_sweep.json").write_text(json.dumps(c1_sweep()))
    print("written")
elif __name__ == "__main__":
    (HERE / "bessel_mpmath.json").write_text(json.dumps({"dps": 40, "values": bessel_rows()}, indent=1))
    (HERE / "circle_eigs.json").write_text(json.dumps({"ranges": {"40_42": circle_eigs(40.0, 42.0),
                                                                  "14.6_15.4": circle_eigs(14.6, 15.4)}},
                                                      indent=1))
    print("written")
