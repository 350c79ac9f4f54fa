"""The C restatement of the CFIE Chebyshev route (oracle/cpu_cfie.c) against
the NumPy one (oracle/chebyshev.py) on the same panels: one smooth curve at
complex k and a circle with a hole (cross-component terms), entries to
1e-13 of the max-norm; its small-argument Hankel series against SciPy's AMOS
to 1e-14 relative; and the CPU Beyn disk against the NumPy Beyn restatement
on the same probes. Also the CPU panel tuner reaches its tolerance."""
import numpy as np
from scipy import special as sp

from oracle import beyn as OB, chebyshev as OC, cpu as OCPU, geometry as OG


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_small_argument_series():
    rng = np.random.default_rng(4)
    z = rng.uniform(0.001, 0.2, 64) * np.exp(1j * rng.uniform(-0.4, 0.4, 64))
    h0, h1 = OCPU.hankel01_small(z)
    assert np.max(np.abs(h0 - sp.hankel1(0, z)) / np.abs(sp.hankel1(0, z))) < 1e-14
    assert np.max(np.abs(h1 - sp.hankel1(1, z)) / np.abs(sp.hankel1(1, z))) < 1e-14


def test_c_assembly_equals_numpy_chebyshev_route():
    params = (1500, 7, 600, 7)
    for b, N, k in ((OG.star(0.2, 5), 240, 30.0 + 0.4j), (OG.circle_with_holes(1.0, ((0.3, 0.1, 0.2),)), 200, 20.0 - 0.3j)):
        pts, _ = OG.points_with_n("cfie_kress", b, N, 30.0)
        ref = OC.cfie_matrix(pts, k, params)
        got = OCPU.cfie_matrix(OCPU.Geometry(pts), k, params)
        assert _rel(got, ref) < 1e-13


def test_cpu_beyn_disk_and_tuner():
    b = OG.star(0.2, 5)
    pts, _ = OG.points_with_n("cfie_kress", b, 260, 30.0)
    g = OCPU.Geometry(pts)
    zj, _ = OB.contour(30.0 + 0j, 0.3, 16)
    nh, Mh, nj, Mj, e = OCPU.chebyshev_params(g, zj, tol=1e-12, npanels_h_init=300, npanels_j_init=100,
                                              sampling_points=4000)
    assert np.all(e < 1e-12)
    cb = OCPU.BeynCPU(pts, 30.0, 0.3, 16, 12, 1e-12, 5, (nh, Mh, nj, Mj), threads=4)
    for j in range(16):
        cb.node(j)
    lam, rk, r = cb.finish()
    cb.close()
    ref, *_ = OB.solve_beyn(lambda zs: [OC.cfie_matrix(pts, z, (nh, Mh, nj, Mj)) for z in zs], pts[0].n, 30.0 + 0j,
                            0.3, nq=16, r=12, svd_tol=1e-12, rng=np.random.default_rng(5))
    sel = lambda l: np.sort_complex(l[(np.abs(l - 30.0) < 0.3) & (np.abs(l.imag) < 1e-6)])
    assert len(sel(lam)) == len(sel(ref)) > 0
    assert np.max(np.abs(sel(lam) - sel(ref))) < 1e-10
