"""GPU: the Beyn spectrum driver (compute_spectrum_beyn, beyn.jl:778-921) and
its residual filters.

* candidate residuals: ||T(lambda) phi||_2, ||T phi||_1, opnorm(T, 1) and the
  phi norms equal NumPy's on the oracle operator (1e-12 relative);
* on the unit disk (DLP Kress) the driver returns exactly the Dirichlet
  eigenvalues j_{m,n} in [k1, k2] (zeros of J_m, m > 0 twice) to 1e-9, with
  both filters and with and without the batched disks.
"""
import numpy as np
import pytest
from scipy import special as sp

from oracle import assembly as OA

pytestmark = pytest.mark.gpu


def _bessel_zeros(k1, k2):
    out = []
    for m in range(0, 60):
        z = sp.jn_zeros(m, 40)
        z = z[(z >= k1) & (z <= k2)]
        out += list(z) * (1 if m == 0 else 2)
    return np.sort(np.array(out))


def test_candidate_residuals_vs_numpy(qb):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 300, 20.0)
    ws = qb.Workspace(sol, pts)
    rng = np.random.default_rng(0)
    lam = np.array([20.1 - 0.01j, 19.7 + 0.002j, 20.3 + 0j])
    Phi = rng.standard_normal((ws.dim, 3)) + 1j * rng.standard_normal((ws.dim, 3))
    got = qb.candidate_residuals(ws, lam, Phi, cheb=None)
    for j, z in enumerate(lam):
        T = OA.cfie_matrix(qb.solvers.as_list(pts), z)
        y = T @ Phi[:, j]
        ref = [np.linalg.norm(y), np.linalg.norm(y, 1), np.linalg.norm(T, 1), np.linalg.norm(Phi[:, j], 1),
               np.linalg.norm(Phi[:, j])]
        assert np.allclose(got[j], ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("batched,imag_check", [(True, True), (False, False)])
def test_compute_spectrum_beyn_unit_disk(qb, batched, imag_check):
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(10.0, b)
    k1, k2 = 10.0, 11.5
    ks, tens, us, pts, tensN = qb.compute_spectrum_beyn(sol, b, k1, k2, m=8, Rmax=0.5, nq=32, svd_tol=1e-10,
                                                        res_tol=1e-8, mixed=True, batched=batched,
                                                        use_imag_check=imag_check, sampling_points=20000,
                                                        rng=np.random.default_rng(1))
    ks = np.sort(np.array(ks))
    ref = _bessel_zeros(k1, k2)
    assert len(ks) == len(ref)
    assert np.max(np.abs(ks - ref) / ref) < 1e-9
    assert len(us) == len(ks) and all(u.shape[0] == p.n for u, p in zip(us, pts))
