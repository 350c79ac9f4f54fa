"""GPU parity at the configurations the benchmarks time, against eigenvalues
the oracle computed alone (tests/golden/make_golden.py: oracle geometry,
direct AMOS kernel values, LAPACK, the same seeded probes and regrowth).

* C2: star r = 1 + 0.2 cos 5 theta, CFIE Kress, N = 2048, k0 = 200, R = 0.5,
  48 nodes, L = 64 (rank saturates, r -> 2r): the plain FP64 form, through
  Chebyshev panels tuned to 1e-13 and through direct Hankel values, matches
  every eigenvalue inside the disk to 1e-12 relative; the mixed form to 1e-11
  (the target is 1e-10; measured 2e-13).
* C3 sample: one disk of the desymmetrised stadium (XY reflection (-1, -1),
  N = 4096, m = 1024, k0 = 300.5, L = 96): plain direct FP64 to 1e-12, mixed
  through panels to 1e-11, and the same disk as the first of a 32-disk batch.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"
IMAG = 1e-6


def _fixture(name):
    g = json.loads((GOLD / name).read_text())
    return g, np.array([complex(*x) for x in g["eigenvalues"]])


def _sel(lam, k0, R):
    lam = np.asarray(lam)
    return np.sort_complex(lam[(np.abs(lam - k0) <= R) & (np.abs(lam.imag) < IMAG)])


def _check(lam, ref_all, k0, R, tol):
    got, ref = _sel(lam, k0, R), _sel(ref_all, k0, R)
    assert len(got) == len(ref) > 0
    err = np.array([np.min(np.abs(ref_all - x)) / abs(x) for x in got])
    back = np.array([np.min(np.abs(got - x)) / abs(x) for x in ref])
    assert err.max() <= tol, (err.max(), int(np.sum(err > tol)))
    assert back.max() <= tol
    return err.max()


@pytest.fixture(scope="module")
def c2(qb):
    g, ref = _fixture("c2_beyn.json")
    b = qb.make_star(0.2, 5)
    pts, sol = qb.points_with_n(qb.CFIE_kress(1.0, b), b, g["N"], g["k0"])
    ws = qb.Workspace(sol, pts)
    zref = g["k0"] + g["R"] * np.exp(2j * math.pi * np.arange(g["nq"]) / g["nq"])
    cheb = qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=1e-13)[:4]
    yield g, ref, sol, pts, ws, cheb
    ws.close()


def _solve_c2(qb, c2, **kw):
    g, ref, sol, pts, ws, cheb = c2
    return qb.solve(sol, pts, g["k0"] + 0j, g["R"], nq=g["nq"], r=g["L"], svd_tol=g["svd_tol"],
                    rng=np.random.default_rng(g["seed"]), ws=ws, **kw)


def test_c2_plain_fp64_vs_oracle(qb, c2):
    g, ref = c2[0], c2[1]
    _check(_solve_c2(qb, c2, mixed=False, cheb=c2[5]), ref, g["k0"], g["R"], 1e-12)
    _check(_solve_c2(qb, c2, mixed=False, use_chebyshev=False), ref, g["k0"], g["R"], 1e-12)


def test_c2_mixed_vs_oracle(qb, c2):
    g, ref = c2[0], c2[1]
    _check(_solve_c2(qb, c2, mixed=True, cheb=c2[5]), ref, g["k0"], g["R"], 1e-11)


def test_c3_disk_vs_oracle(qb):
    g, ref = _fixture("c3_beyn.json")
    bs = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, bs, symmetry=qb.XYReflection(-1, -1))
    pts, sol = qb.points_with_n(sol, bs, g["N"], 332.0)
    ws = qb.Workspace(sol, pts)
    assert ws.dim == g["m"]
    k0, R = g["k0"], g["R"]
    kw = dict(nq=g["nq"], r=g["L"], svd_tol=g["svd_tol"], ws=ws)
    lam = qb.solve(sol, pts, k0 + 0j, R, mixed=False, use_chebyshev=False, rng=np.random.default_rng(g["seed"]), **kw)
    _check(lam, ref, k0, R, 1e-12)
    zref = 331.5 + R * np.exp(2j * math.pi * np.arange(g["nq"]) / g["nq"])
    cheb = qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=1e-12, terms_per_entry=4.0)[:4]
    lam = qb.solve(sol, pts, k0 + 0j, R, mixed=True, cheb=cheb, rng=np.random.default_rng(g["seed"]), **kw)
    _check(lam, ref, k0, R, 1e-11)
    lams = qb.solve_disks(sol, pts, k0 + np.arange(4), R, nq=g["nq"], r=g["L"], svd_tol=g["svd_tol"],
                          rng=np.random.default_rng(g["seed"]), mixed=True, ws=ws, cheb=cheb)
    _check(lams[0], ref, k0, R, 1e-11)
    ws.close()
