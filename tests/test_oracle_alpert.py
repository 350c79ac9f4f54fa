"""Alpert quadrature checks on the CPU.

* the rule table (Alpert 1999, log-singular end correction) is pinned by what
  the rules are for: the corrected trapezoid rule on the periodic grid
  integrates log(4 sin^2(s/2)) cos(m s) (exact value -2 pi/m) and smooth
  periodic functions to the order of the rule;
* the oracle's Alpert CFIE discretises the same operator as the Kress CFIE:
  the Beyn eigenvalues of both agree on a star.
"""
import math

import numpy as np
import pytest

from oracle import alpert as OAL, assembly as OA, beyn as OB

TWO_PI = 2 * math.pi


def _corrected_sum(f, N, rule):
    a, x, w = rule
    h = TWO_PI / N
    j = np.arange(-N // 2 + 1, N // 2 + 1)
    j = j[np.abs(j) >= a]
    s = h * np.sum(f(j * h))
    x, w = np.asarray(x), np.asarray(w)
    return s + h * np.sum(w * (f(x * h) + f(-x * h)))


@pytest.mark.parametrize("order", [4, 6, 8, 10, 12, 16])
def test_rule_integrates_log_singularity(qb, order):
    from qbgpu.alpert import ALPERT_LOG_RULES
    rule = ALPERT_LOG_RULES[order]
    m = 3
    f = lambda s: np.log(4 * np.sin(s / 2) ** 2) * np.cos(m * s) + np.cos(2 * s) + 1.0
    exact = -TWO_PI / m + TWO_PI
    errs = [abs(_corrected_sum(f, N, rule) - exact) for N in (64, 128, 256)]
    # convergence at about the rule's order until rounding
    assert errs[-1] < max(1e-13, 10.0 * errs[0] * 4.0 ** (-order))
    assert errs[-1] < 1e-6 if order < 6 else errs[-1] < 1e-11


def test_alpert_and_kress_cfie_share_eigenvalues(qb):
    b = qb.make_star(0.2, 5)
    crv = b.components[0][0]
    sol_k = qb.CFIE_kress(1.0, b)
    pk, sol_k = qb.points_with_n(sol_k, b, 200, 12.0)
    sol_a = qb.CFIE_alpert(1.0, b, alpert_order=12)
    pa, sol_a = qb.points_with_n(sol_a, b, 200, 12.0)
    from qbgpu.alpert import ALPERT_LOG_RULES
    rule = ALPERT_LOG_RULES[12]
    k0, R, nq, r = 12.0 + 0j, 0.4, 24, 16
    sel = lambda l: np.sort_complex(l[(np.abs(l - k0) < R) & (np.abs(l.imag) < 1e-4)])
    lk, *_ = OB.solve_beyn(lambda zj: [OA.cfie_matrix(pk, z) for z in zj], pk[0].n, k0, R, nq=nq, r=r,
                           svd_tol=1e-12, rng=np.random.default_rng(1))
    la, *_ = OB.solve_beyn(lambda zj: [OAL.cfie_alpert_matrix([crv], pa, z, rule, 12) for z in zj], pa[0].n, k0,
                           R, nq=nq, r=r, svd_tol=1e-12, rng=np.random.default_rng(1))
    lk, la = sel(lk), sel(la)
    assert len(lk) == len(la) > 0
    assert np.max(np.abs(lk - la) / np.abs(lk)) < 1e-7
