"""GPU: the library's FP64 dense path through qbg_dense_inverse -- batched LU
(own panel and GEMM kernels), explicit inverses, and sigma_min by the device
subspace iteration on the inverse (the :svd branch, macros.jl:159-161).

* matrices with a prescribed spectrum A = U diag(s) V^H (U, V Haar-random
  unitary, n = 100 and 257, so no tile divides n), including a doubly
  degenerate smallest singular value: |A X - I| <= 1e-12 * cond(A) and
  sigma_min to 1e-15 * sigma_max absolute (the backward-stable bound);
* the C1 circle matrices (DLP Kress, N = 512 at k = 42) at the first eight k
  of the golden sweep, whose smallest singular values come in exact pairs
  (the rotational symmetry): sigma_min against the oracle's LAPACK values
  (tests/golden/c1_sweep.json) to 2e-12 relative;
* one complex128 matrix of n = 1700 (a 16-CTA cluster panel where the device
  holds one, split-K FP64 updates): A X - I <= 1e-12 cond;
* the complex64 LU of the Beyn mixed form (panels, interchanges, tcgen05
  trailing updates) through both panel forms (one CTA per panel and the
  8-CTA cluster) and two outer-block depths, n = 700 and 2050, batch 3:
  |A X - I| <= 2e-5 for matrices of condition ~3 (numpy's complex64 inverse
  reaches ~1e-6), and the two panel forms agree to 1e-5.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


def _haar(n, rng):
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _run(lib, L, As):
    batch, n = len(As), As[0].shape[0]
    Ac = np.ascontiguousarray(np.stack(As).transpose(0, 2, 1))  # column-major per matrix
    X = np.empty_like(Ac)
    sig = np.zeros(batch)
    L.check(lib.qbg_dense_inverse(n, batch, 0, L.vptr(Ac), L.vptr(X), L.dptr(sig), None))
    return [x.T for x in X], sig


def _inv32(lib, L, As):
    batch, n = len(As), As[0].shape[0]
    Ac = np.ascontiguousarray(np.stack(As).transpose(0, 2, 1))
    X = np.empty_like(Ac)
    L.check(lib.qbg_dense_inverse(n, batch, 2, L.vptr(Ac), L.vptr(X), None, None))
    return [x.T for x in X]


@pytest.mark.parametrize("n", [100, 257])
def test_prescribed_spectrum(qb, n):
    from qbgpu import _lib as L
    lib = L.load()
    rng = np.random.default_rng(20 + n)
    As, smin, conds = [], [], []
    for case in range(3):
        s = np.sort(rng.uniform(0.5, 3.0, n))[::-1]
        s[-1] = 10.0 ** -(2 + case)
        if case != 1:
            s[-2] = s[-1]  # a degenerate smallest pair
        As.append((_haar(n, rng) * s) @ _haar(n, rng).conj().T)
        smin.append(s[-1])
        conds.append(s[0] / s[-1])
    Xs, sig = _run(lib, L, As)
    for A, X, c in zip(As, Xs, conds):
        assert np.abs(A @ X - np.eye(n)).max() <= 1e-12 * c
    # a backward-stable sigma_min is exact to a few eps * sigma_max in absolute terms
    assert np.all(np.abs(sig - np.array(smin)) <= 1e-15 * 3.0), (sig - np.array(smin))


def test_c1_degenerate_pairs(qb):
    from qbgpu import _lib as L
    lib = L.load()
    g = json.loads((GOLD / "c1_sweep.json").read_text())
    ks, so = np.array(g["ks"][:8]), np.array(g["sigma"][:8])
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(g["pts_scaling_factor"], b)
    pts = qb.evaluate_points(sol, b, 42.0)
    ws = qb.Workspace(sol, pts)
    As = qb.assemble(ws, ks)
    _, sig = _run(lib, L, As)
    assert np.all(np.abs(sig - so) <= 2e-12 * so), np.abs(sig - so) / so


@pytest.mark.parametrize("n", [700, 2050])
def test_complex64_lu_panel_forms(qb, n):
    from qbgpu import _lib as L
    import ctypes as C
    lib = L.load()
    rng = np.random.default_rng(n)
    As = [(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2 * n) + 3.0 * np.eye(n)
          for _ in range(3)]
    o0, c0, p0 = C.c_int32(), C.c_int32(), C.c_int32()
    L.check(lib.qbg_get_lu_plan(C.byref(o0), C.byref(c0), C.byref(p0)))
    out = {}
    try:
        for outer, cluster in ((4, 0), (4, 1), (2, 1)):
            L.check(lib.qbg_set_lu_plan(outer, cluster, 0))
            Xs = _inv32(lib, L, As)
            for A, X in zip(As, Xs):
                assert np.abs(A @ X - np.eye(n)).max() < 2e-5, (outer, cluster)
            out[(outer, cluster)] = Xs
    finally:
        L.check(lib.qbg_set_lu_plan(o0.value, c0.value, p0.value))
    for key in ((4, 1), (2, 1)):
        for X0, X1 in zip(out[(4, 0)], out[key]):
            assert np.abs(X1 - X0).max() < 1e-5 * np.abs(X0).max()


@pytest.mark.parametrize("n", [1700])
def test_fp64_lu_single_large(qb, n):
    """One complex128 matrix taller than an 8-CTA cluster panel holds (n >
    1600): the panel runs on a 16-CTA cluster where the device allows one (one
    CTA otherwise), the small-grid updates split over K; A X - I <= 1e-12 cond."""
    from qbgpu import _lib as L
    lib = L.load()
    rng = np.random.default_rng(n)
    s = np.sort(rng.uniform(0.5, 3.0, n))[::-1]
    s[-1] = 1e-3
    A = (_haar(n, rng) * s) @ _haar(n, rng).conj().T
    Ac = np.ascontiguousarray(A.T)[None]
    X = np.empty_like(Ac)
    L.check(lib.qbg_dense_inverse(n, 1, 0, L.vptr(Ac), L.vptr(X), None, None))
    assert np.abs(A @ X[0].T - np.eye(n)).max() <= 1e-12 * s[0] / s[-1]
