"""GPU: the refinement residual R = V - (hi + lo) X on the tensor cores
(exact 7-bit digit products) against an extended-precision NumPy residual
and against the compensated FP32 kernel.

Elementwise bound |R - R_exact| <= tol (|T| |X|)_il + 2^-52 |R_exact|_il: the
product error against |T| |X| plus the final double rounding of V - T X
(which dominates in rows of T far smaller than V). tol = 6e-14 for the
tensor-core kernel (T and X cut to 49 bits against their row and column
maxima, exact digit products; an exact CPU emulation of the same digits gives
1.6e-14 at n = 200, the value measured), 1e-11 for its six-digit form (the
refinement's first residual: 42 bits of T and X, ~2^-7 of the seven-digit
accuracy) and 1e-12 for the compensated FP32 kernel (double-float sums, error
growing with n). Cases: ragged sizes, rows
spanning 16 orders of magnitude, a zero column of X, two 512-term chunks, two
calls in a row; the Beyn moments of the mixed form agree between the two
residual engines to 1e-10.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(rng, b, n, L, row_scale=False, zero_col=False):
    T = (rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n)))
    if row_scale:
        T *= (10.0 ** rng.uniform(-8, 8, (b, n, 1)))
    Th = T.astype(np.complex64)
    Tl = (T - Th.astype(np.complex128)).astype(np.complex64)
    X = rng.standard_normal((b, n, L)) + 1j * rng.standard_normal((b, n, L))
    if zero_col:
        X[:, :, 1] = 0
    V = rng.standard_normal((b, n, L)) + 1j * rng.standard_normal((b, n, L))
    return Th, Tl, X, V


def _exact(Th, Tl, X, V):
    ld = np.clongdouble
    T = Th.astype(ld) + Tl.astype(ld)
    return (V.astype(ld) - T @ X.astype(ld)), np.abs(Th.astype(np.complex128)) @ np.abs(X)


@pytest.mark.parametrize("n,L,b,row_scale,zero_col", [(200, 40, 2, False, False), (257, 64, 1, True, True),
                                                       (512, 96, 1, False, False), (150, 20, 2, False, False)])
def test_residual_engines_vs_exact(qb, n, L, b, row_scale, zero_col):
    rng = np.random.default_rng(n + L)
    Th, Tl, X, V = _case(rng, b, n, L, row_scale, zero_col)
    ref, bound = _exact(Th, Tl, X, V)
    for engine, tol in ((0, 6e-14), (1, 1e-12), (2, 1e-11)):
        for _ in range(2):
            R, rmax = qb.residual_c64(Th, Tl, X, V, engine=engine)
            err = np.abs(R.astype(np.clongdouble) - ref).astype(np.float64)
            allowed = tol * bound + 2.0 ** -52 * np.abs(ref).astype(np.float64)
            ratio = np.max(err / allowed)
            print(f"n={n} L={L} engine={engine} max err/allowed {ratio:.3e}")
            assert ratio <= 1.0, (engine, ratio)
            assert abs(rmax - np.max(np.abs(R.real) + np.abs(R.imag))) <= 1e-15 * rmax


@pytest.mark.parametrize("mixed", [True, "fp32"])
def test_beyn_moments_both_residual_engines(qb, mixed):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 400, 25.0)
    ws = qb.Workspace(sol, pts)
    V = qb.probe_matrix(ws.dim, 24, np.random.default_rng(9))
    out = []
    for eng in (0, 1):
        bh = qb.BeynHandle(ws, 25.0, 0.4, 16, mixed=mixed, resid_engine=eng)
        out.append(bh.moments(V))
        bh.close()
    for a, r in zip(out[0], out[1]):
        assert np.max(np.abs(a - r)) / np.max(np.abs(r)) < 1e-10


@pytest.mark.parametrize("engine", [0, 1])
def test_residual_nonfinite_rows_and_columns(qb, engine):
    """Inf or NaN in a row of T or a column of X gives a non-finite residual
    there and a non-finite rmax; every other entry keeps its accuracy."""
    rng = np.random.default_rng(17)
    n, L = 160, 24
    Th, Tl, X, V = _case(rng, 1, n, L)
    Th[0, 7, 30] = np.nan
    X[0, 11, 5] = np.inf
    R, rmax = qb.residual_c64(Th, Tl, X, V, engine=engine)
    assert not np.isfinite(rmax)
    assert not np.all(np.isfinite(R[0, 7, :]))
    assert not np.all(np.isfinite(R[0, :, 5]))
    keep_r = np.ones(n, bool); keep_r[7] = False
    keep_c = np.ones(L, bool); keep_c[5] = False
    Th2, Tl2, X2 = Th.copy(), Tl.copy(), X.copy()
    Th2[0, 7, 30] = 0
    X2[0, 11, 5] = 0
    ref, bound = _exact(Th2, Tl2, X2, V)
    sub = np.ix_(keep_r, keep_c)
    err = np.abs(R[0][sub].astype(np.clongdouble) - ref[0][sub]).astype(np.float64)
    allowed = 1e-12 * bound[0][sub] + 2.0 ** -52 * np.abs(ref[0][sub]).astype(np.float64)
    assert np.all(np.isfinite(R[0][sub]))
    assert np.max(err / allowed) <= 1.0
