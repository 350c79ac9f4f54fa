"""CPU: the host part of the pipelined Beyn driver (qbgpu.beyn._finish_ahead
and _finish_host_qr) against the reference's rule restated directly on the
full moments (beyn.jl:283-322): the absolute rank test on the first r probe
columns, one r -> 2r regrowth when that rank saturates, B = U_k^H A1 W_k
S_k^-1 of the block used, eig(B). Synthetic moments A0 = Q diag(s) W^H with
prescribed singular values: a leading block that does not saturate (B from r
columns), one that does (B from 2r), and a rank-0 block; eigenvalues of B agree
to 1e-10 relative (they are those of the same pencil), the rank and the
number of columns used match."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "quantumbilliards.jl_gb300"))


def _reference(A0, A1, r, svd_tol):
    """The reference's rank test and B on the full (N x 2r) moments."""
    N = A0.shape[0]
    S1 = np.linalg.svd(A0[:, :r], compute_uv=False)
    rk = int(np.count_nonzero(S1 >= svd_tol))
    cols = r
    if rk == r and 2 * r < N:
        cols = 2 * r
    if rk == 0:
        return np.zeros(0, complex), 0, r
    U, S, Wh = np.linalg.svd(A0[:, :cols], full_matrices=False)
    rk = int(np.count_nonzero(S >= svd_tol))
    if rk == 0:
        return np.zeros(0, complex), 0, cols
    B = U[:, :rk].conj().T @ (A1[:, :cols] @ Wh.conj().T[:, :rk]) / S[:rk][None, :]
    return np.linalg.eigvals(B), rk, cols


def _moments(rng, N, m, s):
    Q, _ = np.linalg.qr(rng.standard_normal((N, m)) + 1j * rng.standard_normal((N, m)))
    W, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    A0 = (Q * s) @ W.conj().T
    # A1 = A0 Z for a fixed diagonalisable Z: eigenvalues of B are those of Z on the range
    Z = np.diag(rng.uniform(1.0, 2.0, m) + 1j * rng.uniform(-0.1, 0.1, m))
    A1 = A0 @ Z
    return A0, A1


def _match(a, b):
    a, b = np.sort_complex(np.asarray(a)), np.sort_complex(np.asarray(b))
    assert len(a) == len(b)
    if len(a):
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))


@pytest.mark.parametrize("case", ["no_regrowth", "regrowth", "rank0"])
def test_finish_matches_reference_rule(case):
    from qbgpu import beyn
    rng = np.random.default_rng({"no_regrowth": 1, "regrowth": 2, "rank0": 3}[case])
    N, r, tol = 200, 12, 1e-10
    m = 2 * r
    if case == "no_regrowth":
        s = np.concatenate([np.logspace(0, -3, 7), np.full(m - 7, 1e-14)])
    elif case == "regrowth":
        s = np.concatenate([np.logspace(0, -4, 18), np.full(m - 18, 1e-14)])
    else:
        s = np.full(m, 1e-15)
    A0, A1 = _moments(rng, N, m, s)
    ref, rk_ref, cols_ref = _reference(A0, A1, r, tol)
    # the device path's reduction: R and Q^H A1 of the thin QR of A0
    R, Cm = beyn._qr_reduce_host(A0, A1)
    lam, rk, cols, _ = beyn._finish_ahead(R, Cm, r, N, tol)
    assert (rk, cols) == (rk_ref, cols_ref)
    _match(lam, ref)
    lam2, rk2, cols2, _ = beyn._finish_host_qr(A0, A1, r, N, tol)
    assert (rk2, cols2) == (rk_ref, cols_ref)
    _match(lam2, ref)
