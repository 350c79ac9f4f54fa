"""Host eigenvalues of many B matrices (qbgpu.beyn._eigvals_many, the last
step of solve_disks; beyn.jl:371): LAPACK's zgeev on host threads through
LAPACKE when NumPy's bundled OpenBLAS exports it, NumPy's eigvals otherwise.
Against NumPy on the same matrices: every eigenvalue within 1e-12 of the
largest modulus, disks without a B (rank 0) give none, the BLAS thread
count is restored, and LAPACKE's zgesdd reproduces NumPy's thin SVD."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "quantumbilliards.jl_gb300"))


def test_eigvals_many_matches_numpy():
    from qbgpu import beyn
    rng = np.random.default_rng(3)
    Bs = [rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) for n in (1, 7, 64, 150)] + [None]
    z = beyn._lapacke()
    before = int(z["get_threads"]()) if z else None
    got = beyn._eigvals_many(Bs)
    assert len(got) == len(Bs) and len(got[-1]) == 0
    for B, w in zip(Bs[:-1], got[:-1]):
        ref = np.linalg.eigvals(B)
        assert len(w) == len(ref)
        d = max(np.min(np.abs(ref - x)) for x in w)
        assert d <= 1e-12 * np.max(np.abs(ref)), d
    if z:
        assert int(z["get_threads"]()) == before
        A = Bs[3]
        U, S, Vh = beyn._svd_lapacke(z, A)
        assert np.max(np.abs(S - np.linalg.svd(A, compute_uv=False))) <= 1e-12 * S[0]
        assert np.max(np.abs((U * S) @ Vh - A)) <= 1e-12 * S[0]


def test_one_thread_helpers_match_numpy():
    """The single-disk path's SVD values, thin SVD and eigvals (BLAS at one
    thread around each call) against NumPy; the thread count is restored."""
    from qbgpu import beyn
    rng = np.random.default_rng(5)
    A = rng.standard_normal((96, 64)) + 1j * rng.standard_normal((96, 64))
    B = rng.standard_normal((100, 100)) + 1j * rng.standard_normal((100, 100))
    z = beyn._lapacke()
    before = int(z["get_threads"]()) if z else None
    S0 = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(beyn._svdvals(A) - S0)) <= 1e-12 * S0[0]
    U, S, Vh = beyn._svd(A)
    assert np.max(np.abs(S - S0)) <= 1e-12 * S0[0]
    assert np.max(np.abs((U * S) @ Vh - A)) <= 1e-12 * S0[0]
    w, ref = beyn._eigvals(B), np.linalg.eigvals(B)
    assert max(np.min(np.abs(ref - x)) for x in w) <= 1e-12 * np.max(np.abs(ref))
    if z:
        assert int(z["get_threads"]()) == before


def test_host_qr_reduction():
    """The pipelined driver's host QR of the moments (LAPACK zgeqrf / zunmqr):
    R upper triangular with R^H R = A0^H A0 and R^H C = A0^H A1 (1e-12 of
    |A0|^2, |A0||A1|), for tall and for wide moment blocks; the BLAS thread
    count is restored."""
    from qbgpu import beyn
    rng = np.random.default_rng(8)
    z = beyn._lapacke()
    before = int(z["get_threads"]()) if z else None
    for n, m in ((300, 64), (40, 64)):
        A0 = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
        A1 = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
        R, Cm = beyn._qr_reduce_host(A0, A1)
        assert R.shape == (min(n, m), m) and Cm.shape == (min(n, m), m)
        assert np.array_equal(R, np.triu(R))
        s0, s01 = np.linalg.norm(A0) ** 2, np.linalg.norm(A0) * np.linalg.norm(A1)
        assert np.max(np.abs(R.conj().T @ R - A0.conj().T @ A0)) < 1e-12 * s0
        assert np.max(np.abs(R.conj().T @ Cm - A0.conj().T @ A1)) < 1e-12 * s01
    if z:
        assert int(z["get_threads"]()) == before
