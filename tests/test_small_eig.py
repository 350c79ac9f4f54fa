"""CPU: the host eigen-decomposition behind the EBIM Rayleigh-Ritz step
(qbg_small_eig) against numpy.linalg.eig: eigenvalues to 1e-12 of |H| after
matching, eigen-residuals |H v - w v| <= 1e-12 |H| with unit v, on random,
triangular, Hermitian, diagonal (repeated values) and 1 x 1 / 2 x 2 inputs."""
import ctypes

import numpy as np


def small_eig(lib, H):
    p = H.shape[0]
    Hf = np.asfortranarray(H, dtype=np.complex128)
    w = np.zeros(p, np.complex128)
    V = np.zeros((p, p), np.complex128, order="F")
    st = lib.qbg_small_eig(p, Hf.ctypes.data, w.ctypes.data, V.ctypes.data)
    assert st == 0
    return w, V


def _check(lib, H):
    w, V = small_eig(lib, H)
    nrm = max(np.linalg.norm(H, 2), 1e-300)
    ref = np.linalg.eigvals(H)
    used = np.zeros(len(ref), bool)
    for x in w:  # greedy matching
        d = np.where(used, np.inf, np.abs(ref - x))
        i = int(np.argmin(d))
        assert d[i] <= 1e-12 * nrm * max(1, len(ref)), (x, ref[i])
        used[i] = True
    for j in range(len(w)):
        v = V[:, j]
        assert abs(np.linalg.norm(v) - 1.0) < 1e-12
        assert np.linalg.norm(H @ v - w[j] * v) <= 1e-12 * nrm * max(1, len(w))


def test_small_eig_matches_numpy(qb):
    from qbgpu import _lib
    lib = _lib.load()
    rng = np.random.default_rng(3)
    for p in (1, 2, 3, 8, 22, 64, 92):
        _check(lib, rng.standard_normal((p, p)) + 1j * rng.standard_normal((p, p)))
    p = 16
    T = np.triu(rng.standard_normal((p, p)) + 1j * rng.standard_normal((p, p)))
    _check(lib, T)
    Hm = rng.standard_normal((p, p)) + 1j * rng.standard_normal((p, p))
    _check(lib, Hm + Hm.conj().T)
    _check(lib, np.diag([2.0, 2.0, 1.0 + 1j, 1.0 + 1j, -3.0]).astype(np.complex128))
    # a graded spectrum like the shift-invert projections (|mu| from 1e4 down to 1)
    Qm, _ = np.linalg.qr(rng.standard_normal((24, 24)) + 1j * rng.standard_normal((24, 24)))
    D = np.diag(np.logspace(4, 0, 24) * np.exp(1j * rng.uniform(0, 6.28, 24)))
    _check(lib, Qm @ D @ np.linalg.inv(Qm))


def test_small_eig_edge_cases(qb):
    """Zero matrix (eigenvalues 0, unit vectors), a Jordan block (the
    repeated eigenvalue; its eigenvectors are defective, only the values are
    checked), and a NaN input, which returns an error instead of iterating on."""
    from qbgpu import _lib
    lib = _lib.load()
    w, V = small_eig(lib, np.zeros((5, 5), np.complex128))
    assert np.all(w == 0) and np.allclose(np.linalg.norm(V, axis=0), 1.0)
    J = np.diag(np.full(4, 2.0 + 1.0j)) + np.diag(np.ones(3), 1)
    w, _ = small_eig(lib, J)
    assert np.max(np.abs(w - (2.0 + 1.0j))) < 1e-3  # a defective eigenvalue moves by eps^(1/4)
    H = np.ones((4, 4), np.complex128)
    H[1, 2] = np.nan
    Hf = np.asfortranarray(H)
    w = np.zeros(4, np.complex128)
    V = np.zeros((4, 4), np.complex128, order="F")
    assert lib.qbg_small_eig(4, Hf.ctypes.data, w.ctypes.data, V.ctypes.data) != 0
    assert "converge" in _lib.last_error()
