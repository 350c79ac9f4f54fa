"""FP64 restatement of the Beyn contour step and the sigma_min sweep (test only).

* contour nodes/weights, LU of every T(z_j), X = T^-1 V, A0/A1 moments,
  thin SVD rank test with absolute svd_tol, single r -> 2r regrowth, and
  B = U_k^H A1 W_k Sigma_k^-1                          beyn.jl:257-322
* lambda = eig(B)                                      beyn.jl:364-375
* sigma_min = last singular value of A                  macros.jl:159-161
* minima from the 2nd difference of log10(sigma)       sweepmethods.jl:193-217
* beyn_disk: the same step with the contour nodes spread over worker
  processes (each assembles, factors and solves its nodes; the moments are
  summed in node order in the parent)
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla


def contour(k0: complex, R: float, nq: int):
    th = np.linspace(0.0, 2 * math.pi, nq + 1)[:-1]
    e = np.exp(1j * th)
    return k0 + R * e, (R / nq) * e


def probe_matrix(N: int, r: int, rng: np.random.Generator) -> np.ndarray:
    """Complex Gaussian with Re, Im ~ N(0, 1/2) (E|v|^2 = 1), the convention of
    Julia's randn(ComplexF64); the stream itself differs from MersenneTwister."""
    s = math.sqrt(0.5)
    return (rng.standard_normal((N, r)) * s + 1j * (rng.standard_normal((N, r)) * s)).astype(np.complex128)


def moments(Ts, zj, wj, V):
    A0 = np.zeros(V.shape, dtype=np.complex128)
    A1 = np.zeros(V.shape, dtype=np.complex128)
    facs = [sla.lu_factor(T, check_finite=False) for T in Ts]
    for f, z, w in zip(facs, zj, wj):
        X = sla.lu_solve(f, V, check_finite=False)
        A0 += w * X
        A1 += (w * z) * X
    return A0, A1, facs


def construct_B_matrix(assemble_at, N, k0, R, nq=64, r=48, svd_tol=1e-14, rng=None, moments_fn=None):
    """assemble_at(zj) -> list of N x N matrices. Returns (B, Uk, info)."""
    rng = rng if rng is not None else np.random.default_rng(0)
    zj, wj = contour(k0, R, nq)
    Ts = assemble_at(zj)
    V = probe_matrix(N, r, rng)
    if moments_fn is None:
        A0, A1, facs = moments(Ts, zj, wj, V)
    else:
        A0, A1 = moments_fn(V)
        facs = None
    U, S, Wh = np.linalg.svd(A0, full_matrices=False)
    rk = int(np.count_nonzero(S >= svd_tol))
    rused = r
    if rk == 0:
        return np.zeros((0, 0), complex), np.zeros((N, 0), complex), dict(rk=0, r=r, S=S)
    if rk == r:
        r_tmp = 2 * r
        while r_tmp < N:
            V = probe_matrix(N, r_tmp, rng)
            if moments_fn is None:
                A0 = np.zeros((N, r_tmp), complex); A1 = np.zeros((N, r_tmp), complex)
                for f, z, w in zip(facs, zj, wj):
                    X = sla.lu_solve(f, V, check_finite=False)
                    A0 += w * X
                    A1 += (w * z) * X
            else:
                A0, A1 = moments_fn(V)
            U, S, Wh = np.linalg.svd(A0, full_matrices=False)
            rk = int(np.count_nonzero(S >= svd_tol))
            rused = r_tmp
            break  # the reference leaves this loop after one regrowth (beyn.jl:307)
    Uk = U[:, :rk]
    Wk = Wh.conj().T[:, :rk]
    tmp = (A1 @ Wk) / S[:rk][None, :]
    B = Uk.conj().T @ tmp
    return B, Uk, dict(rk=rk, r=rused, S=S)


def solve_beyn(assemble_at, N, k0, R, nq=64, r=48, svd_tol=1e-14, rng=None, moments_fn=None):
    B, Uk, info = construct_B_matrix(assemble_at, N, k0, R, nq, r, svd_tol, rng, moments_fn)
    if B.size == 0:
        return np.zeros(0, complex), Uk, np.zeros((0, 0), complex), info
    lam, Y = np.linalg.eig(B)
    return lam, Uk, Y, info


def sigma_min(A: np.ndarray) -> float:
    return float(np.linalg.svd(A, compute_uv=False)[-1])


def get_eigenvalues(ks, tens, threshold=200.0):
    ks = np.asarray(ks, dtype=np.float64)
    y = np.log10(np.abs(np.asarray(tens, dtype=np.float64)))
    g1 = np.diff(y) / np.diff(ks)
    x1 = 0.5 * (ks[:-1] + ks[1:])
    g2 = np.diff(g1) / np.diff(x1)
    x2 = 0.5 * (x1[:-1] + x1[1:])
    out = []
    for i in range(1, len(g2) - 1):
        if g2[i] > g2[i - 1] and g2[i] > g2[i + 1] and g2[i] > threshold:
            out.append(x2[i])
    return np.array(out)


# --------------------------------------------------------------------------
# one disk with the nodes spread over processes
# --------------------------------------------------------------------------
def assemble_spec(spec, z):
    """T(z) for a picklable operator description:
    ("cfie", [nodes...])                  CFIE Kress, direct AMOS values
    ("dlp", nodes)                        DLP Kress Fredholm matrix
    ("dlp_reduced", nodes, orbits)        symmetry-reduced DLP Fredholm matrix
    ("cfie_cheb", [nodes...], params)     CFIE through Chebyshev panels"""
    from . import assembly as OA, chebyshev as OC
    kind = spec[0]
    if kind == "cfie":
        return OA.cfie_matrix(spec[1], z)
    if kind == "dlp":
        return OA.dlp_fredholm(spec[1], z)
    if kind == "dlp_reduced":
        return OA.dlp_fredholm_reduced(spec[1], z, spec[2])
    if kind == "cfie_cheb":
        return OC.cfie_matrix(spec[1], z, spec[2])
    raise ValueError(kind)


def _node_solve(args):
    spec, z, V = args
    T = assemble_spec(spec, z)
    f = sla.lu_factor(T, check_finite=False)
    return sla.lu_solve(f, V, check_finite=False)


def beyn_disk(spec, N, k0, R, nq, r, svd_tol, seed, regrow="extend", workers=1):
    """construct_B_matrix and eig(B) (beyn.jl:257-322, 364-375) for one disk.

    The probes are drawn from NumPy's PCG64 with ``seed``: V1 = probe(N, r);
    when the rank saturates (rk == r, 2r < N) regrow="extend" appends a
    second draw V2 = probe(N, r) to the solved block, regrow="fresh" draws a
    new N x 2r block (the reference's policy). Both blocks are solved at
    every node in one pass, so a regrowth costs no second factorisation.
    Returns dict(lam=eigenvalues of B, rk, r, S)."""
    import multiprocessing as mp
    rng = np.random.default_rng(seed)
    V1 = probe_matrix(N, r, rng)
    V2 = probe_matrix(N, r, rng) if regrow == "extend" else probe_matrix(N, 2 * r, rng)
    Vall = np.hstack([V1, V2])
    zj, wj = contour(k0, R, nq)
    jobs = [(spec, z, Vall) for z in zj]
    if workers > 1:
        with mp.get_context("spawn").Pool(workers) as pool:
            Xs = pool.map(_node_solve, jobs, chunksize=1)
    else:
        Xs = [_node_solve(j) for j in jobs]
    A0 = np.zeros(Vall.shape, complex)
    A1 = np.zeros(Vall.shape, complex)
    for X, z, w in zip(Xs, zj, wj):
        A0 += w * X
        A1 += (w * z) * X
    M0, M1 = A0[:, :r], A1[:, :r]
    S = np.linalg.svd(M0, compute_uv=False)
    rk = int(np.count_nonzero(S >= svd_tol))
    rused = r
    if rk == r and 2 * r < N:
        M0, M1 = (A0, A1) if regrow == "extend" else (A0[:, r:], A1[:, r:])
        rused = 2 * r
    U, S, Wh = np.linalg.svd(M0, full_matrices=False)
    rk = int(np.count_nonzero(S >= svd_tol))
    if rk == 0:
        return dict(lam=np.zeros(0, complex), rk=0, r=rused, S=S)
    Uk = U[:, :rk]
    Wk = Wh.conj().T[:, :rk]
    B = Uk.conj().T @ ((M1 @ Wk) / S[:rk][None, :])
    return dict(lam=np.linalg.eigvals(B), rk=rk, r=rused, S=S)
