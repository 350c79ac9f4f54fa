"""FP64 restatement of the sweep refinement (test infrastructure only).

* newton_refine_svd!   sweepmethods.jl:307-368: Newton steps on
  lambda_min(G(k)), G = A^H A, G' = A'^H A + A^H A',
  G'' = A''^H A + 2 A'^H A' + A^H A''; lambda1 = x^H G' x,
  lambda2 = x^H G'' x + 2 sum_{j != min} |v_j^H G' x|^2 / (lambda - lambda_j)
  (|lambda - lambda_j| < eps skipped); k <- clamp(k - lambda1 / lambda2, a, b);
  stop on a step below tol, a non-finite lambda1/lambda2 or |lambda2| < sqrt(eps);
  return (k, sqrt(lambda_min)) at the final k, or at the best k seen when smaller.
"""
from __future__ import annotations

import numpy as np

EPS = np.finfo(float).eps


def newton_refine_svd(assemble, k0, a=0.0, b=np.inf, maxiter=8, tol=1e-12):
    """assemble(k) -> (A, A', A'') at real k."""
    k = min(max(k0, a), b)
    kbest, lbest = k, np.inf
    for _ in range(maxiter):
        A, dA, ddA = assemble(k)
        G = A.conj().T @ A
        H = dA.conj().T @ A + A.conj().T @ dA
        H2 = ddA.conj().T @ A + 2 * (dA.conj().T @ dA) + A.conj().T @ ddA
        vals, vecs = np.linalg.eigh(G)
        idx = int(np.argmin(vals))
        lam = vals[idx]
        x = vecs[:, idx]
        if np.isfinite(lam) and lam < lbest:
            lbest, kbest = lam, k
        gx = H @ x
        l1 = np.real(np.vdot(x, gx))
        l2 = np.real(np.vdot(x, H2 @ x))
        c = vecs.conj().T @ gx
        for j in range(len(vals)):
            if j == idx:
                continue
            den = lam - vals[j]
            if abs(den) < EPS:
                continue
            l2 += 2 * abs(c[j]) ** 2 / den
        if not np.isfinite(l1) or not np.isfinite(l2) or abs(l2) < np.sqrt(EPS):
            break
        knew = min(max(k - l1 / l2, a), b)
        if not np.isfinite(knew):
            break
        if abs(knew - k) < tol:
            k = knew
            break
        k = knew
    A = assemble(k)[0]
    lmin = np.linalg.eigvalsh(A.conj().T @ A).min()
    if np.isfinite(lmin) and lmin <= lbest:
        return k, np.sqrt(max(0.0, lmin))
    A = assemble(kbest)[0]
    lmin = np.linalg.eigvalsh(A.conj().T @ A).min()
    return kbest, np.sqrt(max(0.0, lmin))


def adjoint_fredholm(F, ds, fund=None):
    """adjoint_fredholm_matrix! (dlp_kress.jl:1451-1500) from the Fredholm
    matrix F = I - D: A_adj[i, j] = delta_ij - D[j, i] ds_j / ds_i; with a
    reduction, ds is indexed by the fundamental nodes' full indices."""
    d = np.asarray(ds if fund is None else np.asarray(ds)[np.asarray(fund)], dtype=np.float64)
    D = np.eye(F.shape[0]) - F
    return np.eye(F.shape[0]) - D.T * (d[None, :] / d[:, None])


def smallest_nullvec(A):
    """smallest_nullvec_krylov! (dlp.jl:991-1004), dense: the eigenvalue mu of
    largest modulus of A^-1 (KrylovKit there), sigma = 1/|mu|, unit vector u."""
    mu, V = np.linalg.eig(np.linalg.inv(A))
    i = int(np.argmax(np.abs(mu)))
    u = V[:, i] / np.linalg.norm(V[:, i])
    return 1.0 / abs(mu[i]), u
