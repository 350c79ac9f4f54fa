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
