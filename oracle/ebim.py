"""FP64 restatement of the EBIM eigen step (test infrastructure only).

Both variants expand A(k + eps) = A + eps A' + eps^2/2 A'' about the trial k
and solve the pencil A v = lambda A' v; per accepted lambda
eps1 = -lambda, eps2 = -eps1^2/2 (u^H A'' v)/(u^H A' v) (0 when
|u^H A' v| <= 1e-15), corrected k = k + eps1 + eps2, tension |eps1 + eps2|.

* solve_full!    ebim.jl:336-375: all generalized eigenpairs with left
  eigenvectors (LAPACK ggev there, scipy.linalg.eig(A, A') here), filtered to
  |Re lambda|, |Im lambda| < dk; u is the left eigenvector of the pencil.
* solve_krylov!  ebim.jl:464-537: the nev eigenvalues of largest |mu| of
  C = A^{-1} A' (KrylovKit Arnoldi there, a dense eig of C here; the
  converged eigenpairs are the same), u the eigenvector of C^H = A'^H A^{-H}
  (op_l! applies A^{-H} and then A'^H, ebim.jl:499-504) paired by
  mu_l ~ conj(mu_r) (:508); kept when |Re(k_c) - k| < dk (:528).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def _correct(lam, u, v, dA, ddA):
    num = np.vdot(u, ddA @ v)
    den = np.vdot(u, dA @ v)
    c1 = -lam
    c2 = -0.5 * c1 * c1 * (num / den) if abs(den) > 1e-15 else 0.0
    return c1 + c2


def solve_full(A, dA, ddA, k, dk, return_imag_part=False):
    """ebim.jl:336-375. Returns (k_corrected, tens)."""
    lam, VL, VR = sla.eig(A, dA, left=True, right=True)
    valid = (np.abs(lam.real) < dk) & (np.abs(lam.imag) < dk)
    out, tens = [], []
    for i in np.nonzero(valid)[0]:
        t = _correct(lam[i], VL[:, i], VR[:, i], dA, ddA)
        out.append(k + (t if return_imag_part else t.real))
        tens.append(abs(t))
    return np.array(out), np.array(tens)


def _largest(M, nev):
    mu, V = np.linalg.eig(M)
    o = np.argsort(-np.abs(mu), kind="stable")[:nev]
    return mu[o], V[:, o]


def solve_krylov(A, dA, ddA, k, dk, nev=5, return_imag_part=False):
    """ebim.jl:464-537. Returns (k_corrected, tens)."""
    lu = sla.lu_factor(A)
    C = sla.lu_solve(lu, dA)
    mu_r, V = _largest(C, nev)
    lam = 1.0 / mu_r
    o = np.argsort(np.abs(lam), kind="stable")
    lam, mu_r, V = lam[o], mu_r[o], V[:, o]
    mu_l, U = _largest(C.conj().T, nev)
    perm = [int(np.argmin(np.abs(mu_l - np.conj(m)))) for m in mu_r]
    U = U[:, perm]
    out, tens = [], []
    for j in range(len(lam)):
        if not (abs(lam[j].real) < dk and abs(lam[j].imag) < dk):
            continue
        t = _correct(lam[j], U[:, j], V[:, j], dA, ddA)
        kc = complex(k) + t
        if abs(kc.real - k) < dk:
            out.append(kc if return_imag_part else kc.real)
            tens.append(abs(t))
    return np.array(out), np.array(tens)
