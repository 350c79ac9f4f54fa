"""FP64 restatement of the Kress DLP / CFIE assembly (test infrastructure only).

Follows:
* kress_R_even!/kress_R_odd!            boundarypoints.jl:310-358
* cfie_geom_cache                        boundarypoints.jl:854-880
* construct_fredholm_matrix!             dlp_kress.jl:906-932
* construct_dlp_matrix_derivatives!      dlp_kress.jl:975-1019 (real k)
* CFIE construct_matrices!               cfie_kress.jl:416-510
* complex-k multi-k CFIE (Chebyshev)     chebyshev_euclidian_helmholtz_cfie_kress.jl:543-666
* complex-k DLP (Chebyshev)              chebyshev_euclidian_helmholtz_dlp_kress.jl:702-769

For complex k the reference evaluates J0/J1 separately from H0/H1
(chebyshev_bessels.jl:1104-1160); this restatement does the same with the
exact AMOS values (``direct``) or with the reference's Chebyshev panels
(``oracle.chebyshev``).
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special as sp

TWO_PI = 2.0 * math.pi
INV_TWO_PI = 1.0 / TWO_PI
EULER_OVER_PI = float(np.euler_gamma) / math.pi


def kress_R_column(N: int) -> np.ndarray:
    """First column c of the circulant Kress matrix, R[i, j] = c[(i - j) mod N]."""
    a = np.zeros(N, dtype=np.complex128)
    if N % 2 == 0:
        n = N // 2
        for m in range(1, n):
            a[m] = 1.0 / m
            a[N - m] = 1.0 / m
        rjn = np.real(np.fft.ifft(a))
        alt = (-1.0) ** np.arange(N)
        return -TWO_PI * rjn - (2 * TWO_PI / N ** 2) * alt
    n = (N - 1) // 2
    for m in range(1, n + 1):
        a[m] = 1.0 / m
        a[N - m] = 1.0 / m
    return -TWO_PI * np.real(np.fft.ifft(a))


def kress_R(N: int) -> np.ndarray:
    c = kress_R_column(N)
    i = np.arange(N)
    return c[(i[:, None] - i[None, :]) % N]


def geom_cache(p):
    X, Y = p.xy[:, 0], p.xy[:, 1]
    dX, dY = p.tangent[:, 0], p.tangent[:, 1]
    ddX, ddY = p.tangent_2[:, 0], p.tangent_2[:, 1]
    DX = X[:, None] - X[None, :]
    DY = Y[:, None] - Y[None, :]
    R = np.hypot(DX, DY)
    np.fill_diagonal(R, 1.0)
    invR = 1.0 / R
    np.fill_diagonal(invR, 0.0)
    inner = dY[None, :] * DX - dX[None, :] * DY
    dT = p.ts[:, None] - p.ts[None, :]
    with np.errstate(divide="ignore"):
        logterm = np.log(4.0 * np.sin(dT / 2) ** 2)
    np.fill_diagonal(logterm, 0.0)
    speed = np.sqrt(dX ** 2 + dY ** 2)
    kappa = INV_TWO_PI * (-(dX * ddY - dY * ddX)) / (dX ** 2 + dY ** 2)
    return dict(R=R, invR=invR, inner=inner, logterm=logterm, speed=speed, kappa=kappa)


def _bessels(k, r, need_derivs=False):
    """H0, H1, J0, J1 at z = k r (diagonal r==1 placeholder is harmless)."""
    z = k * r
    h0 = sp.hankel1(0, z)
    h1 = sp.hankel1(1, z)
    if np.isrealobj(z) or np.all(np.imag(k) == 0):
        j0 = np.real(h0).astype(np.complex128)
        j1 = np.real(h1).astype(np.complex128)
    else:
        j0 = sp.jv(0, z)
        j1 = sp.jv(1, z)
    return h0, h1, j0, j1


def dlp_fredholm(p, k, derivs: bool = False, funcs=None):
    """F = I - D (dlp_kress.jl:906-932); with derivs also F' = -D', F'' = -D''
    (dlp_kress.jl:975-1075). k may be complex (the reference's complex-k path
    is the Chebyshev one; ``funcs`` lets the caller pass interpolated values)."""
    N = p.n
    g = geom_cache(p)
    Rm = kress_R(N)
    r, invr, lt, inn = g["R"], g["invR"], g["logterm"], g["inner"]
    h0, h1, j0, j1 = funcs if funcs is not None else _bessels(k, r)
    aL1 = -k * INV_TWO_PI
    aL2 = 0.5j * k
    w = p.ws[None, :]
    l1 = aL1 * inn * j1 * invr
    l2 = aL2 * inn * h1 * invr - l1 * lt
    D = Rm * l1 + w * l2
    np.fill_diagonal(D, p.ws * g["kappa"])
    F = np.eye(N, dtype=np.complex128) - D
    if not derivs:
        return F
    kr = k * r
    l1_1 = -(inn * k * j0) * INV_TWO_PI
    l1_2 = (inn * (kr * j1 - j0)) * INV_TWO_PI
    l2_1 = (inn * k * (lt * j0 + 1j * math.pi * h0)) * INV_TWO_PI
    l2_2 = (inn * (lt * (j0 - kr * j1) + 1j * math.pi * (h0 - kr * h1))) * INV_TWO_PI
    D1 = Rm * l1_1 + w * l2_1
    D2 = Rm * l1_2 + w * l2_2
    np.fill_diagonal(D1, 0.0)
    np.fill_diagonal(D2, 0.0)
    return F, -D1, -D2


def component_offsets(pts):
    offs = [0]
    for p in pts:
        offs.append(offs[-1] + p.n)
    return offs


def cfie_matrix(pts, k, funcs_same=None, funcs_off=None):
    """A = I - (D + i k S) over all components (cfie_kress.jl:416-510).

    ``funcs_same[a]`` / ``funcs_off[(a, b)]`` optionally replace the exact
    special-function values by interpolated ones (Chebyshev restatement)."""
    offs = component_offsets(pts)
    Nt = offs[-1]
    A = np.zeros((Nt, Nt), dtype=np.complex128)
    ik = 1j * k
    aL1 = -k * INV_TWO_PI
    aL2 = 0.5j * k
    aM1 = -INV_TWO_PI
    aM2 = 0.5j
    for a, p in enumerate(pts):
        g = geom_cache(p)
        Na = p.n
        Rm = kress_R(Na)
        r, invr, lt, inn = g["R"], g["invR"], g["logterm"], g["inner"]
        s = g["speed"]
        if funcs_same is not None:
            h0, h1, j0, j1 = funcs_same[a]
        else:
            h0, h1, j0, j1 = _bessels(k, r)
        w = p.ws[None, :]
        l1 = aL1 * inn * j1 * invr
        l2 = aL2 * inn * h1 * invr - l1 * lt
        dval = Rm * l1 + w * l2
        m1 = aM1 * j0 * s[None, :]
        m2 = aM2 * h0 * s[None, :] - m1 * lt
        sval = Rm * m1 + w * m2
        blk = -(dval + ik * sval)
        # diagonal (cfie_kress.jl:436-445)
        si, ki, wi = s, g["kappa"], p.ws
        dd = wi * ki
        m1d = aM1 * si
        m2d = ((0.5j - EULER_OVER_PI) - INV_TWO_PI * np.log((k ** 2 / 4) * si ** 2 + 0j)) * si
        sd = np.diag(Rm) * m1d + wi * m2d
        np.fill_diagonal(blk, 1.0 - (dd + ik * sd))
        A[offs[a]:offs[a + 1], offs[a]:offs[a + 1]] = blk
    for a, pa in enumerate(pts):
        for b, pb in enumerate(pts):
            if a == b:
                continue
            dx = pa.xy[:, 0][:, None] - pb.xy[:, 0][None, :]
            dy = pa.xy[:, 1][:, None] - pb.xy[:, 1][None, :]
            r = np.hypot(dx, dy)
            invr = 1.0 / r
            inn = pb.tangent[:, 1][None, :] * dx - pb.tangent[:, 0][None, :] * dy
            sb = np.hypot(pb.tangent[:, 0], pb.tangent[:, 1])[None, :]
            if funcs_off is not None:
                h0, h1 = funcs_off[(a, b)]
            else:
                h0, h1 = sp.hankel1(0, k * r), sp.hankel1(1, k * r)
            wj = pb.ws[None, :]
            dval = wj * (aL2 * inn * h1 * invr)
            sval = wj * (aM2 * h0 * sb)
            A[offs[a]:offs[a + 1], offs[b]:offs[b + 1]] = -(dval + ik * sval)
    return A


def assemble(kind, pts, k, derivs=False):
    """Single entry used by the tests: 'dlp' -> one component, 'cfie' -> list."""
    if kind == "dlp":
        p = pts[0] if isinstance(pts, list) else pts
        return dlp_fredholm(p, k, derivs)
    if derivs:
        raise NotImplementedError
    return cfie_matrix(pts if isinstance(pts, list) else [pts], k)
