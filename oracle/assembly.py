"""FP64 restatement of the Kress DLP / CFIE assembly (test infrastructure only).

Follows:
* kress_R_even!/kress_R_odd!            boundarypoints.jl:310-358
* cfie_geom_cache                        boundarypoints.jl:854-880
* construct_fredholm_matrix!             dlp_kress.jl:906-932
* construct_dlp_matrix_derivatives!      dlp_kress.jl:975-1019 (real k)
* CFIE construct_matrices!               cfie_kress.jl:416-510, derivatives :619-757
* symmetry orbits                        symmetry.jl:214-319
* reduced DLP (images)                   dlp_kress.jl:1081-1100, 1151-1189, 1293-1345
* reduced CFIE (orbit sums)              cfie_kress.jl:512-617, 758-892
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


def cfie_matrix_derivs(pts, k, funcs_same=None, funcs_off=None):
    """(A, dA/dk, d2A/dk2) over all components (cfie_kress.jl:619-757; the
    Chebyshev route chebyshev_euclidian_helmholtz_cfie_kress.jl:881-1060 uses
    the same expressions). The off-component double-layer derivatives carry
    the sign written there (cfie_kress.jl:729-731)."""
    offs = component_offsets(pts)
    Nt = offs[-1]
    A = np.zeros((Nt, Nt), dtype=np.complex128)
    A1 = np.zeros_like(A)
    A2 = np.zeros_like(A)
    ik = 1j * k
    aL1 = -k * INV_TWO_PI
    aL2 = 0.5j * k
    aM1 = -INV_TWO_PI
    aM2 = 0.5j
    pi = math.pi
    for a, p in enumerate(pts):
        g = geom_cache(p)
        Rm = kress_R(p.n)
        r, invr, lt, inn = g["R"], g["invR"], g["logterm"], g["inner"]
        s = g["speed"][None, :]
        h0, h1, j0, j1 = funcs_same[a] if funcs_same is not None else _bessels(k, r)
        w = p.ws[None, :]
        kr = k * r
        l1 = aL1 * inn * j1 * invr
        l2 = aL2 * inn * h1 * invr - l1 * lt
        dval = Rm * l1 + w * l2
        dval1 = Rm * (-(inn * k * j0) * INV_TWO_PI) + w * ((inn * k * (lt * j0 + 1j * pi * h0)) * INV_TWO_PI)
        dval2 = Rm * ((inn * (kr * j1 - j0)) * INV_TWO_PI) + \
            w * ((inn * (lt * (j0 - kr * j1) + 1j * pi * (h0 - kr * h1))) * INV_TWO_PI)
        m1 = aM1 * j0 * s
        m2 = aM2 * h0 * s - m1 * lt
        sval = Rm * m1 + w * m2
        m1_1 = (r * s * j1) * INV_TWO_PI
        m1_2 = (r * s * (kr * j0 - j1)) * INV_TWO_PI / k
        m2_1 = -(r * s * (lt * j1 + 1j * pi * h1)) * INV_TWO_PI
        m2_2 = (r * s * (lt * (j1 - kr * j0) - 1j * pi * kr * h0 + 1j * pi * h1)) * INV_TWO_PI / k
        sval1 = Rm * m1_1 + w * m2_1
        sval2 = Rm * m1_2 + w * m2_2
        blk = -(dval + ik * sval)
        blk1 = -(dval1 + 1j * sval + ik * sval1)
        blk2 = -(dval2 + 2j * sval1 + ik * sval2)
        # diagonal (cfie_kress.jl:636-646)
        si, ki, wi = g["speed"], g["kappa"], p.ws
        m2d = ((0.5j - EULER_OVER_PI) - INV_TWO_PI * np.log((k ** 2 / 4) * si ** 2 + 0j)) * si
        sd = np.diag(Rm) * (aM1 * si) + wi * m2d
        sd1 = wi * (-(si / (pi * k)))
        sd2 = wi * (si / (pi * k ** 2))
        np.fill_diagonal(blk, 1.0 - (wi * ki + ik * sd))
        np.fill_diagonal(blk1, -(1j * sd + ik * sd1))
        np.fill_diagonal(blk2, -(2j * sd1 + ik * sd2))
        sl = slice(offs[a], offs[a + 1])
        A[sl, sl], A1[sl, sl], A2[sl, sl] = blk, blk1, blk2
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
            h0, h1 = funcs_off[(a, b)] if funcs_off is not None else (sp.hankel1(0, k * r), sp.hankel1(1, k * r))
            wj = pb.ws[None, :]
            dval = wj * (aL2 * inn * h1 * invr)
            dval1 = wj * (-0.5j * inn * k * h0)
            dval2 = wj * (-0.5j * inn * (h0 - k * r * h1))
            sval = wj * (aM2 * h0 * sb)
            sval1 = wj * (-0.5j * r * h1 * sb)
            sval2 = wj * (0.5j * r * (h1 - k * r * h0) * sb / k)
            sa, sb_ = slice(offs[a], offs[a + 1]), slice(offs[b], offs[b + 1])
            A[sa, sb_] = -(dval + ik * sval)
            A1[sa, sb_] = -(dval1 + 1j * sval + ik * sval1)
            A2[sa, sb_] = -(dval2 + 2j * sval1 + ik * sval2)
    return A, A1, A2


# --------------------------------------------------------------------------
# symmetry-reduced DLP
# --------------------------------------------------------------------------
def periodic_symmetry_index_orbits(N: int, sym):
    """Orbits of a cyclic node index under a reflection or rotation
    (symmetry.jl:214-319), 0-based. ``sym`` is ("x", p) (x -> -x),
    ("y", p) (y -> -y), ("xy", px, py) or ("rot", n, m).
    Returns (fund, fund_to_full [m, norb], fund_to_scale [m, norb])."""
    kind = sym[0]
    if kind in ("x", "y"):
        if N % 2:
            raise ValueError("reflection symmetry needs even N")
        m = N // 2
        orb = lambda q: ([q, (N - q - 1) % N], [1.0, float(sym[1])])
    elif kind == "xy":
        if N % 4:
            raise ValueError("XY reflection needs N divisible by 4")
        m = N // 4
        px, py = float(sym[1]), float(sym[2])
        orb = lambda q: ([q, (N // 2 - q - 1) % N, (N - q - 1) % N, (q + N // 2) % N], [1.0, px, py, px * py])
    elif kind == "rot":
        n, mm = int(sym[1]), int(sym[2])
        if N % n:
            raise ValueError("rotation order must divide N")
        m = N // n
        chi = [complex(math.cos(2 * math.pi * mm * l / n), math.sin(2 * math.pi * mm * l / n)) for l in range(n)]
        orb = lambda q: ([(q + l * (N // n)) % N for l in range(n)], chi)
    else:
        raise ValueError(kind)
    fund = np.arange(m)
    qs, ss = zip(*(orb(q) for q in fund))
    full = np.array(qs, dtype=np.int64)
    scale = np.array(ss, dtype=np.complex128)
    seen = np.zeros(N, dtype=np.int64)
    np.add.at(seen, full.ravel(), 1)
    if not np.all(seen == 1):
        raise ValueError("orbits do not partition the nodes")
    return fund, full, scale


def dlp_fredholm_reduced(p, k, orbits, derivs: bool = False, funcs=None, image_h=None):
    """Reduced F = I - D_red on the fundamental indices (dlp_kress.jl:1151-1189;
    derivatives :1293-1345): the Kress-split entry of D at (I_a, I_b) plus the
    regular image kernels of the other orbit members of I_b."""
    fund, full, scale = orbits
    m = len(fund)
    res = dlp_fredholm(p, k, derivs, funcs)
    Ffull = res if not derivs else res[0]
    idx = np.ix_(fund, fund)
    F = Ffull[idx].copy()
    if derivs:
        F1, F2 = res[1][idx].copy(), res[2][idx].copy()
    X, Y = p.xy[:, 0], p.xy[:, 1]
    dX, dY = p.tangent[:, 0], p.tangent[:, 1]
    sp_ = np.hypot(dX, dY)
    nx, ny = dY / sp_, -dX / sp_
    xi, yi = X[fund][:, None], Y[fund][:, None]
    for l in range(full.shape[1]):
        q = full[:, l]
        sc = scale[:, l][None, :]
        skip = (q == fund)[None, :]
        dx = xi - X[q][None, :]
        dy = yi - Y[q][None, :]
        r = np.hypot(dx, dy)
        rs = np.where(r < np.finfo(float).eps, 1.0, r)
        c = (nx[q][None, :] * dx + ny[q][None, :] * dy) / rs
        wq = (sp_[q] * p.ws[q])[None, :]
        h0, h1 = image_h(rs) if image_h is not None else (sp.hankel1(0, k * rs), sp.hankel1(1, k * rs))
        mask = (~skip) & (r >= np.finfo(float).eps)
        F -= np.where(mask, sc * (0.5j * k) * c * h1 * wq, 0.0)
        if derivs:
            kr = k * rs
            F1 -= np.where(mask, sc * 0.5j * c * (kr * h0) * wq, 0.0)
            F2 -= np.where(mask, sc * 0.5j * c * (rs * h0 - k * rs ** 2 * h1) * wq, 0.0)
    return (F, F1, F2) if derivs else F


def cfie_reduced(pts, k, orbits, derivs=False, full=None):
    """Reduced CFIE on the fundamental indices (construct_matrices_reduced!,
    cfie_kress.jl:512-617; derivatives :758-892): A_red[a, b] = sum over the
    members q of orbit b of scale_q A[I_a, q], every term the full Kress-split
    entry (the diagonal formula at q == I_a). ``full`` optionally supplies the
    full operator (or the (A, A', A'') triple) already assembled."""
    fund, fullidx, scale = orbits
    mats = full if full is not None else (cfie_matrix_derivs(pts, k) if derivs else cfie_matrix(pts, k))
    mats = mats if isinstance(mats, tuple) else (mats,)
    out = []
    for M in mats:
        R = np.zeros((len(fund), len(fund)), dtype=np.complex128)
        for l in range(fullidx.shape[1]):
            R += M[np.ix_(fund, fullidx[:, l])] * scale[:, l][None, :]
        out.append(R)
    return tuple(out) if derivs else out[0]


def assemble(kind, pts, k, derivs=False):
    """Single entry used by the tests: 'dlp' -> one component, 'cfie' -> list."""
    if kind == "dlp":
        p = pts[0] if isinstance(pts, list) else pts
        return dlp_fredholm(p, k, derivs)
    pl = pts if isinstance(pts, list) else [pts]
    return cfie_matrix_derivs(pl, k) if derivs else cfie_matrix(pl, k)
