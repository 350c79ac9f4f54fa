"""EBIM eigen step on the device (mirrors ebim.jl: solve_full! :336-375,
solve_krylov! :464-537).

``solve_full`` and ``solve_krylov`` take assembled A, A', A'' (host arrays,
left unchanged) like the reference's functions; ``solve`` assembles them on
the device for a workspace first and never copies the matrices to the host.
All return (corrected k, tension), nearest eigenvalue first; the corrected k
are real unless ``return_imag_part``.

On the device: FP64 LU of A, block shift-invert iteration on A^{-1} A' and on
its adjoint (Rayleigh-Ritz on the projection after every step, stopping when
the Ritz values change by less than 1e-13 relative), and the second-order
correction. The reference's conventions are kept: solve_krylov! pairs v with
the eigenvector of (A^{-1} A')^H and keeps a result only when
|Re(k_c) - k| < dk; solve_full! uses the left eigenvectors of the pencil and
returns every eigenvalue inside the dk box.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .operators import Workspace


def _run(call, cap, return_imag_part):
    while True:
        out = np.zeros(2 * max(cap, 1))
        tens = np.zeros(max(cap, 1))
        cnt = C.c_int32()
        its = (C.c_int32 * 3)()
        L.check(call(cap, out.ctypes.data_as(C.POINTER(C.c_double)), tens.ctypes.data_as(C.POINTER(C.c_double)),
                     C.byref(cnt), its))
        m = int(cnt.value)
        if m <= cap:
            break
        cap = m
    kc = out[:2 * m].view(np.complex128)
    info = dict(iters_right=its[0], iters_left=its[1], nev=its[2])
    return (kc.copy() if return_imag_part else kc.real.copy()), tens[:m].copy(), info


def _eig(A, dA, ddA, k, dk, nev, flags, return_imag_part, return_info):
    A = np.asfortranarray(A, dtype=np.complex128)
    dA = np.asfortranarray(dA, dtype=np.complex128)
    ddA = np.asfortranarray(ddA, dtype=np.complex128)
    n = A.shape[0]
    if A.shape != (n, n) or dA.shape != (n, n) or ddA.shape != (n, n):
        raise ValueError("A, dA, ddA must be square and of one size")
    lib = L.load()

    def call(cap, po, pt, pc, its):
        return lib.qbg_ebim_eig(n, A.ctypes.data, dA.ctypes.data, ddA.ctypes.data, float(k), float(dk), int(nev),
                                flags, cap, po, pt, pc, its)

    kc, tens, info = _run(call, max(int(nev), 8), return_imag_part)
    return (kc, tens, info) if return_info else (kc, tens)


def solve_krylov(solver, A, dA, ddA, pts, k, dk, multithreaded=True, nev=5, tol=1e-14, maxiter=5000,
                 krylovdim=None, return_imag_part=False, return_info=False):
    """solve_krylov! (ebim.jl:464-537). tol, maxiter and krylovdim belong to
    the reference's Arnoldi; the device iteration has its own stopping rule."""
    return _eig(A, dA, ddA, k, dk, nev, 0, return_imag_part, return_info)


def solve_full(solver, A, dA, ddA, pts, k, dk, use_lapack_raw=False, multithreaded=True, return_imag_part=False,
               return_info=False, nev=8):
    """solve_full! (ebim.jl:336-375): every eigenvalue in the dk box (nev is
    the starting block of the device iteration, grown as needed)."""
    return _eig(A, dA, ddA, k, dk, nev, L.QBG_EBIM_FULL, return_imag_part, return_info)


def solve(ws: Workspace, k, dk, nev=5, full=False, return_imag_part=False, return_info=False):
    """A, A', A'' of the workspace at k assembled on the device (direct FP64),
    then the eigen step of solve_krylov! (or solve_full! with full=True)."""
    lib = L.load()
    flags = L.QBG_EBIM_FULL if full else 0

    def call(cap, po, pt, pc, its):
        return lib.qbg_ebim_solve(ws.handle, float(k), float(dk), int(nev), flags, cap, po, pt, pc, its)

    kc, tens, info = _run(call, max(int(nev), 8), return_imag_part)
    return (kc, tens, info) if return_info else (kc, tens)


def _local_gap(xs, i, w=4):
    """_local_gap (ebim.jl:1021-1029): median positive gap of xs within +-w."""
    seg = np.diff(xs[max(0, i - w):min(len(xs), i + w + 1)])
    seg = seg[seg > 0]
    return float(np.median(seg)) if len(seg) else np.inf


def _score(k, t):
    """_ebim_scoring_logic (ebim.jl:1001-1003): lower is better."""
    eps = np.finfo(float).eps
    return np.log10(abs(complex(k).imag) + eps) + np.log10(abs(float(t)) + eps)


def overlap_and_merge_ebim(k_left, ten_left, k_right, ten_right, control_left, kl, kr, tol=1e-5,
                           spacing_frac=0.02, tolmax=5e-3, local_window=4):
    """overlap_and_merge_ebim! (ebim.jl:1059-1107): appends the right window's
    roots, sorts by Re k, clusters neighbours closer than
    min(tolmax, max(tol, spacing_frac * local gap)) and keeps the best-scoring
    root of each cluster (control marks clusters of more than one root).
    Updates the three lists in place."""
    if len(k_right) == 0:
        return
    k_all = list(k_left) + list(k_right)
    t_all = list(ten_left) + list(ten_right)
    c_all = list(control_left) + [False] * len(k_right)
    order = sorted(range(len(k_all)), key=lambda q: np.real(k_all[q]))
    k_all = [k_all[q] for q in order]
    t_all = [t_all[q] for q in order]
    c_all = [c_all[q] for q in order]
    xs = np.array([np.real(x) for x in k_all])
    nk, nt, nc = [], [], []
    i = 0
    while i < len(k_all):
        j = i
        while j < len(k_all) - 1:
            gap = xs[j + 1] - xs[j]
            lgap = min(_local_gap(xs, j, local_window), _local_gap(xs, j + 1, local_window))
            local_tol = min(tolmax, max(tol, spacing_frac * lgap))
            if gap <= local_tol:
                j += 1
            else:
                break
        best = min(range(i, j + 1), key=lambda q: (_score(k_all[q], t_all[q]), q))
        nk.append(k_all[best])
        nt.append(t_all[best])
        nc.append(any(c_all[i:j + 1]) or j > i)
        i = j + 1
    k_left[:], ten_left[:], control_left[:] = nk, nt, nc


def ebim_windows(billiard, k1, k2, dk=lambda k: 0.05 * k ** (-1.0 / 3.0)):
    """The window centres, half-widths and requested nev of compute_spectrum_ebim
    (ebim.jl:1159-1173): k advances by dk(k); nev = ceil((area k / 2 pi -
    length / 4 pi) dk) + 10 (Weyl's law with padding)."""
    ks, dks = [], []
    k = float(k1)
    while k < k2:
        ks.append(k)
        d = float(dk(k))
        dks.append(d)
        k += d
    nevs = [int(np.ceil((billiard.area * kk / (2 * np.pi) - billiard.length / (4 * np.pi)) * d)) + 10
            for kk, d in zip(ks, dks)]
    return ks, dks, nevs


def segment_plan(ks, seg_reuse_frac=0.95):
    """Segments of windows that share one discretisation (ebim.jl:1195-1226):
    a segment runs from first to the last window with
    ks[last] <= ks[first] / seg_reuse_frac. The first segment uses the points
    built at ks[0] (pts0, ebim.jl:1176, 1201); every later segment is
    discretised at its own upper wavenumber ks[last]. Returns a list of
    (first, last, k_disc), 0-based and inclusive."""
    out = []
    first = 0
    while first < len(ks):
        last = first
        while last < len(ks) - 1 and ks[last + 1] <= ks[first] / seg_reuse_frac:
            last += 1
        out.append((first, last, ks[0] if first == 0 else ks[last]))
        first = last + 1
    return out


def compute_spectrum_ebim(solver, billiard, k1, k2, dk=lambda k: 0.05 * k ** (-1.0 / 3.0), tol=1e-5,
                          use_krylov=True, seg_reuse_frac=0.95, return_imag_part=False):
    """compute_spectrum_ebim (ebim.jl:1158-1268) with direct FP64 assembly:
    windows from ebim_windows; the segments are those of segment_plan (the
    first discretised at ks[0], later ones at their upper k); every window runs the
    device eigen step (solve_krylov!, or solve_full! with use_krylov=False) with
    its Weyl nev; overlapping roots are merged (overlap_and_merge_ebim!) and
    those with k1 <= Re k <= k2 kept. Returns (k, tension)."""
    from .solvers import evaluate_points
    ks, dks, nevs = ebim_windows(billiard, k1, k2, dk)
    if not ks:
        return np.zeros(0), np.zeros(0)
    results = [None] * len(ks)
    for first, last, k_disc in segment_plan(ks, seg_reuse_frac):
        ws = Workspace(solver, evaluate_points(solver, billiard, k_disc))
        try:
            for i in range(first, last + 1):
                results[i] = solve(ws, ks[i], dks[i], nev=nevs[i], full=not use_krylov,
                                   return_imag_part=return_imag_part)
        finally:
            ws.close()
    k_all, t_all, ctrl = [], [], []
    for i in range(len(ks)):
        lam, tens = results[i]
        if len(lam):
            overlap_and_merge_ebim(k_all, t_all, list(lam), list(tens), ctrl, ks[i] - dks[i], ks[i] + dks[i], tol=tol)
    keep = [q for q, x in enumerate(k_all) if k1 <= np.real(x) <= k2]
    return np.array([k_all[q] for q in keep]), np.array([t_all[q] for q in keep])


__all__ = ["solve_krylov", "solve_full", "solve", "overlap_and_merge_ebim", "ebim_windows", "segment_plan",
           "compute_spectrum_ebim"]
