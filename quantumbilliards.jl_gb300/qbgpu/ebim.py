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


__all__ = ["solve_krylov", "solve_full", "solve"]
