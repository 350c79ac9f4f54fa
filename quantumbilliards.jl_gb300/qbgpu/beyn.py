"""Beyn contour method, host side (mirrors beyn.jl).

The N^2 and N^3 work of ``construct_B_matrix`` (beyn.jl:257-322) — assembly of
T(z_j) at every contour node, LU of every node, T(z_j)^-1 V and the moment
sums — runs on the GPU behind ``qbg_beyn_create`` / ``qbg_beyn_moments``.
The host keeps what the reference keeps in FP64 on small matrices: the thin
SVD of A0 (N x r), the absolute rank test ``count(S >= svd_tol)``, the single
r -> 2r regrowth (beyn.jl:291-309, leaving the loop after one pass exactly as
the reference's ``;break`` does at :307), B = U_k^H A1 W_k Sigma_k^-1 and
``eigen(B)`` (beyn.jl:371).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import math
import threading
import time
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .operators import Workspace


def probe_matrix(N: int, r: int, rng: np.random.Generator) -> np.ndarray:
    """Complex Gaussian probes, Re and Im ~ N(0, 1/2) (E|v|^2 = 1) like Julia's
    randn(ComplexF64) (beyn.jl:193); the stream is NumPy's PCG64."""
    s = math.sqrt(0.5)
    V = rng.standard_normal((N, r)) * s + 1j * (rng.standard_normal((N, r)) * s)
    return np.asfortranarray(V.astype(np.complex128))


def contour(k0: complex, R: float, nq: int):
    th = 2 * math.pi * np.arange(nq) / nq
    e = np.cos(th) + 1j * np.sin(th)
    return k0 + R * e, (R / nq) * e


class BeynHandle:
    """Contour nodes assembled and factored on the device (owns a qbg_beyn).

    k0 may be a sequence of disk centres (R a scalar or one radius per disk):
    all disks' nodes are then assembled in one launch and factored as one
    batch, and moments() returns arrays of shape (ndisk, N, L).
    node_chunk > 0 keeps at most that many node operators resident and
    streams the nodes through them in every moments() call."""

    def __init__(self, ws: Workspace, k0, R, nq: int, mixed: bool = False, max_refine: int = 10,
                 refine_tol: float = 1e-6, nb: int = 0, use_chebyshev: bool = True, cheb=None, fp32_sweeps: int = 0,
                 solve_block: int = 0, node_chunk: int = 0, resid_engine: int = 0):
        lib = L.load()
        self.multi = np.ndim(k0) > 0
        k0s = np.atleast_1d(np.asarray(k0, dtype=np.complex128))
        Rs = np.broadcast_to(np.asarray(R, dtype=np.float64), k0s.shape).copy()
        self.ws, self.nq, self.ndisk = ws, int(nq), len(k0s)
        self.k0s, self.Rs = k0s, Rs
        self.k0, self.R = complex(k0s[0]), float(Rs[0])
        self.prec = L.prec_code(mixed)
        self.refine_tol = float(refine_tol)
        cp = L.ChebParams(*(cheb if cheb else (0, 0, 0, 0)))
        o = L.BeynOpts(0, int(max_refine), float(refine_tol), int(nb), 0 if use_chebyshev else 1, cp,
                       int(fp32_sweeps), int(solve_block), int(node_chunk), int(resid_engine))
        h = C.c_void_p()
        if self.multi:
            kk = np.ascontiguousarray(k0s).view(np.float64)
            L.check(lib.qbg_beyn_create_disks(ws.handle, L.dptr(kk), L.dptr(Rs), self.ndisk, self.nq, self.prec,
                                              C.byref(o), C.byref(h)))
        else:
            L.check(lib.qbg_beyn_create(ws.handle, self.k0.real, self.k0.imag, self.R, self.nq, self.prec,
                                        C.byref(o), C.byref(h)))
        self._h = h
        self.N = ws.dim
        self.last_stats = None
        self._m = None

    def moments(self, V: np.ndarray):
        lib = L.load()
        V = np.asfortranarray(V, dtype=np.complex128)
        N, r = V.shape
        if N != self.N:
            raise ValueError(f"V has {N} rows, the operator has {self.N}")
        # per disk an N x r column-major block
        A0 = np.empty((self.ndisk, r, N), dtype=np.complex128)
        A1 = np.empty((self.ndisk, r, N), dtype=np.complex128)
        st = L.BeynStats()
        L.check(lib.qbg_beyn_moments(self._h, L.vptr(V), r, L.vptr(A0), L.vptr(A1), C.byref(st)))
        self._take_stats(st)
        self._m = None  # the kept device blocks are not touched by this call
        A0 = A0.transpose(0, 2, 1)
        A1 = A1.transpose(0, 2, 1)
        if self.multi:
            return A0, A1
        return np.asfortranarray(A0[0]), np.asfortranarray(A1[0])

    def _take_stats(self, st):
        if self.prec != L.QBG_PREC_FP64 and st.nhist and not st.refine_residual <= self.refine_tol:
            warnings.warn(f"qbgpu: mixed refinement stopped at relative residual {st.refine_residual:.2e} > "
                          f"refine_tol {self.refine_tol:.1e} (history {list(st.refine_history[:st.nhist])}); "
                          "the moments are less accurate than requested", RuntimeWarning, stacklevel=3)
        self.last_stats = dict(refine_sweeps=st.refine_sweeps, refine_residual=st.refine_residual,
                               singular=st.singular, ms_assemble=st.ms_assemble, ms_factor=st.ms_factor,
                               ms_solve=st.ms_solve, refine_history=list(st.refine_history[:st.nhist]),
                               ms_residual=st.ms_residual, n_residual=st.n_residual,
                               fp32_history=list(st.fp32_history[:st.nfp32]), ms_solves=st.ms_solves,
                               n_solves=st.n_solves)

    def moments_qr(self, V: np.ndarray, append: bool = False):
        """Moments of V kept on the device and reduced there: returns (R, C)
        with A0 = Q R (thin QR of all kept columns) and C = Q^H A1, each m x m
        (per disk for a multi-disk handle). append=True keeps the columns of
        the previous moments_qr call in front of this call's."""
        lib = L.load()
        V = np.asfortranarray(V, dtype=np.complex128)
        N, r = V.shape
        if N != self.N:
            raise ValueError(f"V has {N} rows, the operator has {self.N}")
        if append and not self._m:
            raise ValueError("append needs an earlier moments_qr call on this handle")
        m = (self._m if append else 0) + r
        Rm = np.empty((self.ndisk, m, m), dtype=np.complex128)
        Cm = np.empty((self.ndisk, m, m), dtype=np.complex128)
        st = L.BeynStats()
        L.check(lib.qbg_beyn_moments_qr(self._h, L.vptr(V), r, int(bool(append)), m, L.vptr(Rm), L.vptr(Cm),
                                        C.byref(st)))
        self._take_stats(st)
        self._m = m
        Rm = Rm.transpose(0, 2, 1)
        Cm = Cm.transpose(0, 2, 1)
        if self.multi:
            return Rm, Cm
        return np.asfortranarray(Rm[0]), np.asfortranarray(Cm[0])

    def B_matrix(self, V: np.ndarray, V2: np.ndarray = None, svd_tol: float = 1e-14, basis: bool = True):
        """construct_B_matrix in one library call (qbg_beyn_B): moments of V,
        the absolute rank test, one regrowth with V2 appended when the rank
        saturates, B = U_k^H A1 W_k S_k^-1 and U_k. Returns (B, U_k or None,
        info with rk, r and the singular values S)."""
        lib = L.load()
        if self.multi:
            raise ValueError("B_matrix takes a single-disk handle")
        V = np.asfortranarray(V, dtype=np.complex128)
        N, r = V.shape
        if N != self.N:
            raise ValueError(f"V has {N} rows, the operator has {self.N}")
        if V2 is not None:
            V2 = np.asfortranarray(V2, dtype=np.complex128)
            if V2.shape != V.shape:
                raise ValueError("V2 must have the shape of V")
        B = np.empty(4 * r * r, dtype=np.complex128)
        U = np.empty((N, 2 * r), dtype=np.complex128, order="F") if basis else None
        S = np.empty(2 * r, dtype=np.float64)
        rk, rused = C.c_int64(), C.c_int64()
        st = L.BeynStats()
        L.check(lib.qbg_beyn_B(self._h, L.vptr(V), r, L.vptr(V2) if V2 is not None else None, float(svd_tol),
                               L.vptr(B), L.vptr(U) if basis else None, L.dptr(S), C.byref(rk), C.byref(rused),
                               C.byref(st)))
        self._take_stats(st)
        self._m = None
        k, m = int(rk.value), int(rused.value)
        Bm = B[:k * k].reshape((k, k), order="F").copy()
        Uk = np.asfortranarray(U[:, :k]) if basis else None
        return Bm, Uk, dict(rk=k, r=m, S=S[:m].copy())

    def close(self):
        if getattr(self, "_h", None) and L.alive():
            L.load().qbg_beyn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_LAPACKE = None


def _lapacke():
    """dict(zgeev, zgesdd, set_threads, get_threads) of LAPACKE in NumPy's
    bundled OpenBLAS, found by their exported names, or None."""
    global _LAPACKE
    if _LAPACKE is None:
        _LAPACKE = False
        try:
            d = os.path.join(os.path.dirname(np.__file__), os.pardir, "numpy.libs")
            for path in sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so*"))):
                lib = C.CDLL(path)
                names = ("scipy_LAPACKE_zgeev64_", "scipy_LAPACKE_zgesdd64_", "scipy_openblas_set_num_threads64_",
                         "scipy_openblas_get_num_threads64_")
                if all(hasattr(lib, x) for x in names):
                    ev, sd = lib.scipy_LAPACKE_zgeev64_, lib.scipy_LAPACKE_zgesdd64_
                    ev.restype = sd.restype = C.c_int64
                    ev.argtypes = [C.c_int, C.c_char, C.c_char, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
                    sd.argtypes = [C.c_int, C.c_char, C.c_int64, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
                    _LAPACKE = dict(zgeev=ev, zgesdd=sd, set_threads=lib.scipy_openblas_set_num_threads64_,
                                    get_threads=lib.scipy_openblas_get_num_threads64_)
                    if hasattr(lib, "scipy_LAPACKE_zgeqrf64_") and hasattr(lib, "scipy_LAPACKE_zunmqr64_"):
                        qf, qm = lib.scipy_LAPACKE_zgeqrf64_, lib.scipy_LAPACKE_zunmqr64_
                        qf.restype = qm.restype = C.c_int64
                        qf.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
                        qm.argtypes = [C.c_int, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                       C.c_int64, C.c_void_p, C.c_void_p, C.c_int64]
                        _LAPACKE.update(zgeqrf=qf, zunmqr=qm)
                    break
        except OSError:
            _LAPACKE = False
    return _LAPACKE or None


def _svd_lapacke(z, A, vals_only=False):
    """Thin SVD U, S, W^H of A through LAPACKE's zgesdd (jobz 'S'), as
    numpy.linalg.svd; vals_only: S alone (jobz 'N')."""
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    m, n = A.shape
    k = min(m, n)
    S = np.empty(k, np.float64)
    if vals_only:
        d = np.empty(1, np.complex128)
        info = z["zgesdd"](102, b"N", m, n, A.ctypes.data, m, S.ctypes.data, d.ctypes.data, 1, d.ctypes.data, 1)
        if info != 0:
            raise np.linalg.LinAlgError(f"zgesdd info {info}")
        return S
    U = np.empty((m, k), np.complex128, order="F")
    Vh = np.empty((k, n), np.complex128, order="F")
    info = z["zgesdd"](102, b"S", m, n, A.ctypes.data, m, S.ctypes.data, U.ctypes.data, m, Vh.ctypes.data, k)
    if info != 0:
        raise np.linalg.LinAlgError(f"zgesdd info {info}")
    return U, S, Vh


# OpenBLAS's thread count is one process-wide setting: the calls that change
# it for their own duration hold this lock, so that two host workers cannot
# interleave their set and restore
_BLAS_THREADS_LOCK = threading.RLock()


def _with_threads(z, threads, fn):
    with _BLAS_THREADS_LOCK:
        n0 = int(z["get_threads"]())
        z["set_threads"](C.c_int(max(1, threads)))
        try:
            return fn()
        finally:
            z["set_threads"](C.c_int(max(1, n0)))


def _one_thread(fn):
    """fn(lapacke) with the BLAS at one thread, or fn(None) without LAPACKE.
    The moments' SVDs and eig(B) are dense problems of at most a few hundred
    rows, which the threaded BLAS runs slower than one thread does (zgeev of a
    128 x 128 matrix: 13 ms at one thread against 16 ms at eight)."""
    z = _lapacke()
    if z is None:
        return fn(None)
    return _with_threads(z, 1, lambda: fn(z))


def _svdvals(A):
    return _one_thread(lambda z: _svd_lapacke(z, A, vals_only=True) if z else np.linalg.svd(A, compute_uv=False))


def _svd(A):
    return _one_thread(lambda z: _svd_lapacke(z, A) if z else np.linalg.svd(A, full_matrices=False))


def _eigvals(B):
    return _one_thread(lambda z: _eigvals_lapacke(z, B) if z else np.linalg.eigvals(B))


def _eigvals_lapacke(z, B):
    A = np.array(B, dtype=np.complex128, order="F", copy=True)
    n = A.shape[0]
    w = np.empty(n, np.complex128)
    info = z["zgeev"](102, b"N", b"N", n, A.ctypes.data, n, w.ctypes.data, None, 1, None, 1)
    if info != 0:
        raise np.linalg.LinAlgError(f"zgeev info {info}")
    return w


def _per_disk_host(jobs, fn):
    """fn(job, lapacke) for every job: on host threads with the BLAS at one
    thread per call when LAPACKE is found (ctypes releases the interpreter
    lock, NumPy's svd and eigvals hold it), else one after another with
    lapacke = None (NumPy). Same LAPACK routines either way. fn runs on pool
    threads while this thread holds the BLAS-thread lock, so it calls the
    LAPACKE wrappers directly (not _svd / _eigvals, which take the lock)."""
    z = _lapacke() if len(jobs) > 1 else None
    if z is None:
        return [fn(j, None) for j in jobs]
    from concurrent.futures import ThreadPoolExecutor

    def run():
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 1)) as pool:
            return list(pool.map(lambda j: fn(j, z), jobs))

    return _with_threads(z, 1, run)


def _eigvals_many(Bs):
    """eigvals of every matrix of Bs (None: no eigenvalues), beyn.jl:371,
    on host threads (see _per_disk_host)."""
    empty = np.zeros(0, complex)

    def one(B, z):
        if B is None:
            return empty
        return _eigvals_lapacke(z, B) if z else np.linalg.eigvals(B)

    return _per_disk_host(list(Bs), one)


def _B_from_moments(A0, A1, svd_tol, svd=None):
    """Thin SVD of A0, absolute rank, B = U_k^H A1 W_k Sigma_k^-1 (beyn.jl:286-320).
    Also takes (R, Q^H A1) of a device QR A0 = Q R: same S, W and B, U_R for U.
    svd: a thin-SVD function in place of numpy.linalg.svd."""
    U, S, Wh = svd(A0) if svd else _svd(A0)
    rk = int(np.count_nonzero(S >= svd_tol))
    Uk = U[:, :rk]
    Wk = Wh.conj().T[:, :rk]
    B = Uk.conj().T @ ((A1 @ Wk) / S[:rk][None, :])
    return B, Uk, rk, S


def solve_disks(solver, pts, k0s, R, nq=32, r=48, svd_tol=1e-14, rng=None, mixed=False, ws=None,
                return_info=False, regrow_ahead=True, **kw):
    """Eigenvalues of several disks from one device batch: construct_B_matrix
    for every disk (beyn.jl:257-322, one r -> 2r regrowth per disk, extending
    the probe block) with the contour nodes of all disks resident together.
    Returns a list of eigenvalue arrays, one per disk."""
    rng = rng if rng is not None else np.random.default_rng(0)
    ws = ws if ws is not None else Workspace(solver, pts)
    N = ws.dim
    k0s = np.atleast_1d(np.asarray(k0s, dtype=np.complex128))
    clk = time.perf_counter
    host = dict(create=0.0, moments=0.0, svd=0.0, B_eigvals=0.0)  # wall-clock ms of the host-visible phases
    ahead = regrow_ahead and 2 * r < N

    def draw():  # the probe block (and the regrowth block, see construct_B_matrix), drawn during the factorisation
        V = probe_matrix(N, r, rng)
        return np.asfortranarray(np.hstack([V, probe_matrix(N, r, rng)])) if ahead else V

    from concurrent.futures import ThreadPoolExecutor
    t = clk()
    with ThreadPoolExecutor(max_workers=1) as ex:
        fut = ex.submit(draw)
        bh = BeynHandle(ws, k0s, R, nq, mixed, **kw)
        host["create"] += (clk() - t) * 1e3
        try:
            V = fut.result()
        except BaseException:
            bh.close()
            raise
    info = dict(stats=[], rk=[], r=[], host_ms=host)
    # moments reduced on the device: per disk R (A0 = Q R) and Q^H A1, m x m
    try:
        t = clk()
        Rf, Cf = bh.moments_qr(V)
        host["moments"] += (clk() - t) * 1e3
        info["stats"].append(bh.last_stats)
        R1, C1 = ([a[:r, :r] for a in Rf], [c[:r, :r] for c in Cf]) if ahead else (Rf, Cf)
        t = clk()
        S = _per_disk_host(list(R1), lambda a, z: _svd_lapacke(z, a, vals_only=True) if z else np.linalg.svd(a, compute_uv=False))
        host["svd"] += (clk() - t) * 1e3
        rks = [int(np.count_nonzero(s >= svd_tol)) for s in S]
        grow = [rk == r and 2 * r < N for rk in rks]
        if ahead:
            R2, C2 = Rf, Cf
        elif any(grow):
            Vn = probe_matrix(N, r, rng)
            t = clk()
            R2, C2 = bh.moments_qr(Vn, append=True)
            host["moments"] += (clk() - t) * 1e3
            info["stats"].append(bh.last_stats)
    finally:
        t = clk()
        bh.close()
        host["create"] += (clk() - t) * 1e3
    t = clk()

    def one_disk(d, z):  # SVD of R, B and eig(B) of disk d
        Rd, Cd = (R2[d], C2[d]) if grow[d] else (R1[d], C1[d])
        if rks[d] == 0:
            return np.zeros(0, complex), 0, r
        B, _, rk, _ = _B_from_moments(Rd, Cd, svd_tol, svd=(lambda A: _svd_lapacke(z, A)) if z else None)
        if not rk:
            return np.zeros(0, complex), 0, Rd.shape[1]
        return (_eigvals_lapacke(z, B) if z else np.linalg.eigvals(B)), rk, Rd.shape[1]

    res = _per_disk_host(list(range(len(k0s))), one_disk)
    out = [x[0] for x in res]
    info["rk"] = [x[1] for x in res]
    info["r"] = [x[2] for x in res]
    host["B_eigvals"] += (clk() - t) * 1e3
    return (out, info) if return_info else out


def construct_B_matrix(solver, pts, N, k0, R, nq=64, r=48, svd_tol=1e-14, rng=None, mixed=False, ws=None,
                       max_refine=10, refine_tol=1e-6, return_info=False, regrow="extend", use_chebyshev=True,
                       cheb=None, fp32_sweeps=0, solve_block=0, node_chunk=0, resid_engine=0, basis=True, nb=0,
                       regrow_ahead=True):
    """construct_B_matrix (beyn.jl:257-322). Returns (B, Uk) [, info].

    regrow: when the rank saturates (rk == r) the reference draws a fresh
    N x 2r probe block and solves all 2r columns again (beyn.jl:291-309).
    "fresh" does the same; "extend" (default) keeps the r columns already
    solved and draws only r new ones, so the moments of the 2r block cost r
    new solves. The eigenvalues of B do not depend on the probe block.

    regrow_ahead (with "extend"): the r regrowth columns are drawn up front
    and solved together with the first r, so the nodes' solves and the mixed
    form's refinement run once on 2r columns instead of twice on r (the
    operators' residual digit planes are streamed half as often). The rank
    test still looks at the first r columns only (the leading r x r block of
    R in A0 = Q R is the R of those columns), and without saturation B comes
    from them alone, as in the reference; the extra columns are then work
    spent for nothing, so pass False when r is expected to exceed the count.

    basis=False skips U_k (returned as None): the moments stay on the device,
    A0 = Q R is factored there and only R and Q^H A1 (m x m) come back, so the
    SVD runs on R (same singular values and W as A0's, U = Q U_R) and
    B = U_R,k^H (Q^H A1) W_k Sigma_k^-1. The rank test, the regrowth and B are
    the reference's; only the order of the dense algebra differs."""
    rng = rng if rng is not None else np.random.default_rng(0)
    ws = ws if ws is not None else Workspace(solver, pts)
    if ws.dim != N:
        raise ValueError(f"N={N} does not match the operator dimension {ws.dim}")
    clk = time.perf_counter
    host = dict(create=0.0, moments=0.0, svd=0.0, B=0.0)  # wall-clock ms of the host-visible phases
    ahead = regrow == "extend" and regrow_ahead and 2 * r < N

    def draw():  # the probe block, drawn while the library assembles and factors
        V = probe_matrix(N, r, rng)
        return np.asfortranarray(np.hstack([V, probe_matrix(N, r, rng)])) if ahead else V

    from concurrent.futures import ThreadPoolExecutor
    t = clk()
    with ThreadPoolExecutor(max_workers=1) as ex:
        fut = ex.submit(draw)
        bh = BeynHandle(ws, k0, R, nq, mixed, max_refine, refine_tol, nb=nb, use_chebyshev=use_chebyshev, cheb=cheb,
                        fp32_sweeps=fp32_sweeps, solve_block=solve_block, node_chunk=node_chunk,
                        resid_engine=resid_engine)
        host["create"] += (clk() - t) * 1e3
        try:
            V = fut.result()
        except BaseException:
            bh.close()
            raise
    info = dict(stats=[], host_ms=host)
    moments = bh.moments if basis else bh.moments_qr
    try:
        t = clk()
        M0, M1 = moments(V)  # (A0, A1), or (R, Q^H A1)
        host["moments"] += (clk() - t) * 1e3
        info["stats"].append(bh.last_stats)
        if ahead:
            M0f, M1f = M0, M1
            if basis:
                M0, M1 = np.asfortranarray(M0f[:, :r]), np.asfortranarray(M1f[:, :r])
            else:
                M0, M1 = np.asfortranarray(M0f[:r, :r]), np.asfortranarray(M1f[:r, :r])
        # the saturation test needs only the singular values; the factors are
        # computed once, for the block that is finally used
        t = clk()
        S = _svdvals(M0)
        rk = int(np.count_nonzero(S >= svd_tol))
        if not (rk == r and 2 * r < N) and rk > 0:
            U, S, Wh = _svd(M0)
        host["svd"] += (clk() - t) * 1e3
        rused = r
        if rk == 0:
            out = (np.zeros((0, 0), complex), np.zeros((N, 0), complex) if basis else None)
            info.update(rk=0, r=r, S=S)
            return (*out, info) if return_info else out
        if rk == r:
            r_tmp = 2 * r
            if r_tmp < N and ahead:
                M0, M1 = M0f, M1f
                t = clk()
                U, S, Wh = _svd(M0)
                rk = int(np.count_nonzero(S >= svd_tol))
                host["svd"] += (clk() - t) * 1e3
                rused = r_tmp
            elif r_tmp < N:
                t = clk()
                if regrow == "extend":
                    Vn = probe_matrix(N, r_tmp - r, rng)
                    if basis:
                        A0n, A1n = bh.moments(Vn)
                        M0 = np.asfortranarray(np.hstack([M0, A0n]))
                        M1 = np.asfortranarray(np.hstack([M1, A1n]))
                    else:
                        M0, M1 = bh.moments_qr(Vn, append=True)
                else:
                    V = probe_matrix(N, r_tmp, rng)
                    M0, M1 = moments(V)
                host["moments"] += (clk() - t) * 1e3
                info["stats"].append(bh.last_stats)
                t = clk()
                U, S, Wh = _svd(M0)
                rk = int(np.count_nonzero(S >= svd_tol))
                host["svd"] += (clk() - t) * 1e3
                rused = r_tmp
    finally:
        t = clk()
        bh.close()
        host["create"] += (clk() - t) * 1e3
    t = clk()
    Uk = U[:, :rk]
    Wk = Wh.conj().T[:, :rk]
    tmp = (M1 @ Wk) / S[:rk][None, :]
    B = Uk.conj().T @ tmp
    host["B"] += (clk() - t) * 1e3
    info.update(rk=rk, r=rused, S=S)
    if not basis:
        Uk = None
    return (B, Uk, info) if return_info else (B, Uk)


def solve_vect(solver, pts, k0, R, nq=32, r=48, svd_tol=1e-14, rng=None, mixed=False, ws=None, **kw):
    """solve_vect (beyn.jl:364-375): eigenvalues lambda, U_k and eigenvectors Y of B."""
    N = ws.dim if ws is not None else None
    if N is None:
        ws = Workspace(solver, pts)
        N = ws.dim
    B, Uk, info = construct_B_matrix(solver, pts, N, k0, R, nq, r, svd_tol, rng, mixed, ws, return_info=True, **kw)
    if B.size == 0:
        return np.zeros(0, complex), Uk, np.zeros((0, 0), complex), info
    lam, Y = np.linalg.eig(B)
    return lam, Uk, Y, info


def solve(solver, pts, k0, R, nq=32, r=48, svd_tol=1e-14, rng=None, mixed=False, ws=None, return_info=False,
          **kw):
    """Eigenvalues only (beyn.jl:388-397): eigvals(B), no eigenvectors."""
    if ws is None:
        ws = Workspace(solver, pts)
    kw.setdefault("basis", False)  # eigenvalues only: U_k is not needed
    B, Uk, info = construct_B_matrix(solver, pts, ws.dim, k0, R, nq, r, svd_tol, rng, mixed, ws, return_info=True,
                                     **kw)
    t = time.perf_counter()
    lam = np.zeros(0, complex) if B.size == 0 else _eigvals(B)
    info["host_ms"]["eigvals"] = (time.perf_counter() - t) * 1e3
    return (lam, info) if return_info else lam


def _qr_reduce_host(A0, A1, threads=4):
    """(R, Q^H A1), m x m each, of the thin Householder QR A0 = Q R: LAPACK's
    zgeqrf and zunmqr (the routines behind the device path's cuSOLVER calls)
    with the BLAS at `threads`, or NumPy's qr without LAPACKE."""
    z = _lapacke()
    m = A0.shape[1]
    if not z or "zgeqrf" not in z:
        Q, R = np.linalg.qr(A0)
        return R, Q.conj().T @ A1
    a = np.array(A0, dtype=np.complex128, order="F", copy=True)
    c = np.array(A1, dtype=np.complex128, order="F", copy=True)
    n = a.shape[0]
    k = min(n, m)  # reflectors
    tau = np.empty(k, np.complex128)
    def run():
        info = z["zgeqrf"](102, n, m, a.ctypes.data, n, tau.ctypes.data)
        if info == 0:
            info = z["zunmqr"](102, b"L", b"C", n, m, k, a.ctypes.data, n, tau.ctypes.data, c.ctypes.data, n)
        return info

    info = _with_threads(z, threads, run)
    if info != 0:
        raise np.linalg.LinAlgError(f"zgeqrf / zunmqr info {info}")
    return np.asfortranarray(np.triu(a[:k, :m])), np.asfortranarray(c[:k, :m])


def _finish_host_qr(A0, A1, r, N, svd_tol):
    """_finish_ahead after the QR reduction of the moments on the host."""
    t = time.perf_counter()
    R, Cm = _qr_reduce_host(A0, A1)
    lam, rk, rused, _ = _finish_ahead(R, Cm, r, N, svd_tol)
    return lam, rk, rused, (time.perf_counter() - t) * 1e3


def _finish_ahead(M0f, M1f, r, N, svd_tol):
    """The host part of construct_B_matrix after moments_qr of the 2r-column
    block drawn up front (regrow_ahead, basis=False): the rank test on the
    leading r x r block of R, the thin SVD of the block finally used, B and
    eig(B) (beyn.jl:283-322, 371). Returns (eigenvalues, rk, r used, host ms)."""
    clk = time.perf_counter
    t = clk()
    ahead = M0f.shape[0] == 2 * r
    M0, M1 = (np.asfortranarray(M0f[:r, :r]), np.asfortranarray(M1f[:r, :r])) if ahead else (M0f, M1f)
    S = _svdvals(M0)
    rk = int(np.count_nonzero(S >= svd_tol))
    rused = r
    U = Wh = None
    if rk == r and ahead:
        M0, M1 = M0f, M1f
        U, S, Wh = _svd(M0)
        rk = int(np.count_nonzero(S >= svd_tol))
        rused = 2 * r
    elif rk > 0:
        U, S, Wh = _svd(M0)
    if rk == 0:
        return np.zeros(0, complex), 0, rused, (clk() - t) * 1e3
    B = U[:, :rk].conj().T @ ((M1 @ Wh.conj().T[:, :rk]) / S[:rk][None, :])
    lam = _eigvals(B)
    return lam, rk, rused, (clk() - t) * 1e3


def solve_pipelined(solver, pts, k0s, R, nq=32, r=48, svd_tol=1e-14, rngs=None, mixed=False, ws=None,
                    return_info=False, nb=0, use_chebyshev=True, cheb=None, max_refine=10, refine_tol=1e-6,
                    host_qr=True, overlap=True):
    """Eigenvalues of a sequence of disks (as `solve` on each, beyn.jl:388-397)
    through a pipeline:

    * overlap=True: two disks in flight on the device. A creator thread builds
      the next disk's handle (assembly and factorisation of its nodes, on the
      handle's own streams) while the calling thread runs the current disk's
      solves and moments, so the factorisation's panel chains and the solves'
      GEMMs and residuals of two disks share the GPU; two handles' operators
      are resident at once. overlap=False: one disk at a time on the device.
    * each disk's host part (the QR reduction of the moments with host_qr, the
      SVDs of R, B and eig(B)) on a worker thread, and the next disk's probe
      block drawn on another.

    The library, LAPACKE and NumPy's normal fills release the interpreter
    lock, so all of these run at once. The regrowth block is drawn up front
    (as `solve`'s default); a disk whose 2r probes would not fit (2r >= N) is
    finished the same way without regrowth, as construct_B_matrix does.

    host_qr: the moments come back whole and their QR reduction (A0 = Q R,
    Q^H A1) runs on the worker too (LAPACK zgeqrf / zunmqr), off the device's
    path (the last disk's, which nothing follows, stay on the device); False
    reduces them on the device (moments_qr) as `solve` does.

    rngs: one numpy Generator per disk (default: default_rng(d) for disk d);
    disk d draws its probes as `solve(..., rng=rngs[d])` would, so the
    eigenvalues are those of `solve` disk by disk. Returns the list of
    eigenvalue arrays [, info with per-disk rk, r and host times]."""
    from concurrent.futures import ThreadPoolExecutor
    ws = ws if ws is not None else Workspace(solver, pts)
    N = ws.dim
    k0s = list(np.atleast_1d(np.asarray(k0s, dtype=np.complex128)))
    Rs = np.broadcast_to(np.asarray(R, dtype=np.float64), (len(k0s),))
    rngs = rngs if rngs is not None else [np.random.default_rng(d) for d in range(len(k0s))]
    if len(rngs) != len(k0s):
        raise ValueError("one generator per disk")
    ahead = 2 * r < N
    clk = time.perf_counter

    def probes(g):  # numpy fills the normals without the interpreter lock
        V = probe_matrix(N, r, g)
        return np.asfortranarray(np.hstack([V, probe_matrix(N, r, g)])) if ahead else V

    def create(d):
        t = clk()
        bh = BeynHandle(ws, complex(k0s[d]), float(Rs[d]), nq, mixed, max_refine, refine_tol, nb=nb,
                        use_chebyshev=use_chebyshev, cheb=cheb)
        return bh, (clk() - t) * 1e3

    futs, stats, dev_ms, split = [], [], [], []
    nd = len(k0s)
    handles = []  # every handle made, closed on the way out whatever happens
    # host workers: the next disk's probes and the previous disk's host part;
    # the creator: the next disk's handle (overlap)
    with ThreadPoolExecutor(max_workers=2) as pool, ThreadPoolExecutor(max_workers=1) as maker:
        try:
            nxt = pool.submit(probes, rngs[0]) if nd else None
            hnext = maker.submit(create, 0) if (nd and overlap) else None
            for d in range(nd):
                t = clk()
                V = nxt.result()
                if d + 1 < nd:
                    nxt = pool.submit(probes, rngs[d + 1])
                t1 = clk()
                if overlap:
                    bh, c_ms = hnext.result()
                    handles.append(bh)
                    if d + 1 < nd:
                        hnext = maker.submit(create, d + 1)
                else:
                    bh, c_ms = create(d)
                    handles.append(bh)
                t2 = clk()
                # the last disk has no successor to overlap its host QR with:
                # its moments are reduced on the device
                hq = host_qr and d + 1 < nd
                try:
                    M0f, M1f = bh.moments(V) if hq else bh.moments_qr(V)
                    stats.append(bh.last_stats)
                finally:
                    t3 = clk()
                    bh.close()
                t4 = clk()
                dev_ms.append((t4 - t) * 1e3)
                split.append(((t1 - t) * 1e3, (t2 - t1) * 1e3, c_ms, (t3 - t2) * 1e3, (t4 - t3) * 1e3))
                futs.append(pool.submit(_finish_host_qr if hq else _finish_ahead, M0f, M1f, r, N, svd_tol))
            res = [f.result() for f in futs]
        finally:
            if overlap and hnext is not None and nd:
                try:
                    extra, _ = hnext.result()
                    if extra not in handles:
                        extra.close()
                except Exception:
                    pass
            for h in handles:
                h.close()
    out = [x[0] for x in res]
    if not return_info:
        return out
    info = dict(stats=stats, rk=[x[1] for x in res], r=[x[2] for x in res], host_ms=[x[3] for x in res],
                device_call_ms=dev_ms,
                call_split_ms=dict(zip(("probe_wait", "handle_wait", "create", "moments", "close"),
                                       [float(np.mean(c)) for c in zip(*split)])) if split else {})
    return out, info


def inside(lam, k0, R):
    return np.abs(lam - k0) <= R
