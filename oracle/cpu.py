"""Host-core restatement of the reference's CFIE Beyn path (test
infrastructure and the timed CPU baseline only).

The reference's default complex-k route (use_chebyshev = true,
beyn.jl:778-921 and 257-322): the panels are tuned once by
chebyshev_params (tol 1e-13 in compute_spectrum_beyn), every contour node's
tables are fitted to AMOS values, the CFIE matrix is assembled by Clenshaw on
those panels (cpu_cfie.c, OpenMP over columns), factored by LAPACK (lu!) and
solved for the r probe columns and, after the rank saturates, for a fresh
block of 2r (beyn.jl:291-309). The tables are fitted in a thread pool and
LAPACK uses its own threads, so every host core is busy.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import scipy.linalg as sla
from scipy import special as sp

from . import assembly as OA, beyn as OB, chebyshev as OC

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_cfie.c"
LIB = HERE / "liboracle_cpu.so"
_lib = None


def build(force: bool = False) -> Path:
    """gcc -O3 -fopenmp; rebuilt when the source is newer than the library."""
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        dp, i64 = C.POINTER(C.c_double), C.POINTER(C.c_int64)
        L.oracle_cfie_cheb.restype = C.c_int
        L.oracle_cfie_cheb.argtypes = ([C.c_int, i64] + [dp] * 9 + [C.c_double, C.c_double, C.c_int, C.c_int,
                                        C.c_double, C.c_double, dp, dp, C.c_int, C.c_int, C.c_double, dp, dp,
                                        C.c_double, dp])
        L.oracle_hankel01_small.restype = None
        L.oracle_hankel01_small.argtypes = [dp, C.c_int64, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def hankel01_small(z):
    z = np.ascontiguousarray(np.asarray(z, dtype=np.complex128))
    out = np.empty((len(z), 2), dtype=np.complex128)
    lib().oracle_hankel01_small(_p(z.view(np.float64)), len(z), _p(out.view(np.float64)))
    return out[:, 0], out[:, 1]


class Geometry:
    """Concatenated node arrays of the CFIE components (outer first)."""

    def __init__(self, pts):
        pts = pts if isinstance(pts, list) else [pts]
        self.pts = pts
        cat = lambda f: np.ascontiguousarray(np.concatenate([f(p) for p in pts]), dtype=np.float64)
        self.x, self.y = cat(lambda p: p.xy[:, 0]), cat(lambda p: p.xy[:, 1])
        self.dx, self.dy = cat(lambda p: p.tangent[:, 0]), cat(lambda p: p.tangent[:, 1])
        self.ddx, self.ddy = cat(lambda p: p.tangent_2[:, 0]), cat(lambda p: p.tangent_2[:, 1])
        self.sig, self.w = cat(lambda p: p.ts), cat(lambda p: p.ws)
        self.rcol = cat(lambda p: OA.kress_R_column(p.n))
        self.offs = np.array(OA.component_offsets(pts), dtype=np.int64)
        self.N = int(self.offs[-1])
        self.rmin, self.rmax = OC.r_range(pts)


def tables(k, g: Geometry, params, pool=None):
    """Panel coefficients of H0, H1 (on [rmin, rmax]) and J0, J1 (on [0, rmax])."""
    nh, Mh, nj, Mj = params
    jobs = [(g.rmin, g.rmax, nh, Mh, lambda z: sp.hankel1(0, z)), (g.rmin, g.rmax, nh, Mh, lambda z: sp.hankel1(1, z)),
            (0.0, g.rmax, nj, Mj, OC._jfun(k, 0)), (0.0, g.rmax, nj, Mj, OC._jfun(k, 1))]
    mk = lambda a: np.ascontiguousarray(OC.Plan(k, *a).c, dtype=np.complex128)
    return list(pool.map(mk, jobs)) if pool is not None else [mk(a) for a in jobs]


def cfie_matrix(g: Geometry, k, params, pool=None, small_cut=0.2):
    """T(k) = I - (D + i k S) through the panels, N x N complex128 (Fortran order)."""
    c = tables(complex(k), g, params, pool)
    out = np.empty((g.N, g.N), dtype=np.complex128, order="F")
    nh, Mh, nj, Mj = params
    L = lib()
    L.oracle_cfie_cheb(len(g.pts), g.offs.ctypes.data_as(C.POINTER(C.c_int64)), _p(g.x), _p(g.y), _p(g.dx),
                       _p(g.dy), _p(g.ddx), _p(g.ddy), _p(g.sig), _p(g.w), _p(g.rcol), float(np.real(k)),
                       float(np.imag(k)), int(nh), int(Mh), float(g.rmin), float(g.rmax), _p(c[0].view(np.float64)),
                       _p(c[1].view(np.float64)), int(nj), int(Mj), float(g.rmax), _p(c[2].view(np.float64)),
                       _p(c[3].view(np.float64)), float(small_cut),
                       C.cast(out.ctypes.data, C.POINTER(C.c_double)))
    return out


def chebyshev_params(g: Geometry, zj, tol=1e-13, npanels_h_init=15000, M_h_init=5, npanels_j_init=3000, M_j_init=5,
                     sampling_points=50000, max_iter=20, grow_panels=1.5, grow_M=2, pool=None):
    """chebyshev_params (chebyshev_optimal_panelization.jl:221-307): the
    maximum absolute error of the interpolated H0, H1 (on linspace(rmin, rmax))
    and J0, J1 (on linspace(0, rmax)) over every contour node must fall below
    tol; otherwise the failing family grows its panel count by 1.5, or its
    degree by 2 on every fifth iteration. Returns (nh, Mh, nj, Mj, errors)."""
    rsH = np.linspace(g.rmin, g.rmax, sampling_points)
    rsJ = np.linspace(0.0, g.rmax, sampling_points)
    nh, Mh, nj, Mj = npanels_h_init, M_h_init, npanels_j_init, M_j_init

    def errs(job):
        k, rs, lo, n, M, nu, fam = job
        f = (lambda z: sp.hankel1(nu, z)) if fam == "h" else OC._jfun(k, nu)
        p = OC.Plan(k, lo, g.rmax, n, M, f)
        return float(np.max(np.abs(p(rs) - f(k * rs))))

    e = None
    for it in range(1, max_iter + 1):
        jobs = []
        for z in zj:
            jobs += [(z, rsH, g.rmin, nh, Mh, 0, "h"), (z, rsH, g.rmin, nh, Mh, 1, "h"),
                     (z, rsJ, 0.0, nj, Mj, 0, "j"), (z, rsJ, 0.0, nj, Mj, 1, "j")]
        ev = np.array(list(pool.map(errs, jobs)) if pool is not None else [errs(j) for j in jobs]).reshape(-1, 4)
        e = ev.max(axis=0)
        okH = e[0] < tol and e[1] < tol
        okJ = e[2] < tol and e[3] < tol
        if okH and okJ:
            return nh, Mh, nj, Mj, e
        if not okH:
            if it % 5 == 0:
                Mh += grow_M
            else:
                nh = int(math.ceil(grow_panels * nh))
        if not okJ:
            if it % 5 == 0:
                Mj += grow_M
            else:
                nj = int(math.ceil(grow_panels * nj))
    return nh, Mh, nj, Mj, e


class BeynCPU:
    """One Beyn disk on the host cores, node by node (the reference's
    construct_B_matrix with its single r -> 2r regrowth drawing a fresh 2r
    block). ``node(j)`` does node j's assembly, LU and both solves;
    ``finish()`` forms the moments, the rank test, B and eig(B)."""

    def __init__(self, pts, k0, R, nq, r, svd_tol, seed, params, threads=None):
        self.g = Geometry(pts)
        self.k0, self.R, self.nq, self.r, self.svd_tol = complex(k0), float(R), int(nq), int(r), float(svd_tol)
        self.params = tuple(int(x) for x in params[:4])
        self.zj, self.wj = OB.contour(self.k0, self.R, self.nq)
        rng = np.random.default_rng(seed)
        self.V1 = OB.probe_matrix(self.g.N, self.r, rng)
        self.V2 = OB.probe_matrix(self.g.N, 2 * self.r, rng)
        self.pool = ThreadPoolExecutor(threads or os.cpu_count())
        self.X1 = [None] * self.nq
        self.X2 = [None] * self.nq

    def node(self, j):
        T = cfie_matrix(self.g, self.zj[j], self.params, self.pool)
        f = sla.lu_factor(T, overwrite_a=True, check_finite=False)
        self.X1[j] = sla.lu_solve(f, self.V1, check_finite=False)
        self.X2[j] = sla.lu_solve(f, self.V2, check_finite=False)

    def finish(self):
        def mom(Xs):
            A0 = sum(w * X for w, X in zip(self.wj, Xs))
            A1 = sum((w * z) * X for w, z, X in zip(self.wj, self.zj, Xs))
            return A0, A1

        A0, A1 = mom(self.X1)
        S = np.linalg.svd(A0, compute_uv=False)
        rk = int(np.count_nonzero(S >= self.svd_tol))
        rused = self.r
        if rk == self.r and 2 * self.r < self.g.N:
            A0, A1 = mom(self.X2)
            rused = 2 * self.r
        U, S, Wh = np.linalg.svd(A0, full_matrices=False)
        rk = int(np.count_nonzero(S >= self.svd_tol))
        if rk == 0:
            return np.zeros(0, complex), rk, rused
        B = U[:, :rk].conj().T @ ((A1 @ Wh.conj().T[:, :rk]) / S[:rk][None, :])
        return np.linalg.eigvals(B), rk, rused

    def close(self):
        self.pool.shutdown()
