"""Device workspaces and operator assembly (host mirror of the reference API).

Reference seams replaced here:
* ``build_dlp_kress_workspace`` / ``build_cfie_kress_workspace``
  (dlp_kress.jl:679-712, cfie_kress.jl:230-270)  -> ``Workspace``
* ``construct_matrices!`` (dlp_kress.jl:1627-1679, cfie_kress.jl:893-929)
* ``construct_boundary_matrices!`` and ``..._with_derivatives!``
  (chebyshev_euclidian_helmholtz_dlp_kress.jl:1110-1144,
  chebyshev_euclidian_helmholtz_cfie_kress.jl:1431-1573)

All arithmetic runs in libqbgpu on the GPU; this module only packs the
O(N) geometry and moves matrices.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import _lib as L
from .solvers import as_list


def _concat(pts):
    pts = as_list(pts)
    offs = np.zeros(len(pts) + 1, dtype=np.int64)
    for a, p in enumerate(pts):
        offs[a + 1] = offs[a] + p.n
    cat = lambda f: np.ascontiguousarray(np.concatenate([f(p) for p in pts]), dtype=np.float64)
    arrs = dict(x=cat(lambda p: p.xy[:, 0]), y=cat(lambda p: p.xy[:, 1]),
                dx=cat(lambda p: p.tangent[:, 0]), dy=cat(lambda p: p.tangent[:, 1]),
                ddx=cat(lambda p: p.tangent_2[:, 0]), ddy=cat(lambda p: p.tangent_2[:, 1]),
                ts=cat(lambda p: p.ts), ws=cat(lambda p: p.ws))
    return offs, arrs


def _alpert_arrays(solver, pts_l):
    """Periodic Alpert caches of every component (cfie_alpert.jl:1351-1363),
    flattened for qbg_geom_create: nodes [6][j][n] with the components in
    their global order."""
    from .alpert import alpert_log_rule, periodic_cache
    rule = alpert_log_rule(solver.alpert_order)
    comps = solver.billiard.components
    caches = []
    for comp, p in zip(comps, pts_l):
        if len(comp) != 1:
            raise NotImplementedError("CFIE_alpert components must be single closed curves")
        caches.append(periodic_cache(comp[0], p, rule, solver.alpert_order))
    c0 = caches[0]
    nodes = np.concatenate([np.stack([c.rp, c.rm, c.innp, c.innm, c.sp, c.sm]) for c in caches], axis=2)
    return dict(a=rule.a, j=rule.j, ninterp=c0.ninterp, w=np.ascontiguousarray(rule.w),
                off=np.ascontiguousarray(np.stack([c0.offp, c0.offm]).astype(np.int64)),
                wt=np.ascontiguousarray(np.stack([c0.wtp, c0.wtm])),
                nodes=np.ascontiguousarray(nodes))


class Workspace:
    """Device-resident geometry for one discretisation (owns a qbg_geom)."""

    def __init__(self, solver, pts, reduction=None):
        """reduction: orbit maps (fund, fund_to_full, fund_to_scale); by default
        they follow the solver's symmetry (none: the full operator)."""
        lib = L.load()
        if reduction is None:
            from .symmetry import reduction as _red
            reduction = _red(solver, pts)
        self.solver = solver
        self.kind = solver.kind
        pts_l = as_list(pts)
        self.ds = np.ascontiguousarray(np.concatenate([np.asarray(p.ds, dtype=np.float64) for p in pts_l]))
        if self.kind == "dlp" and len(pts_l) != 1:
            raise ValueError("DLP_kress expects one BoundaryPointsCFIE component")
        self._offs, self._arrs = _concat(pts_l)
        d = L.GeomDesc()
        d.form = L.QBG_FORM_DLP if self.kind == "dlp" else L.QBG_FORM_CFIE
        d.ncomp = len(pts_l)
        d.comp_offsets = L.dptr(self._offs, C.c_int64)
        for f in ("x", "y", "dx", "dy", "ddx", "ddy", "ts", "ws"):
            setattr(d, f, L.dptr(self._arrs[f]))
        d.m = 0
        self._red = None
        if reduction is not None:
            fund, orbit, scale = reduction
            self._red = (np.ascontiguousarray(fund, dtype=np.int64), np.ascontiguousarray(orbit, dtype=np.int64),
                         np.ascontiguousarray(scale, dtype=np.complex128).view(np.float64))
            d.m = len(fund)
            d.norb = orbit.shape[1]
            d.fund = L.dptr(self._red[0], C.c_int64)
            d.orbit = L.dptr(self._red[1], C.c_int64)
            d.orbit_scale = L.dptr(self._red[2])
        d.quad = 0
        self._alp = None
        if getattr(solver, "alpert_order", None) is not None:
            self._alp = _alpert_arrays(solver, pts_l)
            a = self._alp
            d.quad = 1
            d.alpert_a, d.alpert_j, d.alpert_ninterp = a["a"], a["j"], a["ninterp"]
            d.alpert_w = L.dptr(a["w"])
            d.alpert_off = L.dptr(a["off"], C.c_int64)
            d.alpert_wt = L.dptr(a["wt"])
            d.alpert_nodes = L.dptr(a["nodes"])
        h = C.c_void_p()
        L.check(lib.qbg_geom_create(C.byref(d), C.byref(h)))
        self._h = h
        dim = C.c_int64()
        L.check(lib.qbg_geom_dim(h, C.byref(dim)))
        self.dim = int(dim.value)
        self.n_full = int(self._offs[-1])

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) and L.alive():
            L.load().qbg_geom_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_workspace(solver, pts, reduction=None) -> Workspace:
    return Workspace(solver, pts, reduction)


def _ks_array(ks) -> np.ndarray:
    k = np.ascontiguousarray(np.atleast_1d(np.asarray(ks, dtype=np.complex128)))
    return k


DEFAULT_CHEB = (15000, 5, 3000, 5)  # the reference's n_panels_h, M_h, n_panels_j, M_j


def assemble(ws: Workspace, ks, deriv: bool = False, mixed: bool = False, cheb=None,
             split_lo: bool = False) -> List[np.ndarray]:
    """Return [A(k)...] (+ [A'(k)...], [A''(k)...]) as Fortran-ordered arrays.

    cheb: None for direct evaluation of H0, H1, J0, J1; True or a tuple
    (n_panels_h, M_h, n_panels_j, M_j) for the Chebyshev-panel route.
    split_lo (mixed form only): also return the complex64 low words,
    [hi(k)..., lo(k)...] with hi + lo the kernel value to ~2^-48."""
    lib = L.load()
    k = _ks_array(ks)
    nk = len(k)
    nout = 2 if split_lo else (3 if deriv else 1)
    pc = L.prec_code(mixed)
    dt = np.complex128 if pc == L.QBG_PREC_FP64 else np.complex64
    outs = [np.empty((ws.dim, ws.dim), dtype=dt, order="F") for _ in range(nk * nout)]
    ptrs = (C.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
    kd = k.view(np.float64)
    flags = L.QBG_SPLIT_LO if split_lo else 0
    if cheb is None or cheb is False:
        L.check(lib.qbg_assemble(ws.handle, L.dptr(kd), nk, 1 if deriv else 0, pc, flags, ptrs))
    else:
        prm = L.ChebParams(*(DEFAULT_CHEB if cheb is True else cheb))
        L.check(lib.qbg_assemble_cheb(ws.handle, L.dptr(kd), nk, 1 if deriv else 0, pc, flags, C.byref(prm), ptrs))
    return outs


NOALLOC_MAX_K = 512  # QBG_NOALLOC_MAX_K in include/qbgpu.h


def assemble_noalloc(ws: Workspace, ks, dev_ptrs, deriv: bool = False, prec="fp64"):
    """Assembly into caller-owned device buffers without any device allocation
    inside the call (qbg_assemble_noalloc). ``dev_ptrs`` are integer device
    addresses, ordered as for ``assemble``; at most NOALLOC_MAX_K wavenumbers."""
    lib = L.load()
    k = _ks_array(ks)
    ptrs = (C.c_void_p * len(dev_ptrs))(*[int(p) for p in dev_ptrs])
    L.check(lib.qbg_assemble_noalloc(ws.handle, L.dptr(k.view(np.float64)), len(k), 1 if deriv else 0,
                                     L.prec_code(prec), ptrs))


def construct_matrices(solver, pts, ws: Workspace, k, derivs: bool = False):
    """construct_matrices!(solver, A[, A1, A2], pts, ws, k) -> A or (A, A1, A2)."""
    out = assemble(ws, [k], deriv=derivs)
    return tuple(out) if derivs else out[0]


def construct_boundary_matrices(solver, pts, zj: Sequence[complex], ws: Workspace = None, mixed=False):
    """construct_boundary_matrices!(Tbufs, solver, pts, zj) -> list of T(z_j)."""
    ws = ws if ws is not None else Workspace(solver, pts)
    return assemble(ws, zj, mixed=mixed)


def construct_boundary_matrices_with_derivatives(solver, pts, zj, ws: Workspace = None):
    ws = ws if ws is not None else Workspace(solver, pts)
    out = assemble(ws, zj, deriv=True)
    nk = len(np.atleast_1d(zj))
    return out[:nk], out[nk:2 * nk], out[2 * nk:]


def chebyshev_params(solver, pts, zj, ws: Workspace = None, npanels_h_init=15000, M_h_init=5, npanels_j_init=3000,
                     M_j_init=5, tol=1e-10, sampling_points=50000, max_iter=20, grow_M=2, strict=False):
    """chebyshev_params (chebyshev_optimal_panelization.jl:221-307) on the device.

    Returns (n_panels_h, M_h, n_panels_j, M_j, errors[H0, H1, J0, J1]). When
    max_iter is reached the best effort is returned (strict=True raises)."""
    ws = ws if ws is not None else Workspace(solver, pts)
    k = _ks_array(zj)
    prm = L.ChebParams(int(npanels_h_init), int(M_h_init), int(npanels_j_init), int(M_j_init))
    err = np.zeros(4)
    st = L.load().qbg_cheb_autotune(ws.handle, L.dptr(k.view(np.float64)), len(k), float(tol), int(sampling_points),
                                    int(max_iter), int(grow_M), C.byref(prm), L.dptr(err))
    if st != L.QBG_OK and (strict or st != L.QBG_ETIMEOUT):
        L.check(st)
    return prm.n_panels_h, prm.M_h, prm.n_panels_j, prm.M_j, err


def chebyshev_params_min_cost(solver, pts, zj, ws: Workspace = None, tol=1e-10, entries=None, terms_per_entry=1.0,
                              degrees=(5, 7, 9, 11, 13, 15), sampling_points=50000, bessel_cost=None,
                              tables_per_call=None, mixed: bool = True):
    """Panels of the lowest estimated assembly cost that still meet tol.

    For every degree M in ``degrees`` (kept fixed) the device tuner grows the
    panel counts until every interpolated H0, H1, J0, J1 is within tol. The
    cost of a candidate is the table build (one device Bessel evaluation,
    about ``bessel_cost`` series steps, per Lobatto node per panel per
    wavenumber) plus the series steps of the assembly (``entries`` matrix
    entries, ``terms_per_entry`` H evaluations each plus one J evaluation).
    The default ``bessel_cost`` is measured on GB300: one FP64 device Bessel
    evaluation costs about 150 steps of the complex64 forms' double-float
    series (1.55 ns vs 10.5 ps) and about 60 FP64 Clenshaw steps (FP64 form,
    ``mixed=False``). Returns (n_panels_h, M_h, n_panels_j, M_j, errors, cost)."""
    if bessel_cost is None:
        bessel_cost = 150.0 if mixed else 60.0
    ws = ws if ws is not None else Workspace(solver, pts)
    nk = len(np.atleast_1d(zj)) if tables_per_call is None else int(tables_per_call)
    entries = float(ws.dim) ** 2 * nk if entries is None else float(entries)
    best = None
    for M in degrees:
        # start from few panels; the tuner only grows them
        nh, Mh, nj, Mj, err = chebyshev_params(solver, pts, zj, ws=ws, npanels_h_init=200, M_h_init=M,
                                               npanels_j_init=50, M_j_init=M, tol=tol,
                                               sampling_points=sampling_points, max_iter=40, grow_M=0)
        if not np.all(err < tol):
            continue
        cost = nk * (nh * (Mh + 1) + nj * (Mj + 1)) * bessel_cost + entries * (terms_per_entry * Mh + Mj)
        if best is None or cost < best[-1]:
            best = (nh, Mh, nj, Mj, err, cost)
    if best is None:
        raise RuntimeError(f"no degree in {degrees} reached tol = {tol}")
    return best


def bessel01(z, f32: bool = False) -> np.ndarray:
    """Device J0, J1, Y0, Y1 at complex z (validation helper): shape (n, 4)."""
    lib = L.load()
    zz = np.ascontiguousarray(np.atleast_1d(np.asarray(z, dtype=np.complex128)))
    out = np.empty(4 * len(zz), dtype=np.complex128)
    L.check(lib.qbg_bessel01(L.dptr(zz.view(np.float64)), len(zz), 1 if f32 else 0, L.dptr(out.view(np.float64))))
    return out.reshape(-1, 4)


def cgemm(A, B, C=None, alpha=1.0, beta=0.0, engine: int = 1) -> np.ndarray:
    """Device complex64 GEMM alpha A B + beta C (validation helper).

    A: (M, K) or (batch, M, K); B: (K, N) or (batch, K, N). engine 0 = CUDA-core
    FMA tiles, 1 = tcgen05 tensor cores (the engine of the FP32 LU)."""
    lib = L.load()
    A = np.asarray(A, dtype=np.complex64)
    B = np.asarray(B, dtype=np.complex64)
    single = A.ndim == 2
    if single:
        A, B = A[None], B[None]
    nb, M, K = A.shape
    N = B.shape[2]
    if B.shape[:2] != (nb, K):
        raise ValueError("A and B shapes do not chain")
    Cin = np.zeros((nb, M, N), np.complex64) if C is None else np.asarray(C, np.complex64).reshape(nb, M, N)
    a = np.ascontiguousarray(A.transpose(0, 2, 1))  # column-major per matrix
    b = np.ascontiguousarray(B.transpose(0, 2, 1))
    c = np.array(Cin.transpose(0, 2, 1), order="C", copy=True)  # never write into the caller's C
    al = np.array([complex(alpha).real, complex(alpha).imag], np.float32)
    be = np.array([complex(beta).real, complex(beta).imag], np.float32)
    L.check(lib.qbg_cgemm_c64(int(engine), M, N, K, al.ctypes.data_as(L.C.POINTER(L.C.c_float)), L.vptr(a), M,
                              L.vptr(b), K, be.ctypes.data_as(L.C.POINTER(L.C.c_float)), L.vptr(c), M, nb))
    out = c.transpose(0, 2, 1)
    return out[0] if single else out


def zgemm_sub_tc(A, B, C):
    """C - A B in complex128 through the library's eight-digit tensor-core
    product (qbg_zgemm_sub_tc, validation helper). A: (batch, M, K) or (M, K),
    B: (batch, K, N), C: (batch, M, N). Returns the new C."""
    A3, B3, C3 = (np.asarray(x, dtype=np.complex128) for x in (A, B, C))
    single = A3.ndim == 2
    if single:
        A3, B3, C3 = A3[None], B3[None], C3[None]
    bsz, M, K = A3.shape
    N = B3.shape[2]
    a = np.ascontiguousarray(A3.transpose(0, 2, 1))  # column-major per matrix
    b = np.ascontiguousarray(B3.transpose(0, 2, 1))
    c = np.ascontiguousarray(C3.transpose(0, 2, 1))
    L.check(L.load().qbg_zgemm_sub_tc(M, N, K, L.vptr(a), M, L.vptr(b), K, L.vptr(c), M, bsz))
    out = c.transpose(0, 2, 1)
    return out[0] if single else out


def residual_c64(Th, Tl, X, V, engine: int = 0):
    """Device refinement residual R = V - (Th + Tl) X (validation helper).
    Th, Tl: (batch, n, n) complex64 (Tl may be None); X, V: (batch, n, L)
    complex128. engine 0 = tensor cores, 1 = compensated FP32, 2 = tensor cores
    from the leading six digits (the refinement's first residual). Returns (R, rmax)."""
    Th = np.asarray(Th, np.complex64)
    single = Th.ndim == 2
    Th = Th[None] if single else Th
    bsz, n, _ = Th.shape
    X = np.asarray(X, np.complex128).reshape(bsz, n, -1)
    V = np.asarray(V, np.complex128).reshape(bsz, n, -1)
    L_ = X.shape[2]
    f = lambda a: np.ascontiguousarray(a.transpose(0, 2, 1))
    th = f(Th)
    tl = f(np.asarray(Tl, np.complex64).reshape(bsz, n, n)) if Tl is not None else None
    x, v = f(X), f(V)
    r = np.empty_like(x)
    rmax = C.c_double(0.0)
    L.check(L.load().qbg_residual_c64(int(engine), n, L_, bsz, L.vptr(th), L.vptr(tl) if tl is not None else None,
                                      L.vptr(x), L.vptr(v), L.vptr(r), C.byref(rmax)))
    R = r.transpose(0, 2, 1)
    return (R[0] if single else R), float(rmax.value)


def launch_count() -> int:
    """Kernels launched by the library in this process (its own kernels, not cuSOLVER's)."""
    c = L.C.c_uint64(0)
    L.check(L.load().qbg_launch_count(L.C.byref(c)))
    return int(c.value)


def release_cached_memory() -> None:
    """Return every device block the library's caching allocator holds to the driver."""
    L.check(L.load().qbg_pool_release())


def pool_stats() -> dict:
    """Cached and live bytes of the library's device allocator, reuse hits and driver allocations."""
    v = [L.C.c_uint64(0) for _ in range(4)]
    L.check(L.load().qbg_pool_stats(*[L.C.byref(x) for x in v]))
    return dict(cached_bytes=int(v[0].value), live_bytes=int(v[1].value), hits=int(v[2].value),
                misses=int(v[3].value))


def set_gemm_engine(engine: int) -> None:
    """Engine of the complex64 GEMMs in the FP32 LU and solves: 0 FMA tiles, 1 tcgen05 with
    packed operand tiles (default), 2 tcgen05 with operands split in registers."""
    L.check(L.load().qbg_set_gemm_engine(int(engine)))


def sigma_min(ws: Workspace, ks) -> np.ndarray:
    lib = L.load()
    k = np.ascontiguousarray(np.atleast_1d(np.asarray(ks, dtype=np.float64)))
    sig = np.empty(len(k))
    L.check(lib.qbg_sigma_min(ws.handle, L.dptr(k), len(k), L.dptr(sig)))
    return sig


def adjoint_fredholm_matrix(ws: Workspace, k: float) -> np.ndarray:
    """adjoint_fredholm_matrix! (dlp_kress.jl:1451-1500) for a DLP workspace:
    A_adj[i, j] = delta_ij - D[j, i] ds_j / ds_i at real k (over the fundamental
    nodes on a reduced workspace)."""
    lib = L.load()
    out = np.empty((ws.dim, ws.dim), np.complex128, order="F")
    L.check(lib.qbg_adjoint_fredholm(ws.handle, float(k), ws.ds.ctypes.data, out.ctypes.data, 0))
    return out


def solve_vect_dlp(ws: Workspace, k: float):
    """solve_vect for the DLP solvers (dlp_kress.jl:1914-1949): the adjoint
    Fredholm matrix at k and smallest_nullvec_krylov! (dlp.jl:991-1004) on it.
    Returns (sigma, u): 1/|mu| for the eigenvalue mu of largest modulus of
    A_adj^-1 and its unit eigenvector (the boundary density)."""
    lib = L.load()
    sig = C.c_double()
    u = np.empty(ws.dim, np.complex128)
    L.check(lib.qbg_solve_vect(ws.handle, float(k), ws.ds.ctypes.data, C.byref(sig), u.ctypes.data))
    return sig.value, u
