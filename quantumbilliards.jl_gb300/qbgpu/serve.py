"""Request server over the C ABI (qbg_serve_*): Beyn, EBIM and sweep requests
admitted against an HBM budget, run concurrently on the device, with queued
Beyn requests on the same geometry merged into one multi-disk batch.

The host part of a Beyn request (SVD of A0, rank, B, eigvals; beyn.jl:286-320,
371) runs in the client after the device part returns.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .beyn import _B_from_moments, probe_matrix
from .operators import Workspace

QBG_REQ_BEYN, QBG_REQ_EBIM, QBG_REQ_SWEEP = 0, 1, 2


ServeOpts, RequestDesc, RequestResult = L.ServeOpts, L.RequestDesc, L.RequestResult


def _lib():
    return L.load()


@dataclass
class Request:
    id: int
    kind: int
    t_submit: float
    buffers: dict = field(default_factory=dict)  # host arrays the device writes (kept alive here)
    meta: dict = field(default_factory=dict)
    result: dict = None


class Server:
    """qbg_server: ``hbm_budget`` bytes (0 = 80% of free), ``workers`` requests
    in flight, ``max_batch`` Beyn requests per device batch, ``max_sweeps``
    sigma_min sweeps running at once (others wait; Beyn and EBIM pass them)."""

    def __init__(self, hbm_budget: int = 0, workers: int = 4, max_batch: int = 8, max_sweeps: int = 1):
        lib = _lib()
        o = ServeOpts(int(hbm_budget), int(workers), int(max_batch), int(max_sweeps))
        h = C.c_void_p()
        L.check(lib.qbg_serve_create(C.byref(o), C.byref(h)))
        self._h = h
        self._lock = threading.Lock()

    # -- submission ---------------------------------------------------------
    def _submit(self, d: RequestDesc, req: Request) -> Request:
        rid = C.c_int64()
        L.check(_lib().qbg_serve_submit(self._h, C.byref(d), C.byref(rid)))
        req.id = int(rid.value)
        return req

    def submit_beyn(self, ws: Workspace, k0: complex, R: float, nq: int, V: np.ndarray, mixed=True) -> Request:
        V = np.asfortranarray(V, dtype=np.complex128)
        N, r = V.shape
        A0 = np.empty((N, r), np.complex128, order="F")
        A1 = np.empty((N, r), np.complex128, order="F")
        d = RequestDesc(kind=QBG_REQ_BEYN, geom=ws.handle, prec=L.prec_code(mixed), k0_re=complex(k0).real,
                        k0_im=complex(k0).imag, R=float(R), nq=int(nq), L=r, V=V.ctypes.data, A0=A0.ctypes.data,
                        A1=A1.ctypes.data)
        req = Request(0, QBG_REQ_BEYN, time.perf_counter(), dict(V=V, A0=A0, A1=A1, ws=ws),
                      dict(k0=complex(k0), R=float(R)))
        return self._submit(d, req)

    def submit_ebim(self, ws: Workspace, k: float) -> Request:
        N = ws.dim
        outs = [np.empty((N, N), np.complex128, order="F") for _ in range(3)]
        d = RequestDesc(kind=QBG_REQ_EBIM, geom=ws.handle, prec=0, k=float(k), out_A=outs[0].ctypes.data,
                        out_dA=outs[1].ctypes.data, out_ddA=outs[2].ctypes.data)
        return self._submit(d, Request(0, QBG_REQ_EBIM, time.perf_counter(), dict(outs=outs, ws=ws), dict(k=k)))

    def submit_sweep(self, ws: Workspace, ks) -> Request:
        ks = np.ascontiguousarray(np.asarray(ks, dtype=np.float64))
        sig = np.empty(len(ks))
        d = RequestDesc(kind=QBG_REQ_SWEEP, geom=ws.handle, prec=0, ks=ks.ctypes.data, nk=len(ks),
                        sig=sig.ctypes.data)
        return self._submit(d, Request(0, QBG_REQ_SWEEP, time.perf_counter(), dict(ks=ks, sig=sig, ws=ws)))

    # -- completion ---------------------------------------------------------
    def poll(self, req: Request) -> bool:
        done = C.c_int32()
        L.check(_lib().qbg_serve_poll(self._h, req.id, C.byref(done)))
        return bool(done.value)

    def wait(self, req: Request, timeout: float = -1.0, svd_tol: float = 1e-12) -> dict:
        """Waits for the device part, then finishes a Beyn request on the host
        (rank test, B, eigvals). Raises on a failed request."""
        res = RequestResult()
        L.check(_lib().qbg_serve_wait(self._h, req.id, float(timeout), C.byref(res)))
        L.check(res.status)
        out = dict(batched=res.batched, queue_ms=res.queue_ms, run_ms=res.run_ms)
        b = req.buffers
        if req.kind == QBG_REQ_BEYN:
            B, Uk, rk, S = _B_from_moments(b["A0"], b["A1"], svd_tol)
            out.update(lam=np.linalg.eigvals(B) if rk else np.zeros(0, complex), rk=rk, A0=b["A0"], A1=b["A1"])
        elif req.kind == QBG_REQ_EBIM:
            out.update(A=b["outs"][0], dA=b["outs"][1], ddA=b["outs"][2])
        else:
            out.update(sig=b["sig"])
        out["latency_ms"] = (time.perf_counter() - req.t_submit) * 1e3
        req.result = out
        return out

    def close(self):
        if getattr(self, "_h", None) and L.alive():
            _lib().qbg_serve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Server", "Request", "probe_matrix"]
