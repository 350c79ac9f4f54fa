"""GPU test of qbg_assemble_noalloc, the assembly entry point for callers that
cannot allocate device memory during the call (they own every buffer, e.g. a
pre-reserved arena, or run a loop where cudaMalloc's implicit device
synchronisation is not allowed).

The test owns the device buffers (it may allocate; the entry point may not),
calls the no-allocation entry point twice in a row with different
wavenumbers, and compares each result with the regular qbg_assemble output
(the kernels are the same, so the tolerance is the FP64 assembly tolerance of
the other GPU tests, 1e-12 relative). Around every call it reads the
library's allocator counters: a call may neither take a block from the cache
nor ask the driver for one. Alpert geometries are accepted in FP64 only; their
complex64 forms must be refused before anything is queued. This file is named
so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class DevBuf:
    def __init__(self, rt, nbytes):
        self.rt, self.nbytes = rt, nbytes
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), C.c_size_t(nbytes)) == 0

    def to_host(self, arr):
        assert self.rt.cudaMemcpy(C.c_void_p(arr.ctypes.data), self.ptr, C.c_size_t(self.nbytes), 2) == 0
        return arr

    def free(self):
        self.rt.cudaFree(self.ptr)


def _relerr(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _noalloc(qb, ws, ks, ptrs, **kw):
    """One no-allocation call; asserts the library's allocator saw no request."""
    before = qb.operators.pool_stats()
    qb.assemble_noalloc(ws, ks, ptrs, **kw)
    after = qb.operators.pool_stats()
    for key in ("live_bytes", "hits", "misses"):
        assert after[key] == before[key], (key, before, after)


def test_noalloc_matches_regular_assembly_twice(qb):
    from qbgpu import _lib
    rt = _cudart()
    b = qb.make_star()
    sol = qb.CFIE_kress(8.0, b)
    pts = qb.evaluate_points(sol, b, 30.0)
    ws = qb.Workspace(sol, pts)
    n = ws.dim
    for ks in ([30.0 + 0.5j, 29.8 - 0.2j, 30.1 + 0.0j], [31.0 + 0.1j, 29.5 + 0.3j]):
        bufs = [DevBuf(rt, n * n * 16) for _ in ks]
        try:
            _noalloc(qb, ws, ks, [int(bb.ptr.value) for bb in bufs])
            ref = qb.assemble(ws, ks)
            for bb, r in zip(bufs, ref):
                got = bb.to_host(np.empty((n, n), dtype=np.complex128, order="F"))
                assert _relerr(got, r) < 1e-12
        finally:
            for bb in bufs:
                bb.free()
    # DLP with derivatives: outputs ordered [A..., A'..., A''...]
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(10.0, b)
    pts = qb.evaluate_points(sol, b, 25.0)
    wsd = qb.Workspace(sol, pts)
    n = wsd.dim
    ks = [25.0, 25.3]
    bufs = [DevBuf(rt, n * n * 16) for _ in range(3 * len(ks))]
    try:
        _noalloc(qb, wsd, ks, [int(bb.ptr.value) for bb in bufs], deriv=True)
        ref = qb.assemble(wsd, ks, deriv=True)
        for bb, r in zip(bufs, ref):
            got = bb.to_host(np.empty((n, n), dtype=np.complex128, order="F"))
            assert _relerr(got, r) < 1e-12
    finally:
        for bb in bufs:
            bb.free()


def test_noalloc_alpert_fp64_and_refused_complex64(qb):
    from qbgpu import _lib
    rt = _cudart()
    b = qb.make_circle(1.0)
    sol = qb.CFIE_alpert(8.0, b, alpert_order=12)
    pts = qb.evaluate_points(sol, b, 20.0)
    ws = qb.Workspace(sol, pts)
    n = ws.dim
    ks = [20.0 + 0.2j, 20.4 + 0.0j]
    bufs = [DevBuf(rt, n * n * 16) for _ in ks]
    try:
        for _ in range(2):
            _noalloc(qb, ws, ks, [int(bb.ptr.value) for bb in bufs])
            ref = qb.assemble(ws, ks)
            for bb, r in zip(bufs, ref):
                got = bb.to_host(np.empty((n, n), dtype=np.complex128, order="F"))
                assert _relerr(got, r) < 1e-12
        for prec in ("mixed", "fp32"):
            before = qb.operators.pool_stats()
            with pytest.raises(_lib.QBGError) as ei:
                qb.assemble_noalloc(ws, ks, [int(bb.ptr.value) for bb in bufs], prec=prec)
            assert ei.value.status == _lib.QBG_ENOTSUP
            assert qb.operators.pool_stats() == before
    finally:
        for bb in bufs:
            bb.free()


def test_noalloc_rejects_oversized_request(qb):
    from qbgpu import _lib
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(10.0, b)
    pts = qb.evaluate_points(sol, b, 10.0)
    ws = qb.Workspace(sol, pts)
    ks = np.full(qb.operators.NOALLOC_MAX_K + 1, 10.0 + 0j)
    with pytest.raises(_lib.QBGError) as ei:
        qb.assemble_noalloc(ws, ks, [1] * len(ks))  # rejected before any pointer is used
    assert ei.value.status == _lib.QBG_EINVAL
    assert "at most" in str(ei.value)
