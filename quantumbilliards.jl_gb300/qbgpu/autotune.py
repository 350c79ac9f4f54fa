"""Autotuner of the batched LU plan behind the Beyn step.

The plan has four knobs, none of which changes the mathematics (the factors
and pivots are those of LAPACK's getrf up to rounding in the trailing
updates' summation order):

* ``nb``: panel width of the blocked LU (32 or 64 columns), per Beyn handle;
* ``outer``: panels per outer block of the two-level factorisation (the
  trailing matrix right of an outer block is updated once, with
  K = outer * nb), process-wide;
* ``parts``: contiguous parts of the operator batch factored and solved on
  their own streams, so one part's panels overlap another part's tensor-core
  updates, process-wide (read when a handle is created);
* ``cluster``: the panel form: -1 automatic (the 8-CTA cluster panel for
  batches of at most 4 operators per part, one CTA per panel otherwise),
  0 always one CTA, 1 the cluster wherever the panel fits it.

``tune_beyn`` times whole Beyn steps (assembly, factorisation, solves,
moments and the host rank test and eigenvalues) of the caller's own workload
and keeps the fastest plan, by coordinate descent: parts, then outer, then
nb, then the panel form, each from the best so far. The plan is left set in
the library and returned (pass ``nb`` on to ``solve`` / ``solve_disks``).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib as L

__all__ = ["lu_plan", "set_lu_plan", "tune_beyn"]


def lu_plan() -> dict:
    """The library's current LU plan: outer, cluster (-1 automatic), parts."""
    o, c, p = C.c_int32(), C.c_int32(), C.c_int32()
    L.check(L.load().qbg_get_lu_plan(C.byref(o), C.byref(c), C.byref(p)))
    return {"outer": o.value, "cluster": c.value, "parts": p.value}


def set_lu_plan(outer=None, cluster=None, parts=None):
    """Sets the given knobs (None keeps the current value)."""
    cur = lu_plan()
    L.check(L.load().qbg_set_lu_plan(int(outer if outer is not None else cur["outer"]),
                                     int(cluster if cluster is not None else cur["cluster"]),
                                     int(parts if parts is not None else cur["parts"])))


def tune_beyn(solver, pts, ws, k0, R, nq, r, mixed=True, cheb=None, svd_tol=1e-12, seed=0, reps=2,
              parts=(2, 4, 8), outers=(2, 4, 8), nbs=(64, 32), clusters=(1,), pipelined=0):
    """Times Beyn steps of this workload under candidate plans and keeps the
    fastest. pipelined > 0 times each plan on `solve_pipelined` over that many
    disks (the per-disk time with two disks in flight) instead of one `solve`
    call. Returns dict(nb, outer, parts, cluster, ms, table, tune_s): ``table``
    lists every plan tried with its median time per disk in ms."""
    from .beyn import solve, solve_pipelined

    t_start = time.perf_counter()
    table = []

    def one(kw):
        if pipelined > 0:
            rngs = [np.random.default_rng(seed) for _ in range(pipelined)]
            solve_pipelined(solver, pts, [k0] * pipelined, R, rngs=rngs, **kw)
        else:
            solve(solver, pts, k0, R, rng=np.random.default_rng(seed), **kw)

    def run(nb, outer, npart, cluster=-1):
        set_lu_plan(outer=outer, cluster=cluster, parts=npart)
        kw = dict(nq=nq, r=r, svd_tol=svd_tol, mixed=mixed, ws=ws, cheb=cheb, nb=nb)
        one(kw)  # warm: buffers of this plan
        ts = []
        for _ in range(max(1, reps)):
            t0 = time.perf_counter()
            one(kw)
            ts.append((time.perf_counter() - t0) / max(1, pipelined))
        ms = 1e3 * float(np.median(ts))
        table.append({"nb": nb, "outer": outer, "parts": npart, "cluster": cluster, "ms": ms})
        return ms

    cur = lu_plan()
    best = {"nb": nbs[0], "outer": cur["outer"], "parts": cur["parts"], "cluster": -1}
    best["ms"] = run(best["nb"], best["outer"], best["parts"])
    for p in parts:
        if p != best["parts"]:
            ms = run(best["nb"], best["outer"], p)
            if ms < best["ms"]:
                best.update(parts=p, ms=ms)
    for o in outers:
        if o != best["outer"]:
            ms = run(best["nb"], o, best["parts"])
            if ms < best["ms"]:
                best.update(outer=o, ms=ms)
    for nb in nbs:
        if nb != best["nb"]:
            # the same outer-block width in columns
            o = max(1, min(16, best["outer"] * best["nb"] // nb))
            ms = run(nb, o, best["parts"])
            if ms < best["ms"]:
                best.update(nb=nb, outer=o, ms=ms)
    for c in clusters:
        if c != best["cluster"]:
            ms = run(best["nb"], best["outer"], best["parts"], c)
            if ms < best["ms"]:
                best.update(cluster=c, ms=ms)
    set_lu_plan(outer=best["outer"], cluster=best["cluster"], parts=best["parts"])
    best["table"] = table
    best["tune_s"] = time.perf_counter() - t_start
    return best
