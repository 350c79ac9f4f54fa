"""CPU oracle for the boundary-integral hot path — TEST INFRASTRUCTURE ONLY.

Nothing in the product imports this package. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` use it, and only as the checker or as the timed CPU
restatement of the reference algorithm.

Every function is a plain FP64 NumPy/SciPy restatement of the reference
(QuantumBilliards.jl v0.1.0) and cites the file:line it follows. Special
functions come from SciPy's AMOS wrappers (``hankel1``, ``jv``), which is the
same AMOS code the reference reaches through SpecialFunctions.jl.

Parity status: the reference cannot run here (no Julia on either machine), so
the oracle is pinned by known answers instead of reference-generated vectors:
circle Dirichlet eigenvalues (zeros of J_m), mpmath Hankel values, and the
Kress quadrature weights' closed form (tests/golden/).
"""
