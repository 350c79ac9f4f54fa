"""GPU: the reference's own test of this path, restated (test/solvertests.jl:39-49,
"EBIM DLP_kress_global_corners"): the 2 x 1 rectangle, DLP_kress_global_corners
with b = 15, kressq = 4 and no symmetry, compute_spectrum_ebim over
k in [18, 20] with dk(k) = 0.03 k^(-1/3) and the Krylov convention. The
reference asks that every computed k lie within 1e-3 of an analytical
eigenvalue sqrt((m pi / w)^2 + (n pi / h)^2) and that some be found; here
also that every analytical eigenvalue in the range be found."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rect_ks(w, h, k1, k2, mmax=40, nmax=40):
    return sorted(k for k in (math.sqrt((m * math.pi / w) ** 2 + (n * math.pi / h) ** 2)
                              for m in range(1, mmax + 1) for n in range(1, nmax + 1)) if k1 <= k <= k2)


def test_ebim_dlp_kress_global_corners_rectangle(qb):
    w, h, k1, k2 = 2.0, 1.0, 18.0, 20.0
    b = qb.make_rectangle(w, h)
    sol = qb.DLP_kress_global_corners(15.0, b, kressq=4)
    ks, tens = qb.ebim.compute_spectrum_ebim(sol, b, k1, k2, dk=lambda k: 0.03 * k ** (-1.0 / 3.0), use_krylov=True)
    ks = np.real(np.asarray(ks))
    true = np.array(_rect_ks(w, h, k1, k2))
    assert len(ks) > 0
    assert all(np.min(np.abs(true - k)) <= 1e-3 for k in ks), ks
    assert all(np.min(np.abs(ks - t)) <= 1e-3 for t in true), (true, ks)
