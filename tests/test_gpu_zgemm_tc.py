"""GPU: complex128 products C - A B on the tensor cores from eight 7-bit
digits per operand (qbg_zgemm_sub_tc, the routine behind the FP64 LU's
blocked updates) against an extended-precision NumPy product.

Elementwise bound |C' - C'_exact| <= 4e-15 (|A| |B|)_ij + 2^-52 |C'_exact|_ij:
the digits cut each operand to 56 bits of its row (A) or column (B) maximum,
so a term's error is ~2^-55 max|A_i.| max|B_.j|, and the last term is the
final FP64 rounding of C - A B. Cases: ragged sizes (rows, k and columns off
the 128 / 8 / 32 tiles, whose images are zero-filled), rows of A spanning 16
orders of magnitude, K = 256 (the LU's outer block), a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _exact(A, B, C):
    ld = np.clongdouble
    R = C.astype(ld) - A.astype(ld) @ B.astype(ld)
    return R, np.abs(A) @ np.abs(B)


@pytest.mark.parametrize("M,N,K,b,row_scale", [(300, 70, 64, 2, False), (520, 130, 256, 1, True),
                                               (129, 33, 17, 3, False), (1024, 256, 256, 2, False)])
def test_zgemm_sub_tc_vs_exact(qb, M, N, K, b, row_scale):
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((b, M, K)) + 1j * rng.standard_normal((b, M, K))
    if row_scale:
        A *= 10.0 ** rng.uniform(-8, 8, (b, M, 1))
    B = rng.standard_normal((b, K, N)) + 1j * rng.standard_normal((b, K, N))
    C = rng.standard_normal((b, M, N)) + 1j * rng.standard_normal((b, M, N))
    out = qb.zgemm_sub_tc(A, B, C)
    ref, bound = _exact(A, B, C)
    err = np.abs(out.astype(np.clongdouble) - ref).astype(np.float64)
    allowed = 4e-15 * bound + 2.0 ** -52 * np.abs(ref).astype(np.float64)
    ratio = np.max(err / allowed)
    print(f"M={M} N={N} K={K} b={b}: max err/allowed {ratio:.3e}")
    assert ratio <= 1.0
