"""Complex64 GEMM engines of the FP32 LU: tcgen05 tensor cores (3xTF32) with
packed operand tiles streamed by bulk copies for large products (engine 1:
128 x 128 complex tiles, real N = 256 per MMA, when N spans two such tiles and
the grid fills the device or N fills most of one tile, else 128 x 32) or
with operands split in registers (engine 2), and CUDA-core FMA tiles (engine
0), against a complex128 NumPy product of the same inputs.

Tolerance: |C - C_ref| <= 4e-6 * (|alpha| |A| |B| + |beta| |C0|) elementwise,
i.e. FP32-class accuracy (unit roundoff 6e-8 times a K-term accumulation).
A plain 1xTF32 product (10-bit mantissa) fails this by two orders of magnitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


SHAPES = [
    (1, 1, 1, 1),        # smallest
    (200, 70, 40, 2),    # ragged tiles in M, N, K
    (64, 64, 64, 3),     # triangular-solve update shape
    (1984, 1984, 64, 2), # LU trailing update at n = 2048, nb = 64
    (2048, 64, 2048, 1), # refinement product T X
    (1792, 1792, 256, 2),# LU trailing update of an outer block (K = 256)
    (257, 33, 17, 3),    # ragged everywhere, KT = 2
    (1000, 40, 334, 3),  # ragged rows and columns, k tail of one pair
    (512, 64, 512, 2),   # triangular-solve product shape
    (640, 1, 96, 1),     # one column
    (1000, 1100, 77, 3), # wide 128 x 128 tiles: ragged M, N and K
    (129, 257, 33, 60),  # wide tiles, one row and one column past a tile, many matrices
    (1792, 128, 256, 6), # one wide tile in N: a triangular-solve product of a 128-column block
    (1000, 100, 64, 8),  # one mostly full wide tile, ragged M and N
]


@pytest.mark.parametrize("M,N,K,batch", SHAPES)
@pytest.mark.parametrize("engine", [1, 2, 0])
def test_cgemm_engines(qb, M, N, K, batch, engine):
    rng = np.random.default_rng(M * 7 + N * 3 + K + batch)
    A, B, C0 = _rand(rng, (batch, M, K)), _rand(rng, (batch, K, N)), _rand(rng, (batch, M, N))
    alpha, beta = complex(-1.0, 0.25), complex(0.5, -1.0)
    got = qb.cgemm(A, B, C0, alpha, beta, engine=engine)
    A64, B64, C64 = A.astype(np.complex128), B.astype(np.complex128), C0.astype(np.complex128)
    ref = alpha * (A64 @ B64) + beta * C64
    bound = abs(alpha) * (np.abs(A64) @ np.abs(B64)) + abs(beta) * np.abs(C64)
    err = np.abs(got - ref) / bound
    assert err.max() < 4e-6, (engine, err.max())


def test_cgemm_beta_zero_ignores_c(qb):
    rng = np.random.default_rng(5)
    A, B = _rand(rng, (130, 17)), _rand(rng, (17, 33))
    C0 = np.full((130, 33), np.nan + 1j * np.nan, np.complex64)
    got = qb.cgemm(A, B, C0, 1.0, 0.0, engine=1)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-5


def test_beyn_mixed_same_eigenvalues_both_engines(qb):
    """The FP32 LU with either engine refines to the same FP64-accurate moments."""
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 512, 40.0)
    ws = qb.Workspace(sol, pts)
    # physical eigenvalues: inside the disk with |Im| < 1e-6 (spurious ones sit off the axis)
    sel = lambda l: np.sort_complex(l[qb.beyn.inside(l, 40.0, 0.5) & (np.abs(l.imag) < 1e-6)])
    res = {}
    try:
        for eng in (0, 1, 2):
            qb.set_gemm_engine(eng)
            lam = qb.solve(sol, pts, 40.0 + 0j, 0.5, nq=24, r=24, svd_tol=1e-12, rng=np.random.default_rng(3),
                           mixed=True, ws=ws)
            res[eng] = sel(lam)
    finally:
        qb.set_gemm_engine(1)
    plain = qb.solve(sol, pts, 40.0 + 0j, 0.5, nq=24, r=24, svd_tol=1e-12, rng=np.random.default_rng(3),
                     mixed=False, ws=ws)
    plain = sel(plain)
    assert len(res[0]) == len(res[1]) == len(res[2]) == len(plain) > 0
    for eng in (0, 1, 2):
        assert np.max(np.abs(res[eng] - plain) / np.abs(plain)) < 1e-10, eng


@pytest.mark.parametrize("n_nodes,L", [(1000, 24), (390, 8), (2050, 136)])
def test_mixed_moments_ragged_solve_blocks(qb, n_nodes, L):
    """Mixed moments equal the FP64 moments for sizes that are not multiples of
    the 256-row solve block (partial doubling pairs) and for more probe columns
    than one solve chunk (128)."""
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, n_nodes, 20.0)
    ws = qb.Workspace(sol, pts)
    V = qb.probe_matrix(ws.dim, L, np.random.default_rng(11))
    out = {}
    for mixed in (False, True):
        bh = qb.BeynHandle(ws, 20.0 + 0.1j, 0.4, 8, mixed=mixed, use_chebyshev=False)
        out[mixed] = bh.moments(V)
        bh.close()
    for a, r in zip(out[True], out[False]):
        assert np.max(np.abs(a - r)) / np.max(np.abs(r)) < 1e-10


def test_lu_split_streams_bitwise_equal(qb):
    """The LU and the triangular solves of the mixed form run parts of the
    operator batch on several streams (QBG_LU_SPLIT parts); that changes
    nothing in the results: moments bit-identical to the one-stream run
    (QBG_LU_SPLIT=0) for 2, 3 and 4 parts, also for an odd batch (parts of
    different sizes)."""
    import os
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, 700, 30.0)
    ws = qb.Workspace(sol, pts)
    V = qb.probe_matrix(ws.dim, 24, np.random.default_rng(5))
    for nq in (16, 15):
        out = {}
        for split in ("0", "2", "3", "4"):
            os.environ["QBG_LU_SPLIT"] = split
            try:
                bh = qb.BeynHandle(ws, 30.0 + 0.05j, 0.4, nq, mixed=True)
                out[split] = bh.moments(V)
                bh.close()
            finally:
                os.environ.pop("QBG_LU_SPLIT", None)
        for split in ("2", "3", "4"):
            for a, r in zip(out[split], out["0"]):
                assert np.array_equal(a, r), (nq, split)
