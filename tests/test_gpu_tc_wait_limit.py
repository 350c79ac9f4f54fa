"""The failure path of the tensor-core GEMM's bounded waits, driven without a
fault: with the pipeline-wait poll limit set to 0 every pipeline mbarrier wait
gives up at once, the kernel records its sticky error flag, drains what it
started (with the full limit), frees its tensor memory and returns without
writing C; the entry reports QBG_ECUDA and delivers no product. After the
limit is restored and the flag cleared the same product runs and is correct.
Both engines: packed operands with bulk copies (engine 1) and
register-staged operands (engine 2)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_limit_gives_up_cleanly_then_recovers(qb):
    from qbgpu import _lib
    lib = _lib.load()
    rng = np.random.default_rng(7)
    M, N, K = 512, 256, 256
    A = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))).astype(np.complex64)
    B = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))).astype(np.complex64)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    try:
        for engine in (1, 2):
            _lib.check(lib.qbg_set_tc_wait_limit(0))
            with pytest.raises(_lib.QBGError) as ei:
                qb.cgemm(A, B, engine=engine)
            assert ei.value.status == _lib.QBG_ECUDA
            assert "gave up" in str(ei.value)
            _lib.check(lib.qbg_set_tc_wait_limit(-1))
            with pytest.raises(_lib.QBGError):  # the flag is sticky until cleared
                qb.cgemm(A, B, engine=engine)
            _lib.check(lib.qbg_clear_tc_error())
            C = qb.cgemm(A, B, engine=engine)
            assert np.max(np.abs(C - ref)) < 1e-5 * np.max(np.abs(A)) * np.max(np.abs(B)) * K
    finally:
        lib.qbg_set_tc_wait_limit(-1)
        lib.qbg_clear_tc_error()
