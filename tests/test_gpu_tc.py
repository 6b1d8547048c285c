"""tcgen05 split-BF16 GEMM against an FP64 numpy reference.

Three BF16 planes carry ~24 significant bits of every operand and the six
cross products accumulate in FP32, so the result must match FP64 to FP32
accumulation level: |C - A B| <= 2^-24 * sqrt(K) * 4 * (|A| |B|) elementwise.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import api, build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 100, 80), (37, 13, 5), (1, 1, 1),
                                   (1000, 700, 250), (129, 65, 129)])
def test_tc_gemm_matches_fp64(ctx, M, N, K):
    from ultradmrg_gb300 import _lib
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((K, N))
    Cm = np.zeros((M, N))
    p = lambda a: a.ctypes.data_as(_lib.c_double_p)
    _lib.call("udmrg_selftest_tc_gemm", ctx.h, M, N, K, p(A), p(B), p(Cm))
    ref = A @ B
    bound = np.abs(A) @ np.abs(B)
    err = np.max(np.abs(Cm - ref) / bound)
    assert err < 4 * 2.0 ** -24 * np.sqrt(K + 16), err
