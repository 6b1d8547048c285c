"""The allocation-free norm entry point against the allocating one.

``udmrg_norm_noalloc`` serves callers that cannot allocate device memory at
the point of the call (device memory owned by an allocator they do not
control or fully reserved, loops that must not touch an allocator); its
scratch is a static device array instead of a pool allocation.  Here it must
agree with ``udmrg_tensor_norm`` (the same reduction with allocated scratch)
on two calls in a row, also at the largest accepted length.  The file name
sorts after every other test file (``pytest --collect-only`` lists it last),
so a run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import api, build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _vector_tensor(ctx, values):
    """A one-block rank-1 tensor holding `values` (device resident)."""
    from ultradmrg_gb300 import api
    from ultradmrg_gb300.tensor_data import OUT, BlockTensorData, Index
    idx = Index.make([((0,), len(values))], OUT)
    return api.DeviceTensor.from_data(ctx, BlockTensorData([idx], {(0,): np.asarray(values)}))


def test_norm_noalloc_matches_allocating_norm(ctx):
    import torch

    from ultradmrg_gb300 import _lib
    rng = np.random.default_rng(7)
    x = _vector_tensor(ctx, rng.standard_normal(3_000_001))
    out = _vector_tensor(ctx, np.zeros(1))
    ref = x.norm()  # udmrg_tensor_norm: scratch from the stream-ordered pool
    xp = C.cast(C.c_void_p(x.device_ptr()), _lib.c_double_p)
    op = C.cast(C.c_void_p(out.device_ptr()), _lib.c_double_p)
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        _lib.call("udmrg_norm_noalloc", xp, 3_000_001, op, None)
        torch.cuda.synchronize()
        got = float(out.download_packed()[0])
        assert abs(got - ref) <= RTOL * ref
    # a short vector after a long one: stale partials must not leak in
    y = _vector_tensor(ctx, np.array([3.0, 4.0]))
    yp = C.cast(C.c_void_p(y.device_ptr()), _lib.c_double_p)
    _lib.call("udmrg_norm_noalloc", yp, 2, op, None)
    torch.cuda.synchronize()
    assert abs(float(out.download_packed()[0]) - 5.0) <= RTOL * 5.0


def test_norm_noalloc_at_the_maximum(ctx):
    """16,777,216 doubles: every slot of the static scratch array is written."""
    import torch

    from ultradmrg_gb300 import _lib
    n = 16_777_216
    rng = np.random.default_rng(11)
    x = _vector_tensor(ctx, rng.standard_normal(n))
    out = _vector_tensor(ctx, np.zeros(1))
    ref = x.norm()
    xp = C.cast(C.c_void_p(x.device_ptr()), _lib.c_double_p)
    op = C.cast(C.c_void_p(out.device_ptr()), _lib.c_double_p)
    for _ in range(2):
        _lib.call("udmrg_norm_noalloc", xp, n, op, None)
        torch.cuda.synchronize()
        assert abs(float(out.download_packed()[0]) - ref) <= RTOL * ref


def test_norm_noalloc_rejects_oversize(ctx):
    from ultradmrg_gb300 import _lib
    out = _vector_tensor(ctx, np.zeros(1))
    op = C.cast(C.c_void_p(out.device_ptr()), _lib.c_double_p)
    with pytest.raises(_lib.UdmrgError, match="maximum"):
        _lib.call("udmrg_norm_noalloc", op, 16_777_217, op, None)
