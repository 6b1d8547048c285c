"""Finite-MPS measurements through the device backend (environment updates and
contraction through the C ABI) against the oracle's direct measurements.

The composition itself is checked on the host (``test_measure_host.py``);
here the same code runs on the device primitives.  The file name sorts
last so that a run stopping at the first failure has run every other test
before this one.
"""
import numpy as np
import pytest

from oracle import measure as om
from ultradmrg_gb300 import api, measure as dm, models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _agree(a, b, tol=1e-11):
    assert [x.sites for x in a] == [y.sites for y in b]
    for x, y in zip(a, b):
        assert abs(x.avg - y.avg) <= tol, (x, y)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_device_measurements_match_oracle(ctx, dtype):
    pb, o = M.spinless_fermion_site(dtype)
    mps = M.random_mps([pb] * 7, (1,), 12, seed=5, dtype=dtype)
    dmps = [api.DeviceTensor.from_data(ctx, t) for t in mps]
    m = dm.MPSMeasurer(dm.device_backend(ctx), dmps)
    n = np.diag([0.0, 1.0]).astype(dtype)
    _agree(dm.measure_one_site_op(m, n), om.measure_one_site_op(mps, n))
    f, cd, c = o["f"].mat, o["cdag"].mat, o["c"].mat
    pairs = [[0, 3], [1, 2], [2, 6], [0, 6]]
    _agree(dm.measure_two_site_op(m, [cd, c], f, pairs),
           om.measure_two_site_op(mps, [cd, c], f, pairs))
    ev = ([[cd, c]], [[[f], [f, f]]], [[1, 3]])
    _agree(dm.measure_multi_site_op(m, *ev), om.measure_multi_site_op(mps, *ev))
    m.close()
    for t in dmps:
        t.close()


def test_device_measurement_of_a_device_ground_state(ctx):
    """<Sz_i Sz_j> and <S+_i S-_j> of the N = 8 Heisenberg ground state from
    the device sweep, measured on the device and by the oracle on the
    downloaded MPS."""
    N = 8
    mpo, pb = M.heisenberg_chain_mpo(N)
    _, ops = M.spin_half_site()
    dmps = [api.DeviceTensor.from_data(ctx, t)
            for t in M.direct_product_mps([pb] * N, [i % 2 for i in range(N)])]
    api.two_site_finite_vmps(ctx, dmps, [api.DeviceTensor.from_data(ctx, w) for w in mpo],
                             api.FiniteVMPSSweepParams(4, 16, 16, 1e-10, 1e-10, 100))
    host = [t.to_data() for t in dmps]
    m = dm.MPSMeasurer(dm.device_backend(ctx), dmps)
    pairs = [[0, 1], [0, 4], [3, 7]]
    for a, b in ((ops["sz"], ops["sz"]), (ops["sp"], ops["sm"])):
        _agree(dm.measure_two_site_op(m, [a.mat, b.mat], ops["id"].mat, pairs),
               om.measure_two_site_op(host, [a.mat, b.mat], ops["id"].mat, pairs))
    sz = dm.measure_one_site_op(m, ops["sz"].mat)
    assert abs(sum(r.avg for r in sz)) < 1e-9  # total Sz = 0 sector
    m.close()


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_device_cal_psi1_op_psi2(ctx, dtype):
    """CalPsi1OpPsi2 on the device (contract and dag through the C ABI)."""
    pb, o = M.spinless_fermion_site(dtype)
    a = M.random_mps([pb] * 6, (0,), 8, seed=1, dtype=dtype)
    c = M.random_mps([pb] * 6, (2,), 8, seed=3, dtype=dtype)
    da = [api.DeviceTensor.from_data(ctx, t) for t in a]
    dc = [api.DeviceTensor.from_data(ctx, t) for t in c]
    got = dm.cal_psi1_op_psi2(dm.device_backend(ctx), da, dc, o["cdag"].mat, o["f"].mat)
    want = om.cal_psi1_op_psi2(a, c, o["cdag"].mat, o["f"].mat)
    assert np.allclose(got, want, atol=1e-12 * np.abs(want).max())
    for t in da + dc:
        t.close()
