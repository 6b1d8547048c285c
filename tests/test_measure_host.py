"""The device measurement composition (``ultradmrg_gb300.measure``) run on the
oracle's primitives (environment updates, contraction), against the oracle's
direct measurements (``oracle.measure``) and the reference's known answers.

The composition is host logic; with ``device_backend`` the same code calls
the C ABI's environment updates and contraction, which the GPU tests cover.
"""
import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import measure as om
from oracle import vmps as ov
from ultradmrg_gb300 import measure as dm
from ultradmrg_gb300 import models as M
from ultradmrg_gb300.tensor_data import OUT, Index

ORACLE = dm.Backend(ov.update_site_lenvs, ov.update_site_renvs, bs.contract,
                    lambda t: t, lambda t: t, lambda t: (t.indexes, t.dtype), lambda t: None)


def _close(a, b):
    return all(np.isclose(x.avg, y.avg, atol=1e-12) and x.sites == y.sites for x, y in zip(a, b))


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_composition_matches_oracle(dtype):
    pb, o = M.spinless_fermion_site(dtype)
    mps = M.random_mps([pb] * 7, (1,), 12, seed=5, dtype=dtype)
    m = dm.MPSMeasurer(ORACLE, mps)
    n = np.diag([0.0, 1.0]).astype(dtype)
    assert _close(dm.measure_one_site_op(m, n), om.measure_one_site_op(mps, n))
    f, cd, c = o["f"].mat, o["cdag"].mat, o["c"].mat
    pairs = [[0, 3], [1, 2], [2, 6], [0, 6]]
    assert _close(dm.measure_two_site_op(m, [cd, c], f, pairs),
                  om.measure_two_site_op(mps, [cd, c], f, pairs))
    ev = ([[cd, c]], [[[f], [f, f]]], [[1, 3]])
    assert _close(dm.measure_multi_site_op(m, *ev), om.measure_multi_site_op(mps, *ev))
    assert _close(dm.measure_two_site_op_group(m, cd, c, 1, [2, 4, 6], f),
                  om.measure_two_site_op_group(mps, cd, c, 1, [2, 4, 6], f))
    # an operator string whose total charge is not zero has no expectation value
    assert dm.measure_two_site_op(m, [cd, cd], f, [[0, 2]])[0].avg == 0.0
    m.close()


def test_hubbard_spin_correlation_matches_oracle():
    """U(1) x U(1) sites: <Sz_i Sz_j> and <S+_i S-_j> on a random Hubbard MPS."""
    pb, o = M.hubbard_site_nsz()
    mps = M.random_mps([pb] * 6, (5, 1), 10, seed=3)
    m = dm.MPSMeasurer(ORACLE, mps)
    idm = o["id"].mat
    for ops in ([o["sz"].mat, o["sz"].mat], [o["sp"].mat, o["sm"].mat]):
        pairs = [[0, 1], [1, 4], [2, 5]]
        assert _close(dm.measure_two_site_op(m, ops, idm, pairs),
                      om.measure_two_site_op(mps, ops, idm, pairs))
    m.close()


def test_known_answers():
    """test_finite_mps_measu.cc:100-167 on the composition."""
    pb = Index.make([((0,), 1), ((1,), 1)], OUT)
    ntot, idm = np.diag([0.0, 1.0]), np.eye(2)
    lab = [i % 2 for i in range(6)]
    m = dm.MPSMeasurer(ORACLE, M.direct_product_mps([pb] * 6, lab))
    assert [r.avg for r in dm.measure_one_site_op(m, ntot)] == lab
    sites = [[0, 1], [0, 2], [0, 5], [1, 2], [1, 3], [4, 5]]
    assert [r.avg for r in dm.measure_two_site_op(m, [ntot, ntot], idm, sites)] == \
        [0, 0, 0, 0, 1, 0]


ORACLE2 = dm.Backend(ov.update_site_lenvs, ov.update_site_renvs, bs.contract,
                     lambda t: t, lambda t: t, lambda t: (t.indexes, t.dtype), lambda t: None,
                     bs.dag)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_cal_psi1_op_psi2(dtype):
    """<psi2| F...F O_i |psi1> between two random MPS: a neutral operator with
    and without the string, and c^dag between states whose charges differ by
    its charge (+2 in units where the basis states carry +1 and -1; six sites
    reach even totals only)."""
    pb, o = M.spinless_fermion_site(dtype)
    f, cd = o["f"].mat, o["cdag"].mat
    n = np.diag([0.0, 1.0]).astype(dtype)
    a = M.random_mps([pb] * 6, (0,), 8, seed=1, dtype=dtype)
    b = M.random_mps([pb] * 6, (0,), 8, seed=2, dtype=dtype)
    c = M.random_mps([pb] * 6, (2,), 8, seed=3, dtype=dtype)
    for psi1, psi2, op, inst in ((a, b, n, None), (a, b, n, f), (a, c, cd, f), (a, c, cd, None)):
        got = dm.cal_psi1_op_psi2(ORACLE2, psi1, psi2, op, inst)
        want = om.cal_psi1_op_psi2(psi1, psi2, op, inst)
        assert np.abs(want).max() > 1e-3
        assert np.allclose(got, want, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_act_operator_on_mps(dtype):
    """The host ActOperatorOnMps against the oracle's contraction of the
    operator tensor (block keys and values) and against the state vector."""
    from systems import act_operator, apply_dense, mps_dense
    pb, o = M.spinless_fermion_site(dtype)
    mps = M.random_mps([pb] * 6, (0,), 8, seed=4, dtype=dtype)
    cd, f = o["cdag"].mat, o["f"].mat
    got = M.act_operator_on_mps(mps, cd, f, 3)
    want = act_operator(mps, M.operator_tensor(cd, pb), M.operator_tensor(f, pb), 3)
    for g, w in zip(got, want):
        assert set(g.blocks) == set(w.blocks)
        for k in w.blocks:
            assert np.allclose(g.blocks[k], w.blocks[k], rtol=0, atol=1e-14)
    v = apply_dense(mps_dense(mps), cd, 3, f)
    assert np.allclose(mps_dense(got), v, atol=1e-12)
    # without a string only the site's tensor changes
    only = M.act_operator_on_mps(mps, cd, None, 2)
    assert all(a is b for i, (a, b) in enumerate(zip(only, mps)) if i != 2)
