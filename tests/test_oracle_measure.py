"""The oracle's finite-MPS measurements (``oracle.measure``).

* the known answers of
  ``tests/test_one_dim_tn/test_finite_mps/test_finite_mps_measu.cc:41-215``:
  particle number and identity operators on two product states of six
  sites, one- and two-site forms and the grouped two-site form, real and
  complex;
* the entanglement entropies of the N = 6 Heisenberg ground state
  (``tests/test_one_dim_tn/test_finite_mps/test_finite_mps.cc:304-333``);
* random MPS against the dense state vector: one-site values, two-site
  values with a Jordan-Wigner string in between and a tail string, Renyi
  entropies.
"""
import json
import os

import numpy as np
import pytest

from oracle import krylov, measure, vmps
from systems import mps_dense
from ultradmrg_gb300 import models as M
from ultradmrg_gb300.tensor_data import OUT, Index

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
N = 6
SITES = [[0, 1], [0, 2], [0, 5], [1, 2], [1, 3], [4, 5]]  # test_finite_mps_measu.cc:141-145


def site():
    """N = 0 and N = 1 sectors, one state each (test_finite_mps_measu.cc:44-50)."""
    pb = Index.make([((0,), 1), ((1,), 1)], OUT)
    return pb, np.diag([0.0, 1.0]), np.eye(2)


LABELS = {"all_one": [1] * N, "alternating": [i % 2 for i in range(N)]}


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("labels", sorted(LABELS))
def test_one_site_known_answers(dtype, labels):
    pb, ntot, _ = site()
    lab = LABELS[labels]
    mps = M.direct_product_mps([pb] * N, lab, dtype=dtype)
    res = measure.measure_one_site_op(mps, ntot.astype(dtype))
    assert [r.sites for r in res] == [[i] for i in range(N)]
    assert all(r.avg == lab[i] for i, r in enumerate(res))


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_two_site_known_answers(dtype):
    pb, ntot, idm = site()
    ntot, idm = ntot.astype(dtype), idm.astype(dtype)
    ones = [1.0] * len(SITES)
    m1 = M.direct_product_mps([pb] * N, LABELS["all_one"], dtype=dtype)
    m2 = M.direct_product_mps([pb] * N, LABELS["alternating"], dtype=dtype)
    for mps, ops, want in ((m1, [idm, idm], ones), (m1, [ntot, ntot], ones),
                           (m2, [idm, idm], ones), (m2, [ntot, ntot], [0, 0, 0, 0, 1, 0])):
        res = measure.measure_two_site_op(mps, ops, idm, SITES)
        assert [r.sites for r in res] == SITES
        assert [r.avg for r in res] == want


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_two_site_group_known_answers(dtype):
    """test_finite_mps_measu.cc:196-215 (site1 = 0, site2 in {1, 2, 5})."""
    pb, ntot, idm = site()
    ntot, idm = ntot.astype(dtype), idm.astype(dtype)
    m1 = M.direct_product_mps([pb] * N, LABELS["all_one"], dtype=dtype)
    m2 = M.direct_product_mps([pb] * N, LABELS["alternating"], dtype=dtype)
    for mps, a, b, want in ((m1, idm, idm, [1, 1, 1]), (m1, ntot, ntot, [1, 1, 1]),
                            (m2, idm, idm, [1, 1, 1]), (m2, ntot, ntot, [0, 0, 0])):
        res = measure.measure_two_site_op_group(mps, a, b, 0, [1, 2, 5], idm)
        assert [r.avg for r in res] == want


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_heisenberg_entanglement_entropy_golden(dtype):
    g = GOLD["ee_heisenberg6"]
    mpo, pb = M.heisenberg_chain_mpo(N, dtype=dtype, builder="reference")
    mps = M.direct_product_mps([pb] * N, [i % 2 for i in range(N)], dtype=dtype)
    vmps.two_site_finite_vmps(mps, mpo, vmps.FiniteVMPSSweepParams(
        4, 16, 16, 1e-9, krylov.LanczosParams(1e-9)))
    ee = measure.entanglement_entropy(mps)
    assert len(ee) == N - 1
    assert max(abs(a - b) for a, b in zip(ee, g["ee"])) < g["tol"]


def _dense_expect(v, ops_at):
    w = v
    for site_, m in ops_at.items():
        w = np.moveaxis(np.tensordot(m, w, axes=([0], [site_])), 0, site_)
    return np.vdot(v, w) / np.vdot(v, v)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_random_mps_against_dense(dtype):
    """Spinless fermions (U(1) charge): <c^dag_i F ... F c_j>, a tail string,
    one-site densities, Renyi entropies, all against the state vector."""
    pb, o = M.spinless_fermion_site(dtype)
    L = 7
    mps = M.random_mps([pb] * L, (1,), 12, seed=5, dtype=dtype)
    v = mps_dense(mps)
    nmat = np.diag([0.0, 1.0]).astype(dtype)  # occupation of the basis state 1
    res = measure.measure_one_site_op(mps, nmat)
    for i, r in enumerate(res):
        assert np.isclose(r.avg, _dense_expect(v, {i: nmat}), atol=1e-12)
    f, cd, c = o["f"].mat, o["cdag"].mat, o["c"].mat
    pairs = [[0, 3], [1, 2], [2, 6]]
    res = measure.measure_two_site_op(mps, [cd, c], f, pairs)
    for (i, j), r in zip(pairs, res):
        ops = {i: cd, j: c}
        for k in range(i + 1, j):
            ops[k] = f
        assert np.isclose(r.avg, _dense_expect(v, ops), atol=1e-12)
    # a tail string after the last physical operator (MultiSiteOpAvg)
    res = measure.measure_multi_site_op(mps, [[cd, c]], [[[f], [f, f]]], [[1, 3]])
    ops = {1: cd, 2: f, 3: c, 4: f, 5: f}
    assert np.isclose(res[0].avg, _dense_expect(v, ops), atol=1e-12)
    # entropies against the SVD of the state vector
    vv = v.reshape(-1) / np.linalg.norm(v)
    for n in (1, 2):
        ee = measure.entanglement_entropy(mps, n)
        for bond in range(L - 1):
            s = np.linalg.svd(vv.reshape(2 ** (bond + 1), -1), compute_uv=False)
            p = s[s > 1e-12] ** 2
            want = -(p * np.log(p)).sum() if n == 1 else -np.log((p ** n).sum()) / (n - 1)
            assert abs(ee[bond] - want) < 1e-10
