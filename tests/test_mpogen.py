"""The restated MPO generator (``ultradmrg_gb300.mpogen``) against the
reference's own unit tests, and its MPOs against the Hamiltonians they encode.

* compressed FSM matrices of ``tests/test_one_dim_tn/test_mpogen/test_mpogen_fsm.cc:334-496``
  (cases 1-7) and of the generator tests
  ``tests/test_one_dim_tn/test_mpogen/test_mpogen.cc:72-237`` (cases 1-6,
  including the sign normalisation and label conversion);
* ``LabelConvertor`` (``test_mpogen_fsm.cc:508-518``);
* MPOs from the generator equal, as operators, the MPOs of the package's
  prefix-sharing builder (Heisenberg chain, Hubbard 2x2, Hubbard cylinder
  with Jordan-Wigner strings), and the two-site VMPS golden energies
  (Heisenberg N = 6, Hubbard 2x2) come out of the oracle sweep on them.
"""
import json
import os

import numpy as np
import pytest

from oracle import krylov, vmps as ovmps
from ultradmrg_gb300 import models as M
from ultradmrg_gb300.mpogen import (FSM, ID_COEF, ID_OP, Coef, LabelConvertor, MPOGenerator,
                                    Op, SparMat)
from ultradmrg_gb300.tensor_data import OUT, Index

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def mat(rows, cols, elems):
    m = SparMat(rows, cols)
    for (x, y), v in elems.items():
        m.set(x, y, v)
    return m


def s_(lab=1, coef=None):
    return Op.of(lab) if coef is None else Op.of(lab, Coef(coef))


def assert_mats(got, want):
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert (g.rows, g.cols) == (w.rows, w.cols)
        assert g == w, (g.cells, w.cells)


# ---- FSM (test_mpogen_fsm.cc) ----


def test_fsm_compressed_case1():
    f = FSM(1)
    f.add_path(0, 0, [ID_OP])
    assert_mats(f.gen_compressed_mat_repr(), [mat(1, 1, {(0, 0): ID_OP})])
    f = FSM(1)
    f.add_path(0, 0, [s_()])
    assert_mats(f.gen_compressed_mat_repr(), [mat(1, 1, {(0, 0): s_()})])


def test_fsm_compressed_case2():
    f = FSM(2)
    f.add_path(0, 0, [s_()])
    f.add_path(1, 1, [s_()])
    assert_mats(f.gen_compressed_mat_repr(),
                [mat(1, 2, {(0, 0): ID_OP, (0, 1): s_()}),
                 mat(2, 1, {(0, 0): s_(), (1, 0): ID_OP})])


def test_fsm_compressed_case3():
    f = FSM(2)
    f.add_path(0, 1, [s_(), s_()])
    f.add_path(0, 1, [s_(), s_()])
    assert_mats(f.gen_compressed_mat_repr(),
                [mat(1, 1, {(0, 0): s_()}), mat(1, 1, {(0, 0): s_() + s_()})])


def _case4_mats():
    s = s_()
    return [mat(1, 2, {(0, 0): s, (0, 1): ID_OP}),
            mat(2, 3, {(0, 2): s, (1, 0): ID_OP, (1, 1): s}),
            mat(3, 2, {(0, 0): s, (1, 1): s, (2, 1): ID_OP}),
            mat(2, 1, {(0, 0): s, (1, 0): ID_OP})]


def _case5_mats():
    """test_mpogen_fsm.cc:410-421.  The source sets the last matrix (2 x 1) at
    (0, 0) and (0, 1); SetElem on column 1 of a one-column matrix writes flat
    offset 1, which is element (1, 0)."""
    s = s_()
    return [mat(1, 2, {(0, 0): ID_OP, (0, 1): s}),
            mat(2, 2, {(0, 1): s, (1, 0): ID_OP}),
            mat(2, 2, {(0, 0): ID_OP, (1, 1): s}),
            mat(2, 2, {(0, 1): ID_OP, (1, 0): s, (1, 1): ID_OP}),
            mat(2, 1, {(0, 0): ID_OP, (1, 0): s})]


def test_fsm_compressed_case4():
    f = FSM(4)
    for a in range(3):
        f.add_path(a, a + 1, [s_(), s_()])
    assert_mats(f.gen_compressed_mat_repr(), _case4_mats())


def test_fsm_compressed_case5():
    s = s_()
    f = FSM(5)
    f.add_path(0, 4, [s, ID_OP, ID_OP, ID_OP, s])
    f.add_path(1, 4, [s, s, ID_OP, s])
    f.add_path(1, 3, [s, s, s])
    assert_mats(f.gen_compressed_mat_repr(), _case5_mats())


def _case6_mats():
    j1, j2, s = 1, 2, 1
    op_s = Op.of(s)
    return [mat(1, 2, {(0, 0): ID_OP, (0, 1): op_s}),
            mat(2, 4, {(0, 0): Op.of(0, Coef(j1)), (0, 3): op_s, (1, 1): Op.of(s, Coef(j1)),
                       (1, 2): ID_OP}),
            mat(4, 2, {(0, 0): op_s, (1, 1): ID_OP, (2, 0): Op.of(0, Coef(j2)),
                       (2, 1): Op.of(s, Coef(j1)), (3, 0): Op.of(0, Coef(j1)),
                       (3, 1): Op.of(s, Coef(j2))}),
            mat(2, 1, {(0, 0): op_s, (1, 0): ID_OP})]


def test_fsm_compressed_case6():
    j1, j2, s = 1, 2, 1
    op_s = Op.of(s)
    f = FSM(4)
    f.add_path(0, 1, [Op.of(s, Coef(j1)), op_s])
    f.add_path(0, 2, [Op.of(s, Coef(j1)), ID_OP, op_s])
    f.add_path(1, 3, [Op.of(s, Coef(j1)), ID_OP, op_s])
    f.add_path(2, 3, [Op.of(s, Coef(j1)), op_s])
    f.add_path(0, 3, [Op.of(s, Coef(j2)), ID_OP, ID_OP, op_s])
    f.add_path(1, 2, [Op.of(s, Coef(j2)), op_s])
    assert_mats(f.gen_compressed_mat_repr(), _case6_mats())


def _case7_mats(j=1, k=2, sx=1, sy=2, sz=3):
    return [mat(1, 4, {(0, 0): Op.sum_of([Coef(k), Coef(j)], [sx, sx]),
                       (0, 1): Op.of(sy, Coef(j)), (0, 2): Op.of(sz, Coef(j)), (0, 3): ID_OP}),
            mat(4, 4, {(0, 3): Op.of(sx), (1, 3): Op.of(sy), (2, 3): Op.of(sz),
                       (3, 0): Op.of(sx, Coef(j)), (3, 1): Op.of(sy, Coef(j)),
                       (3, 2): Op.sum_of([Coef(j), Coef(k)], [sz, sz])}),
            mat(4, 1, {(0, 0): Op.of(sx), (1, 0): Op.of(sy), (2, 0): Op.of(sz), (3, 0): ID_OP})]


def test_fsm_compressed_case7():
    j, k, sx, sy, sz = 1, 2, 1, 2, 3
    f = FSM(3)
    for a in (0, 1):
        for o in (sx, sy, sz):
            f.add_path(a, a + 1, [Op.of(o, Coef(j)), Op.of(o)])
    f.add_path(0, 1, [Op.of(sx, Coef(k)), Op.of(sx)])
    f.add_path(1, 2, [Op.of(sz, Coef(k)), Op.of(sz)])
    assert_mats(f.gen_compressed_mat_repr(), _case7_mats())


def test_label_convertor():
    c = LabelConvertor(1.0)
    assert c.convert(1) == 0 and c.convert(1.0) == 0
    assert c.convert(2.0) == 1 and c.convert(2.0) == 1
    assert c.convert(1.0) == 0


def test_coef_and_op_algebra():
    # CoefRepr equality is up to permutation (coef_op_alg.h:71-74)
    assert Coef((1, 2)) == Coef((2, 1)) and Coef((1, 2)) != Coef((1, 1))
    # OpRepr(coefs, labels) merges repeated labels (coef_op_alg.h:189-201)
    assert Op.sum_of([Coef(1), Coef(2)], [3, 3]) == Op.of(3, Coef((2, 1)))
    assert Op.of(1) + Op.of(2) == Op.sum_of([ID_COEF, ID_COEF], [2, 1])


# ---- generator (test_mpogen.cc) ----


def spin_site():
    """test_mpogen.cc:31-69: sectors Sz = -1, +1 (one state each)."""
    pb = Index.make([((-1,), 1), ((1,), 1)], OUT)
    sz = np.diag([-0.5, 0.5])
    return pb, sz


def test_generator_case1():
    pb, sz = spin_site()
    g = MPOGenerator([pb] * 2)
    g.add_term(1.0, [-sz], [0])
    want = [mat(1, 1, {(0, 0): s_()}), mat(1, 1, {(0, 0): ID_OP})]
    assert_mats(g.mat_repr(), want)
    g = MPOGenerator([pb] * 2)
    g.add_term(1.0, [-sz], [0])
    g.add_term(0.0, [-sz], [0])
    assert_mats(g.mat_repr(), want)


def test_generator_case2():
    pb, sz = spin_site()
    g = MPOGenerator([pb] * 2)
    g.add_term(1.0, [sz, sz], [0, 1])
    g.add_term(1.0, [sz, sz], [0, 1])
    assert_mats(g.mat_repr(), [mat(1, 1, {(0, 0): s_()}), mat(1, 1, {(0, 0): s_() + s_()})])


def test_generator_case3():
    pb, sz = spin_site()
    g = MPOGenerator([pb] * 4)
    for a in range(3):
        g.add_term(1.0, [sz, sz], [a, a + 1])
    assert_mats(g.mat_repr(), _case4_mats())


def test_generator_case4():
    pb, sz = spin_site()
    g = MPOGenerator([pb] * 5)
    g.add_term(1.0, [sz, sz], [0, 4])
    g.add_term(1.0, [-sz, -sz, -sz], [1, 2, 4])
    g.add_term(1.0, [-sz, -sz, -sz], [1, 2, 3])
    assert_mats(g.mat_repr(), _case5_mats())


def test_generator_case5():
    pb, sz = spin_site()
    g = MPOGenerator([pb] * 4)
    ja, jb = 0.5, 2.0
    for (a, b) in ((0, 1), (0, 2), (1, 3), (2, 3)):
        g.add_term(ja, [sz, sz], [a, b])
    g.add_term(jb, [sz, sz], [0, 3])
    g.add_term(jb, [sz, sz], [1, 2])
    assert_mats(g.mat_repr(), _case6_mats())


def test_generator_case6_complex():
    pb, _ = spin_site()
    zsz = np.diag([-0.5, 0.5]).astype(np.complex128)
    zsx = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    zsy = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    g = MPOGenerator([pb] * 3, dtype=np.complex128)
    J, K = 0.5, 2.0
    for a in (0, 1):
        for o in (zsx, zsy, zsz):
            g.add_term(J, [o, o], [a, a + 1])
    g.add_term(K, [zsx, zsx], [0, 1])
    g.add_term(K, [zsz, zsz], [1, 2])
    assert_mats(g.mat_repr(), _case7_mats())


# ---- the operators the MPOs encode ----


def mpo_dense(mpo):
    """The operator an MPO encodes, as a (d^N x d^N) matrix [in, out]."""
    T = mpo[0].to_dense()[0]  # (in, out, r)
    for W in mpo[1:]:
        w = W.to_dense()  # (l, in, out, r)
        din, dout, _ = T.shape
        T = np.einsum("ijl,lpqr->ipjqr", T, w).reshape(din * w.shape[1], dout * w.shape[2],
                                                       w.shape[3])
    return T[..., 0]


def test_heisenberg_operator_matches():
    N = 6
    mpo_ref, pb = M.heisenberg_chain_mpo(N)
    _, ops = M.spin_half_site()
    g = MPOGenerator([pb] * N)
    for i in range(N - 1):
        g.add_term(1.0, [ops["sz"], ops["sz"]], [i, i + 1])
        g.add_term(0.5, [ops["sp"], ops["sm"]], [i, i + 1])
        g.add_term(0.5, [ops["sm"], ops["sp"]], [i, i + 1])
    mpo = g.gen()
    assert np.allclose(mpo_dense(mpo), mpo_dense(mpo_ref), atol=1e-13)
    # bulk bond dimension 5 (Id, Sz, S+, S-, done); the edge bonds need 4
    assert g.bond_dims == [4] + [5] * (N - 3) + [4, 1]


MODELS = {
    "heisenberg6": lambda b: M.heisenberg_chain_mpo(6, builder=b)[0],
    "heisenberg2d": lambda b: M.heisenberg_chain_mpo(
        6, pairs=[(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)], builder=b)[0],
    "ising6": lambda b: M.ising_chain_mpo(6, builder=b)[0],
    "free_fermion6": lambda b: M.free_fermion_chain_mpo(6, builder=b)[0],
    "hubbard2x2": lambda b: M.hubbard_2x2_test_mpo(builder=b)[0],
    "hubbard_cyl2x2": lambda b: M.hubbard_cylinder_mpo(2, 2, builder=b)[0],
    "hubbard_cyl1x3": lambda b: M.hubbard_cylinder_mpo(1, 3, builder=b)[0],
    "hubbard_cyl1x4": lambda b: M.hubbard_cylinder_mpo(1, 4, builder=b)[0],
    "tj1d": lambda b: M.tj_mpo(4, builder=b)[0],
    "tj2d": lambda b: M.tj_mpo(4, pairs=[(0, 1), (0, 2), (2, 3), (1, 3)], builder=b)[0],
    "rashba_tj": lambda b: M.rashba_tj_mpo(builder=b)[0],
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_builders_encode_the_same_operator(name):
    """Both generators, the same term list: the same operator (the Hubbard
    cylinders include the periodic bond with its Jordan-Wigner string)."""
    a = mpo_dense(MODELS[name]("reference"))
    b = mpo_dense(MODELS[name]("prefix"))
    assert np.allclose(a, b, atol=1e-12 * max(1.0, np.abs(b).max()))


def _oracle_energy(mpo, pb, labels, params):
    mps = M.direct_product_mps([pb] * len(labels), labels)
    return ovmps.two_site_finite_vmps(mps, mpo, params)


@pytest.mark.parametrize("case", ["1DHeisenberg", "2DHeisenberg", "1DIsing", "Hubbard2x2"])
def test_vmps_goldens_on_reference_layout(case):
    """The two-site VMPS golden energies of
    ``tests/test_algorithm/test_two_site_update_finite_vmps.cc`` (whose MPOs
    the reference's generator makes) from the oracle sweep on this
    generator's MPOs."""
    g = GOLD["vmps"][case]
    P = ovmps.FiniteVMPSSweepParams
    if case == "1DHeisenberg":
        mpo, pb = M.heisenberg_chain_mpo(6, builder="reference")
        labels, p = [i % 2 for i in range(6)], P(4, 8, 8, 1e-9, krylov.LanczosParams(1e-7))
    elif case == "2DHeisenberg":
        mpo, pb = M.heisenberg_chain_mpo(
            6, pairs=[(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)], builder="reference")
        labels, p = [i % 2 for i in range(6)], P(4, 8, 8, 1e-9, krylov.LanczosParams(1e-7))
    elif case == "1DIsing":
        mpo, pb = M.ising_chain_mpo(6, builder="reference")
        labels, p = [i % 2 for i in range(6)], P(4, 1, 10, 1e-5, krylov.LanczosParams(1e-7))
    else:
        mpo, pb = M.hubbard_2x2_test_mpo(builder="reference")
        labels = [1 if i % 2 == 0 else 2 for i in range(4)]
        p = P(10, 16, 16, 1e-9, krylov.LanczosParams(1e-8, 20))
    e0 = _oracle_energy(mpo, pb, labels, p)
    assert abs(e0 - g["energy"]) < g["tol"]


@pytest.mark.parametrize("Lx,Ly", [(8, 4), (16, 4)])
def test_hubbard_cylinder_reference_layout(Lx, Ly):
    """The benchmark's cylinders (``benchmark/ultradmrg_hubbard2d.cpp:138-181``,
    t2 = 0) through the reference's generator: divergence-free tensors, bulk
    bonds of 18 channels in five (N, Sz) sectors, and in the bulk the same
    sector sizes as the prefix-sharing builder (in another order)."""
    mpo, _ = M.hubbard_cylinder_mpo(Lx, Ly, builder="reference")
    pre, _ = M.hubbard_cylinder_mpo(Lx, Ly)
    assert len(mpo) == Lx * Ly
    for W in mpo:
        for key in W.blocks:
            q = [0, 0]
            for ind, sid in zip(W.indexes, key):
                for c in range(2):
                    q[c] += ind.dir * ind.qns[sid][c]
            assert q == [0, 0]
    dims = [W.indexes[3].dim for W in mpo]
    assert max(dims) == 18 and dims[-1] == 1
    mid = len(mpo) // 2
    a, b = mpo[mid].indexes[3], pre[mid].indexes[3]
    assert sorted(zip(a.qns, a.dims)) == sorted(zip(b.qns, b.dims))
    assert a.nsec == 5
    print(f"Hubbard {Ly}x{Lx} (reference layout): bond dims {dims}")
