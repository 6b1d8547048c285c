"""Pin the CPU oracle against the reference's own golden values.

Golden numbers come from ``tests/golden/reference_goldens.json`` (extracted
from the reference test sources by ``tests/golden/extract_reference_goldens.py``).
"""
import json
import os

import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov, vmps
from ultradmrg_gb300 import models as M
from ultradmrg_gb300.tensor_data import IN, OUT, BlockTensorData, Index

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "reference_goldens.json")))


def _run(mpo, pb, labels, params):
    mps = M.direct_product_mps([pb] * len(labels), labels)
    return vmps.two_site_finite_vmps(mps, mpo, params)


def test_vmps_ising_golden():
    g = GOLD["vmps"]["1DIsing"]
    mpo, pb = M.ising_chain_mpo(6)
    e = _run(mpo, pb, [i % 2 for i in range(6)],
             vmps.FiniteVMPSSweepParams(4, 1, 10, 1e-5, krylov.LanczosParams(1e-7)))
    assert abs(e - g["energy"]) < g["tol"]


def test_vmps_heisenberg_golden():
    g = GOLD["vmps"]["1DHeisenberg"]
    mpo, pb = M.heisenberg_chain_mpo(6)
    e = _run(mpo, pb, [i % 2 for i in range(6)],
             vmps.FiniteVMPSSweepParams(4, 8, 8, 1e-9, krylov.LanczosParams(1e-7)))
    assert abs(e - g["energy"]) < g["tol"]


def test_vmps_heisenberg2d_golden():
    g = GOLD["vmps"]["2DHeisenberg"]
    pairs = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]
    mpo, pb = M.heisenberg_chain_mpo(6, pairs=pairs)
    e = _run(mpo, pb, [i % 2 for i in range(6)],
             vmps.FiniteVMPSSweepParams(4, 8, 8, 1e-9, krylov.LanczosParams(1e-7)))
    assert abs(e - g["energy"]) < g["tol"]


def test_vmps_hubbard2x2_golden():
    g = GOLD["vmps"]["Hubbard2x2"]
    mpo, pb = M.hubbard_2x2_test_mpo()
    e = _run(mpo, pb, [1 if i % 2 == 0 else 2 for i in range(4)],
             vmps.FiniteVMPSSweepParams(10, 16, 16, 1e-9, krylov.LanczosParams(1e-8, 20)))
    assert abs(e - g["energy"]) < g["tol"]


@pytest.mark.parametrize("case", [0, 1])
def test_tridiag_expme1_known_answers(case):
    c = GOLD["expme1"][case]
    n = len(c["a"])
    res = krylov.tridiag_expme1_solver(c["a"], c["b"], n, c["delta"])
    ref = np.array([complex(x, y) for x, y in c["res"]])
    assert krylov.distance(res, ref) < 1e-13


def _random_single_sector_eff_ham(D=20, d=2, dh=2, seed=0, dtype=np.float64):
    """Random Hermitian L, W, R on one-sector indexes, the layout of
    ``tests/test_algorithm/test_lanczos_solver.cc:114-150``."""
    rng = np.random.default_rng(seed)
    q0 = (0,)
    iD = lambda dr: Index.make([(q0, D)], dr)
    id_ = lambda dr: Index.make([(q0, d)], dr)
    iv = lambda dr: Index.make([(q0, dh)], dr)

    def sym(n):
        a = rng.random((n, n))
        if dtype == np.complex128:
            a = a + 1j * rng.random((n, n))
        return a + a.conj().T

    blk = sym(D)
    L = BlockTensorData([iD(IN), iv(OUT), iD(OUT)], {}, dtype)
    R = BlockTensorData([iD(OUT), iv(IN), iD(IN)], {}, dtype)
    Lb = np.zeros((D, dh, D), dtype)
    Rb = np.zeros((D, dh, D), dtype)
    for k in range(dh):
        Lb[:, k, :] = blk
        Rb[:, k, :] = blk.T
    L.blocks[(0, 0, 0)] = Lb
    R.blocks[(0, 0, 0)] = Rb
    site = sym(d)
    Wb = np.zeros((dh, d, d, dh), dtype)
    for k in range(dh):
        Wb[k, :, :, k] = site
    W = BlockTensorData([iv(IN), id_(IN), id_(OUT), iv(OUT)], {(0, 0, 0, 0): Wb}, dtype)
    psi = BlockTensorData([iD(IN), id_(OUT), id_(OUT), iD(OUT)],
                          {(0, 0, 0, 0): rng.standard_normal((D, d, d, D)).astype(dtype)},
                          dtype)
    return [L, W, W.copy(), R], psi


def dense_eff_ham(eff_ham):
    """Dense matrix of H_eff (rows: output (a,s1,s2,b), cols: input)."""
    L, W1, W2, R = [t.to_dense() for t in eff_ham]
    H = np.einsum('xwa,wsty,yuvz,bzc->xtvbasuc', L, W1, W2, R)
    n = H.shape[0] * H.shape[1] * H.shape[2] * H.shape[3]
    return H.reshape(n, n)


@pytest.mark.parametrize("dtype,params", [(np.float64, (1e-9, 200)),
                                          (np.float64, (1e-16, 20)),
                                          (np.complex128, (1e-9, 200))])
def test_lanczos_vs_dense_ed(dtype, params):
    """Cases of ``tests/test_algorithm/test_lanczos_solver.cc:145-207``: tolerance
    stop and max-iteration stop (real), tolerance stop (complex)."""
    eff_ham, psi = _random_single_sector_eff_ham(dtype=dtype)
    H = dense_eff_ham(eff_ham)
    assert np.allclose(H, H.conj().T)
    w = np.linalg.eigvalsh(H)
    res = krylov.lanczos_solver(eff_ham, psi, krylov.eff_ham_mul_two_site_state,
                                krylov.LanczosParams(*params))
    assert abs(res.gs_eng - w[0]) < 1e-8


def test_matvec_matches_dense():
    eff_ham, psi = _random_single_sector_eff_ham(D=6, seed=3)
    H = dense_eff_ham(eff_ham)
    out = krylov.eff_ham_mul_two_site_state(eff_ham, psi)
    ref = H @ psi.to_dense().ravel()
    assert np.allclose(out.to_dense().ravel(), ref, atol=1e-12)


def test_svd_truncation_rule():
    sv = [np.array([0.9, 0.3, 0.1]), np.array([0.3, 0.05])]
    kept, D, err = bs.select_kept(sv, 1e-2, 1, 10)
    # weights .81 .09 .09 .01 .0025 ; keep until discarded <= 1e-2 of total
    tot = 0.81 + 0.09 + 0.09 + 0.01 + 0.0025
    assert D == 4 and kept == [3, 1]
    assert abs(err - 0.0025 / tot) < 1e-15
    kept, D, _ = bs.select_kept(sv, 1e-2, 1, 2)
    assert D == 2 and kept == [2, 0]  # tie 0.3/0.3 broken by sector order


# ---- fermionic two-site goldens (test_fermion_two_site_update_finite_vmps.cc) ----
# The reference runs these with fermionic tensors; here the same Hamiltonians
# carry explicit Jordan-Wigner strings.  A dense exact diagonalisation of each
# MPO pins the Hamiltonian, the oracle sweep with the reference's parameters
# and initial product state pins the energy.

FERMION = {
    "free_fermion8": lambda dt: M.free_fermion_chain_mpo(8, dtype=dt)[:2],
    "tj1d": lambda dt: M.tj_mpo(4, dtype=dt),
    "tj2d": lambda dt: M.tj_mpo(4, pairs=[(0, 1), (0, 2), (2, 3), (1, 3)], dtype=dt),
}


def _sweep_params(text):
    """FiniteVMPSSweepParams(sweeps, Dmin, Dmax, trunc, LanczosParams(err, max_it))."""
    import re
    nums = [float(x) for x in re.findall(r"[-0-9.]+(?:[eE][-+]?[0-9]+)?", text)]
    sweeps, dmin, dmax, trunc, err = nums[:5]
    it = int(nums[5]) if len(nums) > 5 else 200
    return vmps.FiniteVMPSSweepParams(int(sweeps), int(dmin), int(dmax), trunc,
                                      krylov.LanczosParams(err, it))


def _sector_ground_energy(mpo, pb, labels):
    import itertools
    from test_mpogen import mpo_dense
    N = len(labels)
    qs = [pb.qns[pb.sector_of(i)[0]] for i in range(pb.dim)]
    tgt = tuple(np.sum([qs[x] for x in labels], axis=0))
    idx = [k for k, c in enumerate(itertools.product(range(pb.dim), repeat=N))
           if tuple(np.sum([qs[x] for x in c], axis=0)) == tgt]
    H = mpo_dense(mpo)[np.ix_(idx, idx)]
    return np.linalg.eigvalsh((H + H.conj().T) / 2)[0]


@pytest.mark.parametrize("case", sorted(FERMION))
def test_fermion_hamiltonians_by_exact_diagonalisation(case):
    g = GOLD["fermion_vmps"][case]
    mpo, pb = FERMION[case](np.float64)
    assert abs(_sector_ground_energy(mpo, pb, g["labels"]) - g["energy"]) < max(g["tol"], 1e-11)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("case", sorted(FERMION))
def test_fermion_vmps_goldens(case, dtype):
    g = GOLD["fermion_vmps"][case]
    mpo, pb = FERMION[case](dtype)
    mps = M.direct_product_mps([pb] * len(g["labels"]), g["labels"], dtype=dtype)
    e = vmps.two_site_finite_vmps(mps, mpo, _sweep_params(g["sweep_params"]))
    assert abs(e - g["energy"]) < g["tol"]


def _kitaev():
    g = GOLD["dmrg_kitaev_gamma"]
    mpo, pb = M.kitaev_gamma_mpo(g["Nx"], g["Ny"], g["J"], g["K"], g["Gm"], g["h"])
    return g, mpo, pb


def test_kitaev_gamma_by_exact_diagonalisation():
    """test_finite_dmrg.cc:346-444 (no symmetry, complex, 12 sites): the
    ground energy of the dense Hamiltonian (4096 states)."""
    from test_mpogen import mpo_dense
    g, mpo, _ = _kitaev()
    H = mpo_dense(mpo)
    assert np.allclose(H, H.conj().T, atol=1e-13)
    assert abs(np.linalg.eigvalsh(H)[0] - g["energy"]) < g["tol"]


def test_kitaev_gamma_oracle_sweep():
    """The same energy from the oracle's two-site sweep with the test's
    parameters (D = 60, truncation 1e-4) from the alternating product state."""
    g, mpo, pb = _kitaev()
    N = g["Nx"] * g["Ny"]
    mps = M.direct_product_mps([pb] * N, [i % 2 for i in range(N)], dtype=np.complex128)
    e = vmps.two_site_finite_vmps(mps, mpo, _sweep_params(g["sweep_params"]))
    assert abs(e - g["energy"]) < g["tol"]


def test_kondo_double_chain():
    """test_two_site_update_finite_vmps.cc:976-1084: alternating four-state
    electron and two-state spin sites; exact diagonalisation (4096 states)
    and the oracle sweep with the test's parameters, both builders."""
    from test_mpogen import mpo_dense
    g = GOLD["vmps"]["KondoDoubleChain"]
    mpo, sites = M.kondo_chain_mpo()
    H = mpo_dense(mpo)
    assert abs(np.linalg.eigvalsh((H + H.T) / 2)[0] - g["energy"]) < g["tol"]
    for builder in ("prefix", "reference"):
        mpo, sites = M.kondo_chain_mpo(builder=builder)
        mps = M.direct_product_mps(sites, [i % 2 for i in range(len(sites))])
        e = vmps.two_site_finite_vmps(mps, mpo, _sweep_params(g["sweep_params"]))
        assert abs(e - g["energy"]) < g["tol"]


def test_rashba_tj():
    """test_two_site_update_finite_vmps.cc:627-751: complex spin-orbit hopping,
    periodic x; exact diagonalisation in the charge sector of the initial
    state and the oracle sweep with the test's parameters."""
    from test_mpogen import mpo_dense
    g = GOLD["vmps"]["RashbaTJ"]
    mpo, pb = M.rashba_tj_mpo()
    assert abs(_sector_ground_energy(mpo, pb, g["labels"]) - g["energy"]) < g["tol"]
    mps = M.direct_product_mps([pb] * len(g["labels"]), g["labels"], dtype=np.complex128)
    e = vmps.two_site_finite_vmps(mps, mpo, _sweep_params(g["sweep_params"]))
    assert abs(e - g["energy"]) < g["tol"]


@pytest.mark.parametrize("case", ["tj1d", "tj2d", "Hubbard2x2"])
def test_finite_dmrg_golden_hamiltonians(case):
    """The FiniteDMRG goldens of test_finite_dmrg.cc:484-835 are the ground
    energies of the Hamiltonians built here (exact diagonalisation in the
    sector of the test's initial state)."""
    g = GOLD["dmrg"][case]
    if case == "Hubbard2x2":
        mpo, pb = M.hubbard_2x2_test_mpo()
        labels = [1 if i % 2 == 0 else 2 for i in range(4)]
    else:
        mpo, pb = FERMION[case](np.float64)
        labels = g["labels"]
    assert abs(_sector_ground_energy(mpo, pb, labels) - g["energy"]) < g["tol"]


def test_lanczos_expmv_vs_dense():
    """``tests/test_algorithm/test_lanczos_expmv_solver.cc:222-315``: the Krylov
    exp(-i dt H) psi of a random complex Hermitian H_eff (dt = 0.1, Lanczos
    1e-14 / 100) against the dense matrix exponential, relative distance
    below 1e-13."""
    from scipy.linalg import expm
    eff_ham, psi = _random_single_sector_eff_ham(dtype=np.complex128, seed=3)
    psi.blocks[(0, 0, 0, 0)] = psi.blocks[(0, 0, 0, 0)] + 0.5j * np.random.default_rng(4) \
        .standard_normal(psi.blocks[(0, 0, 0, 0)].shape)
    H = dense_eff_ham(eff_ham)
    v = psi.to_dense().reshape(-1)
    want = expm(-1j * 0.1 * H) @ v
    res = krylov.lanczos_expmv_solver(eff_ham, psi.copy(), krylov.eff_ham_mul_two_site_state,
                                      0.1, krylov.LanczosParams(1e-14, 100))
    got = res.expmv.to_dense().reshape(-1)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-13


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_single_site_lanczos_vs_dense_ed(dtype):
    """``tests/test_algorithm/test_lanczos_solver.cc:209-394``: Lanczos with
    the single-site matvec against the ground energy of the dense operator
    (built column by column from the same matvec), 1e-8."""
    eff_ham, _ = _random_single_sector_eff_ham(D=12, dtype=dtype, seed=5)
    L, W, _, R = eff_ham
    D, d = 12, 2
    q0 = (0,)
    psi = BlockTensorData([Index.make([(q0, D)], IN), Index.make([(q0, d)], OUT),
                           Index.make([(q0, D)], OUT)],
                          {(0, 0, 0): np.random.default_rng(6).standard_normal((D, d, D)).astype(dtype)},
                          dtype)
    n = D * d * D
    H = np.zeros((n, n), dtype=dtype)
    for c in range(n):
        e = psi.copy()
        blk = np.zeros(n, dtype=dtype)
        blk[c] = 1.0
        e.blocks[(0, 0, 0)] = blk.reshape(D, d, D)
        H[:, c] = krylov.eff_ham_mul_single_site_state([L, W, R], e).to_dense().reshape(-1)
    assert np.allclose(H, H.conj().T, atol=1e-10)
    w0 = np.linalg.eigvalsh((H + H.conj().T) / 2)[0]
    res = krylov.lanczos_solver([L, W, R], psi, krylov.eff_ham_mul_single_site_state,
                                krylov.LanczosParams(1e-9, 200))
    assert abs(res.gs_eng - w0) < 1e-8
