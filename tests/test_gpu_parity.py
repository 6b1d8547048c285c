"""GPU parity: the C-ABI path against the FP64 oracle on seeded inputs.

Tolerances: FP64 block GEMMs in a different summation order than numpy, so
element-wise results agree to ~1e-13 relative; energies to 1e-10.
"""
import json
import os

import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov, vmps as ovmps
from ultradmrg_gb300 import api, models as M
from systems import heisenberg_system, hubbard_system, max_block_diff, two_site_problem

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def up(ctx, t, dtype=None):
    return api.DeviceTensor.from_data(ctx, t, dtype)


SYSTEMS = {
    "heis": lambda: heisenberg_system(N=10, D=24, seed=0),
    "hub": lambda: hubbard_system(Lx=3, Ly=2, D=40, seed=1),
    "heis_c": lambda: heisenberg_system(N=8, D=16, seed=2, dtype=np.complex128),
}


@pytest.mark.parametrize("name,l", [("heis", 4), ("heis", 0), ("heis", 8), ("hub", 2),
                                    ("heis_c", 3)])
def test_matvec_parity(ctx, name, l):
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    dev = [up(ctx, t, psi.dtype) for t in eff]
    out = api.eff_ham_mul_two_site_state(ctx, dev, up(ctx, psi)).to_data()
    assert [i for i in out.indexes] == [i for i in ref.indexes]
    assert set(ref.blocks) <= set(out.blocks)
    d, s = max_block_diff(out, ref)
    assert d <= RTOL * s * 10


@pytest.mark.parametrize("name,l", [("heis", 4), ("hub", 2)])
def test_lanczos_parity(ctx, name, l):
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    params = krylov.LanczosParams(1e-12, 100)
    ref = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state, params)
    dev = [up(ctx, t) for t in eff]
    res = api.lanczos_solver(ctx, dev, up(ctx, psi), 1e-12, 100)
    # 1e-10 relative; absolute below |E| = 1 (both solvers stop at an energy
    # change of 1e-12, so a near-zero energy agrees only to that level)
    assert abs(res.gs_eng - ref.gs_eng) <= 1e-10 * max(abs(ref.gs_eng), 1.0)
    g = res.gs_vec.to_data()
    ov = abs(bs.inner(ref.gs_vec, g)) / (bs.norm(ref.gs_vec) * bs.norm(g))
    assert abs(ov - 1.0) < 1e-8


def test_lanczos_dense_ed(ctx):
    """The dense-ED check of ``tests/test_algorithm/test_lanczos_solver.cc`` on the GPU."""
    from test_oracle_golden import _random_single_sector_eff_ham, dense_eff_ham
    for dtype in (np.float64, np.complex128):
        eff, psi = _random_single_sector_eff_ham(dtype=dtype)
        w = np.linalg.eigvalsh(dense_eff_ham(eff))
        res = api.lanczos_solver(ctx, [up(ctx, t) for t in eff], up(ctx, psi), 1e-9, 200)
        assert abs(res.gs_eng - w[0]) < 1e-8


@pytest.mark.parametrize("name,l", [("heis", 3), ("hub", 2)])
def test_env_update_parity(ctx, name, l):
    mpo, mps = SYSTEMS[name]()
    L, R = (two_site_problem(mpo, mps, l)[0][i] for i in (0, 3))
    refL = ovmps.update_site_lenvs(L, mps[l], mpo[l])
    refR = ovmps.update_site_renvs(R, mps[l + 1], mpo[l + 1])
    gL = api.update_site_lenvs(ctx, up(ctx, L), up(ctx, mps[l]), up(ctx, mpo[l])).to_data()
    gR = api.update_site_renvs(ctx, up(ctx, R), up(ctx, mps[l + 1]), up(ctx, mpo[l + 1])).to_data()
    for g, r in ((gL, refL), (gR, refR)):
        assert g.indexes == r.indexes
        assert set(g.blocks) == set(r.blocks)  # bit-exact block bookkeeping
        d, s = max_block_diff(g, r)
        assert d <= RTOL * s * 10


@pytest.mark.parametrize("name,l,D,trunc", [("heis", 4, 12, 1e-6), ("hub", 2, 20, 1e-8),
                                            ("heis", 4, 1000, 1e-12)])
def test_svd_parity(ctx, name, l, D, trunc):
    mpo, mps = SYSTEMS[name]()
    psi = bs.contract(mps[l], mps[l + 1], [2], [0])
    bs.normalize(psi)
    ldiv = mps[l].div()
    u, s, vt, err, Dk = bs.svd(psi, 2, ldiv, trunc, 1, D)
    gu, gs, gvt, gerr, gD = api.svd(ctx, up(ctx, psi), 2, ldiv, trunc, 1, D)
    assert gD == Dk
    assert abs(gerr - err) <= 1e-10
    gu, gs, gvt = gu.to_data(), gs.to_data(), gvt.to_data()
    # identical kept-state set: same bond sectors and sizes, same block lists
    assert gu.indexes == u.indexes and gvt.indexes == vt.indexes
    assert set(gu.blocks) == set(u.blocks) and set(gvt.blocks) == set(vt.blocks)
    sv_ref = np.concatenate([np.diag(b) for _, b in sorted(s.blocks.items())])
    sv_gpu = np.concatenate([np.diag(b) for _, b in sorted(gs.blocks.items())])
    # Schmidt weights s^2 agree to FP64 accuracy of the Gram-matrix spectrum
    assert np.allclose(sv_gpu ** 2, sv_ref ** 2, rtol=1e-9, atol=1e-13)
    # gauge-invariant reconstruction of the truncated state
    rec_ref = bs.contract(bs.contract(u, s, [2], [0]), vt, [2], [0])
    rec_gpu = bs.contract(bs.contract(gu, gs, [2], [0]), gvt, [2], [0])
    d, sc = max_block_diff(rec_gpu, rec_ref)
    assert d <= 1e-9 * sc


def _gpu_vmps(ctx, mpo, pb, labels, params):
    mps0 = M.direct_product_mps([pb] * len(labels), labels)
    dmps = [up(ctx, t) for t in mps0]
    dmpo = [up(ctx, t) for t in mpo]
    e0, log = api.two_site_finite_vmps(ctx, dmps, dmpo, params)
    return e0, log, dmps


def test_vmps_golden_heisenberg(ctx):
    g = GOLD["vmps"]["1DHeisenberg"]
    mpo, pb = M.heisenberg_chain_mpo(6)
    e0, log, _ = _gpu_vmps(ctx, mpo, pb, [i % 2 for i in range(6)],
                           api.FiniteVMPSSweepParams(4, 8, 8, 1e-9, 1e-7))
    assert abs(e0 - g["energy"]) < g["tol"]


def test_vmps_golden_ising(ctx):
    g = GOLD["vmps"]["1DIsing"]
    mpo, pb = M.ising_chain_mpo(6)
    e0, _, _ = _gpu_vmps(ctx, mpo, pb, [i % 2 for i in range(6)],
                         api.FiniteVMPSSweepParams(4, 1, 10, 1e-5, 1e-7))
    assert abs(e0 - g["energy"]) < g["tol"]


def test_vmps_golden_heisenberg2d(ctx):
    g = GOLD["vmps"]["2DHeisenberg"]
    pairs = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]
    mpo, pb = M.heisenberg_chain_mpo(6, pairs=pairs)
    e0, _, _ = _gpu_vmps(ctx, mpo, pb, [i % 2 for i in range(6)],
                         api.FiniteVMPSSweepParams(4, 8, 8, 1e-9, 1e-7))
    assert abs(e0 - g["energy"]) < g["tol"]


def test_vmps_golden_hubbard2x2(ctx):
    g = GOLD["vmps"]["Hubbard2x2"]
    mpo, pb = M.hubbard_2x2_test_mpo()
    e0, _, _ = _gpu_vmps(ctx, mpo, pb, [1 if i % 2 == 0 else 2 for i in range(4)],
                         api.FiniteVMPSSweepParams(10, 16, 16, 1e-9, 1e-8, 20))
    assert abs(e0 - g["energy"]) < g["tol"]


def test_vmps_heisenberg16_vs_oracle(ctx):
    """A truncating sweep (L=16, D=24): per-site energies, truncation errors and
    bond dimensions against the oracle run with the same parameters.  Lanczos
    runs to 1e-12 on both sides: a truncating sweep carries each local
    solve's residual into the next environments, so a looser tolerance lets
    summation order alone move the final energy by about that tolerance."""
    N = 16
    mpo, pb = M.heisenberg_chain_mpo(N)
    labels = M.random_sz0_labels(N, 0)
    params = api.FiniteVMPSSweepParams(2, 24, 24, 1e-8, 1e-12, 100)
    e0, log, _ = _gpu_vmps(ctx, mpo, pb, labels, params)
    mps = M.direct_product_mps([pb] * N, labels)
    olog = []
    oe = ovmps.two_site_finite_vmps(
        mps, mpo, ovmps.FiniteVMPSSweepParams(2, 24, 24, 1e-8, krylov.LanczosParams(1e-12, 100)),
        olog)
    assert abs(e0 - oe) <= 1e-9 * abs(oe)
    assert len(log) == len(olog)
    for a, b in zip(log, olog):
        assert a["D"] == b.D
        assert abs(a["trunc_err"] - b.trunc_err) <= 1e-10
