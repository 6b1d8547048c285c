"""Sector-wise randomized SVD against the exact block SVD (and the oracle).

The randomized path must reproduce the exact truncation: same kept count per
bond sector, truncation error and kept Schmidt weights within 1e-10
absolute; too-small sketches must be detected (misses) and grown until the
result is exact.
"""
import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov
from systems import canonical_system, two_site_problem
from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ground_state():
    """Lanczos ground state of a two-site problem (a decaying Schmidt spectrum)."""
    mpo, mps = canonical_system("hub_big", 3, seed=5)
    eff, psi = two_site_problem(mpo, mps, 3, normalize=False)
    res = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state,
                                krylov.LanczosParams(1e-12, 100))
    g = res.gs_vec
    bs.normalize(g)
    return g, mps[3].div()


def _weights(s):
    return np.concatenate([np.diag(b) for _, b in sorted(s.blocks.items())]) ** 2


def _sector_kept(u):
    bond = u.indexes[-1]
    return {q: d for q, d in zip(bond.qns, bond.dims)}


@pytest.mark.parametrize("how", ["exact_guess", "small_guess", "no_guess"])
@pytest.mark.parametrize("D,trunc", [(40, 1e-8), (400, 1e-10)])
def test_rsvd_matches_exact(ctx, ground_state, how, D, trunc):
    psi, ldiv = ground_state
    u, s, vt, err, Dk = bs.svd(psi, 2, ldiv, trunc, 1, D)
    kept = _sector_kept(u)
    if how == "exact_guess":
        sketch = list(kept.items())
    elif how == "small_guess":
        sketch = [(q, 1) for q in kept]
    else:
        sketch = []
    dpsi = api.DeviceTensor.from_data(ctx, psi)
    gu, gs, gvt, gerr, gD, rounds = api.svd_randomized(ctx, dpsi, 2, ldiv, trunc, 1, D, sketch,
                                                       oversample=4)
    gu, gs, gvt = gu.to_data(), gs.to_data(), gvt.to_data()
    assert gD == Dk
    assert abs(gerr - err) <= 1e-10
    assert _sector_kept(gu) == kept
    assert set(gu.blocks) == set(u.blocks) and set(gvt.blocks) == set(vt.blocks)
    # kept Schmidt weights: within the same 1e-10 absolute bar as the truncation error
    assert np.allclose(_weights(gs), _weights(s), rtol=1e-9, atol=1e-10)
    # the kept subspace agrees up to the sketch error (sigma_{k+p}/sigma_k)^(2q+1)
    rec_ref = bs.contract(bs.contract(u, s, [2], [0]), vt, [2], [0])
    rec_gpu = bs.contract(bs.contract(gu, gs, [2], [0]), gvt, [2], [0])
    diff = bs.linear_combine([1.0, -1.0], [rec_gpu, rec_ref], 0.0,
                             bs.T(list(rec_ref.indexes), {}, rec_ref.dtype))
    rel = bs.norm(diff) / bs.norm(rec_ref)
    print(f"{how} D={D}: truncated-state distance {rel:.2e}, grow rounds {rounds}")
    assert rel <= 1e-5  # energy effect is second order: <= ~1e-10
    if how == "small_guess":
        assert rounds >= 1  # the too-small sketches were detected and grown


def _vmps(ctx, mpo, pb, labels, params):
    mps0 = M.direct_product_mps([pb] * len(labels), labels)
    dmps = [api.DeviceTensor.from_data(ctx, t) for t in mps0]
    dmpo = [api.DeviceTensor.from_data(ctx, t) for t in mpo]
    return api.two_site_finite_vmps(ctx, dmps, dmpo, params)


def test_sweep_randomized_svd_matches_exact(ctx):
    N = 16
    mpo, pb = M.heisenberg_chain_mpo(N)
    labels = M.random_sz0_labels(N, 1)
    e_ex, log_ex = _vmps(ctx, mpo, pb, labels, api.FiniteVMPSSweepParams(4, 24, 24, 1e-9, 1e-10, 100))
    e_rs, log_rs = _vmps(ctx, mpo, pb, labels,
                         api.FiniteVMPSSweepParams(4, 24, 24, 1e-9, 1e-10, 100, svd_mode=1))
    assert abs(e_rs - e_ex) <= 1e-10 * abs(e_ex)
    for a, b in zip(log_rs, log_ex):
        assert a["D"] == b["D"]
        assert abs(a["trunc_err"] - b["trunc_err"]) <= 1e-10
