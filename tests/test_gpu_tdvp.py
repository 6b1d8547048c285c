"""Two-site TDVP path on the device against the oracle and the reference's
analytic free-fermion test.

* complex truncated SVD: kept states, truncation error (1e-10) and the
  truncated state against the oracle's numpy SVD;
* single-site matvec (eff_ham_mul_single_site_state) element-wise;
* Krylov exp(-i dt H) (two-site and single-site forms) against the oracle;
* TDVP sweeps against the oracle's restatement (state amplitudes, 1e-10);
* the free-fermion Green's function after a c^dag insertion, 30 steps of
  dt = 0.01, against its closed form (1e-10), with the ground state from the
  device sweep driver (energy 1e-12 from the reference's golden value).
"""
import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov
from oracle import tdvp as otdvp
from oracle.krylov import LanczosParams
from systems import (act_operator, apply_dense, canonical_system, free_fermion_green,
                     max_block_diff, mps_dense, op_tensor, two_site_problem)
from ultradmrg_gb300 import _lib, api, models as M

pytestmark = pytest.mark.gpu

GOLD_E0 = -3.4939592074349334893668128643185  # test_two_site_finite_tdvp.cc:125


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def up(ctx, t):
    return api.DeviceTensor.from_data(ctx, t)


def _complex_system(kind, l, seed):
    mpo, mps = canonical_system(kind, l, seed=seed, dtype=np.complex128)
    return [bs.scale(w, 1.0 + 0j) for w in mpo], mps


@pytest.mark.parametrize("kind,l,D", [("heis", 4, 16), ("hub", 2, 40), ("hub_big", 3, 60)])
def test_complex_svd_parity(ctx, kind, l, D):
    mpo, mps = _complex_system(kind, l, 3)
    eff, psi = two_site_problem(mpo, mps, l)
    res = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state,
                                krylov.LanczosParams(1e-12, 60))
    g = res.gs_vec
    bs.normalize(g)
    ldiv = mps[l].div()
    u, s, vt, err, Dk = bs.svd(g, 2, ldiv, 1e-8, 1, D)
    gu, gs, gvt, gerr, gD = api.svd(ctx, up(ctx, g), 2, ldiv, 1e-8, 1, D)
    gu, gs, gvt = gu.to_data(), gs.to_data(), gvt.to_data()
    assert gD == Dk and abs(gerr - err) <= 1e-10
    assert set(gu.blocks) == set(u.blocks) and set(gvt.blocks) == set(vt.blocks)
    w = np.concatenate([np.diag(b) for _, b in sorted(s.blocks.items())])
    gw = np.concatenate([np.diag(b) for _, b in sorted(gs.blocks.items())])
    assert np.allclose(gw ** 2, w ** 2, atol=1e-13)
    rec = bs.contract(bs.contract(u, s, [2], [0]), vt, [2], [0])
    grec = bs.contract(bs.contract(gu, gs, [2], [0]), gvt, [2], [0])
    d, _ = max_block_diff(grec, rec)
    assert d <= 1e-10
    # left factor isometric
    uu = bs.contract(bs.dag(gu), gu, [0, 1], [0, 1])
    for k, b in uu.blocks.items():
        assert np.allclose(b, np.eye(b.shape[0]), atol=1e-12)


def _single_site_problem(mpo, mps, site):
    N = len(mps)
    from oracle import vmps as ovmps
    lenv = ovmps.trivial_lenv(mps[0], mpo[0])
    for i in range(site):
        lenv = ovmps.update_site_lenvs(lenv, mps[i], mpo[i])
    renv = ovmps.trivial_renv(mps[N - 1], mpo[N - 1])
    for i in range(N - 1, site, -1):
        renv = ovmps.update_site_renvs(renv, mps[i], mpo[i])
    return [lenv, mpo[site], renv], mps[site]


@pytest.mark.parametrize("kind,site", [("heis", 4), ("heis", 0), ("hub", 3)])
def test_single_site_matvec_parity(ctx, kind, site):
    mpo, mps = _complex_system(kind, site, 5)
    eff, psi = _single_site_problem(mpo, mps, site)
    ref = krylov.eff_ham_mul_single_site_state(eff, psi)
    out = api.eff_ham_mul_single_site_state(ctx, [up(ctx, t) for t in eff], up(ctx, psi))
    out = out.to_data()
    assert set(ref.blocks) <= set(out.blocks)
    d, scale = max_block_diff(out, ref)
    assert d <= 1e-12 * scale


@pytest.mark.parametrize("form", ["two", "one"])
def test_expmv_parity(ctx, form):
    mpo, mps = _complex_system("heis", 4, 7)
    if form == "two":
        eff, psi = two_site_problem(mpo, mps, 4)
        mv = krylov.eff_ham_mul_two_site_state
    else:
        eff, psi = _single_site_problem(mpo, mps, 4)
        mv = krylov.eff_ham_mul_single_site_state
    step = 0.05
    ref = krylov.lanczos_expmv_solver(eff, psi.copy(), mv, step, LanczosParams(1e-12, 30))
    it, out = api.lanczos_expmv_solver(ctx, [up(ctx, t) for t in eff], up(ctx, psi), step,
                                       1e-12, 30)
    out = out.to_data()
    d, scale = max_block_diff(out, ref.expmv)
    assert d <= 1e-10 * scale


def _fermion_gs(ctx, N=6):
    mpo, pb, ops = M.free_fermion_chain_mpo(N, dtype=np.complex128)
    mps0 = M.direct_product_mps([pb] * N, [i % 2 for i in range(N)], dtype=np.complex128)
    dmps = [up(ctx, t) for t in mps0]
    dmpo = [up(ctx, t) for t in mpo]
    e0, _ = api.two_site_finite_vmps(ctx, dmps, dmpo,
                                     api.FiniteVMPSSweepParams(8, 1, 16, 1e-12, 1e-13, 200))
    return e0, [t.to_data() for t in dmps], mpo, pb, ops


def test_tdvp_matches_oracle(ctx):
    N = 8
    mpo, pb = M.heisenberg_chain_mpo(N, dtype=np.complex128)
    mps = M.random_mps([pb] * N, (0,), 12, seed=4, dtype=np.complex128)
    p = otdvp.TDVPParams(0.05, 4, 12, 1e-9, LanczosParams(1e-12, 30))
    ref = otdvp.two_site_finite_tdvp([t.copy() for t in mps], mpo, p, 2)
    dmps = [up(ctx, t) for t in mps]
    log = api.two_site_finite_tdvp(ctx, dmps, [up(ctx, t) for t in mpo],
                                   api.TDVPEvolveParams(0.05, 2, 4, 12, 1e-9, 1e-12, 30))
    assert len(log) == 2 * (4 * N - 7)
    v = mps_dense([t.to_data() for t in dmps])
    vr = mps_dense(ref)
    assert np.linalg.norm(v - vr) <= 1e-10 * np.linalg.norm(vr)


def test_tdvp_free_fermion_dynamics(ctx):
    N, site0, dt, steps = 6, 3, 0.01, 30
    e0, gs, mpo, pb, ops = _fermion_gs(ctx, N)
    assert abs(e0 - GOLD_E0) <= 1e-12
    gs_v = mps_dense(gs)
    cdag, f = op_tensor(ops["cdag"], pb), op_tensor(ops["f"], pb)
    dmps = [up(ctx, t) for t in act_operator(gs, cdag, f, site0)]
    dmpo = [up(ctx, t) for t in mpo]
    params = api.TDVPEvolveParams(dt, 1, 10, 16, 1e-10, 1e-12, 40)
    worst = 0.0
    for step in range(1, steps + 1):
        api.two_site_finite_tdvp(ctx, dmps, dmpo, params)
        v = mps_dense([t.to_data() for t in dmps])
        t = step * dt
        for x2 in range(N):
            g = np.vdot(gs_v, apply_dense(v, ops["c"].mat, x2, ops["f"].mat))
            g *= np.exp(1j * e0 * t)
            d = abs(g - free_fermion_green(t, N, site0, x2))
            worst = max(worst, d)
            assert d <= 1e-10, (step, x2, d)
    print(f"max |G - G_exact| over {steps} steps: {worst:.2e}")


# ---- complex mixed precision (real embedding of the split-BF16 pipeline) ----

@pytest.mark.parametrize("kind,l", [("heis", 4), ("hub", 2)])
def test_complex_mixed_matvec_parity(ctx, kind, l):
    """Complex L, R, psi with a (promoted) real MPO: element-wise 2e-5 of the
    largest element against the oracle, as the real mixed form."""
    mpo, mps = _complex_system(kind, l, 3)
    eff, psi = two_site_problem(mpo, mps, l)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    plan = api.MatvecPlan(ctx, dev, dpsi, precision=api.PREC_MIXED)
    x, y = plan.embed(dpsi), plan.embed(dpsi)
    plan.apply(x, y)
    d, s = max_block_diff(y.to_data(), ref)
    assert d <= 2e-5 * s, (d, s)


def test_complex_mixed_rejects_complex_mpo(ctx):
    """MPO tensors with nonzero imaginary parts are refused by the mixed form
    (its fused coefficients are real); the FP64 form takes them."""
    mpo, mps = _complex_system("heis", 4, 3)
    mpo = [bs.scale(w, 1.0 + 0.5j) for w in mpo]
    eff, psi = two_site_problem(mpo, mps, 4)
    dev = [up(ctx, t) for t in eff]
    with pytest.raises(_lib.UdmrgError):
        api.MatvecPlan(ctx, dev, up(ctx, psi), precision=api.PREC_MIXED)
    api.MatvecPlan(ctx, dev, up(ctx, psi), precision=api.PREC_FP64).close()


def test_mixed_expmv(ctx):
    """exp(-i dt H) psi with the mixed two-site matvec against the oracle."""
    mpo, mps = _complex_system("heis", 4, 7)
    eff, psi = two_site_problem(mpo, mps, 4)
    step = 0.05
    ref = krylov.lanczos_expmv_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state, step,
                                      LanczosParams(1e-12, 30))
    it, out = api.lanczos_expmv_solver(ctx, [up(ctx, t) for t in eff], up(ctx, psi), step,
                                       1e-12, 30, precision=api.PREC_MIXED)
    d, scale = max_block_diff(out.to_data(), ref.expmv)
    print(f"mixed expmv: iters {it}, max diff {d / scale:.2e} of the largest element")
    assert d <= 1e-5 * scale


def test_mixed_tdvp_vs_fp64(ctx):
    """Two TDVP sweeps of a complex Heisenberg chain with the mixed two-site
    matvec against the FP64 form on the device: state and energy."""
    N = 8
    mpo, pb = M.heisenberg_chain_mpo(N, dtype=np.complex128)
    mps = M.random_mps([pb] * N, (0,), 12, seed=4, dtype=np.complex128)
    dmpo = [up(ctx, t) for t in mpo]
    out = {}
    for prec in (api.PREC_FP64, api.PREC_MIXED):
        dmps = [up(ctx, t) for t in mps]
        api.two_site_finite_tdvp(ctx, dmps, dmpo,
                                 api.TDVPEvolveParams(0.05, 2, 4, 12, 1e-9, 1e-12, 30,
                                                      precision=prec))
        out[prec] = mps_dense([t.to_data() for t in dmps])
    a, b = out[api.PREC_MIXED], out[api.PREC_FP64]
    err = np.linalg.norm(a - b) / np.linalg.norm(b)
    print(f"mixed TDVP vs FP64: relative state difference {err:.2e}")
    assert err <= 1e-5


def test_tdvp_ladder_quench_vs_oracle(ctx):
    """The ladder TDVP benchmark script (``ultradmrg_gb300.tdvp_ladder``) at a
    reduced size: 2x4 ladder, ground state at D = 16, S+ quench at the centre,
    four steps of dt = 0.05 with Krylov 20.  The FP64 device evolution against
    the oracle's TDVP from the same quenched state (amplitudes, 1e-10), the
    mixed form against the FP64 one (local <Sz> and overlap)."""
    from ultradmrg_gb300 import tdvp_ladder as TL
    out, final, quenched, mpo_c = TL.run(ctx, Lx=4, D=16, steps=4, dt=0.05, krylov=20, every=2,
                                         gs_schedule="2:8,2:16")
    p = otdvp.TDVPParams(0.05, 1, 16, 1e-10, LanczosParams(1e-10, 20))
    ref = otdvp.two_site_finite_tdvp([t.copy() for t in quenched], mpo_c, p, 4)
    v, vr = mps_dense(final["fp64"]), mps_dense(ref)
    assert np.linalg.norm(v - vr) <= 1e-10 * np.linalg.norm(vr)
    for cp in out["checkpoints"]:
        assert cp["max_abs_dSz"] <= 1e-6, cp
        assert cp["overlap_err"] <= 1e-8, cp


def test_tdvp_measured_driver_free_fermion(ctx):
    """The TwoSiteFiniteTDVP driver with its measurements
    (``ultradmrg_gb300.tdvp``): c^dag inserted at site 3 with the f string,
    ten steps of dt = 0.01, c measured with the f string; every record
    <GS| c_x(t) c^dag_3 |GS> e^{i E0 t} against the closed form (1e-10), the
    records in the reference's order (step-major, sites (site0, x))."""
    from ultradmrg_gb300 import tdvp as T
    N, site0, dt, steps = 6, 3, 0.01, 10
    e0, gs, mpo, pb, ops = _fermion_gs(ctx, N)
    dmpo = [up(ctx, t) for t in mpo]
    params = api.TDVPEvolveParams(dt, steps, 10, 16, 1e-10, 1e-12, 40)
    res, log = T.two_site_finite_tdvp_measured(ctx, gs, dmpo, params, site0, ops["cdag"],
                                               ops["c"], e0, ops["f"], ops["f"])
    assert len(res) == (steps + 1) * N
    assert len(log) == steps * (4 * N - 7)
    for k in range(steps + 1):
        for x in range(N):
            r = res[k * N + x]
            assert r.sites == (site0, x) and abs(r.times[1] - k * dt) < 1e-15
            assert abs(r.avg - free_fermion_green(k * dt, N, site0, x)) <= 1e-10, (k, x)
    for t in dmpo:
        t.close()
