"""Mixed-precision matvec (split-BF16 tcgen05 GEMMs, FP32 accumulation)
against the FP64 oracle.

Element-wise the mixed matvec is FP32-accurate (tolerance 2e-5 of the
largest element); energies from Lanczos and from whole sweeps must stay
within |dE/E| <= 1e-9 of the FP64 results, the accuracy bar of the
mixed-precision form.
"""
import json
import os

import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov
from systems import (canonical_system, heisenberg_system, hubbard_system, max_block_diff,
                     two_site_problem)
from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
MIXED = api.PREC_MIXED


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def up(ctx, t):
    return api.DeviceTensor.from_data(ctx, t)


SYSTEMS = {
    "heis": lambda: heisenberg_system(N=10, D=24, seed=0),
    "hub": lambda: hubbard_system(Lx=3, Ly=2, D=40, seed=1),
    "hub_big": lambda: hubbard_system(Lx=4, Ly=2, D=120, seed=3),
}


@pytest.mark.parametrize("name,l", [("heis", 4), ("heis", 0), ("heis", 8), ("hub", 2),
                                    ("hub_big", 3)])
def test_mixed_matvec_parity(ctx, name, l):
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    plan = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    x = plan.embed(dpsi)
    y = plan.embed(dpsi)
    plan.apply(x, y)
    out = y.to_data()
    assert set(ref.blocks) <= set(out.blocks)
    d, s = max_block_diff(out, ref)
    assert d <= 2e-5 * s, (d, s)


@pytest.mark.parametrize("name,l", [("heis", 4), ("hub", 2), ("hub_big", 3), ("hub_big", 1)])
def test_mixed_lanczos_energy(ctx, name, l):
    """Mixed-canonical environments (the scale of a DMRG run): the FP64
    Rayleigh quotient of the mixed-precision ground state vs FP64 Lanczos."""
    mpo, mps = canonical_system(name, l, seed=5)
    eff, psi = two_site_problem(mpo, mps, l, normalize=False)
    ref = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state,
                                krylov.LanczosParams(1e-12, 100))
    res = api.lanczos_solver(ctx, [up(ctx, t) for t in eff], up(ctx, psi), 1e-12, 100,
                             precision=MIXED)
    rel = abs(res.gs_eng - ref.gs_eng) / abs(ref.gs_eng)
    print(f"{name}: mixed Lanczos |dE/E| = {rel:.2e} ({res.iters} iterations)")
    assert rel <= 1e-9


@pytest.mark.parametrize("name,l", [("heis", 4), ("hub", 2), ("hub_big", 3)])
def test_anchor_dw_matvec_vs_oracle(ctx, name, l):
    """The mixed solver's anchor matvec in double-word FP32 arithmetic against
    the oracle's FP64 matvec: 1e-13 of the largest element (48-bit operands,
    error-free products and sums)."""
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    plan = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    x, y = plan.embed(dpsi), plan.embed(dpsi)
    plan.apply_anchor(x, y)
    d, s = max_block_diff(y.to_data(), ref)
    assert d <= 1e-13 * s, (d, s)


def test_anchor_dw_workload(ctx):
    """The anchor at the 4x8 D=256 workload: double-word against the FP64
    pipe, 1e-13 of the largest element and in norm."""
    from ultradmrg_gb300.workloads import WORKLOADS, build_host
    w = WORKLOADS["hubbard4x8_D256"]
    mpo, mps = build_host(w)
    l = w.centre
    L, R = api.build_envs(ctx, mpo, mps, l, normalize=False)
    psi = api.contract(ctx, up(ctx, mps[l]), up(ctx, mps[l + 1]), [2], [0])
    plan = api.MatvecPlan(ctx, [L, up(ctx, mpo[l]), up(ctx, mpo[l + 1]), R], psi,
                          precision=MIXED)
    x, ya, yb = plan.embed(psi), plan.embed(psi), plan.embed(psi)
    try:
        plan.apply_anchor(x, ya)
        ctx.set_anchor_dw(False)
        plan.apply_anchor(x, yb)
    finally:
        ctx.set_anchor_dw(True)
    a, b = ya.download_packed(), yb.download_packed()
    assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b))
    assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(b)


@pytest.mark.parametrize("name,l", [("hub", 2), ("hub_big", 3)])
def test_mixed_lanczos_anchor_forms(ctx, name, l):
    """Mixed Lanczos with the double-word anchor and with the FP64-pipe
    anchor: energies within 1e-12 relative of each other and of the oracle's
    FP64 Lanczos to 1e-10."""
    mpo, mps = canonical_system(name, l, seed=5)
    eff, psi = two_site_problem(mpo, mps, l, normalize=False)
    ref = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state,
                                krylov.LanczosParams(1e-12, 100))
    dev = [up(ctx, t) for t in eff]
    e = {}
    try:
        for dw in (True, False):
            ctx.set_anchor_dw(dw)
            e[dw] = api.lanczos_solver(ctx, dev, up(ctx, psi), 1e-12, 100,
                                       precision=MIXED).gs_eng
    finally:
        ctx.set_anchor_dw(True)
    assert abs(e[True] - e[False]) <= 1e-12 * abs(e[False])
    assert abs(e[True] - ref.gs_eng) <= 1e-10 * abs(ref.gs_eng)


@pytest.mark.parametrize("name,l", [("hub", 2), ("hub_big", 3)])
def test_gemm_tile_policies_bit_identical(ctx, name, l):
    """The FP64 matvec and the double-word anchor under both tile policies of
    the grouped GEMMs: bit-identical (every output sums in the same order)."""
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    out = {}
    try:
        for pol in (0, 1):
            ctx.set_gemm_tiles(pol)
            p64 = api.MatvecPlan(ctx, dev, dpsi, precision=api.PREC_FP64)
            pmx = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
            assert p64.gemm_policy() == pol and pmx.gemm_policy() == pol
            x, y, z = p64.embed(dpsi), p64.embed(dpsi), p64.embed(dpsi)
            p64.apply(x, y)
            pmx.apply_anchor(x, z)
            out[pol] = (y.download_packed(), z.download_packed())
    finally:
        ctx.set_gemm_tiles(-1)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_gemm_tile_autotuner(ctx):
    """With the autotuner on, the first plan of a shape class runs the timed
    trials; a second plan of the class reuses the decision."""
    mpo, mps = SYSTEMS["hub_big"]()
    eff, psi = two_site_problem(mpo, mps, 3)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    ctx.set_gemm_tiles(-1)
    api.MatvecPlan(ctx, dev, dpsi, precision=api.PREC_FP64)
    t0, c0 = ctx.gemm_tuning()
    p = api.MatvecPlan(ctx, dev, dpsi, precision=api.PREC_FP64)
    t1, c1 = ctx.gemm_tuning()
    assert c0 >= 1 and t1 == t0 and c1 == c0
    assert p.gemm_policy() in (0, 1)


def test_plan_host_threads_bit_identical(ctx):
    """The first mixed plan of a fresh context builds its tables on this
    thread (tile trials); later plans build them on host threads beside the
    contraction plans.  Both give bit-identical matvecs, and the plan reports
    its build phases."""
    mpo, mps = SYSTEMS["hub_big"]()
    eff, psi = two_site_problem(mpo, mps, 3)
    c2 = api.Context(0)
    dev = [up(c2, t) for t in eff]
    dpsi = up(c2, psi)
    out = []
    for rep in range(3):
        pmx = api.MatvecPlan(c2, dev, dpsi, precision=MIXED)
        p64 = api.MatvecPlan(c2, dev, dpsi, precision=api.PREC_FP64)
        bt = pmx.build_times()
        assert set(bt) == set(api.MatvecPlan.PLAN_PHASES)
        assert all(v >= 0.0 for v in bt.values())
        x, y, z, w = (pmx.embed(dpsi) for _ in range(4))
        pmx.apply(x, y)
        pmx.apply_anchor(x, z)
        p64.apply(x, w)
        out.append([t.download_packed() for t in (y, z, w)])
    for rep in (1, 2):
        for k in range(3):
            assert np.array_equal(out[0][k], out[rep][k])


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_apply_host_modes(ctx, mode):
    """apply_host with page-locked buffers (used in place under modes 1 and 2)
    and with pageable ones (always copied): the device-buffer product, bit for
    bit, every entry written."""
    torch = pytest.importorskip("torch")
    mpo, mps = SYSTEMS["hub_big"]()
    eff, psi = two_site_problem(mpo, mps, 3)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    plan = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    x, y = plan.embed(dpsi), plan.embed(dpsi)
    plan.apply(x, y)
    want = y.download_packed()
    xin = x.download_packed()
    n = xin.size
    before = ctx.host_mapped()
    try:
        ctx.set_host_mapped(mode)
        assert ctx.host_mapped() == mode
        hx = torch.from_numpy(xin.copy()).pin_memory()
        hy = torch.full((n,), float("nan"), dtype=torch.float64).pin_memory()
        for _ in range(2):
            plan.apply_host_ptr(hx.data_ptr(), hy.data_ptr())
            assert np.array_equal(hy.numpy(), want)
        px, py = xin.copy(), np.full(n, np.nan)
        plan.apply_host_ptr(px.ctypes.data, py.ctypes.data)
        assert np.array_equal(py, want)
    finally:
        ctx.set_host_mapped(before)


def _gpu_vmps(ctx, mpo, pb, labels, params):
    mps0 = M.direct_product_mps([pb] * len(labels), labels)
    dmps = [up(ctx, t) for t in mps0]
    dmpo = [up(ctx, t) for t in mpo]
    return api.two_site_finite_vmps(ctx, dmps, dmpo, params)


def test_mixed_vmps_golden_heisenberg(ctx):
    g = GOLD["vmps"]["1DHeisenberg"]
    mpo, pb = M.heisenberg_chain_mpo(6)
    e0, _ = _gpu_vmps(ctx, mpo, pb, [i % 2 for i in range(6)],
                      api.FiniteVMPSSweepParams(4, 8, 8, 1e-9, 1e-7, precision=MIXED))
    assert abs(e0 - g["energy"]) <= 1e-9 * abs(g["energy"])


def test_mixed_vmps_golden_hubbard2x2(ctx):
    g = GOLD["vmps"]["Hubbard2x2"]
    mpo, pb = M.hubbard_2x2_test_mpo()
    e0, _ = _gpu_vmps(ctx, mpo, pb, [1 if i % 2 == 0 else 2 for i in range(4)],
                      api.FiniteVMPSSweepParams(10, 16, 16, 1e-9, 1e-8, 20, precision=MIXED))
    assert abs(e0 - g["energy"]) <= 1e-9 * abs(g["energy"])


def test_mixed_vmps_heisenberg16_vs_fp64(ctx):
    N = 16
    mpo, pb = M.heisenberg_chain_mpo(N)
    labels = M.random_sz0_labels(N, 0)
    e_mixed, log_m = _gpu_vmps(ctx, mpo, pb, labels,
                               api.FiniteVMPSSweepParams(6, 32, 32, 1e-10, 1e-10, 100,
                                                         precision=MIXED))
    e_fp64, log_d = _gpu_vmps(ctx, mpo, pb, labels,
                              api.FiniteVMPSSweepParams(6, 32, 32, 1e-10, 1e-10, 100))
    per_sweep = 2 * (N - 2)
    for s in range(6):
        em, ed = log_m[(s + 1) * per_sweep - 1]["e0"], log_d[(s + 1) * per_sweep - 1]["e0"]
        print(f"sweep {s + 1}: mixed {em:.12f} fp64 {ed:.12f} |dE/E| {abs(em - ed) / abs(ed):.2e}")
    rel = abs(e_mixed - e_fp64) / abs(e_fp64)
    print(f"L=16 D=32 sweep: |dE/E| mixed vs FP64 = {rel:.2e}")
    assert rel <= 1e-9


@pytest.mark.parametrize("workload", ["hubbard4x8_D256"])
def test_mixed_matvec_workload(ctx, workload):
    """The benchmark's synthetic Hubbard workload, whose sector pairs carry
    more than 32 MPO output channels (several channel chunks per warp):
    mixed against the device FP64 form, element-wise 2e-5 of the largest
    element."""
    from ultradmrg_gb300.workloads import WORKLOADS, build_host
    w = WORKLOADS[workload]
    mpo, mps = build_host(w)
    l = w.centre
    L, R = api.build_envs(ctx, mpo, mps, l, normalize=False)
    psi = api.contract(ctx, up(ctx, mps[l]), up(ctx, mps[l + 1]), [2], [0])
    eh = [L, up(ctx, mpo[l]), up(ctx, mpo[l + 1]), R]
    pm = api.MatvecPlan(ctx, eh, psi, precision=MIXED)
    p64 = api.MatvecPlan(ctx, eh, psi, precision=api.PREC_FP64)
    x, ym, yd = pm.embed(psi), pm.embed(psi), pm.embed(psi)
    pm.apply(x, ym)
    p64.apply(x, yd)
    a, b = ym.download_packed(), yd.download_packed()
    assert np.max(np.abs(a - b)) <= 2e-5 * np.max(np.abs(b))
    assert np.linalg.norm(a - b) <= 2e-5 * np.linalg.norm(b)


@pytest.mark.parametrize("name,l,cplx", [("heis", 4, False), ("hub", 2, False),
                                         ("hub_big", 3, False), ("heis", 4, True)])
def test_fused_mpo_gemm_bit_identical(ctx, name, l, cplx):
    """The MPO step fused into the .R GEMM's producers against the separate MPO
    kernel + image GEMM: the same FP32 sums in the same order, the same BF16
    split, the same MMAs, so the results agree bit for bit."""
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    dt = np.complex128 if cplx else None
    dev = [api.DeviceTensor.from_data(ctx, t, dt) for t in eff]
    dpsi = api.DeviceTensor.from_data(ctx, psi, dt)
    plan = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    x, yf, yu = plan.embed(dpsi), plan.embed(dpsi), plan.embed(dpsi)
    plan.set_fused(True)
    plan.apply(x, yf)
    plan.set_fused(False)
    plan.apply(x, yu)
    a, b = yf.download_packed(), yu.download_packed()
    assert np.array_equal(a, b)
    if not cplx:
        ref = krylov.eff_ham_mul_two_site_state(eff, psi)
        d, s = max_block_diff(yf.to_data(), ref)
        assert d <= 2e-5 * s, (d, s)


def test_fused_mpo_gemm_workload(ctx):
    """The same on the benchmark's synthetic Hubbard 4x8 D=256 workload."""
    from ultradmrg_gb300.workloads import WORKLOADS, build_host
    w = WORKLOADS["hubbard4x8_D256"]
    mpo, mps = build_host(w)
    l = w.centre
    L, R = api.build_envs(ctx, mpo, mps, l, normalize=False)
    psi = api.contract(ctx, up(ctx, mps[l]), up(ctx, mps[l + 1]), [2], [0])
    pm = api.MatvecPlan(ctx, [L, up(ctx, mpo[l]), up(ctx, mpo[l + 1]), R], psi, precision=MIXED)
    x, yf, yu = pm.embed(psi), pm.embed(psi), pm.embed(psi)
    pm.set_fused(True)
    pm.apply(x, yf)
    pm.set_fused(False)
    pm.apply(x, yu)
    assert np.array_equal(yf.download_packed(), yu.download_packed())


@pytest.mark.parametrize("tiles", [(128, 128), (64, 128), (128, 64)])
@pytest.mark.parametrize("name,l", [("hub", 2), ("hub_big", 3)])
def test_tc_tile_shapes(ctx, tiles, name, l):
    """B tiles of 128 rows (either GEMM) against the oracle and against 64-row
    tiles; the fused form with the same tiles bit for bit."""
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    try:
        ctx.set_tc_tiles(64, 64)
        p64 = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
        ctx.set_tc_tiles(*tiles)
        pt = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    finally:
        ctx.set_tc_tiles(0, 0)
    assert pt.tiles()[:2] == tiles
    x, y64, yt, yf = pt.embed(dpsi), pt.embed(dpsi), pt.embed(dpsi), pt.embed(dpsi)
    p64.apply(x, y64)
    pt.apply(x, yt)
    pt.set_fused(True)
    pt.apply(x, yf)
    a, b = yt.download_packed(), y64.download_packed()
    assert np.array_equal(yf.download_packed(), a)
    assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b))
    d, s = max_block_diff(yt.to_data(), ref)
    assert d <= 2e-5 * s, (d, s)


def test_tc_tile_autotuner(ctx):
    """With no tiles set, the first plan of a shape class runs the timed
    trials and later plans of the class reuse the choice."""
    mpo, mps = SYSTEMS["hub_big"]()
    eff, psi = two_site_problem(mpo, mps, 3)
    dev = [up(ctx, t) for t in eff]
    dpsi = up(ctx, psi)
    t0, _ = ctx.tc_tuning()
    p1 = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    t1, classes = ctx.tc_tuning()
    p2 = api.MatvecPlan(ctx, dev, dpsi, precision=MIXED)
    t2, _ = ctx.tc_tuning()
    assert p1.tiles()[2] and p2.tiles()[2] and classes >= 1
    assert p1.tiles() == p2.tiles()
    assert t2 == t1 and t1 <= t0 + 1
