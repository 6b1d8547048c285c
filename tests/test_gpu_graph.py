"""Krylov steps replayed as CUDA graphs against direct kernel launches.

Every kernel of a Krylov step reads the step index from device memory, so a
solve captures its step once and replays it.  Both modes run the same
kernels on the same data: energies, vectors and iteration counts agree
exactly (bit for bit), and a replay counts the same kernels as the direct
launch sequence.  Covered: the Lanczos ground state (FP64 real and complex,
mixed precision), the Krylov exponential (two-site and single-site FP64,
mixed), and a TDVP run and a truncating VMPS sweep through the drivers.
"""
import numpy as np
import pytest

from oracle import blocksparse as bs
from systems import canonical_system, heisenberg_system, hubbard_system, mps_dense, \
    two_site_problem
from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.set_krylov_graph(True)
    c.close()


def up(ctx, t):
    return api.DeviceTensor.from_data(ctx, t)


def both_modes(ctx, fn):
    """fn() with direct launches, then with graph replays: [(result, launches)].
    One untimed call first fills the context's per-shape caches (the tile
    autotuner's timed trials run once per shape class), so both counted calls
    launch the same work."""
    out = []
    fn()
    ctx.sync()
    try:
        for graph in (False, True):
            ctx.set_krylov_graph(graph)
            l0 = ctx.launches()
            r = fn()
            ctx.sync()
            out.append((r, ctx.launches() - l0))
    finally:
        ctx.set_krylov_graph(True)
    return out


def same_blocks(a, b):
    assert a.indexes == b.indexes and set(a.blocks) == set(b.blocks)
    for k in a.blocks:
        assert np.array_equal(a.blocks[k], b.blocks[k])


SYSTEMS = {
    "heis": lambda: heisenberg_system(N=10, D=24, seed=0),
    "hub": lambda: hubbard_system(Lx=3, Ly=2, D=40, seed=1),
    "hub_big": lambda: hubbard_system(Lx=4, Ly=2, D=120, seed=3),
    "heis_c": lambda: heisenberg_system(N=8, D=16, seed=2, dtype=np.complex128),
}


@pytest.mark.parametrize("name,l,prec", [("heis", 4, api.PREC_FP64), ("hub", 2, api.PREC_FP64),
                                         ("heis_c", 3, api.PREC_FP64),
                                         ("hub_big", 3, api.PREC_MIXED),
                                         ("heis", 4, api.PREC_MIXED)])
def test_lanczos_graph_identical(ctx, name, l, prec):
    mpo, mps = SYSTEMS[name]()
    eff, psi = two_site_problem(mpo, mps, l)
    dev = [up(ctx, t) for t in eff]

    def solve():
        r = api.lanczos_solver(ctx, dev, up(ctx, psi), 1e-12, 100, precision=prec)
        return r.iters, r.gs_eng, r.matvecs, r.gs_vec.to_data()

    (r0, l0), (r1, l1) = both_modes(ctx, solve)
    assert r0[0] == r1[0] and r0[2] == r1[2]
    assert r0[1] == r1[1]  # bitwise
    same_blocks(r0[3], r1[3])
    assert l0 == l1


def _complex_system(kind, l, seed):
    mpo, mps = canonical_system(kind, l, seed=seed, dtype=np.complex128)
    return [bs.scale(w, 1.0 + 0j) for w in mpo], mps


@pytest.mark.parametrize("form,prec", [("two", api.PREC_FP64), ("one", api.PREC_FP64),
                                       ("two", api.PREC_MIXED)])
def test_expmv_graph_identical(ctx, form, prec):
    from test_gpu_tdvp import _single_site_problem
    mpo, mps = _complex_system("heis", 4, 7)
    if form == "two":
        eff, psi = two_site_problem(mpo, mps, 4)
    else:
        eff, psi = _single_site_problem(mpo, mps, 4)
    dev = [up(ctx, t) for t in eff]

    def solve():
        it, out = api.lanczos_expmv_solver(ctx, dev, up(ctx, psi), 0.05, 1e-12, 30,
                                           precision=prec)
        return it, out.to_data()

    (r0, l0), (r1, l1) = both_modes(ctx, solve)
    assert r0[0] == r1[0]
    same_blocks(r0[1], r1[1])
    assert l0 == l1


def test_tdvp_graph_identical(ctx):
    N = 8
    mpo, pb = M.heisenberg_chain_mpo(N, dtype=np.complex128)
    mps = M.random_mps([pb] * N, (0,), 12, seed=4, dtype=np.complex128)
    dmpo = [up(ctx, t) for t in mpo]

    def run():
        dmps = [up(ctx, t) for t in mps]
        api.two_site_finite_tdvp(ctx, dmps, dmpo,
                                 api.TDVPEvolveParams(0.05, 2, 4, 12, 1e-9, 1e-12, 30))
        return mps_dense([t.to_data() for t in dmps])

    (a, l0), (b, l1) = both_modes(ctx, run)
    assert np.array_equal(a, b)
    assert l0 == l1


def test_vmps_graph_identical(ctx):
    N = 12
    mpo, pb = M.heisenberg_chain_mpo(N)
    labels = M.random_sz0_labels(N, 0)
    dmpo = [up(ctx, t) for t in mpo]

    def run():
        dmps = [up(ctx, t) for t in M.direct_product_mps([pb] * N, labels)]
        e0, log = api.two_site_finite_vmps(ctx, dmps, dmpo,
                                           api.FiniteVMPSSweepParams(2, 16, 16, 1e-8, 1e-10, 60))
        return e0, [(x["D"], x["trunc_err"]) for x in log]

    (a, l0), (b, l1) = both_modes(ctx, run)
    assert a == b
    assert l0 == l1


def test_krylov_step_probe(ctx):
    """The vector-kernel probe times every kernel of one step and counts the
    bytes each moves: 3, 2 and 4 vectors for normalise, alpha and update,
    2 (s + 1) + 3 for a re-orthogonalisation pass against v_0 .. v_s."""
    n, s = 200_003, 6
    pr = ctx.krylov_step_probe(n, s)
    v = 8.0 * n
    assert pr["bytes"]["normalise"] == 3 * v
    assert pr["bytes"]["alpha"] == 2 * v
    assert pr["bytes"]["update"] == 4 * v
    assert pr["bytes"]["reorth_pass1"] == (2 * (s + 1) + 3) * v
    assert pr["bytes"]["reorth_pass2"] == (pr["bytes"]["reorth_pass1"] if pr["second_pass_ran"]
                                           else 0.0)
    assert all(t > 0.0 for t in pr["ms"].values())
