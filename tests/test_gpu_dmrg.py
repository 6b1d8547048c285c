"""FiniteDMRG over a matrix-representation MPO (MatReprMPO) through the C ABI.

The reference's FiniteDMRG goldens (tests/test_algorithm/test_finite_dmrg.cc,
values in tests/golden/reference_goldens.json) with the reference's sweep
parameters, and equality with the MPO-tensor sweep (same Hamiltonian, same
start state) site by site.
"""
import json
import os

import pytest

from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _run(ctx, mpo, pb, labels, params, mat_repr=True):
    mps0 = M.direct_product_mps([pb] * len(labels), labels)
    dmps = [api.DeviceTensor.from_data(ctx, t) for t in mps0]
    if mat_repr:
        return api.finite_dmrg(ctx, dmps, M.mat_repr_mpo(mpo), params)
    return api.two_site_finite_vmps(ctx, dmps, [api.DeviceTensor.from_data(ctx, t) for t in mpo],
                                    params)


CASES = {
    # test_finite_dmrg.cc: 1DIsing (4 sweeps, D 1..10, 1e-5, Lanczos 1e-7)
    "1DIsing": (lambda: M.ising_chain_mpo(6), api.FiniteVMPSSweepParams(4, 1, 10, 1e-5, 1e-7)),
    "1DHeisenberg": (lambda: M.heisenberg_chain_mpo(6),
                     api.FiniteVMPSSweepParams(4, 8, 8, 1e-9, 1e-7)),
    "2DHeisenberg": (lambda: M.heisenberg_chain_mpo(
        6, pairs=[(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]),
        api.FiniteVMPSSweepParams(4, 8, 8, 1e-9, 1e-7)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_finite_dmrg_golden(ctx, name):
    g = GOLD["dmrg"][name]
    build, params = CASES[name]
    mpo, pb = build()
    labels = [i % 2 for i in range(6)]
    e0, log = _run(ctx, mpo, pb, labels, params)
    assert abs(e0 - g["energy"]) < g["tol"]
    # the same sweep on the MPO tensors: equal site by site
    e1, log1 = _run(ctx, mpo, pb, labels, params, mat_repr=False)
    assert len(log) == len(log1)
    for a, b in zip(log, log1):
        assert a["D"] == b["D"]
        assert abs(a["e0"] - b["e0"]) <= 1e-12 * max(1.0, abs(b["e0"]))


def test_mat_repr_hubbard_matches_mpo(ctx):
    """A U(1)xU(1) model whose MPO bond carries several channels per quantum
    number (channel grouping into bond sectors)."""
    mpo, pb = M.hubbard_cylinder_mpo(3, 2, t=1.0, U=8.0)
    labels = M.hubbard_cylinder_holes(6, 1)
    params = api.FiniteVMPSSweepParams(3, 1, 32, 1e-10, 1e-10, 60)
    e0, log = _run(ctx, mpo, pb, labels, params)
    e1, log1 = _run(ctx, mpo, pb, labels, params, mat_repr=False)
    assert abs(e0 - e1) <= 1e-10 * abs(e1)
    for a, b in zip(log, log1):
        assert a["D"] == b["D"]
