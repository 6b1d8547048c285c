"""Golden energies through the device drivers:

* the fermionic two-site VMPS goldens
  (``tests/test_algorithm/test_fermion_two_site_update_finite_vmps.cc``): free
  fermions N = 8, t-J 1D and 2D with explicit Jordan-Wigner strings, real
  and complex;
* the FiniteDMRG golden of the J-K-Gamma model without symmetry
  (``tests/test_algorithm/test_finite_dmrg.cc:346-444``): one sector of
  dimension 2 per site and an MPO with imaginary entries.

Each runs with the reference's sweep parameters and initial product states,
and with both MPO builders: the prefix-sharing one and the restated
reference generator (``mpogen``: the reference's bond dimensions, sector and
channel order).  The host side (the Hamiltonians by exact diagonalisation,
the oracle sweeps) is pinned in ``test_oracle_golden.py`` and
``test_mpogen.py``.
"""
import json
import os
import re

import numpy as np
import pytest

from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))

BUILDERS = ["prefix", "reference"]

FERMION = {
    "free_fermion8": lambda dt, b: M.free_fermion_chain_mpo(8, dtype=dt, builder=b)[:2],
    "tj1d": lambda dt, b: M.tj_mpo(4, dtype=dt, builder=b),
    "tj2d": lambda dt, b: M.tj_mpo(4, pairs=[(0, 1), (0, 2), (2, 3), (1, 3)], dtype=dt,
                                   builder=b),
}


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _params(text):
    nums = [float(x) for x in re.findall(r"[-0-9.]+(?:[eE][-+]?[0-9]+)?", text)]
    sweeps, dmin, dmax, trunc, err = nums[:5]
    it = int(nums[5]) if len(nums) > 5 else 200
    return api.FiniteVMPSSweepParams(int(sweeps), int(dmin), int(dmax), trunc, err, it)


@pytest.mark.parametrize("builder", BUILDERS)
@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("case", sorted(FERMION))
def test_fermion_vmps_goldens_device(ctx, case, dtype, builder):
    g = GOLD["fermion_vmps"][case]
    mpo, pb = FERMION[case](dtype, builder)
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * len(g["labels"]), g["labels"], dtype=dtype)]
    e0, _ = api.two_site_finite_vmps(ctx, mps, [api.DeviceTensor.from_data(ctx, w) for w in mpo],
                                     _params(g["sweep_params"]))
    assert abs(e0 - g["energy"]) < g["tol"]


def test_kitaev_gamma_finite_dmrg_device(ctx):
    g = GOLD["dmrg_kitaev_gamma"]
    mpo, pb = M.kitaev_gamma_mpo(g["Nx"], g["Ny"], g["J"], g["K"], g["Gm"], g["h"])
    N = g["Nx"] * g["Ny"]
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * N, [i % 2 for i in range(N)],
                                         dtype=np.complex128)]
    e0, _ = api.finite_dmrg(ctx, mps, M.mat_repr_mpo(mpo), _params(g["sweep_params"]))
    assert abs(e0 - g["energy"]) < g["tol"]


@pytest.mark.parametrize("builder", BUILDERS)
def test_kondo_double_chain_device(ctx, builder):
    """Alternating four-state and two-state sites through the device sweep."""
    g = GOLD["vmps"]["KondoDoubleChain"]
    mpo, sites = M.kondo_chain_mpo(builder=builder)
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps(sites, [i % 2 for i in range(len(sites))])]
    e0, _ = api.two_site_finite_vmps(ctx, mps, [api.DeviceTensor.from_data(ctx, w) for w in mpo],
                                     _params(g["sweep_params"]))
    assert abs(e0 - g["energy"]) < g["tol"]


@pytest.mark.parametrize("builder", BUILDERS)
def test_rashba_tj_device(ctx, builder):
    """Complex spin-orbit hopping (an MPO with imaginary entries) through the
    device sweep."""
    g = GOLD["vmps"]["RashbaTJ"]
    mpo, pb = M.rashba_tj_mpo(builder=builder)
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * len(g["labels"]), g["labels"],
                                         dtype=np.complex128)]
    e0, _ = api.two_site_finite_vmps(ctx, mps, [api.DeviceTensor.from_data(ctx, w) for w in mpo],
                                     _params(g["sweep_params"]))
    assert abs(e0 - g["energy"]) < g["tol"]


DMRG = {
    "tj1d": lambda dt, b: M.tj_mpo(4, dtype=dt, builder=b),
    "tj2d": lambda dt, b: M.tj_mpo(4, pairs=[(0, 1), (0, 2), (2, 3), (1, 3)], dtype=dt,
                                   builder=b),
    "Hubbard2x2": lambda dt, b: M.hubbard_2x2_test_mpo(dtype=dt, builder=b),
}


@pytest.mark.parametrize("builder", BUILDERS)
@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("case", sorted(DMRG))
def test_finite_dmrg_goldens_device(ctx, case, dtype, builder):
    """test_finite_dmrg.cc:484-835 through udmrg_finite_dmrg (MatReprMPO in);
    the Hubbard case starts from labels 1, 2, 1, 2 (the test's loop)."""
    g = GOLD["dmrg"][case]
    mpo, pb = DMRG[case](dtype, builder)
    labels = g["labels"] or [1 if i % 2 == 0 else 2 for i in range(len(mpo))]
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * len(labels), labels, dtype=dtype)]
    e0, _ = api.finite_dmrg(ctx, mps, M.mat_repr_mpo(mpo), _params(g["sweep_params"]))
    assert abs(e0 - g["energy"]) < g["tol"]
