"""The noised two-site VMPS (subspace expansion) through the device driver
``udmrg_two_site_finite_vmps_noise``:

* the reference's noise-test goldens (1D and 2D Heisenberg, N = 6, D = 8,
  ``tests/test_algorithm/test_two_site_noise_update_finite_vmps.cc``), real and
  complex, with both MPO builders;
* a truncating case against the oracle's noised sweep (``oracle/noise.py``):
  per-update energies, bond dimensions, truncation errors and the noise each
  update applied;
* the mixed-precision matvec against the FP64 one on the same case.
"""
import json
import os

import numpy as np
import pytest

from oracle import krylov, noise as ON
from ultradmrg_gb300 import api, models as M

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
PAIRS_2D = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]
KEYS = ("max_noise", "noise_increase", "noise_decrease", "alpha")


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _run(ctx, mpo, pb, labels, sweeps, D, trunc, lerr, noises, dtype=np.float64, prec=0,
         dmin=None, **kw):
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * len(labels), labels, dtype=dtype)]
    dmpo = [api.DeviceTensor.from_data(ctx, w) for w in mpo]
    p = api.FiniteVMPSSweepParams(sweeps, D if dmin is None else dmin, D, trunc, lerr, 200,
                                  precision=prec)
    return api.two_site_finite_vmps_noise(ctx, mps, dmpo, p, noises, **kw)


@pytest.mark.parametrize("builder", ["prefix", "reference"])
@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("case", ["1DHeisenberg", "2DHeisenberg"])
def test_noise_vmps_goldens_device(ctx, case, dtype, builder):
    g = GOLD["noise_vmps"][case]
    mpo, pb = M.heisenberg_chain_mpo(6, pairs=PAIRS_2D if case == "2DHeisenberg" else None,
                                     dtype=dtype, builder=builder)
    kw = {k: g[k] for k in KEYS if k in g}
    e0, log, used = _run(ctx, mpo, pb, [i % 2 for i in range(6)], g["sweeps"], g["Dmax"],
                         g["trunc_err"], g["lanczos_error"], g["noises"], dtype=dtype, **kw)
    assert abs(e0 - g["energy"]) < g["tol"], (e0, g["energy"])
    assert any(u > 0 for u in used)


def test_noise_vmps_vs_oracle(ctx):
    """Heisenberg chain N = 12, Dmax = 12 (truncating), noises 0.1, 0.01,
    0.001, Lanczos 1e-12: the device sweep against the oracle's, update by
    update.  Dmin = 1: with Dmin = Dmax the first updates keep numerically null
    states (a product-state start has fewer than Dmin non-zero singular
    values), whose vectors are any orthonormal completion; the next update's
    variational space, and so its energy, then depends on that arbitrary
    choice (it differs between two platforms' LAPACK already).

    Per-update energies agree to 1e-7 relative, the final energy to 1e-9.  The
    first sweep starts from a product state with noise 0.1, and its updates
    keep states whose singular values lie 1e-5 below their sector's largest.
    The device takes singular vectors from the sector's Gram matrix, so such a
    vector carries an error of about eps * s_1^2 / (s_k^2 - s_k+1^2) (7e-7 at
    site 4 here), which rotates the next update's variational space; LAPACK's
    direct SVD in the oracle has eps * s_1 / (s_k - s_k+1) instead."""
    N, D = 12, 12
    mpo, pb = M.heisenberg_chain_mpo(N, builder="reference")
    labels = M.random_sz0_labels(N, 5)
    noises = [0.1, 0.01, 0.001]
    e0, log, used = _run(ctx, mpo, pb, labels, 4, D, 1e-10, 1e-12, noises, dmin=1)
    olog, oused, margins = [], [], []
    oe = ON.two_site_finite_vmps_with_noise(
        M.direct_product_mps([pb] * N, labels), mpo,
        ON.NoiseSweepParams(4, 1, D, 1e-10, krylov.LanczosParams(1e-12, 200), noises),
        olog, oused, margins)
    assert abs(e0 - oe) <= 1e-9 * abs(oe)
    assert len(log) == len(olog)
    # Update by update until the applied noises part.  Where an update neither
    # truncates nor changes the state, the next energy expectation equals the
    # last energy up to rounding, and the sign that raises or keeps the noise
    # (the reference's sharp rule) is a coin toss on either side: the two
    # noise sequences may part there, and only there.  Up to the update that
    # first applies a different noise the states are the same.
    compared, coin_toss = 0, False
    for a, b, u, ou, mg in zip(log, olog, used, oused, margins):
        assert a["site"] == b.site
        assert abs(a["e0"] - b.e0) <= 1e-7 * abs(b.e0)
        coin_toss = coin_toss or abs(mg) < 1e-10
        if abs(u - ou) > 1e-12 * max(ou, 1e-300):
            assert coin_toss, (compared, u, ou)
            break
        assert a["D"] == b.D
        assert abs(a["trunc_err"] - b.trunc_err) <= 1e-10
        compared += 1
    assert compared >= 5
    assert sum(1 for u in used if u > 0) > 0


def test_noise_vmps_mixed_vs_fp64(ctx):
    N, D = 12, 12
    mpo, pb = M.heisenberg_chain_mpo(N, builder="reference")
    labels = M.random_sz0_labels(N, 5)
    noises = [0.1, 0.01, 0.001]
    e64, _, _ = _run(ctx, mpo, pb, labels, 4, D, 1e-10, 1e-12, noises)
    emx, _, _ = _run(ctx, mpo, pb, labels, 4, D, 1e-10, 1e-12, noises, prec=api.PREC_MIXED)
    assert abs(emx - e64) <= 1e-9 * abs(e64)
