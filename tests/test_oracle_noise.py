"""The noised two-site VMPS of the oracle (``oracle/noise.py``) against the
reference's noise-test goldens (``tests/test_algorithm/
test_two_site_noise_update_finite_vmps.cc``: 1D and 2D Heisenberg, N = 6,
D = 8, noises 1e-2 .. 1e-5, 1e-12), with both MPO builders, and its index
operations (fusion, expansion, combiners, boundaries) on their own."""
import json
import os

import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import krylov, noise as ON
from ultradmrg_gb300 import models as M

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
PAIRS_2D = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 5), (4, 5)]


def noise_params(g):
    kw = {k: g[k] for k in ("max_noise", "noise_increase", "noise_decrease", "alpha") if k in g}
    return ON.NoiseSweepParams(g["sweeps"], g["Dmin"], g["Dmax"], g["trunc_err"],
                               krylov.LanczosParams(g["lanczos_error"], 200), list(g["noises"]),
                               **kw)


@pytest.mark.parametrize("builder", ["prefix", "reference"])
@pytest.mark.parametrize("case", ["1DHeisenberg", "2DHeisenberg"])
def test_noise_vmps_goldens(case, builder):
    g = GOLD["noise_vmps"][case]
    mpo, pb = M.heisenberg_chain_mpo(6, pairs=PAIRS_2D if case == "2DHeisenberg" else None,
                                     builder=builder)
    mps = M.direct_product_mps([pb] * 6, [i % 2 for i in range(6)])
    used = []
    e0 = ON.two_site_finite_vmps_with_noise(mps, mpo, noise_params(g), None, used)
    assert abs(e0 - g["energy"]) < g["tol"]
    assert any(u > 0 for u in used)  # the bonds were expanded


def test_fuse_and_expand():
    mpo, pb = M.heisenberg_chain_mpo(8)
    mps = M.random_mps([pb] * 8, (0,), 12, seed=3)
    t = bs.contract(mps[3], mps[4], [2], [0])  # (a, s1, s2, b)
    f = ON.fuse_axes(t, 0, 3, t.indexes[3].dir)
    assert f.rank == 3 and abs(bs.norm(f) - bs.norm(t)) <= 1e-14 * bs.norm(t)
    assert f.div() == t.div()
    # expansion by zeros keeps the norm and the old blocks
    e = ON.expand(t, None, 3, t.indexes[3])
    assert abs(bs.norm(e) - bs.norm(t)) <= 1e-14 * bs.norm(t)
    assert e.indexes[3].dim == 2 * t.indexes[3].dim
    # appending a tensor adds its weight
    e2 = ON.expand(t, t, 3)
    assert abs(bs.norm(e2) ** 2 - 2 * bs.norm(t) ** 2) <= 1e-12 * bs.norm(t) ** 2


def test_combiner_isometry_and_boundaries():
    idx = M.spin_half_site()[0]
    c = ON.combiner(idx.inverse(), idx, 1)
    cc = bs.contract(bs.dag(c), c, [0, 1], [0, 1])
    for k, b in cc.blocks.items():
        assert np.allclose(b, np.eye(b.shape[0]))
    # the boundaries keep the state
    from systems import mps_dense
    mpo, pb = M.heisenberg_chain_mpo(8)
    mps = M.random_mps([pb] * 8, (0,), 6, seed=1)
    v0 = mps_dense(mps)
    work = [t.copy() for t in mps]
    left, right = ON.boundaries(work, 6)
    v1 = mps_dense(work)
    ov = abs(np.vdot(v0, v1)) / (np.linalg.norm(v0) * np.linalg.norm(v1))
    assert abs(ov - 1.0) < 1e-12
    assert 0 <= left < right <= 7
