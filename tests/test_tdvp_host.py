"""Argument checks of the measured TDVP driver (``ultradmrg_gb300.tdvp``),
raised before any device call."""
import numpy as np
import pytest

from ultradmrg_gb300 import api, models as M, tdvp as T


def _chain(N=4):
    mpo, pb = M.heisenberg_chain_mpo(N)
    gs = M.direct_product_mps([pb] * N, [i % 2 for i in range(N)])
    _, ops = M.spin_half_site()
    return gs, ops


@pytest.mark.parametrize("site0", [-1, 4])
def test_site_out_of_range(site0):
    gs, ops = _chain()
    with pytest.raises(ValueError):
        T.two_site_finite_tdvp_measured(None, gs, [], api.TDVPEvolveParams(0.1, 1, 1, 4, 0.0),
                                        site0, ops["sp"], ops["sm"], 0.0)


def test_negative_steps():
    gs, ops = _chain()
    with pytest.raises(ValueError):
        T.two_site_finite_tdvp_measured(None, gs, [], api.TDVPEvolveParams(0.1, -1, 1, 4, 0.0),
                                        1, ops["sp"], ops["sm"], 0.0)


def test_records_layout():
    """DynamicMeasuResElem carries (site0, i) and (0, t) like the reference's."""
    r = T.DynamicMeasuResElem((2, 5), (0.0, 0.3), 1.0 + 0.5j)
    assert r.sites == (2, 5) and r.times == (0.0, 0.3) and np.isclose(r.avg, 1.0 + 0.5j)
