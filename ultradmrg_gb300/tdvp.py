"""``TwoSiteFiniteTDVP`` with its operator insertion and correlation output
(algorithm/tdvp/two_site_update_finite_tdvp_impl.h:123-202), on the device.

The reference driver acts ``local_op0`` on ``site_0`` of the ground state
(with ``inst0`` on every site left of it, ``ActOperatorOnMps``, :23-54),
evolves the result by ``step`` two-site TDVP sweeps and, before the first
sweep and after each one, measures ``CalPsi1OpPsi2`` (:540-614) between the
evolved state and the ground state: res[i] = <gs| inst1_{j<i} op1_i |phi(t)>
for every site i, multiplied by exp(i e0 t) after a sweep (t = (step + 1)
tau).  Element k N + i of the result carries sites (site_0, i) and times
(0, k tau), as the reference's ``DynamicMeasuRes``.

Here the insertion is host work on the ground state's blocks
(``models.act_operator_on_mps``), the sweeps are ``api.two_site_finite_tdvp``
one step at a time, and the correlations are ``measure.cal_psi1_op_psi2`` on
the device backend.  States stay in HBM between steps; the reference's disk
paths have no counterpart.  The state's canonical form does not enter the
correlations (the device driver right-canonicalises before each step; a
complete sweep ends with the centre at site 0 again).
"""
from __future__ import annotations

from dataclasses import dataclass, replace
from typing import List, Sequence, Tuple

import numpy as np

from . import api, measure as dm, models as M
from .tensor_data import BlockTensorData


@dataclass
class DynamicMeasuResElem:
    """``DynamicMeasuResElem`` (two_site_update_finite_tdvp_impl.h:103-112)."""

    sites: Tuple[int, int]
    times: Tuple[float, float]
    avg: complex


def _matrix(op):
    if op is None:
        return None
    return np.asarray(op.mat if hasattr(op, "mat") else op).astype(np.complex128)


def _complex(t: BlockTensorData) -> BlockTensorData:
    return BlockTensorData(list(t.indexes),
                           {k: np.asarray(v, dtype=np.complex128) for k, v in t.blocks.items()},
                           np.complex128)


def two_site_finite_tdvp_measured(ctx, gs: Sequence[BlockTensorData], mpo: Sequence,
                                  params: api.TDVPEvolveParams, site0: int, op0, op1,
                                  e0: float, inst0=None, inst1=None
                                  ) -> Tuple[List[DynamicMeasuResElem], list]:
    """The reference's ``TwoSiteFiniteTDVP(mps, mpo, params, ...)`` with
    ``local_op_corr``: ``gs`` the ground state (host blocks), ``mpo`` the
    Hamiltonian's device tensors, ``params.steps`` sweeps of ``params.tau``;
    ``op0``/``inst0`` the inserted operator and its string, ``op1``/``inst1``
    the measured one, ``e0`` the ground-state energy of the phase factor.
    Operators are matrices O[in, out] over the site's physical index (or
    objects with a ``mat``).  Returns the (steps + 1) N measurement records
    and the per-update TDVP log."""
    N = len(gs)
    if N < 2 or not 0 <= site0 < N:
        raise ValueError("two_site_finite_tdvp_measured: need N >= 2 and 0 <= site0 < N")
    if params.steps < 0:
        raise ValueError("two_site_finite_tdvp_measured: steps must be >= 0")
    phi = M.act_operator_on_mps(list(gs), _matrix(op0), _matrix(inst0), site0)
    dphi = [api.DeviceTensor.from_data(ctx, _complex(t)) for t in phi]
    dgs = [api.DeviceTensor.from_data(ctx, _complex(t)) for t in gs]
    backend = dm.device_backend(ctx)
    one = replace(params, steps=1)
    op1m, inst1m = _matrix(op1), _matrix(inst1)
    res: List[DynamicMeasuResElem] = []
    log: list = []
    try:
        for k in range(params.steps + 1):
            if k > 0:
                log += api.two_site_finite_tdvp(ctx, dphi, list(mpo), one)
            t = k * params.tau
            phase = np.exp(1j * e0 * t) if k > 0 else 1.0
            corr = dm.cal_psi1_op_psi2(backend, dphi, dgs, op1m, inst1m)
            res += [DynamicMeasuResElem((site0, i), (0.0, t), complex(corr[i]) * phase)
                    for i in range(N)]
    finally:
        for x in dphi + dgs:
            x.close()
    return res, log
