"""Two-site finite VMPS (oracle restatement, in memory instead of on disk).

* ``update_site_renvs`` / ``update_site_lenvs`` <- ``algorithm/vmps/vmps_init.h:343-373``
* ``init_envs``          <- ``algorithm/vmps/two_site_update_finite_vmps_impl.h:146-190``
* ``two_site_update``    <- ``two_site_update_finite_vmps_impl.h:232-373``
* ``two_site_sweep``     <- ``two_site_update_finite_vmps_impl.h:197-222``
* ``two_site_finite_vmps`` <- ``two_site_update_finite_vmps_impl.h:95-125``
* ``measure_ee``         <- ``two_site_update_finite_vmps_impl.h:38-49``

The reference keeps MPS tensors and environments on disk between site
updates (``Load/DumpRelatedTensTwoSiteAlg``); that changes no arithmetic, so
here everything stays in lists.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from ultradmrg_gb300.tensor_data import BlockTensorData

from . import blocksparse as bs
from .krylov import LanczosParams, eff_ham_mul_two_site_state, lanczos_solver


@dataclass
class FiniteVMPSSweepParams:
    """``FiniteVMPSSweepParams`` (``algorithm/finite_vmps_sweep_params.h:31-107``)."""

    sweeps: int
    Dmin: int
    Dmax: int
    trunc_err: float
    lancz_params: LanczosParams = field(default_factory=LanczosParams)


def update_site_renvs(renv, mps_ten, mpo_ten):
    mps_dag = bs.dag(mps_ten)
    t = bs.contract_cyclic(mps_dag, renv, 2, 0, 1)
    t2 = bs.contract_cyclic(t, mpo_ten, 1, 2, 2)
    return bs.contract_cyclic(t2, mps_ten, 3, 1, 2)


def update_site_lenvs(lenv, mps_ten, mpo_ten):
    mps_dag = bs.dag(mps_ten)
    t = bs.contract_cyclic(lenv, mps_ten, 2, 0, 1)
    t2 = bs.contract_cyclic(t, mpo_ten, 1, 0, 2)
    return bs.contract_cyclic(mps_dag, t2, 0, 1, 2)


def trivial_renv(mps_last, mpo_last):
    i0 = mps_last.indexes[2]
    R = BlockTensorData([i0, mpo_last.indexes[3].inverse(), i0.inverse()], {},
                        np.result_type(mps_last.dtype, mpo_last.dtype))
    R.set_elem((0, 0, 0), 1.0)
    return R


def trivial_lenv(mps_first, mpo_first):
    i0 = mps_first.indexes[0]
    L = BlockTensorData([i0, mpo_first.indexes[0].inverse(), i0.inverse()], {},
                        np.result_type(mps_first.dtype, mpo_first.dtype))
    L.set_elem((0, 0, 0), 1.0)
    return L


def init_envs(mps, mpo, update_site_num=2):
    N = len(mps)
    renvs: List[Optional[BlockTensorData]] = [None] * N
    lenvs: List[Optional[BlockTensorData]] = [None] * N
    renvs[0] = trivial_renv(mps[N - 1], mpo[N - 1])
    for i in range(1, N - update_site_num + 1):
        renvs[i] = update_site_renvs(renvs[i - 1], mps[N - i], mpo[N - i])
    lenvs[0] = trivial_lenv(mps[0], mpo[0])
    return lenvs, renvs


def measure_ee(s, D):
    ee = 0.0
    for blk in s.blocks.values():
        for v in np.diag(blk):
            p = v * v
            if p > 0:
                ee += -p * np.log(p)
    return ee


@dataclass
class SiteLog:
    site: int
    e0: float
    trunc_err: float
    D: int
    iters: int
    ee: float
    # smallest kept singular value over the largest (test bookkeeping: where
    # Dmin keeps states far below the largest, which ones are kept is decided
    # by rounding-level differences)
    s_min_kept: float = float("nan")


def two_site_update(mps, lenvs, renvs, mpo, params: FiniteVMPSSweepParams, dir, target,
                    log: Optional[list] = None):
    N = len(mps)
    if dir == 'r':
        l, r = target, target + 1
        lenv_len, renv_len = target, N - (target + 2)
    elif dir == 'l':
        l, r = target - 1, target
        lenv_len, renv_len = target - 1, N - target - 1
    else:
        raise ValueError("dir must be 'r' or 'l'")
    eff_ham = [lenvs[lenv_len], mpo[l], mpo[r], renvs[renv_len]]
    init_state = bs.contract(mps[l], mps[r], [2], [0])
    res = lanczos_solver(eff_ham, init_state, eff_ham_mul_two_site_state,
                         params.lancz_params)
    ldiv = mps[l].div()
    u, s, vt, err, D = bs.svd(res.gs_vec, 2, ldiv, params.trunc_err, params.Dmin,
                              params.Dmax)
    ee = measure_ee(s, D)
    if dir == 'r':
        mps[l] = u
        mps[r] = bs.contract(s, vt, [1], [0])
        lenvs[lenv_len + 1] = update_site_lenvs(lenvs[lenv_len], mps[target], mpo[target])
    else:
        mps[l] = bs.contract(u, s, [2], [0])
        mps[r] = vt
        renvs[renv_len + 1] = update_site_renvs(renvs[renv_len], mps[target], mpo[target])
    if log is not None:
        sv = [float(x) for blk in s.blocks.values() for x in np.diag(blk)]
        smin = min(sv) / max(sv) if sv and max(sv) > 0 else float("nan")
        log.append(SiteLog(target, res.gs_eng, err, D, res.iters, ee, smin))
    return res.gs_eng


def two_site_sweep(mps, mpo, params, lenvs, renvs, log=None):
    N = len(mps)
    e0 = None
    for i in range(0, N - 2):
        e0 = two_site_update(mps, lenvs, renvs, mpo, params, 'r', i, log)
    for i in range(N - 1, 1, -1):
        e0 = two_site_update(mps, lenvs, renvs, mpo, params, 'l', i, log)
    return e0


def two_site_finite_vmps(mps, mpo, params: FiniteVMPSSweepParams, log=None):
    """Returns the energy of the last site update of the last sweep.  ``mps``
    is updated in place; its centre must be at site 0 or 1 on entry."""
    lenvs, renvs = init_envs(mps, mpo)
    e0 = None
    for _ in range(params.sweeps):
        e0 = two_site_sweep(mps, mpo, params, lenvs, renvs, log)
    return e0
