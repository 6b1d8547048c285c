"""Two-site finite TDVP (oracle restatement, test infrastructure only).

* ``right_canonicalize``    <- the ``RightCanonicalizeTen`` loop of
  ``algorithm/tdvp/two_site_update_finite_tdvp_impl.h:145-152``
* ``two_site_evolution``    <- ``TwoSiteFiniteTDVPEvolution`` (:261-417)
* ``single_site_backward``  <- ``SingleSiteFiniteTDVPBackwardEvolution``
  with dir ``'n'`` (:419-531)
* ``tdvp_sweep``            <- ``TwoSiteFiniteTDVPSweep`` (:196-259)

Environments and MPS tensors stay in lists instead of on disk.  Operator
insertion and the correlation measurements of ``TwoSiteFiniteTDVP`` are left
to the caller (the tests compose them from ``measure.py``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import blocksparse as bs
from .krylov import (LanczosParams, eff_ham_mul_single_site_state,
                     eff_ham_mul_two_site_state, lanczos_expmv_solver)
from .vmps import init_envs, update_site_lenvs, update_site_renvs


@dataclass
class TDVPParams:
    tau: float
    Dmin: int
    Dmax: int
    trunc_err: float
    lancz_params: LanczosParams


def _complex(t):
    return bs.scale(t, 1.0 + 0j) if t.dtype != np.complex128 else t


def right_canonicalize(mps):
    """Sites N-1 .. 1 right-isometric; the centre ends at site 0."""
    for i in range(len(mps) - 1, 0, -1):
        u, s, vt, _, _ = bs.svd(mps[i], 1, mps[i].div(), 0.0, 1, 1 << 40)
        mps[i] = vt
        us = bs.contract(u, s, [1], [0])
        mps[i - 1] = bs.contract(mps[i - 1], us, [2], [0])


def two_site_evolution(mps, lenvs, renvs, mpo, p: TDVPParams, dir, target, step):
    N = len(mps)
    if dir == 'r':
        l, r = target, target + 1
        lenv_len, renv_len = target, N - (target + 2)
    else:
        l, r = target - 1, target
        lenv_len, renv_len = target - 1, N - target - 1
    eff_ham = [lenvs[lenv_len], mpo[l], mpo[r], renvs[renv_len]]
    init_state = bs.contract(mps[l], mps[r], [2], [0])
    res = lanczos_expmv_solver(eff_ham, init_state, eff_ham_mul_two_site_state, step,
                               p.lancz_params)
    u, s, vt, err, D = bs.svd(res.expmv, 2, mps[l].div(), p.trunc_err, p.Dmin, p.Dmax)
    if dir == 'r':
        mps[l] = u
        mps[r] = bs.contract(s, vt, [1], [0])
        lenvs[lenv_len + 1] = update_site_lenvs(lenvs[lenv_len], mps[target], mpo[target])
    else:
        mps[l] = bs.contract(u, s, [2], [0])
        mps[r] = vt
        renvs[renv_len + 1] = update_site_renvs(renvs[renv_len], mps[target], mpo[target])
    return err, D, res.iters


def single_site_backward(mps, lenvs, renvs, mpo, p: TDVPParams, site, step):
    N = len(mps)
    eff_ham = [lenvs[site], mpo[site], renvs[N - site - 1]]
    res = lanczos_expmv_solver(eff_ham, mps[site], eff_ham_mul_single_site_state, step,
                               p.lancz_params)
    mps[site] = res.expmv
    return res.iters


def tdvp_sweep(mps, mpo, p: TDVPParams, lenvs, renvs):
    N = len(mps)
    half = p.tau / 2
    for i in range(0, N - 2):
        two_site_evolution(mps, lenvs, renvs, mpo, p, 'r', i, half)
        single_site_backward(mps, lenvs, renvs, mpo, p, i + 1, -half)
    for i in range(N - 1, 1, -1):
        two_site_evolution(mps, lenvs, renvs, mpo, p, 'l', i, p.tau if i == N - 1 else half)
        single_site_backward(mps, lenvs, renvs, mpo, p, i - 1, -half)
    two_site_evolution(mps, lenvs, renvs, mpo, p, 'r', 0, half)


def two_site_finite_tdvp(mps, mpo, p: TDVPParams, steps: int):
    """``steps`` TDVP sweeps after right-canonicalisation; ``mps`` is updated in place."""
    for i in range(len(mps)):
        mps[i] = _complex(mps[i])
    mpo = [_complex(w) for w in mpo]
    right_canonicalize(mps)
    lenvs, renvs = init_envs(mps, mpo)
    for _ in range(steps):
        tdvp_sweep(mps, mpo, p, lenvs, renvs)
    return mps
