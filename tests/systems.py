"""Seeded test systems: MPO + random MPS + environments built by the oracle."""
import numpy as np

from oracle import blocksparse as bs
from oracle import vmps as ovmps
from ultradmrg_gb300 import models as M


def heisenberg_system(N=10, D=24, seed=0, dtype=np.float64):
    mpo, pb = M.heisenberg_chain_mpo(N)
    mps = M.random_mps([pb] * N, (0,), D, seed=seed, dtype=dtype)
    return mpo, mps


def hubbard_system(Lx=3, Ly=2, D=32, seed=1, dtype=np.float64, holes=1):
    mpo, pb = M.hubbard_cylinder_mpo(Lx, Ly, t=1.0, U=8.0)
    N = Lx * Ly
    div = (N - holes, 0 if (N - holes) % 2 == 0 else 1)
    mps = M.random_mps([pb] * N, div, D, seed=seed, dtype=dtype)
    return mpo, mps


def canonical_system(kind, l, seed=0, D=None, dtype=np.float64):
    """Mixed-canonical random MPS around site l (environments at physical scale)."""
    if kind == "heis":
        N = 10
        mpo, pb = M.heisenberg_chain_mpo(N)
        mps = M.random_canonical_mps([pb] * N, (0,), D or 24, l, seed=seed, dtype=dtype)
    else:
        Lx, Ly = (3, 2) if kind == "hub" else (4, 2)
        N = Lx * Ly
        mpo, pb = M.hubbard_cylinder_mpo(Lx, Ly, t=1.0, U=8.0)
        ne = N - 1
        mps = M.random_canonical_mps([pb] * N, (ne, ne % 2), D or (40 if kind == "hub" else 120),
                                     l, seed=seed, dtype=dtype)
    return mpo, mps


def envs_at(mpo, mps, l, normalize=True):
    """Left env of sites [0, l) and right env of sites (l+1, N) via the oracle."""
    N = len(mps)
    L = ovmps.trivial_lenv(mps[0], mpo[0])
    for i in range(l):
        L = ovmps.update_site_lenvs(L, mps[i], mpo[i])
        if normalize:
            L = bs.scale(L, 1.0 / max(1e-300, bs.norm(L)))
    R = ovmps.trivial_renv(mps[N - 1], mpo[N - 1])
    for i in range(N - 1, l + 1, -1):
        R = ovmps.update_site_renvs(R, mps[i], mpo[i])
        if normalize:
            R = bs.scale(R, 1.0 / max(1e-300, bs.norm(R)))
    return L, R


def two_site_problem(mpo, mps, l, normalize=True):
    L, R = envs_at(mpo, mps, l, normalize)
    psi = bs.contract(mps[l], mps[l + 1], [2], [0])
    return [L, mpo[l], mpo[l + 1], R], psi


def max_block_diff(gpu, ref):
    """max |gpu - ref| over blocks, and whether gpu's extra blocks are zero."""
    diff = 0.0
    for k, v in ref.blocks.items():
        g = gpu.blocks.get(k)
        if g is None:
            diff = max(diff, float(np.max(np.abs(v))))
        else:
            diff = max(diff, float(np.max(np.abs(g - v))))
    for k, g in gpu.blocks.items():
        if k not in ref.blocks:
            diff = max(diff, float(np.max(np.abs(g))))
    scale = max(1e-300, max(float(np.max(np.abs(v))) for v in ref.blocks.values()))
    return diff, scale
