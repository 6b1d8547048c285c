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


# ---- free fermions (TDVP pins, tests/test_algorithm/test_two_site_finite_tdvp.cc:82-150) ----

def op_tensor(op, pb, dtype=np.complex128):
    """Operator tensor {pb_in, pb_out} of an ``models.Operator``."""
    from ultradmrg_gb300.tensor_data import BlockTensorData
    t = BlockTensorData([pb.inverse(), pb], {}, dtype)
    for (i, o) in np.argwhere(op.mat != 0):
        t.set_elem((int(i), int(o)), op.mat[i, o])
    return t


def act_operator(mps, op_t, inst_t, site):
    """``ActOperatorOnMps``: op on ``site``, the string operator on every site
    left of it (two_site_update_finite_tdvp_impl.h:25-54)."""
    out = list(mps)
    for i, o in [(site, op_t)] + [(j, inst_t) for j in range(site - 1, -1, -1)]:
        t = bs.contract(o, out[i], [0], [1])  # (s_out, l, r)
        out[i] = bs.transpose(t, [1, 0, 2])
    return out


def mps_dense(mps):
    """The state vector (shape (d,)*N) of a short MPS."""
    v = mps[0].to_dense()[0]  # (s, r)
    for A in mps[1:]:
        v = np.tensordot(v, A.to_dense(), axes=([v.ndim - 1], [0]))
    return v[..., 0]


def apply_dense(v, mat, site, string=None):
    """(op ket)_out = sum_in mat[in, out] ket_in on ``site`` (and the string left of it)."""
    ops = [(site, mat)] + ([(j, string) for j in range(site)] if string is not None else [])
    for j, m in ops:
        v = np.moveaxis(np.tensordot(m, v, axes=([0], [j])), 0, j)
    return v


def free_fermion_green(time, L, x1, x2):
    """<GS| c_{x2}(t) c^dag_{x1}(0) |GS> of the open chain (H = -sum c^dag c + h.c.),
    half filling (test_two_site_finite_tdvp.cc:82-101)."""
    res = 0j
    for k in range(1, L + 1):
        eps = -2 * np.cos(k * np.pi / (L + 1))
        if eps > 0:
            res += (np.exp(-1j * eps * time) * np.sin(k * np.pi / (L + 1) * (x1 + 1)) *
                    np.sin(k * np.pi / (L + 1) * (x2 + 1)))
    return res * 2.0 / (L + 1)


def config_problem(name):
    """The two-site problem at the centre bond of a benchmark workload
    (``ultradmrg_gb300.workloads``: seeded MPS with the configuration's
    sizes), environments built by the oracle's environment updates without
    normalisation (their physical scale), as host tensors:
    ([L, W1, W2, R], psi, left divergence of the bond, workload)."""
    from ultradmrg_gb300.workloads import WORKLOADS, build_host
    w = WORKLOADS[name]
    mpo, mps = build_host(w)
    l = w.centre
    eff, psi = two_site_problem(mpo, mps, l, normalize=False)
    return eff, psi, tuple(mps[l].div()), w
