"""Two-site VMPS with noise (subspace expansion), oracle restatement.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``algorithm/vmps/two_site_update_noise_finite_vmps_impl.h``:

* ``two_site_finite_vmps_with_noise`` <- ``TwoSiteFiniteVMPSWithNoise`` (:81-126):
  boundaries, then sweeps whose starting noise is ``noises[sweep]`` (the last
  one repeats);
* ``boundaries``     <- ``CheckAndUpdateBoundaryMPSTensors``
  (``algorithm/vmps/vmps_init.h:135-246``): edge tensors whose bond can hold
  the whole block Hilbert space become index combiners, and sweeps run only
  between the first sites where ``Dmax`` binds;
* ``noise_sweep``    <- ``TwoSiteFiniteVMPSSweep`` (:132-200): the noise
  adapts from the energy expectation before each update
  (``CalEnergyEptTwoSite``, :688-721) against the previous update's;
* ``noise_update``   <- ``TwoSiteFiniteVMPSUpdate`` (:216-404): Lanczos, the
  quantum-number coverage test (``IsQNCovered``, :727-765), the expansion,
  truncated SVD, MPS and environment update;
* ``expand``         <- ``TwoSiteFiniteVMPSExpand`` (:406-556): the term
  noise * (L psi W1 W2) with the right MPO bond left open and fused with the
  right bond (moving right), or noise * (psi R W2 W1) with the left MPO bond
  fused with the left bond (moving left), appended to psi's bond sectors; the
  next-next MPS tensor grows by zeros along that bond.

Conventions of the absent tensor library that this restatement fixes itself
(the device form follows the same ones): a fused index has one sector per
quantum number, in order of first appearance while the first index's
sectors run slowest; inside a sector the (first, second) sector pairs come in
that order, each pair's elements row-major (first index slowest).  An
expanded index keeps the original sectors in order, each followed by the
added part of the same quantum number; added quantum numbers come after, in
the added index's order.  Index combiners are built from the same fused
index.  Left / right canonicalisation uses the SVD keeping every singular
value, so a bond keeps min(rows, cols) states per sector, as a QR would.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from ultradmrg_gb300.tensor_data import IN, OUT, BlockTensorData, Index

from . import blocksparse as bs
from .krylov import LanczosParams, eff_ham_mul_two_site_state, lanczos_solver
from .vmps import SiteLog, measure_ee, trivial_lenv, trivial_renv, update_site_lenvs, \
    update_site_renvs


@dataclass
class NoiseSweepParams:
    """``FiniteVMPSSweepParams`` with its noise fields
    (``algorithm/finite_vmps_sweep_params.h:31-107``)."""

    sweeps: int
    Dmin: int
    Dmax: int
    trunc_err: float
    lancz_params: LanczosParams = field(default_factory=LanczosParams)
    noises: List[float] = field(default_factory=list)
    # defaults: kVMPSMaxNoise, kVMPSNoiseIncreaseRate, kVMPSNoiseDecreaseRate,
    # kVMPSNoiseAlpha (finite_vmps_sweep_params.h:25-28)
    noise_decrease: float = 0.95
    noise_increase: float = 1.02
    max_noise: float = 1.0
    alpha: float = 0.3


# ---------------------------------------------------------------------------
# fused and expanded indexes
# ---------------------------------------------------------------------------

def fuse_index(i1: Index, i2: Index, out_dir: int):
    """The fused index of (i1, i2) with direction out_dir and, for every sector
    pair (s1, s2), its (fused sector, offset inside it).  dir_f q_f =
    dir_1 q_1 + dir_2 q_2, so replacing the two indexes by it keeps a block's
    divergence."""
    qns, dims, where = [], [], {}
    for s1, (q1, d1) in enumerate(zip(i1.qns, i1.dims)):
        for s2, (q2, d2) in enumerate(zip(i2.qns, i2.dims)):
            q = tuple(out_dir * (i1.dir * a + i2.dir * b) for a, b in zip(q1, q2))
            if q in qns:
                f = qns.index(q)
            else:
                f = len(qns)
                qns.append(q)
                dims.append(0)
            where[(s1, s2)] = (f, dims[f])
            dims[f] += d1 * d2
    return Index(tuple(qns), tuple(dims), out_dir), where


def fuse_axes(t: BlockTensorData, ax1: int, ax2: int, out_dir: int) -> BlockTensorData:
    """Fuse axes ax1, ax2 of t into one index at position 0 (``FuseIndex``);
    the other axes follow in their order."""
    f, where = fuse_index(t.indexes[ax1], t.indexes[ax2], out_dir)
    rest = [k for k in range(t.rank) if k not in (ax1, ax2)]
    idx = [f] + [t.indexes[k] for k in rest]
    out = BlockTensorData(idx, {}, t.dtype)
    for key, blk in sorted(t.blocks.items()):
        fs, off = where[(key[ax1], key[ax2])]
        d1, d2 = blk.shape[ax1], blk.shape[ax2]
        moved = np.transpose(blk, [ax1, ax2] + rest).reshape((d1 * d2,) + tuple(
            blk.shape[k] for k in rest))
        nk = (fs,) + tuple(key[k] for k in rest)
        if nk not in out.blocks:
            out.blocks[nk] = np.zeros(out.block_shape(nk), dtype=t.dtype)
        out.blocks[nk][off:off + d1 * d2] += moved
    return out


def expanded_index(a: Index, b: Index) -> Tuple[Index, List[int], List[Tuple[int, int]]]:
    """a's sectors each followed by b's part of the same quantum number, then
    b's other quantum numbers.  Returns the index, the sector of every a sector
    and the (sector, offset) of every b sector."""
    assert a.dir == b.dir
    qns, dims = list(a.qns), list(a.dims)
    amap = list(range(a.nsec))
    bmap = []
    for q, d in zip(b.qns, b.dims):
        if q in qns:
            s = qns.index(q)
            bmap.append((s, dims[s]))
            dims[s] += d
        else:
            bmap.append((len(qns), 0))
            qns.append(q)
            dims.append(d)
    return Index(tuple(qns), tuple(dims), a.dir), amap, bmap


def expand(t: BlockTensorData, p: Optional[BlockTensorData], axis: int,
           extra: Optional[Index] = None) -> BlockTensorData:
    """``ExpandQNBlocks``: t with p appended along axis (p = None: zeros whose
    index along axis is ``extra``; the other indexes equal t's)."""
    if p is not None:
        assert all(p.indexes[k] == t.indexes[k] for k in range(t.rank) if k != axis)
    add = extra if p is None else p.indexes[axis]
    e, amap, bmap = expanded_index(t.indexes[axis], add)
    idx = list(t.indexes)
    idx[axis] = e
    dt = t.dtype if p is None else np.result_type(t.dtype, p.dtype)
    out = BlockTensorData(idx, {}, dt)

    def put(key, blk, s, off):
        nk = key[:axis] + (s,) + key[axis + 1:]
        if nk not in out.blocks:
            out.blocks[nk] = np.zeros(out.block_shape(nk), dtype=dt)
        sl = [slice(None)] * blk.ndim
        sl[axis] = slice(off, off + blk.shape[axis])
        out.blocks[nk][tuple(sl)] = blk

    for key, blk in sorted(t.blocks.items()):
        put(key, blk, amap[key[axis]], 0)
    if p is not None:
        for key, blk in sorted(p.blocks.items()):
            put(key, blk, *bmap[key[axis]])
    return out


def combiner(i1: Index, i2: Index, out_dir: int) -> BlockTensorData:
    """``IndexCombine``: (i1, i2, f), the isometry taking (x1, x2) to its place
    in the fused index, ones on those entries.  f has direction out_dir and
    the tensor divergence zero: dir_f q_f = -(dir_1 q_1 + dir_2 q_2)."""
    F, where = fuse_index(i1, i2, -out_dir)
    f = F.inverse()
    t = BlockTensorData([i1, i2, f], {}, np.float64)
    for (s1, s2), (fs, off) in where.items():
        d1, d2 = i1.dims[s1], i2.dims[s2]
        blk = np.zeros((d1, d2, f.dims[fs]))
        for x in range(d1):
            for y in range(d2):
                blk[x, y, off + x * d2 + y] = 1.0
        t.blocks[(s1, s2, fs)] = blk
    return t


# ---------------------------------------------------------------------------
# boundaries (CheckAndUpdateBoundaryMPSTensors)
# ---------------------------------------------------------------------------

KEEP_ALL = 1 << 40  # Dmin = Dmax: every singular value kept (min(rows, cols) per sector)


def _left_canonicalize(mps, i):
    u, s, vt, _, _ = bs.svd(mps[i], 2, mps[i].div(), 0.0, KEEP_ALL, KEEP_ALL)
    mps[i] = u
    mps[i + 1] = bs.contract(bs.contract(s, vt, [1], [0]), mps[i + 1], [1], [0])


def _right_canonicalize(mps, i):
    u, s, vt, _, _ = bs.svd(mps[i], 1, mps[i].div(), 0.0, KEEP_ALL, KEEP_ALL)
    mps[i] = vt
    mps[i - 1] = bs.contract(mps[i - 1], bs.contract(u, s, [1], [0]), [2], [0])


def boundaries(mps, Dmax):
    """Edge tensors whose bond can hold the whole block space become index
    combiners (the state is unchanged); returns (left_boundary,
    right_boundary), the outermost sites the sweeps update.  The centre must
    be at site 0 on entry and is at left_boundary + 1 on return."""
    N = len(mps)
    lmid, rmid = (N // 2 - 1, N // 2) if N % 2 == 0 else (N // 2, N // 2)
    left = right = 0
    for i in range(lmid):
        _left_canonicalize(mps, i)
        a, s, b = (ind.dim for ind in mps[i].indexes)
        if a * s > Dmax:
            left = i
            break
        if a * s > b:
            c = combiner(mps[i].indexes[0], mps[i].indexes[1], mps[i].indexes[2].dir)
            r = bs.contract(bs.dag(c), mps[i], [0, 1], [0, 1])
            mps[i + 1] = bs.contract(r, mps[i + 1], [1], [0])
            mps[i] = c
        if i == lmid - 1:
            left = i
    for i in range(N - 1, rmid, -1):
        _right_canonicalize(mps, i)
        b, s, c = (ind.dim for ind in mps[i].indexes)
        if s * c > Dmax:
            right = i
            break
        if s * c > b:
            cb = combiner(mps[i].indexes[1], mps[i].indexes[2], IN)
            cb = bs.transpose(cb, [2, 0, 1])  # (f, s, c)
            r = bs.contract(mps[i], bs.dag(cb), [1, 2], [1, 2])
            mps[i - 1] = bs.contract(mps[i - 1], r, [2], [0])
            mps[i] = cb
        if i == rmid + 1:
            right = i
    return left, right


# ---------------------------------------------------------------------------
# the noised update and sweep
# ---------------------------------------------------------------------------

def qn_covered(cover, sub) -> bool:
    """``IsQNCovered``: every quantum number of sub is one of cover's."""
    return set(sub) <= set(cover)


def _side_qns(t: BlockTensorData, left: bool):
    """The quantum numbers the coverage test reads
    (two_site_update_noise_finite_vmps_impl.h:286-312): for a two-state site
    the outer bond's sectors; otherwise the outer bond fused with the physical
    index, both taken with the same direction (the left tensor's physical
    index inverted), whose fused sectors carry the sums q_bond + q_phys."""
    if left:
        if t.indexes[1].dim == 2:
            return set(t.indexes[0].qns)
        return {tuple(x + y for x, y in zip(qa, qs))
                for qa in t.indexes[0].qns for qs in t.indexes[1].qns}
    if t.indexes[1].dim == 2:
        return set(t.indexes[2].qns)
    return {tuple(x + y for x, y in zip(qs, qc))
            for qs in t.indexes[1].qns for qc in t.indexes[2].qns}


def expansion_term(gs, eff_ham, dir):
    L, W1, W2, R = eff_ham
    if dir == 'r':
        t1 = bs.contract(L, gs, [2], [0])                  # (a', w, s1, s2, b)
        t2 = bs.contract_cyclic(t1, W1, 1, 0, 2)           # (s2, b, a', s1', wr)
        t3 = bs.contract_cyclic(t2, W2, 4, 0, 2)           # (b, a', s1', s2', w2)
        return fuse_axes(t3, 0, 4, gs.indexes[3].dir)      # (f, a', s1', s2')
    t1 = bs.contract(gs, R, [3], [2])                      # (a, s1, s2, b', w2)
    t2 = bs.contract(t1, W2, [2, 4], [1, 3])               # (a, s1, b', wl2, s2')
    t3 = bs.contract(t2, W1, [1, 3], [1, 3])               # (a, b', s2', wl1, s1')
    t3 = bs.transpose(t3, [0, 3, 4, 2, 1])                 # (a, wl1, s1', s2', b')
    return fuse_axes(t3, 0, 1, gs.indexes[0].dir)          # (f, s1', s2', b')


def noise_update(mps, lenvs, renvs, mpo, p: NoiseSweepParams, dir, target, noise, log=None):
    N = len(mps)
    if dir == 'r':
        l, r = target, target + 1
        lenv_len, renv_len = target, N - (target + 2)
    else:
        l, r = target - 1, target
        lenv_len, renv_len = target - 1, N - target - 1
    eff_ham = [lenvs[lenv_len], mpo[l], mpo[r], renvs[renv_len]]
    init = bs.contract(mps[l], mps[r], [2], [0])
    res = lanczos_solver(eff_ham, init, eff_ham_mul_two_site_state, p.lancz_params)
    gs = res.gs_vec
    expand_now = abs(noise) >= 1e-10
    if expand_now:
        ql, qr = _side_qns(mps[l], True), _side_qns(mps[r], False)
        if (dir == 'r' and qn_covered(qr, ql)) or (dir == 'l' and qn_covered(ql, qr)):
            expand_now = False
    if expand_now:
        term = bs.scale(expansion_term(gs, eff_ham, dir), noise)
        if dir == 'r':
            g = bs.transpose(gs, [3, 0, 1, 2])
            gs = bs.transpose(expand(g, term, 0), [1, 2, 3, 0])
            nn = target + 2
            mps[nn] = expand(mps[nn], None, 0, term.indexes[0].inverse())
        else:
            gs = expand(gs, term, 0)
            nn = target - 2
            mps[nn] = expand(mps[nn], None, 2, term.indexes[0].inverse())
    u, s, vt, err, D = bs.svd(gs, 2, mps[l].div(), p.trunc_err, p.Dmin, p.Dmax)
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
        log.append(SiteLog(target, res.gs_eng, err, D, res.iters, ee))
    return res.gs_eng, (noise if expand_now else 0.0)


def energy_expectation(mps, lenvs, renvs, mpo, l, r):
    """``CalEnergyEptTwoSite``: <psi|H|psi> of the current two-site tensor."""
    N = len(mps)
    eff = [lenvs[l], mpo[l], mpo[r], renvs[N - r - 1]]
    psi = bs.contract(mps[l], mps[r], [2], [0])
    return float(np.real(bs.inner(psi, eff_ham_mul_two_site_state(eff, psi))))


def noise_sweep(mps, mpo, p, lenvs, renvs, left, right, noise, log=None, noises_used=None,
                margins=None):
    """``margins`` (optional list) receives, per update, the energy expectation
    minus the previous update's energy, relative to the latter: the quantity
    whose sign and size decide the noise adaptation."""
    e0 = 0.0
    last = 0.0

    def adapt(actual, noise):
        if margins is not None:
            margins.append((actual - e0) / abs(e0) if e0 != 0.0 else np.inf)
        if actual - e0 <= 0.0:
            return noise
        if actual - e0 >= p.alpha * abs(last - e0):
            return noise * p.noise_decrease
        return min(noise * p.noise_increase, p.max_noise)

    for i in range(left, right - 1):
        actual = energy_expectation(mps, lenvs, renvs, mpo, i, i + 1)
        noise = adapt(actual, noise)
        e0, used = noise_update(mps, lenvs, renvs, mpo, p, 'r', i, noise, log)
        last = actual
        if noises_used is not None:
            noises_used.append(used)
    for i in range(right, left + 1, -1):
        actual = energy_expectation(mps, lenvs, renvs, mpo, i - 1, i)
        noise = adapt(actual, noise)
        e0, used = noise_update(mps, lenvs, renvs, mpo, p, 'l', i, noise, log)
        last = actual
        if noises_used is not None:
            noises_used.append(used)
    return e0, noise


def two_site_finite_vmps_with_noise(mps, mpo, p: NoiseSweepParams, log=None, noises_used=None,
                                    margins=None):
    """Returns the last update's energy; ``mps`` (centre at site 0 on entry) is
    updated in place."""
    from .vmps import FiniteVMPSSweepParams, two_site_finite_vmps
    if not p.noises:
        return two_site_finite_vmps(mps, mpo, FiniteVMPSSweepParams(
            p.sweeps, p.Dmin, p.Dmax, p.trunc_err, p.lancz_params), log)
    N = len(mps)
    left, right = boundaries(mps, p.Dmax)
    lenvs, renvs = [None] * N, [None] * N
    lenvs[0] = trivial_lenv(mps[0], mpo[0])
    for i in range(left):
        lenvs[i + 1] = update_site_lenvs(lenvs[i], mps[i], mpo[i])
    renvs[0] = trivial_renv(mps[N - 1], mpo[N - 1])
    for k in range(1, N - left - 1):
        renvs[k] = update_site_renvs(renvs[k - 1], mps[N - k], mpo[N - k])
    e0 = None
    noise = p.noises[0]
    for s in range(p.sweeps):
        if s < len(p.noises):
            noise = p.noises[s]
        e0, noise = noise_sweep(mps, mpo, p, lenvs, renvs, left, right, noise, log,
                                noises_used, margins)
    return e0
