"""Finite-MPS measurements on the device: ``MeasureOneSiteOp``,
``MeasureTwoSiteOp``, ``MeasureMultiSiteOp`` and ``MeasureTwoSiteOpGroup``
(``one_dim_tn/mps/finite_mps/finite_mps_measu_memory.h:141-478``,
``finite_mps_measu_disk.h``).

A measured value is a chain of environment updates: the same
``L' = A^dag (L A) W`` contraction the two-site sweep runs
(``update_site_lenvs``).  Here ``W`` is the measured operator written as an
MPO tensor with one-dimensional virtual bonds.  A charged operator
(c^dag, S+) moves that bond's quantum number, and the identity or string
operators after it carry the number on.  The measurer caches the identity
chains from the left (sites < i) and from the right (sites >= i).  An event
on sites h..t then costs t - h + 1 updates from the cached left chain at h,
and one contraction against the cached right chain at t + 1.  The result is
divided by <psi|psi>, so the MPS needs no particular canonical form.  The
reference centralises the MPS at the first operator's site instead, and gets
the same number for the normalised MPS it measures.

Everything runs through a ``Backend``: the environment updates, a
contraction, upload and download.  ``device_backend`` binds them to the C
ABI (``udmrg_update_site_lenvs`` / ``renvs``, ``udmrg_contract``).  The
tests bind them to the FP64 oracle, so the composition is checked on the
host and the primitives on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from .mpogen import op_div
from .tensor_data import IN, OUT, BlockTensorData, Index, qn_sub


@dataclass
class MeasuResElem:
    """``MeasuResElem`` (finite_mps_measu_memory.h:40-48)."""
    sites: List[int]
    avg: complex


@dataclass
class Backend:
    """update_left(L, A, W) / update_right(R, A, W): the sweep's environment
    updates; contract(a, b, axes_a, axes_b); upload(BlockTensorData) and
    download(t) -> BlockTensorData; info(t) -> (indexes, dtype);
    release(t) frees a backend tensor; dag(t) flips the index directions and
    conjugates."""
    update_left: Callable
    update_right: Callable
    contract: Callable
    upload: Callable
    download: Callable
    info: Callable
    release: Callable
    dag: Optional[Callable] = None


def device_backend(ctx) -> Backend:
    from . import api

    def info(t):
        return t.indexes(), (np.complex128 if t.is_complex else np.float64)

    return Backend(
        update_left=lambda L, A, W: api.update_site_lenvs(ctx, L, A, W),
        update_right=lambda R, A, W: api.update_site_renvs(ctx, R, A, W),
        contract=lambda a, b, xa, xb: api.contract(ctx, a, b, xa, xb),
        upload=lambda t: api.DeviceTensor.from_data(ctx, t),
        download=lambda t: t.to_data(),
        info=info,
        release=lambda t: t.close(),
        dag=lambda t: api.dag(ctx, t),
    )


def op_tensor(mat: np.ndarray, pb_out: Index, q_left, dtype):
    """The operator O[in, out] as W(lvb IN, pb_in IN, pb_out OUT, rvb OUT) with
    one-dimensional bonds: lvb carries q_left, rvb q_left - Div(O).  Returns
    (W, the right bond's quantum number)."""
    m = np.asarray(mat.mat if hasattr(mat, "mat") else mat)
    q_right = qn_sub(q_left, op_div(m, pb_out))
    W = BlockTensorData([Index.make([(q_left, 1)], IN), pb_out.inverse(), pb_out,
                         Index.make([(q_right, 1)], OUT)], {}, dtype)
    for a, o in np.argwhere(m != 0):
        W.set_elem((0, int(a), int(o), 0), m[a, o])
    return W, q_right


class MPSMeasurer:
    """Expectation values <psi| prod O |psi> / <psi|psi> of one MPS."""

    def __init__(self, backend: Backend, mps: Sequence):
        self.b = backend
        self.mps = list(mps)
        self.N = len(self.mps)
        if self.N < 2:
            raise ValueError("measurements need at least two sites")
        infos = [backend.info(t) for t in self.mps]
        self.idx = [i for i, _ in infos]
        self.pb = [ix[1] for ix in self.idx]
        self.dtype = np.result_type(*[d for _, d in infos])
        self.zero = tuple(0 for _ in range(self.pb[0].nq))
        self._id: Dict[int, object] = {}
        self._left: List[Optional[object]] = [None] * (self.N + 1)
        self._right: List[Optional[object]] = [None] * (self.N + 1)
        self._norm = None

    # ---- cached pieces ----

    def _identity(self, site):
        if site not in self._id:
            eye = np.eye(self.pb[site].dim, dtype=self.dtype)
            self._id[site] = self.b.upload(op_tensor(eye, self.pb[site], self.zero, self.dtype)[0])
        return self._id[site]

    def _trivial(self, side):
        z = Index.make([(self.zero, 1)], OUT)
        i0 = self.idx[0][0] if side == "l" else self.idx[-1][2]
        iw = z if side == "l" else z.inverse()  # inverse of W's lvb (IN) / rvb (OUT)
        t = BlockTensorData([i0, iw, i0.inverse()], {}, self.dtype)
        t.set_elem((0, 0, 0), 1.0)
        return self.b.upload(t)

    def left(self, i):
        """Identity chain over the sites < i."""
        if self._left[i] is None:
            self._left[i] = self._trivial("l") if i == 0 else \
                self.b.update_left(self.left(i - 1), self.mps[i - 1], self._identity(i - 1))
        return self._left[i]

    def right(self, i):
        """Identity chain over the sites >= i."""
        if self._right[i] is None:
            self._right[i] = self._trivial("r") if i == self.N else \
                self.b.update_right(self.right(i + 1), self.mps[i], self._identity(i))
        return self._right[i]

    def _close(self, L, R):
        """<L|R> over the bra and ket bonds; the one-dimensional operator bonds
        stay (a 1 x 1 result, or no block when the quantum numbers differ)."""
        t = self.b.download(self.b.contract(L, R, [0, 2], [0, 2]))
        return sum((blk.sum() for blk in t.blocks.values()), 0.0)

    def norm2(self):
        if self._norm is None:
            self._norm = self._close(self.left(self.N // 2), self.right(self.N // 2))
        return self._norm

    # ---- events ----

    def expectation(self, head: int, ops: Sequence) -> complex:
        """<psi| O_head O_head+1 ... |psi> / <psi|psi> for the operators ops
        on consecutive sites from head."""
        if head < 0 or head + len(ops) > self.N or not ops:
            raise ValueError("operators must lie on the chain")
        L, q, owned = self.left(head), self.zero, []
        for k, op in enumerate(ops):
            s = head + k
            W, q = op_tensor(op, self.pb[s], q, self.dtype)
            w = self.b.upload(W)
            L = self.b.update_left(L, self.mps[s], w)
            owned += [w, L]
        val = self._close(L, self.right(head + len(ops))) if q == self.zero else 0.0
        for t in owned:
            self.b.release(t)
        val = val / self.norm2()
        return val.real if np.isrealobj(val) or self.dtype == np.float64 else val

    def close(self):
        for t in list(self._id.values()) + self._left + self._right:
            if t is not None:
                self.b.release(t)
        self._id, self._left, self._right = {}, [None] * (self.N + 1), [None] * (self.N + 1)


def _ops_sequence(phys, insts, sites):
    if len(sites) < 2 or list(sites) != sorted(sites):
        raise ValueError("two or more sites in ascending order")
    if len(insts) not in (len(phys) - 1, len(phys)):
        raise ValueError("insertion lists: one per gap, optionally a tail")
    seq = []
    for j in range(len(phys) - 1):
        seq.append(phys[j])
        if len(insts[j]) != sites[j + 1] - sites[j] - 1:
            raise ValueError("one insertion operator per site in between")
        seq.extend(insts[j])
    seq.append(phys[-1])
    if len(insts) == len(phys):
        seq.extend(insts[-1])
    return seq


def measure_one_site_op(m: MPSMeasurer, op) -> List[MeasuResElem]:
    return [MeasuResElem([i], m.expectation(i, [op])) for i in range(m.N)]


def measure_multi_site_op(m: MPSMeasurer, phys_ops_set, inst_ops_set_set,
                          sites_set) -> List[MeasuResElem]:
    """``MeasureMultiSiteOp`` (finite_mps_measu_memory.h:285-311): per event,
    physical operators at sites (ascending) with explicit insertion lists
    between them and optionally a tail string after the last."""
    return [MeasuResElem(list(sites), m.expectation(sites[0], _ops_sequence(phys, insts, sites)))
            for phys, insts, sites in zip(phys_ops_set, inst_ops_set_set, sites_set)]


def measure_two_site_op(m: MPSMeasurer, phys_ops, inst_op, sites_set) -> List[MeasuResElem]:
    """``MeasureTwoSiteOp`` (finite_mps_measu_memory.h:200-265): one insertion
    operator on every site in between, or explicit per-event lists."""
    if len(phys_ops) != 2:
        raise ValueError("two physical operators")
    if isinstance(inst_op, (list, tuple)):
        insts = [[list(x)] for x in inst_op]
    else:
        insts = [[[inst_op] * (s[1] - s[0] - 1)] for s in sites_set]
    return measure_multi_site_op(m, [phys_ops] * len(sites_set), insts, sites_set)


def measure_two_site_op_group(m: MPSMeasurer, op1, op2, site1, site2_set,
                              inst_op) -> List[MeasuResElem]:
    """``MeasureTwoSiteOpGroup``: one first site against a list of second sites."""
    return measure_two_site_op(m, [op1, op2], inst_op, [[site1, s2] for s2 in site2_set])


def _op_data(mat, pb_out: Index, dtype) -> BlockTensorData:
    """O[in, out] as the rank-2 tensor {pb_in, pb_out}."""
    m = np.asarray(mat.mat if hasattr(mat, "mat") else mat)
    t = BlockTensorData([pb_out.inverse(), pb_out], {}, dtype)
    for a, o in np.argwhere(m != 0):
        t.set_elem((int(a), int(o)), m[a, o])
    return t


def _trace(t: BlockTensorData):
    """Trace of a matrix whose two indexes are one bond and its inverse."""
    return np.trace(t.to_dense()) if t.blocks else 0.0


def cal_psi1_op_psi2(b: Backend, mps1: Sequence, mps2: Sequence, op, inst=None) -> list:
    """``CalPsi1OpPsi2`` (algorithm/tdvp/two_site_update_finite_tdvp_impl.h:540-614):
    res[i] = <psi2| inst_0 ... inst_{i-1} op_i |psi1> for every site i (the
    string only when inst is given), not normalised.  Right boundaries are
    built from the right end, the left one is carried site by site; each
    value closes the left boundary, the operator and the right boundary.
    The final contraction keeps the ket bond open and the trace is taken on
    the host (device tensors have rank >= 1)."""
    N = len(mps1)
    if len(mps2) != N or N < 1:
        raise ValueError("two MPS of the same length")
    i1 = [b.info(t)[0] for t in mps1]
    i2 = [b.info(t)[0] for t in mps2]
    dtype = np.result_type(*[b.info(t)[1] for t in list(mps1) + list(mps2)])
    owned = []

    def keep(t):
        owned.append(t)
        return t

    def boundary(a: Index, c: Index):
        t = BlockTensorData([a, c.inverse()], {}, dtype)
        t.set_elem((0, 0), 1.0)
        return keep(b.upload(t))

    # right boundaries: rb[k] covers the sites >= k
    rb = [None] * (N + 1)
    rb[N] = boundary(i2[N - 1][2], i1[N - 1][2])
    for k in range(N - 1, 0, -1):
        t = keep(b.contract(keep(b.dag(mps2[k])), rb[k + 1], [2], [0]))
        rb[k] = keep(b.contract(t, mps1[k], [1, 2], [1, 2]))
    opt = keep(b.upload(_op_data(op, i1[0][1], dtype)))
    instt = None if inst is None else keep(b.upload(_op_data(inst, i1[0][1], dtype)))
    L = boundary(i2[0][0], i1[0][0])
    res = []
    for i in range(N):
        t1 = keep(b.contract(keep(b.dag(mps2[i])), L, [0], [0]))
        t2 = keep(b.contract(opt, t1, [1], [0]))
        t3 = keep(b.contract(t2, mps1[i], [2, 0], [0, 1]))
        t4 = b.contract(t3, rb[i + 1], [0], [0])
        res.append(_trace(b.download(t4)))
        b.release(t4)
        if i < N - 1:
            src = t1 if instt is None else keep(b.contract(instt, t1, [1], [0]))
            L = keep(b.contract(src, mps1[i], [2, 0], [0, 1]))
    for t in owned:
        b.release(t)
    return res
