"""Finite-MPS measurements, restated in numpy.

Test infrastructure: this is the checker for measurements of MPS produced by
the device sweeps, never a product code path.

* ``measure_one_site_op`` follows ``MeasureOneSiteOp`` / ``OneSiteOpAvg``
  (``one_dim_tn/mps/finite_mps/finite_mps_measu_memory.h:141-157, 343-364``).
  The result is <psi| O_i |psi> for every site i.
* ``measure_two_site_op`` follows ``MeasureTwoSiteOp`` (``:200-265``), and
  ``measure_multi_site_op`` follows ``MeasureMultiSiteOp`` / ``MultiSiteOpAvg``
  / ``OpsVecAvg`` (``:285-478``).  The physical operators sit at the given
  sites, with insertion operators (Jordan-Wigner strings) on the sites
  between them and optionally a tail string after the last.  Sites without
  an operator carry the identity.
* ``measure_two_site_op_group`` follows ``MeasureTwoSiteOpGroup``
  (``finite_mps_measu_disk.h``).  One first site is paired with a list of
  second sites, with a uniform insertion operator in between.
* ``cal_psi1_op_psi2`` follows ``CalPsi1OpPsi2``
  (``algorithm/tdvp/two_site_update_finite_tdvp_impl.h:540-614``): for every
  site i, <psi2| inst_0 ... inst_{i-1} O_i |psi1> between two MPS, not
  normalised.
* ``entanglement_entropy`` follows ``FiniteMPS::GetEntanglementEntropy``
  (``one_dim_tn/mps/finite_mps/finite_mps.h:277-310``).  It returns the von
  Neumann entropy -sum p ln p (n = 1) or the Renyi entropy
  -ln(sum p^n) / (n - 1) of the Schmidt weights at every bond.

The reference centralises the MPS at the first operator's site and contracts
locally.  Here the whole network is contracted from the left, one transfer
matrix per site, and the result is divided by <psi|psi>.  For the
normalised MPS the reference measures, the two are the same number.
Operators are dense matrices ``O[in, out]`` (``models.Operator`` or arrays),
in the element layout of ``QLTensor({pb_in, pb_out})``.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np


@dataclass
class MeasuResElem:
    """``MeasuResElem`` (finite_mps_measu_memory.h:40-48)."""
    sites: List[int]
    avg: complex


def _mat(op):
    return np.asarray(op.mat if hasattr(op, "mat") else op)


def _dense(mps):
    return [t.to_dense() for t in mps]  # (l, s, r), sector-ordered coordinates


def _transfer(E, A, O):
    """E'[r', r] = sum conj(A[a', s', r']) E[a', a] O[s, s'] A[a, s, r]."""
    T = np.tensordot(E, A, axes=([1], [0]))          # (a', s, r)
    if O is not None:
        T = np.tensordot(T, O, axes=([1], [0]))      # (a', r, s')
        T = np.transpose(T, (0, 2, 1))               # (a', s', r)
    return np.tensordot(np.conj(A), T, axes=([0, 1], [0, 1]))  # (r', r)


def _expectation(dense, ops_at):
    """<psi| prod_i ops_at[i] |psi> / <psi|psi>; ops_at[i] None = identity."""
    E = np.ones((1, 1), dtype=np.result_type(dense[0], np.float64))
    N0 = E.copy()
    for i, A in enumerate(dense):
        E = _transfer(E, A, ops_at.get(i))
        N0 = _transfer(N0, A, None)
    val = E[0, 0] / N0[0, 0]
    return val.real if np.isrealobj(dense[0]) and all(
        np.isrealobj(o) for o in ops_at.values()) else val


def measure_one_site_op(mps, op) -> List[MeasuResElem]:
    dense = _dense(mps)
    O = _mat(op)
    return [MeasuResElem([i], _expectation(dense, {i: O})) for i in range(len(mps))]


def measure_multi_site_op(mps, phys_ops_set, inst_ops_set_set, sites_set) -> List[MeasuResElem]:
    """Per event k: physical operators phys_ops_set[k] at sites_set[k]
    (ascending) with inst_ops_set_set[k][j] a list of insertion operators
    placed one per site from sites[j] + 1 on (j < len(phys) - 1 in between,
    j = len(phys) - 1 a tail string after the last physical operator)."""
    dense = _dense(mps)
    out = []
    for phys, insts, sites in zip(phys_ops_set, inst_ops_set_set, sites_set):
        if len(sites) < 2 or list(sites) != sorted(sites):
            raise ValueError("two or more sites in ascending order")
        if len(insts) not in (len(phys) - 1, len(phys)):
            raise ValueError("insertion lists: one per gap, optionally a tail")
        seq = []
        for j in range(len(phys) - 1):
            seq.append(_mat(phys[j]))
            seq.extend(_mat(o) for o in insts[j])
        seq.append(_mat(phys[-1]))
        if len(insts) == len(phys):
            seq.extend(_mat(o) for o in insts[-1])
        head = sites[0]
        ops_at = {head + k: o for k, o in enumerate(seq)}
        if head + len(seq) > len(mps):
            raise ValueError("operator string runs past the last site")
        out.append(MeasuResElem(list(sites), _expectation(dense, ops_at)))
    return out


def measure_two_site_op(mps, phys_ops, inst_op, sites_set) -> List[MeasuResElem]:
    """<A_i O_{i+1} ... O_{j-1} B_j> for every (i, j); inst_op is one operator
    used on every site in between, or a list of per-event lists."""
    if len(phys_ops) != 2:
        raise ValueError("two physical operators")
    if isinstance(inst_op, (list, tuple)):
        insts = [[list(x)] for x in inst_op]
        for x, s in zip(inst_op, sites_set):
            if len(x) != s[1] - s[0] - 1:
                raise ValueError("one insertion operator per site in between")
    else:
        insts = [[[inst_op] * (s[1] - s[0] - 1)] for s in sites_set]
    return measure_multi_site_op(mps, [phys_ops] * len(sites_set), insts, sites_set)


def measure_two_site_op_group(mps, op1, op2, site1, site2_set, inst_op) -> List[MeasuResElem]:
    return measure_two_site_op(mps, [op1, op2], inst_op, [[site1, s2] for s2 in site2_set])


def entanglement_entropy(mps, n: int = 1) -> List[float]:
    """Entropy of the Schmidt weights at each of the N - 1 bonds.  At bond i
    the state is Q R X with Q orthonormal (QR of the sites <= i, carried from
    the left) and X the sites > i; the weights are the eigenvalues of
    R (X X^dag) R^dag, normalised to sum 1."""
    dense = _dense(mps)
    out = []
    R = np.ones((1, 1), dtype=np.result_type(dense[0], np.float64))
    for i in range(len(dense) - 1):
        A = np.tensordot(R, dense[i], axes=([1], [0]))
        l, d, r = A.shape
        _, R = np.linalg.qr(A.reshape(l * d, r))
        M = R @ _right_gram(dense, i + 1) @ np.conj(R.T)
        w = np.clip(np.linalg.eigvalsh((M + np.conj(M.T)) / 2).real, 0.0, None)
        p = w[w > 0] / w.sum()
        if n == 1:
            out.append(float(-(p * np.log(p)).sum()))
        else:
            out.append(float(-np.log((p ** n).sum()) / (n - 1)))
    return out


def _right_gram(dense, start):
    """G[b, b'] = sum_y X[b, y] conj(X[b', y]) for X = the sites >= start."""
    G = np.ones((1, 1), dtype=np.result_type(dense[0], np.float64))
    for A in reversed(dense[start:]):
        T = np.tensordot(A, G, axes=([2], [0]))                  # (b, s, r')
        G = np.tensordot(T, np.conj(A), axes=([1, 2], [1, 2]))  # (b, b')
    return G


def cal_psi1_op_psi2(mps1, mps2, op, inst=None) -> list:
    """res[i] = <psi2| inst_0 ... inst_{i-1} op_i |psi1> (the string only when
    inst is given), unnormalised."""
    d1, d2 = _dense(mps1), _dense(mps2)
    O = _mat(op)
    I = None if inst is None else _mat(inst)
    out = []
    for i in range(len(d1)):
        E = np.ones((1, 1), dtype=np.result_type(d1[0], d2[0], O, np.float64))
        for k, (A, B) in enumerate(zip(d1, d2)):
            X = O if k == i else (I if (I is not None and k < i) else None)
            T = np.tensordot(E, A, axes=([1], [0]))              # (a2, s, r1)
            if X is not None:
                T = np.transpose(np.tensordot(T, X, axes=([1], [0])), (0, 2, 1))
            E = np.tensordot(np.conj(B), T, axes=([0, 1], [0, 1]))  # (r2, r1)
        out.append(E[0, 0])
    return out
