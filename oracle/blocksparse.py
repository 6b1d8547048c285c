"""Block-sparse tensor arithmetic (FP64 / complex128), numpy restatement.

Semantics restated from how qlmps calls TensorToolkit:

* ``Contract(A, B, {axes_a, axes_b}, C)``: ordinary tensordot; output axes are
  A's free axes in order, then B's free axes in order
  (``algorithm/vmps/lanczos_vmps_solver_impl.h:268``,
  ``algorithm/vmps/two_site_update_finite_vmps_impl.h:279``).
* ``Contract<T, Q, a_tail, b_head>(A, B, a_start, b_start, n, C)``: contracts
  the ``n`` cyclically consecutive axes of A starting at ``a_start`` with those
  of B starting at ``b_start``; the output is A's remaining axes in cyclic order
  from ``a_start + n`` followed by B's remaining axes in cyclic order from
  ``b_start + n``.  Only this reading makes the four-step matvec of
  ``lanczos_vmps_solver_impl.h:268-272`` and the environment updates of
  ``algorithm/vmps/vmps_init.h:343-373`` land on the layouts the callers use.
* An output block exists iff at least one pair of input blocks contributes to
  it (blocks are created lazily).
* ``Dag``: flip every index direction, complex-conjugate the data.
* ``LinearCombine``: output holds the union of the input block sets.
* ``Normalize`` / ``QuasiNormalize``: divide by the 2-norm and return it (the
  two coincide for bosonic tensors, which are the only ones used here).
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

from ultradmrg_gb300.tensor_data import BlockTensorData, Index

T = BlockTensorData

# algorithmic flop counter of block contractions: 2*M*N*K per block pair
# (x4 for complex data), the same count the device schedule reports
FLOPS = [0.0]


def zeros_like_struct(t: T) -> T:
    return T(list(t.indexes), {k: np.zeros_like(v) for k, v in t.blocks.items()}, t.dtype)


def _result_dtype(a: T, b: T):
    return np.result_type(a.dtype, b.dtype)


def contract(a: T, b: T, axes_a: Sequence[int], axes_b: Sequence[int],
             out_perm: Sequence[int] = None) -> T:
    """Block-sparse tensordot; ``out_perm`` optionally permutes the output axes."""
    axes_a, axes_b = list(axes_a), list(axes_b)
    for x, y in zip(axes_a, axes_b):
        ia, ib = a.indexes[x], b.indexes[y]
        if ia.qns != ib.qns or ia.dims != ib.dims or ia.dir != -ib.dir:
            raise ValueError(f"contracted indexes do not match (axes {x},{y})")
    free_a = [i for i in range(a.rank) if i not in axes_a]
    free_b = [i for i in range(b.rank) if i not in axes_b]
    out_idx = [a.indexes[i] for i in free_a] + [b.indexes[i] for i in free_b]
    dtype = _result_dtype(a, b)
    # group B blocks by their contracted sector ids
    bgroups: Dict[Tuple[int, ...], List[Tuple[int, ...]]] = {}
    for kb in b.sorted_keys():
        bgroups.setdefault(tuple(kb[i] for i in axes_b), []).append(kb)
    out: Dict[Tuple[int, ...], np.ndarray] = {}
    cplx = 4.0 if np.dtype(dtype).kind == 'c' else 1.0
    for ka in a.sorted_keys():
        ck = tuple(ka[i] for i in axes_a)
        for kb in bgroups.get(ck, []):
            key = tuple(ka[i] for i in free_a) + tuple(kb[i] for i in free_b)
            blk_a, blk_b = a.blocks[ka], b.blocks[kb]
            kdim = int(np.prod([blk_a.shape[i] for i in axes_a])) if axes_a else 1
            FLOPS[0] += 2.0 * cplx * (blk_a.size // max(kdim, 1)) * (blk_b.size // max(kdim, 1)) * kdim
            prod = np.tensordot(blk_a, blk_b, axes=(axes_a, axes_b))
            if key in out:
                out[key] += prod
            else:
                out[key] = prod.astype(dtype, copy=True)
    res = T(out_idx, out, dtype)
    if out_perm is not None:
        res = transpose(res, out_perm)
    return res


def contract_cyclic(a: T, b: T, a_start: int, b_start: int, n: int) -> T:
    """``Contract<…, a_tail, b_head>(A, B, a_start, b_start, n)`` (cyclic axes)."""
    ra, rb = a.rank, b.rank
    axes_a = [(a_start + i) % ra for i in range(n)]
    axes_b = [(b_start + i) % rb for i in range(n)]
    rem_a = [(a_start + n + i) % ra for i in range(ra - n)]
    rem_b = [(b_start + n + i) % rb for i in range(rb - n)]
    free_a = [i for i in range(ra) if i not in axes_a]
    free_b = [i for i in range(rb) if i not in axes_b]
    # tensordot output order is free_a (ascending) then free_b (ascending)
    perm = [free_a.index(i) for i in rem_a] + [len(free_a) + free_b.index(i) for i in rem_b]
    return contract(a, b, axes_a, axes_b, out_perm=perm)


def transpose(t: T, perm: Sequence[int]) -> T:
    perm = list(perm)
    if perm == list(range(t.rank)):
        return t
    blocks = {tuple(k[p] for p in perm): np.ascontiguousarray(v.transpose(perm))
              for k, v in t.blocks.items()}
    return T([t.indexes[p] for p in perm], blocks, t.dtype)


def dag(t: T) -> T:
    return T([i.inverse() for i in t.indexes],
             {k: np.conj(v) for k, v in t.blocks.items()}, t.dtype)


def inner(a: T, b: T) -> complex:
    """<a|b> = sum conj(a) * b over common blocks (the ``Dag`` + full contraction
    of ``lanczos_vmps_solver_impl.h:154-161``)."""
    s = 0.0
    for k, v in a.blocks.items():
        w = b.blocks.get(k)
        if w is not None:
            s += np.vdot(v, w)
    return s


def norm(t: T) -> float:
    return float(np.sqrt(sum(np.vdot(v, v).real for v in t.blocks.values())))


def normalize(t: T) -> float:
    """In-place ``Normalize()``; returns the norm before normalisation."""
    nrm = norm(t)
    if nrm != 0.0:
        for k in t.blocks:
            t.blocks[k] = t.blocks[k] / nrm
    return nrm


def linear_combine(coefs: Sequence, tens: Sequence[T], beta, res: T) -> T:
    """``LinearCombine(coefs, tens, beta, res)``: res = beta*res + sum c_i t_i."""
    dtype = np.result_type(res.dtype, *[t.dtype for t in tens], np.asarray(coefs).dtype)
    blocks = {}
    for k, v in res.blocks.items():
        blocks[k] = (beta * v).astype(dtype) if beta != 0 else np.zeros(v.shape, dtype)
    for c, t in zip(coefs, tens):
        for k, v in t.blocks.items():
            if k in blocks:
                blocks[k] = blocks[k] + c * v
            else:
                blocks[k] = (c * v).astype(dtype)
    idx = res.indexes if res.indexes else tens[0].indexes
    res.indexes = list(idx)
    res.blocks = blocks
    res.dtype = dtype
    return res


def scale(t: T, s) -> T:
    dtype = np.result_type(t.dtype, np.asarray(s).dtype)
    return T(list(t.indexes), {k: (s * v).astype(dtype) for k, v in t.blocks.items()}, dtype)


# ---------------------------------------------------------------------------
# Truncated block SVD
# ---------------------------------------------------------------------------

TIE_RTOL = 1e-12


def select_kept(svals: List[np.ndarray], trunc_err: float, Dmin: int, Dmax: int,
                rtol: float = TIE_RTOL):
    """Kept-state selection over all sectors.

    ``svals[q]`` are the singular values of bond sector ``q`` (descending inside
    the sector).  All values are ordered by descending size; values whose
    difference is below ``rtol * s_max`` count as ties and are ordered by
    (sector, position).  The kept count D is the smallest value in
    ``[min(Dmin, n), min(Dmax, n)]`` whose discarded weight
    ``sum_{discarded} s^2 / sum s^2`` is <= ``trunc_err`` (or the upper end).
    Returns (kept per sector, D, discarded weight).
    """
    flat = []
    for q, sv in enumerate(svals):
        for i, s in enumerate(sv):
            flat.append((float(s), q, i))
    n = len(flat)
    if n == 0:
        return [0] * len(svals), 0, 0.0
    smax = max(f[0] for f in flat)
    flat.sort(key=lambda x: (-x[0], x[1], x[2]))
    # tie-cluster reordering: consecutive values within rtol*smax are one cluster
    ordered, i = [], 0
    tol = rtol * smax
    while i < n:
        j = i + 1
        while j < n and flat[j - 1][0] - flat[j][0] <= tol:
            j += 1
        ordered.extend(sorted(flat[i:j], key=lambda x: (x[1], x[2])))
        i = j
    sq = np.array([f[0] ** 2 for f in ordered])
    total = sq.sum()
    # tail[k] = discarded weight when keeping the first k values
    tail = np.concatenate([np.cumsum(sq[::-1])[::-1], [0.0]])
    lo, hi = min(Dmin, n), min(Dmax, n)
    D = hi
    for k in range(lo, hi + 1):
        if total == 0 or tail[k] / total <= trunc_err:
            D = k
            break
    err = 0.0 if total == 0 else float(tail[D] / total)
    kept = [0] * len(svals)
    for f in ordered[:D]:
        kept[f[1]] += 1
    return kept, D, err


def svd_sector_matrices(t: T, ldims: int, ldiv):
    """Group the blocks of ``t`` by the QN of the new bond and assemble one dense
    matrix per bond sector.  Returns a list ordered by ascending bond QN of
    (bond_qn, rows, cols, matrix) where rows/cols are lists of
    (left key, row offset) / (right key, col offset)."""
    nq = t.nq
    sectors = {}
    for key in t.sorted_keys():
        lk, rk = key[:ldims], key[ldims:]
        qrow = tuple(0 for _ in range(nq))
        for ind, s in zip(t.indexes[:ldims], lk):
            qrow = tuple(x + ind.dir * y for x, y in zip(qrow, ind.qns[s]))
        qbond = tuple(x - y for x, y in zip(ldiv, qrow))
        sec = sectors.setdefault(qbond, ({}, {}))
        sec[0].setdefault(lk, None)
        sec[1].setdefault(rk, None)
    out = []
    for qb in sorted(sectors):
        lkeys, rkeys = sorted(sectors[qb][0]), sorted(sectors[qb][1])
        rows, cols = [], []
        r = 0
        for lk in lkeys:
            rows.append((lk, r))
            r += int(np.prod([t.indexes[i].dims[s] for i, s in enumerate(lk)]))
        c = 0
        for rk in rkeys:
            cols.append((rk, c))
            c += int(np.prod([t.indexes[ldims + i].dims[s] for i, s in enumerate(rk)]))
        M = np.zeros((r, c), dtype=t.dtype)
        for lk, ro in rows:
            for rk, co in cols:
                blk = t.blocks.get(lk + rk)
                if blk is not None:
                    m = int(np.prod(blk.shape[:ldims]))
                    M[ro:ro + m, co:co + blk.size // m] = blk.reshape(m, -1)
        out.append((qb, rows, cols, M))
    return out


def svd(t: T, ldims: int, ldiv, trunc_err: float, Dmin: int, Dmax: int):
    """``SVD(T, ldims, ldiv, trunc_err, Dmin, Dmax, &u, &s, &vt, &err, &D)``
    (call site ``two_site_update_finite_vmps_impl.h:302-307``).

    u: (left indexes..., bond OUT), Div(u) = ldiv; s: (bond IN, bond OUT) real
    diagonal; vt: (bond IN, right indexes...).  The new bond's sectors are the
    kept ones in ascending QN order.  Returns (u, s, vt, trunc_err, D).
    """
    secs = svd_sector_matrices(t, ldims, ldiv)
    decomp, svals = [], []
    for qb, rows, cols, M in secs:
        U, S, Vh = np.linalg.svd(M, full_matrices=False)
        decomp.append((U, S, Vh))
        svals.append(S)
    kept, D, err = select_kept(svals, trunc_err, Dmin, Dmax)
    bond_sectors = [(secs[q][0], kept[q]) for q in range(len(secs)) if kept[q] > 0]
    bond = Index.make(bond_sectors, 1)
    lidx, ridx = t.indexes[:ldims], t.indexes[ldims:]
    u = T(list(lidx) + [bond], {}, t.dtype)
    vt = T([bond.inverse()] + list(ridx), {}, t.dtype)
    s = T([bond.inverse(), bond], {}, np.float64)
    b = 0
    for q, (qb, rows, cols, M) in enumerate(secs):
        k = kept[q]
        if k == 0:
            continue
        U, S, Vh = decomp[q]
        for lk, ro in rows:
            shp = tuple(t.indexes[i].dims[s_] for i, s_ in enumerate(lk))
            m = int(np.prod(shp))
            u.blocks[lk + (b,)] = np.ascontiguousarray(U[ro:ro + m, :k]).reshape(shp + (k,))
        for rk, co in cols:
            shp = tuple(t.indexes[ldims + i].dims[s_] for i, s_ in enumerate(rk))
            n = int(np.prod(shp))
            vt.blocks[(b,) + rk] = np.ascontiguousarray(Vh[:k, co:co + n]).reshape((k,) + shp)
        s.blocks[(b, b)] = np.diag(S[:k]).astype(np.float64)
        b += 1
    return u, s, vt, err, D
