"""Host-side model builders: local Hilbert spaces, operators, MPOs, product MPS.

These make the inputs of the two-site update (MPO tensors and initial MPS);
they run once per job on the host and are not part of the GPU hot path.

MPO construction is a finite-state machine over "channels" of each virtual
bond, with prefix sharing: terms that have applied the same operators on the
same sites so far (and carry the same pending string operator) share one
channel.  Channel 0 of every bulk bond is "nothing applied yet" and the last
channel of a bond is "term completed".  The resulting tensors follow the
reference's MPO conventions:

* ``W(lvb IN, pb_in IN, pb_out OUT, rvb OUT)`` and an operator ``O`` given
  as ``O[in, out]`` is written to ``W[l, in, out, r]``
  (``one_dim_tn/mpo/mpogen/mpogen_impl.h:445-545``);
* a right-bond channel carries ``qn(lvb channel) - Div(O)``
  (``mpogen_impl.h:373-381``) so every MPO tensor is divergence free;
* terms with a zero coefficient are skipped (``mpogen_impl.h:92-101``);
* ``AddTerm(coef, op1, s1, op2, s2, inst)`` puts ``inst`` on every site strictly
  between ``s1`` and ``s2`` (Jordan-Wigner strings,
  ``benchmark/ultradmrg_hubbard2d.cpp:149-181``).

The generator in the reference additionally compresses the channel graph; this
one does prefix sharing only, so its bond dimension can differ from the
reference's for the same Hamiltonian (the operator it represents is the same).
The Hamiltonian builders below take ``builder="reference"`` to use
``mpogen`` instead, the reference's generator restated, whose MPOs have the
reference's bond layout.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .tensor_data import IN, OUT, BlockTensorData, Index, qn_sub

# ---------------------------------------------------------------------------
# Local Hilbert spaces and operators.  Operators are dense d x d matrices
# indexed [in, out], i.e. O[i, o] = <o|O|i>, the element layout of
# QLTensor({pb_in, pb_out}) in the reference tests.
# ---------------------------------------------------------------------------


@dataclass
class Operator:
    name: str
    mat: np.ndarray  # [in, out]

    def __mul__(self, s):
        return Operator(f"{s}*{self.name}", self.mat * s)

    __rmul__ = __mul__


def _op(name, d, entries, dtype=np.float64):
    m = np.zeros((d, d), dtype=dtype)
    for (i, o), v in entries.items():
        m[i, o] = v
    return Operator(name, m)


def spin_half_site(dtype=np.float64):
    """S=1/2 with U(1) Sz in units of 1/2: basis [up (+1), down (-1)].

    Operator tables follow ``tests/test_algorithm/test_two_site_update_finite_vmps.cc:64-110``
    (``sp`` sets element {0,1}, ``sm`` element {1,0}).
    """
    pb_out = Index.make([((1,), 1), ((-1,), 1)], OUT)
    ops = {
        "id": _op("id", 2, {(0, 0): 1, (1, 1): 1}, dtype),
        "sz": _op("sz", 2, {(0, 0): 0.5, (1, 1): -0.5}, dtype),
        "sp": _op("sp", 2, {(0, 1): 1}, dtype),
        "sm": _op("sm", 2, {(1, 0): 1}, dtype),
    }
    return pb_out, ops


def hubbard_site_nsz(dtype=np.float64):
    """Hubbard site with U(1)xU(1) (N, Sz): basis [(2,0), (1,1), (1,-1), (0,0)].

    Operator tables (hard-core bosons times the on-site parity F) are those of
    ``benchmark/ultradmrg_hubbard2d.cpp:17-121``.
    """
    pb_out = Index.make([((2, 0), 1), ((1, 1), 1), ((1, -1), 1), ((0, 0), 1)], OUT)
    e = lambda name, t: _op(name, 4, t, dtype)
    ops = {
        "id": e("id", {(0, 0): 1, (1, 1): 1, (2, 2): 1, (3, 3): 1}),
        "f": e("f", {(0, 0): 1, (1, 1): -1, (2, 2): -1, (3, 3): 1}),
        "sz": e("sz", {(1, 1): 0.5, (2, 2): -0.5}),
        "sp": e("sp", {(1, 2): 1.0}),
        "sm": e("sm", {(2, 1): 1.0}),
        "bupc": e("bupc", {(0, 2): 1, (1, 3): 1}),
        "bdnc": e("bdnc", {(0, 1): 1, (2, 3): 1}),
        "bupa": e("bupa", {(2, 0): 1, (3, 1): 1}),
        "bdna": e("bdna", {(1, 0): 1, (3, 2): 1}),
        "bupcF": e("bupcF", {(0, 2): -1, (1, 3): 1}),
        "Fbdnc": e("Fbdnc", {(0, 1): 1, (2, 3): -1}),
        "bupaF": e("bupaF", {(2, 0): 1, (3, 1): -1}),
        "Fbdna": e("Fbdna", {(1, 0): -1, (3, 2): 1}),
        "Uterm": e("Uterm", {(0, 0): 1}),
        "nf": e("nf", {(0, 0): 2, (1, 1): 1, (2, 2): 1}),
    }
    return pb_out, ops


def hubbard_site_nupndn(dtype=np.float64):
    """Hubbard site with U(1)xU(1) (Nup, Ndn): basis [(0,0), (1,0), (0,1), (1,1)].

    Operator tables of ``tests/test_algorithm/test_two_site_update_finite_vmps.cc:759-843``.
    """
    pb_out = Index.make([((0, 0), 1), ((1, 0), 1), ((0, 1), 1), ((1, 1), 1)], OUT)
    e = lambda name, t: _op(name, 4, t, dtype)
    ops = {
        "id": e("id", {(0, 0): 1, (1, 1): 1, (2, 2): 1, (3, 3): 1}),
        "f": e("f", {(0, 0): 1, (1, 1): -1, (2, 2): -1, (3, 3): 1}),
        "nupdn": e("nupdn", {(3, 3): 1}),
        "adagupf": e("adagupf", {(1, 0): 1, (3, 2): -1}),
        "aup": e("aup", {(0, 1): 1, (2, 3): 1}),
        "adagdn": e("adagdn", {(2, 0): 1, (3, 1): 1}),
        "fadn": e("fadn", {(0, 2): 1, (1, 3): -1}),
        "naupf": e("naupf", {(0, 1): 1, (2, 3): -1}),
        "adagup": e("adagup", {(1, 0): 1, (3, 2): 1}),
        "nadn": e("nadn", {(0, 2): -1, (1, 3): -1}),
        "fadagdn": e("fadagdn", {(2, 0): -1, (3, 1): 1}),
    }
    return pb_out, ops


def op_div(op: Operator, pb_out: Index):
    """Div of an operator tensor {pb_in, pb_out}: qn(out) - qn(in)."""
    nz = np.argwhere(op.mat != 0)
    if len(nz) == 0:
        return None
    divs = set()
    for i, o in nz:
        si, _ = pb_out.sector_of(int(i))
        so, _ = pb_out.sector_of(int(o))
        divs.add(qn_sub(pb_out.qns[so], pb_out.qns[si]))
    if len(divs) != 1:
        raise ValueError(f"operator {op.name} does not conserve the quantum numbers")
    return divs.pop()


# ---------------------------------------------------------------------------
# MPO generator
# ---------------------------------------------------------------------------


@dataclass
class _Term:
    coef: float
    sites: List[int]
    ops: List[Operator]
    insts: List[Optional[Operator]]  # string operator after ops[k] (len = len(ops)-1)


class MPOGenerator:
    """Sum-of-products Hamiltonian -> MPO tensors (host side).

    Mirrors the ``AddTerm`` surface of ``one_dim_tn/mpo/mpogen/mpogen.h:38-127``.
    """

    def __init__(self, sites: Sequence[Index], ops_id: Sequence[Operator], dtype=np.float64):
        self.sites = list(sites)
        self.N = len(self.sites)
        self.ids = list(ops_id)
        self.dtype = dtype
        self.terms: List[_Term] = []
        self.zero = tuple(0 for _ in range(self.sites[0].nq))

    def add_term(self, coef, ops: Sequence[Operator], sites: Sequence[int],
                 insts: Optional[Sequence[Optional[Operator]]] = None):
        if coef == 0:
            return
        order = np.argsort(sites, kind="stable")
        sites = [int(sites[i]) for i in order]
        ops = [ops[i] for i in order]
        if len(set(sites)) != len(sites):
            raise ValueError("one operator per site per term")
        if insts is None:
            insts = [None] * (len(ops) - 1)
        elif not isinstance(insts, (list, tuple)):
            insts = [insts] * (len(ops) - 1)
        self.terms.append(_Term(coef, sites, list(ops), list(insts)))

    def add_two_site(self, coef, op1, s1, op2, s2, inst=None):
        """``AddTerm(coef, op1, s1, op2, s2, inst)`` of the reference."""
        if s1 > s2:
            raise ValueError("s1 must precede s2")
        self.add_term(coef, [op1, op2], [s1, s2], [inst])

    def gen(self) -> List[BlockTensorData]:
        N = self.N
        # channel keys per bond b (between site b and b+1): key -> channel id
        # key = ("ready",) | ("done",) | (prefix, inst_name)
        bond_keys: List[Dict] = [dict() for _ in range(N - 1)]
        bond_qn: List[List] = [[] for _ in range(N - 1)]

        def key_of(term: _Term, b: int):
            k = max(i for i, s in enumerate(term.sites) if s <= b)
            prefix = tuple((term.sites[i], term.ops[i].name) for i in range(k + 1))
            gap_empty = term.sites[k + 1] == b + 1
            inst = term.insts[k]
            return prefix, (None if inst is None else inst.name), gap_empty, k

        def qn_after(term: _Term, k: int):
            q = self.zero
            for i in range(k + 1):
                q = qn_sub(q, op_div(term.ops[i], self.sites[term.sites[i]]))
            return q

        for b in range(N - 1):
            bond_keys[b][("ready",)] = 0
            bond_qn[b].append(self.zero)
        # pass 1: channels of terms whose pending gap is non-empty; pass 2 reuses
        # a channel with the same prefix for terms whose next operator is adjacent
        for pass_no in (1, 2):
            for term in self.terms:
                if len(term.sites) < 2:
                    continue
                for b in range(term.sites[0], term.sites[-1]):
                    prefix, inst, gap_empty, k = key_of(term, b)
                    if gap_empty != (pass_no == 2):
                        continue
                    keys = bond_keys[b]
                    if (prefix, inst) in keys:
                        continue
                    if gap_empty:
                        hit = [kk for kk in keys if kk[0] == prefix]
                        if hit:
                            continue
                    keys[(prefix, inst)] = len(bond_qn[b])
                    bond_qn[b].append(qn_after(term, k))
        for b in range(N - 1):
            bond_keys[b][("done",)] = len(bond_qn[b])
            bond_qn[b].append(self.zero)

        def chan(term, b):
            prefix, inst, gap_empty, k = key_of(term, b)
            keys = bond_keys[b]
            if (prefix, inst) in keys:
                return keys[(prefix, inst)]
            for kk, v in keys.items():
                if kk[0] == prefix:
                    return v
            raise KeyError("channel missing")

        # per-site operator matrix entries: (l_chan, r_chan) -> accumulated op
        entries: List[Dict[Tuple[int, int], np.ndarray]] = [dict() for _ in range(N)]

        def add(site, l, r, mat):
            e = entries[site]
            if (l, r) in e:
                e[(l, r)] = e[(l, r)] + mat
            else:
                e[(l, r)] = mat.astype(self.dtype).copy()

        ready_l = lambda i: 0
        done_r = lambda i: 0 if i == N - 1 else bond_keys[i][("done",)]
        ready_r = lambda i: 0
        done_l = lambda i: 0 if i == 0 else bond_keys[i - 1][("done",)]

        for i in range(N):
            idm = self.ids[i].mat
            if i < N - 1 and i > 0:
                add(i, ready_l(i), ready_r(i), idm)
                add(i, done_l(i), done_r(i), idm)
            elif i == 0 and N > 1:
                add(i, 0, ready_r(i), idm)
            elif i == N - 1 and N > 1:
                add(i, done_l(i), 0, idm)
        for term in self.terms:
            if len(term.sites) == 1:
                s = term.sites[0]
                l = 0 if s == 0 else ready_l(s)
                r = done_r(s)
                add(s, l, r, term.coef * term.ops[0].mat)
                continue
            first, last = term.sites[0], term.sites[-1]
            for s in range(first, last + 1):
                l = 0 if s == first else chan(term, s - 1)
                r = done_r(s) if s == last else chan(term, s)
                if s in term.sites:
                    k = term.sites.index(s)
                    mat = term.ops[k].mat
                    if s == last:
                        mat = term.coef * mat
                else:
                    k = max(j for j, t in enumerate(term.sites) if t < s)
                    inst = term.insts[k]
                    mat = self.ids[s].mat if inst is None else inst.mat
                # an identical (l, r, mat) entry from another term is the same
                # shared channel transition; only add transitions once
                key = (l, r)
                e = entries[s]
                if s != last and key in e:
                    continue
                add(s, l, r, mat)

        # bond indexes: group channels by QN (ascending), keep creation order
        bond_perm, bond_index = [], []
        for b in range(N - 1):
            qns = bond_qn[b]
            uniq = sorted(set(qns))
            order = []
            sectors = []
            for q in uniq:
                members = [c for c in range(len(qns)) if qns[c] == q]
                order.extend(members)
                sectors.append((q, len(members)))
            pos = {c: p for p, c in enumerate(order)}
            bond_perm.append(pos)
            bond_index.append(Index.make(sectors, OUT))
        triv = Index.make([(self.zero, 1)], OUT)
        mpo = []
        for i in range(N):
            lvb = (triv if i == 0 else bond_index[i - 1]).inverse()
            rvb = triv if i == N - 1 else bond_index[i]
            pb_out = self.sites[i]
            W = BlockTensorData([lvb, pb_out.inverse(), pb_out, rvb], {}, self.dtype)
            for (l, r), mat in entries[i].items():
                lc = l if i == 0 else bond_perm[i - 1][l]
                rc = r if i == N - 1 else bond_perm[i][r]
                for a, o in np.argwhere(mat != 0):
                    W.set_elem((lc, int(a), int(o), rc), mat[a, o])
            mpo.append(W)
        return mpo


class _ReferenceLayoutGenerator:
    """The builder calls of this module on ``mpogen.MPOGenerator`` (the
    reference's compressing generator): MPOs with the reference's bond
    dimensions, sector order and channel order."""

    def __init__(self, sites: Sequence[Index], ops_id: Sequence[Operator], dtype=np.float64):
        from .mpogen import MPOGenerator as RefGen
        self.g = RefGen(sites, [o.mat for o in ops_id], dtype=dtype)

    def add_term(self, coef, ops: Sequence[Operator], sites: Sequence[int], insts=None):
        if insts is not None and not isinstance(insts, (list, tuple)):
            insts = [insts] * (len(ops) - 1)
        if insts is None or all(i is None for i in insts):
            self.g.add_term(coef, [o.mat for o in ops], list(sites))
        else:
            self.g.add_term_insert(coef, [o.mat for o in ops], list(sites),
                                   [o.mat for o in insts])

    def add_two_site(self, coef, op1, s1, op2, s2, inst=None):
        self.g.add_two_body(coef, op1.mat, s1, op2.mat, s2, None if inst is None else inst.mat)

    def gen(self) -> List[BlockTensorData]:
        return self.g.gen()


BUILDERS = ("prefix", "reference")


def _generator(builder: str, sites, ops_id, dtype):
    """builder "prefix": this module's prefix-sharing generator; "reference":
    the reference's FSM generator with symbolic compression (``mpogen``)."""
    if builder == "prefix":
        return MPOGenerator(sites, ops_id, dtype)
    if builder == "reference":
        return _ReferenceLayoutGenerator(sites, ops_id, dtype)
    raise ValueError(f"unknown MPO builder {builder!r}")


# ---------------------------------------------------------------------------
# Hamiltonians used by the tests and the benchmark (builder: see _generator)
# ---------------------------------------------------------------------------


def heisenberg_chain_mpo(N, J=1.0, dtype=np.float64, pairs=None, builder="prefix"):
    pb, ops = spin_half_site(dtype)
    g = _generator(builder, [pb] * N, [ops["id"]] * N, dtype)
    if pairs is None:
        pairs = [(i, i + 1) for i in range(N - 1)]
    for (i, j) in pairs:
        i, j = min(i, j), max(i, j)
        g.add_two_site(J, ops["sz"], i, ops["sz"], j)
        g.add_two_site(0.5 * J, ops["sp"], i, ops["sm"], j)
        g.add_two_site(0.5 * J, ops["sm"], i, ops["sp"], j)
    return g.gen(), pb


def spinless_fermion_site(dtype=np.float64):
    """Spinless fermion site with a U(1) charge: basis [0 (+1), 1 (-1)];
    c sets element {0,1}, c^dag element {1,0}, the Jordan-Wigner string
    f = diag(-1, 1) (``tests/test_algorithm/test_two_site_finite_tdvp.cc:38-80``)."""
    pb_out = Index.make([((1,), 1), ((-1,), 1)], OUT)
    ops = {
        "id": _op("id", 2, {(0, 0): 1, (1, 1): 1}, dtype),
        "c": _op("c", 2, {(0, 1): 1}, dtype),
        "cdag": _op("cdag", 2, {(1, 0): 1}, dtype),
        "f": _op("f", 2, {(0, 0): -1, (1, 1): 1}, dtype),
    }
    return pb_out, ops


def free_fermion_chain_mpo(N, t=1.0, dtype=np.float64, builder="prefix"):
    """H = -t sum_i (c^dag_i c_{i+1} + c_i c^dag_{i+1}) on an open chain
    (``test_two_site_finite_tdvp.cc:108-113``)."""
    pb, ops = spinless_fermion_site(dtype)
    g = _generator(builder, [pb] * N, [ops["id"]] * N, dtype)
    for i in range(N - 1):
        g.add_two_site(-t, ops["cdag"], i, ops["c"], i + 1)
        g.add_two_site(-t, ops["c"], i, ops["cdag"], i + 1)
    return g.gen(), pb, ops


def ising_chain_mpo(N, dtype=np.float64, builder="prefix"):
    pb, ops = spin_half_site(dtype)
    g = _generator(builder, [pb] * N, [ops["id"]] * N, dtype)
    for i in range(N - 1):
        g.add_two_site(1.0, ops["sz"], i, ops["sz"], i + 1)
    return g.gen(), pb


def spin_half_site_nosym(dtype=np.complex128):
    """S=1/2 without symmetry: one sector of dimension 2 (a trivial quantum
    number), basis [up, down]; the operator tables of
    ``include/qlmps/model_relevant/operators/spin/spin_one_half_operators.h``
    (``sp`` sets {down, up}; ``sx``, and ``sy`` with <up|Sy|down> = -i/2)."""
    pb_out = Index.make([((0,), 2)], OUT)
    e = lambda name, t: _op(name, 2, t, dtype)
    ops = {
        "id": e("id", {(0, 0): 1, (1, 1): 1}),
        "sz": e("sz", {(0, 0): 0.5, (1, 1): -0.5}),
        "sp": e("sp", {(1, 0): 1}),
        "sm": e("sm", {(0, 1): 1}),
        "sx": e("sx", {(1, 0): 0.5, (0, 1): 0.5}),
    }
    if np.issubdtype(np.dtype(dtype), np.complexfloating):
        ops["sy"] = e("sy", {(1, 0): -0.5j, (0, 1): 0.5j})
    return pb_out, ops


def kitaev_gamma_mpo(Nx=3, Ny=4, J=-1.0, K=1.0, Gm=0.1, h=0.1, dtype=np.complex128,
                     builder="prefix"):
    """The J-K-Gamma model with a field of ``tests/test_algorithm/test_finite_dmrg.cc:346-436``
    (no symmetry, complex): sites x * Ny + y; per site -h (Sz + Sx + Sy); x
    links (y even, to y + 1) J S.S + K Sx Sx + Gm (Sz Sy + Sy Sz); z links
    (y odd, to (y + 1) mod Ny) J S.S + K Sz Sz + Gm (Sx Sy + Sy Sx); y links
    (y odd, x < Nx - 1, to (x + 1, y - 1)) J S.S + K Sy Sy + Gm (Sz Sx + Sx Sz)."""
    pb, o = spin_half_site_nosym(dtype)
    N = Nx * Ny
    g = _generator(builder, [pb] * N, [o["id"]] * N, dtype)
    idx = lambda x, y: x * Ny + y
    sx, sy, sz = o["sx"], o["sy"], o["sz"]

    def bond(s0, s1, kit, gam):
        s0, s1 = min(s0, s1), max(s0, s1)
        for a in (sz, sx, sy):
            g.add_two_site(J, a, s0, a, s1)
        g.add_two_site(K, kit, s0, kit, s1)
        g.add_two_site(Gm, gam[0], s0, gam[1], s1)
        g.add_two_site(Gm, gam[1], s0, gam[0], s1)

    for x in range(Nx):
        for y in range(Ny):
            s0 = idx(x, y)
            for a in (sz, sx, sy):
                g.add_term(-h, [a], [s0])
            if y % 2 == 0:
                bond(s0, idx(x, y + 1), sx, (sz, sy))
            if y % 2 == 1:
                bond(s0, idx(x, (y + 1) % Ny), sz, (sx, sy))
            if y % 2 == 1 and x != Nx - 1:
                bond(s0, idx(x + 1, y - 1), sy, (sz, sx))
    return g.gen(), pb


def kondo_chain_mpo(Nx=4, t=0.25, Jk=1.0, Jz=0.5, dtype=np.float64, builder="prefix"):
    """Kondo insulator double chain of
    ``tests/test_algorithm/test_two_site_update_finite_vmps.cc:976-1084``: even
    sites conduction electrons (four states in one Sz = 0 sector), odd sites
    localized spins (two states, one sector); hopping between consecutive
    electron sites i, i + 2 (the Jordan-Wigner sign is inside the tables, the
    spin between carries the identity), Jz Sz Sz between consecutive spins
    and the Kondo coupling Jk S_e . S_l on each rung.  Returns (mpo, sites)."""
    pbE = Index.make([((0,), 4)], OUT)
    pbL = Index.make([((0,), 2)], OUT)
    e4 = lambda name, tb: _op(name, 4, tb, dtype)
    e2 = lambda name, tb: _op(name, 2, tb, dtype)
    o = {
        "sz": e4("sz", {(0, 0): 0.5, (1, 1): -0.5}), "sp": e4("sp", {(0, 1): 1.0}),
        "sm": e4("sm", {(1, 0): 1.0}),
        "bupcF": e4("bupcF", {(2, 1): -1, (0, 3): 1}), "Fbdnc": e4("Fbdnc", {(2, 0): 1, (1, 3): -1}),
        "bupaF": e4("bupaF", {(1, 2): 1, (3, 0): -1}), "Fbdna": e4("Fbdna", {(0, 2): -1, (3, 1): 1}),
        "bupc": e4("bupc", {(2, 1): 1, (0, 3): 1}), "bdnc": e4("bdnc", {(2, 0): 1, (1, 3): 1}),
        "bupa": e4("bupa", {(1, 2): 1, (3, 0): 1}), "bdna": e4("bdna", {(0, 2): 1, (3, 1): 1}),
        "Sz": e2("Sz", {(0, 0): 0.5, (1, 1): -0.5}), "Sp": e2("Sp", {(0, 1): 1.0}),
        "Sm": e2("Sm", {(1, 0): 1.0}),
        "idE": e4("idE", {(i, i): 1 for i in range(4)}), "idL": e2("idL", {(0, 0): 1, (1, 1): 1}),
    }
    N = 2 * Nx
    sites = [pbE if i % 2 == 0 else pbL for i in range(N)]
    ids = [o["idE"] if i % 2 == 0 else o["idL"] for i in range(N)]
    g = _generator(builder, sites, ids, dtype)
    for i in range(0, N - 2, 2):
        g.add_two_site(-t, o["bupcF"], i, o["bupa"], i + 2)
        g.add_two_site(-t, o["bdnc"], i, o["Fbdna"], i + 2)
        g.add_two_site(t, o["bupaF"], i, o["bupc"], i + 2)
        g.add_two_site(t, o["bdna"], i, o["Fbdnc"], i + 2)
        g.add_two_site(Jz, o["Sz"], i + 1, o["Sz"], i + 3)
    for i in range(0, N, 2):
        g.add_two_site(Jk, o["sz"], i, o["Sz"], i + 1)
        g.add_two_site(Jk / 2, o["sp"], i, o["Sm"], i + 1)
        g.add_two_site(Jk / 2, o["sm"], i, o["Sp"], i + 1)
    return g.gen(), sites


def rashba_tj_mpo(Nx=3, Ny=2, t=3.0, J=1.0, lamb=0.03, builder="prefix"):
    """t-J model with a Rashba spin-orbit term on an Nx x Ny lattice, periodic
    in x and open in y, of ``tests/test_algorithm/test_two_site_update_finite_vmps.cc:627-751``:
    one U(1) (charge; sectors N = 1 of two states [up, down], N = 0 of one),
    complex.  Operator tables, term list (hard-core operators with the
    parity string f strictly between the two sites) and the swap of a wrapped
    bond's site indices while its operators keep their order are the test's,
    term for term.  Sites x * Ny + y."""
    dtype = np.complex128
    pb = Index.make([((1,), 2), ((0,), 1)], OUT)
    e = lambda name, tb: _op(name, 3, tb, dtype)
    o = {
        "id": e("id", {(0, 0): 1, (1, 1): 1, (2, 2): 1}),
        "f": e("f", {(0, 0): -1, (1, 1): -1, (2, 2): 1}),
        "sz": e("sz", {(0, 0): 0.5, (1, 1): -0.5}), "sp": e("sp", {(1, 0): 1}),
        "sm": e("sm", {(0, 1): 1}),
        "cup": e("cup", {(0, 2): 1}), "cdagup": e("cdagup", {(2, 0): 1}),
        "cdn": e("cdn", {(1, 2): 1}), "cdagdn": e("cdagdn", {(2, 1): 1}),
        "ntot": e("ntot", {(0, 0): 1, (1, 1): 1}),
    }
    N = Nx * Ny
    g = _generator(builder, [pb] * N, [o["id"]] * N, dtype)
    idx = lambda x, y: x * Ny + y
    f = o["f"]
    ilamb = 1j * lamb

    def common(s0, s1):
        for c, a, b_ in ((-t, "cdagup", "cup"), (-t, "cdagdn", "cdn"), (-t, "cup", "cdagup"),
                         (-t, "cdn", "cdagdn")):
            g.add_two_site(c, o[a], s0, o[b_], s1, f)
        g.add_two_site(J, o["sz"], s0, o["sz"], s1)
        g.add_two_site(J / 2, o["sp"], s0, o["sm"], s1)
        g.add_two_site(J / 2, o["sm"], s0, o["sp"], s1)
        g.add_two_site(-J / 4, o["ntot"], s0, o["ntot"], s1)

    for x in range(Nx):
        for y in range(Ny):
            # x bonds, periodic
            s0, s1 = idx(x, y), idx((x + 1) % Nx, y)
            s0, s1 = min(s0, s1), max(s0, s1)
            common(s0, s1)
            so = ((lamb, "cdagup", "cdn"), (lamb, "cup", "cdagdn"), (-lamb, "cdagdn", "cup"),
                  (-lamb, "cdn", "cdagup")) if x != Nx - 1 else \
                 ((lamb, "cdn", "cdagup"), (lamb, "cdagdn", "cup"), (-lamb, "cup", "cdagdn"),
                  (-lamb, "cdagup", "cdn"))
            for c, a, b_ in so:
                g.add_two_site(c, o[a], s0, o[b_], s1, f)
            # y bonds, open
            if y != Ny - 1:
                s0, s2 = idx(x, y), idx(x, (y + 1) % Ny)
                s0, s2 = min(s0, s2), max(s0, s2)
                common(s0, s2)
                for c, a, b_ in ((ilamb, "cdagup", "cdn"), (ilamb, "cdagdn", "cup"),
                                 (-ilamb, "cup", "cdagdn"), (-ilamb, "cdn", "cdagup")):
                    g.add_two_site(c, o[a], s0, o[b_], s2, f)
    return g.gen(), pb


def tj_site(dtype=np.float64):
    """t-J site with U(1)xU(1) (N, Sz): basis [up (1,1), down (1,-1), empty (0,0)];
    operator tables of ``tests/test_algorithm/test_fermion_two_site_update_finite_vmps.cc:110-160``
    (``cup`` sets {0,2}: up -> empty; ``sp`` sets {1,0}: down -> up) and the
    on-site parity ``f = diag(-1, -1, 1)``."""
    pb_out = Index.make([((1, 1), 1), ((1, -1), 1), ((0, 0), 1)], OUT)
    e = lambda name, t: _op(name, 3, t, dtype)
    ops = {
        "id": e("id", {(0, 0): 1, (1, 1): 1, (2, 2): 1}),
        "f": e("f", {(0, 0): -1, (1, 1): -1, (2, 2): 1}),
        "sz": e("sz", {(0, 0): 0.5, (1, 1): -0.5}),
        "sp": e("sp", {(1, 0): 1}),
        "sm": e("sm", {(0, 1): 1}),
        "cup": e("cup", {(0, 2): 1}),
        "cdagup": e("cdagup", {(2, 0): 1}),
        "cdn": e("cdn", {(1, 2): 1}),
        "cdagdn": e("cdagdn", {(2, 1): 1}),
    }
    return pb_out, ops


def tj_mpo(N, t=3.0, J=1.0, pairs=None, dtype=np.float64, builder="prefix"):
    """t-J model of ``test_fermion_two_site_update_finite_vmps.cc:162-270``:
    sum over bonds (i < j) of t (c^dag_i c_j - c_i c^dag_j) per spin plus
    J (Sz Sz + (S+ S- + S- S+) / 2).  The reference's fermionic tensors carry
    the signs; here they are explicit Jordan-Wigner strings:
    c^dag_i c_j = (c^dag f)_i f_{i+1} ... f_{j-1} c_j, where the operator
    product (c^dag f) applies f first (the matrix f @ c^dag in the [in, out]
    layout)."""
    pb, o = tj_site(dtype)
    g = _generator(builder, [pb] * N, [o["id"]] * N, dtype)
    f = o["f"]
    if pairs is None:
        pairs = [(i, i + 1) for i in range(N - 1)]
    after_f = lambda op: Operator(op.name + "F", f.mat @ op.mat)
    for (i, j) in pairs:
        i, j = min(i, j), max(i, j)
        inst = f if j - i > 1 else None
        for s in ("up", "dn"):
            g.add_term(t, [after_f(o["cdag" + s]), o["c" + s]], [i, j], inst)
            g.add_term(-t, [after_f(o["c" + s]), o["cdag" + s]], [i, j], inst)
        g.add_two_site(J, o["sz"], i, o["sz"], j)
        g.add_two_site(J / 2, o["sp"], i, o["sm"], j)
        g.add_two_site(J / 2, o["sm"], i, o["sp"], j)
    return g.gen(), pb


def heisenberg_ladder_pairs(Lx, Ly=2):
    """Nearest-neighbour bonds of an Lx x Ly open ladder, site = x*Ly + y."""
    pairs = []
    for x in range(Lx):
        for y in range(Ly):
            s = x * Ly + y
            if y + 1 < Ly:
                pairs.append((s, s + 1))
            if x + 1 < Lx:
                pairs.append((s, s + Ly))
    return pairs


def hubbard_cylinder_mpo(Lx, Ly, t=1.0, U=8.0, t2=0.0, dtype=np.float64, builder="prefix"):
    """Hubbard cylinder (open x, periodic y) with the site map and hopping terms
    of ``benchmark/ultradmrg_hubbard2d.cpp:138-202`` (site = x*Ly + y)."""
    pb, o = hubbard_site_nsz(dtype)
    N = Lx * Ly
    g = _generator(builder, [pb] * N, [o["id"]] * N, dtype)
    f = o["f"]

    def hop(tt, s1, s2, inst):
        g.add_two_site(-tt, o["bupcF"], s1, o["bupa"], s2, inst)
        g.add_two_site(-tt, o["bdnc"], s1, o["Fbdna"], s2, inst)
        g.add_two_site(tt, o["bupaF"], s1, o["bupc"], s2, inst)
        g.add_two_site(tt, o["bdna"], s1, o["Fbdnc"], s2, inst)

    for i in range(N):
        g.add_term(U, [o["Uterm"]], [i])
    for i in range(N - Ly):
        hop(t, i, i + Ly, f)
    for i in range(N):
        y = i % Ly
        if y < Ly - 1:
            hop(t, i, i + 1, None)
        elif Ly > 2:
            hop(t, i - Ly + 1, i, f)
    if t2 != 0.0:
        for i in range(N - Ly):
            y, x = i % Ly, i // Ly
            for T in ((y + 1) % Ly + (x + 1) * Ly, (y + Ly - 1) % Ly + (x + 1) * Ly):
                hop(t2, min(i, T), max(i, T), f)
    return g.gen(), pb


def hubbard_cylinder_holes(N, n_holes_per=8):
    """Initial product state labels of ``benchmark/ultradmrg_hubbard2d.cpp:206-225``
    (one hole every N/8 sites, alternating up/down elsewhere): basis labels
    0=(2,0), 1=(1,1), 2=(1,-1), 3=(0,0)."""
    per = N // n_holes_per
    labs, sz = [], 0
    for i in range(N):
        if i % per == per - 1:
            labs.append(3)
        else:
            labs.append(sz % 2 + 1)
            sz += 1
    return labs


def hubbard_2x2_test_mpo(dtype=np.float64, t0=1.0, t1=0.5, U=2.0, Nx=2, Ny=2, builder="prefix"):
    """Hubbard model of ``test_two_site_update_finite_vmps.cc:848-905``."""
    pb, o = hubbard_site_nupndn(dtype)
    N = Nx * Ny
    g = _generator(builder, [pb] * N, [o["id"]] * N, dtype)
    f = o["f"]
    idx = lambda i, j: i * Ny + j

    def hop(tt, s0, s1):
        g.add_two_site(1, -tt * o["adagupf"], s0, o["aup"], s1, f)
        g.add_two_site(1, -tt * o["adagdn"], s0, o["fadn"], s1, f)
        g.add_two_site(1, o["naupf"], s0, -tt * o["adagup"], s1, f)
        g.add_two_site(1, o["nadn"], s0, -tt * o["fadagdn"], s1, f)

    for i in range(Nx):
        for j in range(Ny):
            s0 = idx(i, j)
            g.add_term(U, [o["nupdn"]], [s0])
            if i != Nx - 1:
                hop(t0, s0, idx(i + 1, j))
            if j != Ny - 1:
                hop(t0, s0, idx(i, j + 1))
            if j != Ny - 1:
                if i != 0:
                    a, b = sorted((s0, idx(i - 1, j + 1)))
                    hop(t1, a, b)
                if i != Nx - 1:
                    a, b = sorted((s0, idx(i + 1, j + 1)))
                    hop(t1, a, b)
    return g.gen(), pb


def act_operator_on_mps(mps: Sequence[BlockTensorData], op, inst, site: int
                        ) -> List[BlockTensorData]:
    """``ActOperatorOnMps`` (algorithm/tdvp/two_site_update_finite_tdvp_impl.h:23-54):
    the operator ``op`` on ``site`` and, when ``inst`` is given, the string
    operator on every site left of it: ``A'[l, o, r] = sum_i O[i, o] A[l, i, r]``.
    A block (l, o-sector, r) of the result exists where the site has a block
    (l, i-sector, r) and O has a non-zero element between the two sectors.
    The MPS keeps its bonds; the operator's divergence moves into ``site``'s
    tensor.  Host data in, host data out."""
    out = list(mps)
    todo = [(site, op)] + ([] if inst is None else [(j, inst) for j in range(site - 1, -1, -1)])
    for i, o in todo:
        O = np.asarray(o.mat if hasattr(o, "mat") else o)
        A = out[i]
        pb = A.indexes[1]
        off = pb.offsets()
        dtype = np.result_type(A.dtype, O.dtype)
        blocks: Dict[Tuple[int, ...], np.ndarray] = {}
        for (ls, ps, rs), B in A.blocks.items():
            for so in range(pb.nsec):
                sub = O[off[ps]:off[ps + 1], off[so]:off[so + 1]]
                if not sub.any():
                    continue
                C = np.einsum("lir,io->lor", B, sub)
                key = (ls, so, rs)
                blocks[key] = blocks[key] + C if key in blocks else C.astype(dtype)
        out[i] = BlockTensorData(list(A.indexes), blocks, dtype)
    return out


# ---------------------------------------------------------------------------
# MPS initialisation
# ---------------------------------------------------------------------------


def operator_tensor(mat: np.ndarray, pb_out: Index, dtype=None) -> BlockTensorData:
    """One-site operator tensor {pb_in, pb_out} from a dense matrix mat[in, out]."""
    mat = np.asarray(mat)
    t = BlockTensorData([pb_out.inverse(), pb_out], {}, dtype or mat.dtype)
    for (i, o) in np.argwhere(mat != 0):
        t.set_elem((int(i), int(o)), mat[i, o])
    return t


def mat_repr_mpo(mpo: Sequence[BlockTensorData]):
    """The matrix representation (MatReprMPO, ``one_dim_tn/mpo/mat_repr_mpo.h:21``)
    of MPO tensors W(lvb, pb_in, pb_out, rvb): per site (rows, cols, [(x, y,
    operator tensor {pb_in, pb_out})]) for the non-null operators W[x, :, :, y]."""
    out = []
    for W in mpo:
        d = W.to_dense()
        pb = W.indexes[2]
        rows, cols = d.shape[0], d.shape[3]
        elems = []
        for x in range(rows):
            for y in range(cols):
                m = d[x, :, :, y]
                if np.any(m != 0):
                    elems.append((x, y, operator_tensor(m, pb, W.dtype)))
        out.append((rows, cols, elems))
    return out


def direct_product_mps(sites: Sequence[Index], labels: Sequence[int], dtype=np.float64):
    """Product-state MPS with the bond conventions of ``DirectStateInitMps``
    (``one_dim_tn/mps/finite_mps/finite_mps_init.h:213-266``): tensors
    (lvb IN, pb OUT, rvb OUT); site 0 carries the total divergence and
    ``qn(rvb_i) = qn(lvb_i) - qn(pb_i)``.  The reference then calls
    ``Centralize(0)``, which leaves a product state's tensors as they are
    up to signs; this builder returns them unchanged (centre at site 0).
    """
    N = len(sites)
    qn_of = lambda i: sites[i].qns[sites[i].sector_of(labels[i])[0]]
    zero = tuple(0 for _ in range(sites[0].nq))
    div = zero
    for i in range(N):
        div = tuple(a + b for a, b in zip(div, qn_of(i)))
    mps = []
    lvb = Index.make([(zero, 1)], IN)
    rq = qn_sub(div, qn_of(0))
    for i in range(N):
        if i == 0:
            lvb = Index.make([(zero, 1)], IN)
            rvb = Index.make([(rq, 1)], OUT)
        else:
            lvb = rvb.inverse()
            if i == N - 1:
                rvb = Index.make([(zero, 1)], OUT)
            else:
                rvb = Index.make([(qn_sub(lvb.qns[0], qn_of(i)), 1)], OUT)
        A = BlockTensorData([lvb, sites[i], rvb], {}, dtype)
        A.set_elem((0, labels[i], 0), 1.0)
        mps.append(A)
    return mps


def _qn_sum_counts(sites: Sequence[Index]):
    """counts[b][q] = number of product states of sites[0..b] with QN sum q."""
    out = []
    cur = {tuple(0 for _ in range(sites[0].nq)): 1.0}
    for ind in sites:
        nxt = {}
        for q, c in cur.items():
            for sq, d in zip(ind.qns, ind.dims):
                k = tuple(a + b for a, b in zip(q, sq))
                nxt[k] = nxt.get(k, 0.0) + c * d
        out.append(nxt)
        cur = nxt
    return out


def bond_sectors(sites: Sequence[Index], div, D: int, sigma: float = 2.5):
    """Bond QN sectors of an MPS with total QN ``div`` and bond dimension <= D.

    Bond b (right of site b) carries r = div - sum_{i<=b} q_i (the convention of
    ``DirectStateInitMps``).  A sector's weight is a Gaussian of width ``sigma``
    (in QN units) around the mean filling of the right block, the shape of the
    Schmidt-spectrum weight of a converged ground state; the dimensions are the
    weights scaled to fit D, never above c (the smaller of the numbers of left
    and right product states with that QN) and at least 1 for kept sectors.
    """
    N = len(sites)
    left = _qn_sum_counts(sites)
    right = _qn_sum_counts(list(reversed(sites)))
    bonds = []
    for b in range(N - 1):
        cl, cr = left[b], right[N - 2 - b]
        sec = {}
        for ql, c in cl.items():
            r = qn_sub(div, ql)
            if r in cr:
                sec[r] = min(c, cr[r])
        qs = sorted(sec)
        cnt = np.array([sec[q] for q in qs], dtype=float)
        if cnt.sum() <= D:
            dims = cnt
        else:
            mean = np.array(div, dtype=float) * (N - 1 - b) / N
            d2 = np.array([np.sum((np.array(q, dtype=float) - mean) ** 2) for q in qs])
            w = np.exp(-d2 / (2.0 * sigma ** 2))
            keep_min = w > 1e-3 * w.max()
            w = np.where(keep_min, w, 0.0)
            order = np.argsort(-w, kind="stable")
            keep = np.zeros(len(qs), bool)
            keep[order[:D]] = True
            keep &= w > 0
            dims = np.zeros(len(qs))
            budget = D
            # water-filling: sectors capped by their count, the rest share the budget
            active = keep.copy()
            while True:
                share = budget / w[active].sum()
                cand = np.where(active, np.floor(w * share), 0)
                capped = active & (cand >= cnt)
                if not capped.any():
                    dims[active] = np.maximum(1, cand[active])
                    break
                dims[capped] = cnt[capped]
                budget -= cnt[capped].sum()
                active &= ~capped
            while dims.sum() > D:
                dims[np.argmax(dims)] -= 1
        bonds.append([(q, int(d)) for q, d in zip(qs, dims) if d > 0])
    return bonds


def random_mps(sites: Sequence[Index], div, D: int, seed: int = 0, dtype=np.float64,
               sigma: float = 2.5):
    """Random MPS with the block structure of ``bond_sectors`` (site 0 carries the
    divergence); each tensor is scaled to squared norm min(D_l*d, D_r)."""
    rng = np.random.default_rng(seed)
    N = len(sites)
    bonds = bond_sectors(sites, div, D, sigma)
    zero = tuple(0 for _ in range(sites[0].nq))
    mps = []
    for i in range(N):
        lvb = Index.make([(zero, 1)], IN) if i == 0 else Index.make(bonds[i - 1], OUT).inverse()
        rvb = Index.make([(zero, 1)], OUT) if i == N - 1 else Index.make(bonds[i], OUT)
        A = BlockTensorData([lvb, sites[i], rvb], {}, dtype)
        target = div if i == 0 else zero
        rpos = {q: s for s, q in enumerate(rvb.qns)}
        for li, lq in enumerate(lvb.qns):
            for pi, pq in enumerate(sites[i].qns):
                # Div = -lq + pq + rq = target
                rq = tuple(t + a - b for t, a, b in zip(target, lq, pq))
                ri = rpos.get(rq)
                if ri is None:
                    continue
                shp = (lvb.dims[li], sites[i].dims[pi], rvb.dims[ri])
                blk = rng.standard_normal(shp)
                if dtype == np.complex128:
                    blk = blk + 1j * rng.standard_normal(shp)
                A.blocks[(li, pi, ri)] = blk.astype(dtype)
        nrm2 = sum(np.vdot(b, b).real for b in A.blocks.values())
        want = min(lvb.dim * sites[i].dim, rvb.dim)
        if nrm2 > 0:
            s = np.sqrt(want / nrm2)
            for k in A.blocks:
                A.blocks[k] = A.blocks[k] * s
        mps.append(A)
    return mps


def random_canonical_mps(sites: Sequence[Index], div, D: int, centre: int, seed: int = 0,
                         dtype=np.float64, sigma: float = 2.5):
    """Random MPS in mixed-canonical form around ``centre``: sites left of it
    are left isometries, sites right of it right isometries (per bond sector,
    by QR of Gaussian blocks), the centre tensor is Gaussian with unit norm.
    Environments built from it have the scale of a converged DMRG state."""
    mps = random_mps(sites, div, D, seed=seed, dtype=dtype, sigma=sigma)
    N = len(mps)

    def orthonormalize(A: BlockTensorData, left: bool):
        # group blocks by the sector of the open bond (right bond if left-isometry)
        ax = 2 if left else 0
        groups: Dict[int, List[Tuple[int, ...]]] = {}
        for k in sorted(A.blocks):
            groups.setdefault(k[ax], []).append(k)
        for sec, keys in groups.items():
            if left:
                mats = [A.blocks[k].reshape(-1, A.blocks[k].shape[2]) for k in keys]
                M = np.concatenate(mats, axis=0)
            else:
                mats = [A.blocks[k].reshape(A.blocks[k].shape[0], -1) for k in keys]
                M = np.concatenate(mats, axis=1).T
            q, _ = np.linalg.qr(M)
            Q = np.zeros_like(M)
            Q[:, :q.shape[1]] = q
            if not left:
                Q = Q.T
            off = 0
            for k, mt in zip(keys, mats):
                if left:
                    A.blocks[k] = Q[off:off + mt.shape[0], :].reshape(A.blocks[k].shape)
                    off += mt.shape[0]
                else:
                    A.blocks[k] = Q[:, off:off + mt.shape[1]].reshape(A.blocks[k].shape)
                    off += mt.shape[1]

    for i in range(N):
        if i < centre:
            orthonormalize(mps[i], True)
        elif i > centre:
            orthonormalize(mps[i], False)
    c = mps[centre]
    nrm = np.sqrt(sum(np.vdot(b, b).real for b in c.blocks.values()))
    for k in c.blocks:
        c.blocks[k] = c.blocks[k] / nrm
    return mps


def random_sz0_labels(N, seed):
    """Random half-up / half-down spin labels (total Sz=0) from numpy's PCG64."""
    rng = np.random.Generator(np.random.PCG64(seed))
    labs = np.array([0] * (N // 2) + [1] * (N - N // 2))
    return [int(v) for v in rng.permutation(labs)]
