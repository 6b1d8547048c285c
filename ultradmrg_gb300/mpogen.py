"""The reference's MPO generator, restated: finite-state machine plus symbolic
compression (``one_dim_tn/mpo/mpogen/``), so an MPO built here has the
reference's virtual-bond dimensions, sector order and channel order for the
same list of terms.

This is host-side code that runs once per job to make the MPO tensors the
two-site update consumes.  ``models.MPOGenerator`` is a different,
prefix-sharing builder: its MPOs represent the same operators but their
bonds differ from the reference's.

Pieces, each following its reference file:

* ``Coef`` / ``Op`` — ``CoefRepr`` / ``OpRepr`` (``symb_alg/coef_op_alg.h:35-405``).
  A coefficient is a sum of c-number labels, and two coefficients are equal
  when their label lists are permutations of each other.  An operator maps
  basis-operator labels to coefficients.
* ``SparMat`` — ``SparMat`` / ``SparOpReprMat`` (``symb_alg/sparse_mat.h``,
  ``coef_op_alg.h:423-660``).  Rows and columns are sorted by their number
  of non-null elements, common coefficients are separated, and rows or
  columns that are combinations of earlier ones are found.
* compression — ``SparOpReprMatColCompresser`` / ``RowCompresser`` and the
  delinearisations (``coef_op_alg.h:660-940``).
* ``FSM`` — ``fsm.h:116-281``.  Paths become ready / middle / final states,
  there is a matrix per site, and compression runs left to right over columns
  and then right to left over rows.
* ``MPOGenerator`` — ``mpogen_impl.h:50-545``.  It mirrors the three
  ``AddTerm`` forms (sign normalisation by the first non-zero element; label
  conversion of coefficients and operators) and ``Gen``.  ``Gen`` groups a
  bond's columns by quantum number in order of first appearance, and within a
  group the later column goes first.  The tensors are
  ``W(lvb IN, pb_in IN, pb_out OUT, rvb OUT)``.

The delinearisation works on per-row / per-column dictionaries of the
non-null elements, so its cost follows the number of non-null elements.  A
dense scan would be quadratic in the bond dimension per overlap.

Two constants come from TensorToolkit (``qlten``), which is absent here:
``kDoubleEpsilon`` (taken as 1e-15), and the storage order behind
``GetFirstNonZeroElement``.  For the latter this module scans blocks in
lexicographic sector order, each block row-major.  That is the block-sparse
layout the rest of this package uses.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .tensor_data import IN, OUT, BlockTensorData, Index, qn_sub

K_DOUBLE_EPSILON = 1e-15
ID_COEF_LABEL = 0
ID_OP_LABEL = 0
READY = 0
FINAL = -1


# ---------------------------------------------------------------------------
# Symbolic algebra
# ---------------------------------------------------------------------------


class Coef:
    """A sum of c-number labels (``CoefRepr``); equality is up to order."""

    __slots__ = ("labels", "key")

    def __init__(self, labels=()):
        if isinstance(labels, (int, np.integer)):
            labels = (int(labels),)
        self.labels = tuple(int(v) for v in labels)
        self.key = tuple(sorted(self.labels))

    def __eq__(self, other):
        return isinstance(other, Coef) and self.key == other.key

    def __ne__(self, other):
        return not self == other

    def __hash__(self):
        return hash(self.key)

    def __add__(self, other):
        return Coef(self.labels + other.labels)

    def is_null(self):
        return not self.labels

    def realize(self, label_coef):
        c = 0
        for lab in self.labels:
            c = c + label_coef[lab]
        return c

    def __repr__(self):
        return f"Coef{self.labels}"


NULL_COEF = Coef(())
ID_COEF = Coef((ID_COEF_LABEL,))


class Op:
    """Basis-operator label -> coefficient (``OpRepr``), kept in label order."""

    __slots__ = ("terms", "_key")

    def __init__(self, terms: Optional[Dict[int, Coef]] = None):
        self.terms = dict(sorted(terms.items())) if terms else {}
        self._key = None

    @staticmethod
    def of(op_label, coef: Coef = ID_COEF) -> "Op":
        return Op({int(op_label): coef})

    @staticmethod
    def sum_of(coefs: Sequence[Coef], op_labels: Sequence[int]) -> "Op":
        """``OpRepr(coef_reprs, op_labels)``: repeated labels add their coefficients."""
        t: Dict[int, Coef] = {}
        for c, lab in zip(coefs, op_labels):
            t[int(lab)] = t[int(lab)] + c if int(lab) in t else c
        return Op(t)

    @property
    def key(self):
        if self._key is None:
            self._key = tuple((lab, c.key) for lab, c in self.terms.items())
        return self._key

    def __eq__(self, other):
        return isinstance(other, Op) and self.key == other.key

    def __ne__(self, other):
        return not self == other

    def __hash__(self):
        return hash(self.key)

    def is_null(self):
        return not self.terms

    def __add__(self, other: "Op") -> "Op":
        t = dict(self.terms)
        for lab, c in other.terms.items():
            t[lab] = t[lab] + c if lab in t else c
        return Op(t)

    def op_labels(self):
        return list(self.terms)

    def with_coef(self, coef: Coef) -> "Op":
        return Op({lab: coef for lab in self.terms})

    def realize(self, label_coef, label_op):
        out = None
        for lab, c in self.terms.items():
            term = c.realize(label_coef) * label_op[lab]
            out = term if out is None else out + term
        return out

    def __repr__(self):
        return "Op(" + " + ".join(f"{c.labels}*{lab}" for lab, c in self.terms.items()) + ")"


NULL_OP = Op()
ID_OP = Op.of(ID_OP_LABEL)


def separate(op: Op) -> Tuple[Coef, Op]:
    """``SeparateCoefAndBase`` (coef_op_alg.h:375-399): a coefficient common to
    every term and the operator with identity coefficients; (Id, op) when the
    terms' coefficients differ."""
    n = len(op.terms)
    if n == 0:
        return NULL_COEF, NULL_OP
    if n == 1:
        lab, c = next(iter(op.terms.items()))
        return c, Op.of(lab)
    cs = list(op.terms.values())
    if any(c != cs[0] for c in cs[1:]):
        return ID_COEF, op
    return cs[0], op.with_coef(ID_COEF)


def coef_of(op: Op) -> Coef:
    return separate(op)[0]


def incomplete_mul(coef: Coef, op: Op) -> Op:
    """``CoefReprOpReprIncompleteMulti`` (coef_op_alg.h:650-668): every term of
    op takes the coefficient coef (op's own coefficients are identities)."""
    if op.is_null():
        return NULL_OP
    if coef == ID_COEF:
        return op
    return op.with_coef(coef)


# ---------------------------------------------------------------------------
# Sparse matrices of symbols (dense storage, None = null element)
# ---------------------------------------------------------------------------


class SparMat:
    """Row-major matrix of ``Op`` or ``Coef`` elements; ``None`` is the null
    element and setting a null value leaves a cell unchanged, as
    ``SparMat::SetElem`` (sparse_mat.h:67-77) does."""

    def __init__(self, rows: int, cols: int):
        self.rows, self.cols = rows, cols
        self.cells = [[None] * cols for _ in range(rows)]

    @staticmethod
    def _null(v):
        return v is None or v.is_null()

    def __call__(self, x, y):
        return self.cells[x][y]

    def set(self, x, y, v):
        if self._null(v):
            return
        self.cells[x][y] = v

    def row(self, x):
        return list(self.cells[x])

    def col(self, y):
        return [r[y] for r in self.cells]

    def nnz(self):
        return sum(v is not None for r in self.cells for v in r)

    def __eq__(self, other):
        if self.rows != other.rows or self.cols != other.cols:
            return False
        for a, b in zip(self.cells, other.cells):
            for u, v in zip(a, b):
                if (u is None) != (v is None) or (u is not None and u != v):
                    return False
        return True

    def copy(self):
        m = SparMat(self.rows, self.cols)
        m.cells = [list(r) for r in self.cells]
        return m

    def remove_row(self, x):
        if self.rows == 1:
            self.rows, self.cols, self.cells = 0, 0, []
            return
        del self.cells[x]
        self.rows -= 1

    def remove_col(self, y):
        if self.cols == 1:
            self.rows, self.cols, self.cells = 0, 0, []
            return
        for r in self.cells:
            del r[y]
        self.cols -= 1

    def transpose_rows(self, order):
        """new row i = old row order[i] (sparse_mat.h:171-183)"""
        if len(order) != self.rows:
            raise ValueError("row order does not cover the matrix")
        self.cells = [self.cells[o] for o in order]

    def transpose_cols(self, order):
        if len(order) != self.cols:
            raise ValueError("column order does not cover the matrix")
        self.cells = [[r[o] for o in order] for r in self.cells]

    # ---- SparOpReprMat (coef_op_alg.h:423-645) ----

    def sort_rows(self):
        """Rows by ascending number of non-null elements, ties by index."""
        order = sorted(range(self.rows), key=lambda x: (sum(v is not None for v in self.cells[x]), x))
        self.transpose_rows(order)
        return order

    def sort_cols(self):
        order = sorted(range(self.cols),
                       key=lambda y: (sum(r[y] is not None for r in self.cells), y))
        self.transpose_cols(order)
        return order

    @staticmethod
    def _common_coef(elems):
        """``TryCatchRow/ColCommonDivisorCoef``: the coefficient shared by every
        non-null element, Id when they differ, null when there is none."""
        res = NULL_COEF
        first = True
        for v in elems:
            if v is None:
                continue
            c = coef_of(v)
            if first:
                res, first = c, False
            elif c != res:
                return ID_COEF
        return res

    def row_common_coef(self, x):
        return self._common_coef(self.cells[x])

    def col_common_coef(self, y):
        return self._common_coef(r[y] for r in self.cells)

    def remove_row_coef(self, x):
        r = self.cells[x]
        for y, v in enumerate(r):
            if v is not None:
                r[y] = separate(v)[1]

    def remove_col_coef(self, y):
        for r in self.cells:
            if r[y] is not None:
                r[y] = separate(r[y])[1]

    def print(self):
        for r in self.cells:
            print("\t".join("0" if v is None else repr(v) for v in r))


def coef_op_mul(coef_mat: SparMat, op_mat: SparMat) -> SparMat:
    """``SparCoefReprMatSparOpReprMatIncompleteMulti`` (coef_op_alg.h:670-744):
    res(x, y) = sum_i coef(x, i) * op(i, y), terms added in ascending i."""
    if coef_mat.cols != op_mat.rows:
        raise ValueError("shape mismatch")
    res = SparMat(coef_mat.rows, op_mat.cols)
    for x in range(coef_mat.rows):
        crow = [(i, c) for i, c in enumerate(coef_mat.cells[x]) if c is not None]
        for y in range(op_mat.cols):
            acc = NULL_OP
            for i, c in crow:
                o = op_mat.cells[i][y]
                if o is not None:
                    acc = acc + incomplete_mul(c, o)
            res.set(x, y, acc)
    return res


def op_coef_mul(op_mat: SparMat, coef_mat: SparMat) -> SparMat:
    """``SparOpReprMatSparCoefReprMatIncompleteMulti``: res(x, y) = sum_i
    coef(i, y) * op(x, i), ascending i."""
    if op_mat.cols != coef_mat.rows:
        raise ValueError("shape mismatch")
    res = SparMat(op_mat.rows, coef_mat.cols)
    ccols = [[(i, coef_mat.cells[i][y]) for i in range(coef_mat.rows)
              if coef_mat.cells[i][y] is not None] for y in range(coef_mat.cols)]
    for x in range(op_mat.rows):
        orow = op_mat.cells[x]
        for y in range(coef_mat.cols):
            acc = NULL_OP
            for i, c in ccols[y]:
                o = orow[i]
                if o is not None:
                    acc = acc + incomplete_mul(c, o)
            res.set(x, y, acc)
    return res


# ---- linear dependence of rows / columns (dictionaries of non-null elements) ----


def _overlap(vec: Dict[int, Op], base: Dict[int, Op]) -> Coef:
    """``CalcRowOverlap_`` / ``CalcColOverlap_`` (coef_op_alg.h:586-642): the
    coefficient c with vec = c * base on every non-null element of base (the
    scan runs over base's positions in ascending order); null when none."""
    first = None
    for p in sorted(base):
        b = base[p]
        t = vec.get(p)
        if t is None:
            t = NULL_OP
        if t == b:
            c = ID_COEF
        else:
            tc, tb = separate(t)
            if tb != b:
                return NULL_COEF
            c = tc
        if first is None:
            first = c
        elif c != first:
            return NULL_COEF
    return NULL_COEF if first is None else first


def _lin_cmb(vecs: List[Dict[int, Op]], cmb: List[Coef]) -> Dict[int, Op]:
    """``CalcSparOpReprMatRow/ColLinCmb`` (coef_op_alg.h:752-815)."""
    res: Dict[int, Op] = {}
    for i, c in enumerate(cmb):
        if c.is_null():
            continue
        for p, e in vecs[i].items():
            e2 = e if c == ID_COEF else e.with_coef(c)
            res[p] = res[p] + e2 if p in res else e2
    return res


def _same(a: Dict[int, Op], b: Dict[int, Op]) -> bool:
    return a.keys() == b.keys() and all(a[k] == b[k] for k in a)


def _rows_of(m: SparMat):
    return [{y: v for y, v in enumerate(r) if v is not None} for r in m.cells]


def _cols_of(m: SparMat):
    return [{x: m.cells[x][y] for x in range(m.rows) if m.cells[x][y] is not None}
            for y in range(m.cols)]


def row_delinearize(target: SparMat, follower: SparMat) -> None:
    """``SparOpReprMatRowDelinearize`` (coef_op_alg.h:817-849): a row equal to
    a combination of earlier rows is removed and the follower's columns take
    the combination (trans(orig row, kept row))."""
    rows = _rows_of(target)
    n0 = len(rows)
    trans = SparMat(n0, n0)
    trans.set(0, 0, ID_COEF)
    deleted = 0
    i = 1
    while i < len(rows):
        row = rows[i]
        cmb = None
        for x in range(i):  # CalcRowLinCmb: an identical earlier row first
            if _same(row, rows[x]):
                cmb = [NULL_COEF] * i
                cmb[x] = ID_COEF
                break
        if cmb is None:
            cmb = [_overlap(row, rows[x]) for x in range(i)]
        if _same(_lin_cmb(rows, cmb), row):
            del rows[i]
            trans.remove_col(trans.cols - 1)
            for j in range(i):
                trans.set(i + deleted, j, cmb[j])
            deleted += 1
        else:
            trans.set(i + deleted, i, ID_COEF)
            i += 1
    if deleted:
        _rebuild_rows(target, rows)
    if trans.cols < trans.rows:
        new = op_coef_mul(follower, trans)
        follower.rows, follower.cols, follower.cells = new.rows, new.cols, new.cells


def col_delinearize(target: SparMat, follower: SparMat) -> None:
    """``SparOpReprMatColDelinearize`` (coef_op_alg.h:854-883)."""
    cols = _cols_of(target)
    n0 = len(cols)
    trans = SparMat(n0, n0)
    trans.set(0, 0, ID_COEF)
    deleted = 0
    i = 1
    while i < len(cols):
        col = cols[i]
        cmb = [_overlap(col, cols[y]) for y in range(i)]
        if _same(_lin_cmb(cols, cmb), col):
            del cols[i]
            trans.remove_row(trans.rows - 1)
            for j in range(i):
                trans.set(j, i + deleted, cmb[j])
            deleted += 1
        else:
            trans.set(i, i + deleted, ID_COEF)
            i += 1
    if deleted:
        _rebuild_cols(target, cols)
    if trans.rows < trans.cols:
        new = coef_op_mul(trans, follower)
        follower.rows, follower.cols, follower.cells = new.rows, new.cols, new.cells


def _rebuild_rows(m: SparMat, rows):
    m.rows = len(rows)
    m.cells = [[r.get(y) for y in range(m.cols)] for r in rows]


def _rebuild_cols(m: SparMat, cols):
    m.cols = len(cols)
    m.cells = [[c.get(x) for c in cols] for x in range(m.rows)]


def row_compress(target: SparMat, follower: SparMat) -> None:
    """``SparOpReprMatRowCompresser`` (coef_op_alg.h:886-914)."""
    n = target.rows
    if n == 1:
        return
    order = target.sort_rows()
    follower.transpose_cols(order)
    need = False
    coefs = SparMat(n, n)
    for x in range(n):
        c = target.row_common_coef(x)
        coefs.set(x, x, c if not c.is_null() else ID_COEF)
        if not c.is_null() and c != ID_COEF:
            need = True
            target.remove_row_coef(x)
    if need:
        new = op_coef_mul(follower, coefs)
        follower.rows, follower.cols, follower.cells = new.rows, new.cols, new.cells
    row_delinearize(target, follower)


def col_compress(target: SparMat, follower: SparMat) -> None:
    """``SparOpReprMatColCompresser`` (coef_op_alg.h:924-953)."""
    n = target.cols
    if n == 1:
        return
    order = target.sort_cols()
    follower.transpose_rows(order)
    need = False
    coefs = SparMat(n, n)
    for y in range(n):
        c = target.col_common_coef(y)
        coefs.set(y, y, c if not c.is_null() else ID_COEF)
        if not c.is_null() and c != ID_COEF:
            need = True
            target.remove_col_coef(y)
    if need:
        new = coef_op_mul(coefs, follower)
        follower.rows, follower.cols, follower.cells = new.rows, new.cols, new.cells
    col_delinearize(target, follower)


# ---------------------------------------------------------------------------
# Finite-state machine (fsm.h)
# ---------------------------------------------------------------------------


class FSM:
    """Paths of terms through ready (0) / middle (1, 2, ...) / final (-1)
    states on the N + 1 bonds (``FSM``, fsm.h:116-281)."""

    def __init__(self, n_sites: int, id_ops: Optional[Sequence[Op]] = None):
        self.N = n_sites
        self.mid = [0] * (n_sites + 1)
        self.has_ready = [False] * (n_sites + 1)
        self.has_final = [False] * (n_sites + 1)
        self.paths: List[Tuple[List[int], List[Op]]] = []
        self.id_ops = list(id_ops) if id_ops is not None else [ID_OP] * n_sites
        if len(self.id_ops) != n_sites:
            raise ValueError("one identity per site")

    def add_path(self, head: int, tail: int, ntrvl_ops: Sequence[Op]) -> None:
        """``FSM::AddPath`` (fsm.h:183-219)."""
        if head + len(ntrvl_ops) != tail + 1:
            raise ValueError("operators must cover head..tail")
        ops = [self.id_ops[i] if (i < head or i > tail) else ntrvl_ops[i - head]
               for i in range(self.N)]
        stats = [READY] * (self.N + 1)
        self.has_ready[0] = True
        for i in range(self.N):
            t = i + 1
            if i < head:
                stats[t] = READY
                self.has_ready[t] = True
            elif i >= tail:
                stats[t] = FINAL
                self.has_final[t] = True
            else:
                self.mid[t] += 1
                stats[t] = self.mid[t]
        self.paths.append((stats, ops))

    def _dims(self):
        return [self.mid[i] + int(self.has_ready[i]) + int(self.has_final[i])
                for i in range(self.N + 1)]

    def gen_mat_repr(self) -> List[SparMat]:
        """``FSM::GenMatRepr`` (fsm.h:221-276)."""
        dims = self._dims()
        final_idx = [-1] * (self.N + 1)
        for i in range(self.N + 1):
            if self.has_final[i]:
                final_idx[i] = dims[i] - 1 if self.has_ready[i] else 0
        mats = [SparMat(dims[i], dims[i + 1]) for i in range(self.N)]

        def place(i, stat):
            if stat == FINAL:
                return final_idx[i]
            if not self.has_ready[i] and not self.has_final[i]:
                return stat - 1
            return stat

        for stats, ops in self.paths:
            for i in range(self.N):
                r, c = place(i, stats[i]), place(i + 1, stats[i + 1])
                cur = mats[i](r, c)
                if cur is None:
                    mats[i].set(r, c, ops[i])
                elif cur != ops[i]:
                    mats[i].set(r, c, cur + ops[i])
        return mats

    def gen_compressed_mat_repr(self) -> List[SparMat]:
        """``FSM::GenCompressedMatRepr`` (fsm.h:278-295): columns left to
        right, then rows right to left."""
        mats = self.gen_mat_repr()
        for i in range(self.N - 1):
            col_compress(mats[i], mats[i + 1])
        for i in range(self.N - 1, 0, -1):
            row_compress(mats[i], mats[i - 1])
        return mats


class LabelConvertor:
    """Objects -> labels by first appearance (``LabelConvertor``, fsm.h:297-340)."""

    def __init__(self, first=None, eq=None):
        self.hub = [] if first is None else [first]
        self.eq = eq or (lambda a, b: a == b)

    def convert(self, obj) -> int:
        for i, h in enumerate(self.hub):
            if self.eq(h, obj):
                return i
        self.hub.append(obj)
        return len(self.hub) - 1


# ---------------------------------------------------------------------------
# Generator (mpogen_impl.h)
# ---------------------------------------------------------------------------


def first_nonzero(mat: np.ndarray, pb_out: Index):
    """First non-zero element of the operator tensor {pb_in, pb_out} in block
    storage order: blocks in lexicographic (in sector, out sector) order, each
    row-major."""
    off = pb_out.offsets()
    for si in range(pb_out.nsec):
        for so in range(pb_out.nsec):
            blk = mat[off[si]:off[si + 1], off[so]:off[so + 1]]
            nz = np.flatnonzero(blk)
            if len(nz):
                return blk.flat[nz[0]]
    return 0


def op_div(mat: np.ndarray, pb_out: Index):
    """Div of the operator tensor {pb_in IN, pb_out OUT}: qn(out) - qn(in)."""
    divs = set()
    for i, o in np.argwhere(mat != 0):
        si, _ = pb_out.sector_of(int(i))
        so, _ = pb_out.sector_of(int(o))
        divs.add(qn_sub(pb_out.qns[so], pb_out.qns[si]))
    if len(divs) != 1:
        raise ValueError("operator has no definite divergence")
    return divs.pop()


class MPOGenerator:
    """``MPOGenerator`` (mpogen.h:38-127, mpogen_impl.h).

    sites: the physical index (OUT) of each site.  Operators are dense
    matrices ``O[in, out]`` (``models.Operator`` or plain arrays) in the
    layout of ``QLTensor({pb_in, pb_out})``.
    """

    def __init__(self, sites: Sequence[Index], id_ops=None, zero_div=None, dtype=np.float64):
        self.sites = list(sites)
        self.N = len(self.sites)
        self.dtype = dtype
        self.zero = tuple(zero_div) if zero_div is not None else \
            tuple(0 for _ in range(self.sites[0].nq))
        if id_ops is None:
            id_ops = [np.eye(s.dim, dtype=dtype) for s in self.sites]
        self.id_mats = [self._mat(o) for o in id_ops]
        self.coef_labels = LabelConvertor(dtype(1))
        self.op_labels = LabelConvertor(eq=lambda a, b: a.shape == b.shape and np.array_equal(a, b))
        ids = [Op.of(self.op_labels.convert(m)) for m in self.id_mats]
        self.fsm = FSM(self.N, ids)
        self.bond_dims: Optional[List[int]] = None  # right-bond dimensions, set by gen()

    def _mat(self, op):
        m = op.mat if hasattr(op, "mat") else op
        return np.asarray(m, dtype=self.dtype)

    def add_term(self, coef, local_ops: Sequence, local_idxs: Sequence[int]) -> None:
        """The generic ``AddTerm(coef, local_ops, local_ops_idxs)``
        (mpogen_impl.h:92-166)."""
        if len(local_ops) != len(local_idxs):
            raise ValueError("one site per operator")
        if coef == 0:
            return
        if abs(coef) < K_DOUBLE_EPSILON:
            return
        mats = [self._mat(o) for o in local_ops]
        idxs = [int(i) for i in local_idxs]
        if idxs != sorted(idxs):
            order = sorted(range(len(idxs)), key=lambda k: idxs[k])
            mats = [mats[k] for k in order]
            idxs = [idxs[k] for k in order]
        if idxs[-1] >= self.N:
            raise ValueError("site out of range")
        coef = self.dtype(coef)
        for k in range(len(mats)):  # the sign of the first non-zero element goes to coef
            if np.real(first_nonzero(mats[k], self.sites[idxs[k]])) < 0.0:
                coef = -coef
                mats[k] = -mats[k]
        coef_label = self.coef_labels.convert(coef)
        head, tail = idxs[0], idxs[-1]
        ops = []
        for i in range(head, tail + 1):
            if i in idxs:
                loc = idxs.index(i)
                lab = self.op_labels.convert(mats[loc])
                ops.append(Op.of(lab, Coef(coef_label)) if loc == 0 else Op.of(lab))
            else:
                ops.append(Op.of(self.op_labels.convert(self.id_mats[i])))
        self.fsm.add_path(head, tail, ops)

    def add_term_insert(self, coef, phys_ops: Sequence, phys_idxs: Sequence[int],
                        inst_ops: Sequence, inst_idxs_set=None) -> None:
        """``AddTerm(coef, phys_ops, phys_ops_idxs, inst_ops, inst_ops_idxs_set)``
        (mpogen_impl.h:187-234): insertion operators between the physical ones
        (every site in between, or the listed sites), and after the last one
        as a tail string when there are as many insertion as physical
        operators."""
        if len(phys_ops) < 2 or len(phys_ops) != len(phys_idxs):
            raise ValueError("at least two physical operators, one site each")
        if len(inst_ops) not in (len(phys_ops) - 1, len(phys_ops)):
            raise ValueError("one insertion operator per gap (and optionally a tail)")
        ops, idxs = [], []
        for k in range(len(phys_ops) - 1):
            ops.append(phys_ops[k])
            idxs.append(phys_idxs[k])
            sites = range(phys_idxs[k] + 1, phys_idxs[k + 1]) if inst_idxs_set is None \
                else inst_idxs_set[k]
            for j in sites:
                ops.append(inst_ops[k])
                idxs.append(j)
        ops.append(phys_ops[-1])
        idxs.append(phys_idxs[-1])
        if len(inst_ops) == len(phys_ops):
            sites = range(phys_idxs[-1], self.N) if inst_idxs_set is None else inst_idxs_set[-1]
            for j in sites:
                ops.append(inst_ops[-1])
                idxs.append(j)
        self.add_term(coef, ops, idxs)

    def add_two_body(self, coef, op1, i1: int, op2=None, i2: Optional[int] = None,
                     inst=None, inst_idxs=None) -> None:
        """``AddTerm(coef, op1, op1_idx, op2, op2_idx, inst_op, inst_op_idxs)``
        (mpogen_impl.h:250-283): one-body when op2 is None."""
        if op2 is None:
            self.add_term(coef, [op1], [i1])
        elif inst is None:
            self.add_term(coef, [op1, op2], [i1, i2])
        elif inst_idxs is None:
            if not i1 < i2:
                raise ValueError("uniform insertion needs op1 before op2")
            self.add_term_insert(coef, [op1, op2], [i1, i2], [inst])
        else:
            self.add_term_insert(coef, [op1, op2], [i1, i2], [inst], [list(inst_idxs)])

    # ---- tensors ----

    def mat_repr(self, compress: bool = True) -> List[SparMat]:
        return self.fsm.gen_compressed_mat_repr() if compress else self.fsm.gen_mat_repr()

    @staticmethod
    def _sort_cols_by_qn(m: SparMat, lvb: Index, pb_out: Index,
                         label_op) -> Tuple[List[int], Index]:
        """``SortSparOpReprMatColsByQN_`` (mpogen_impl.h:383-429): right-bond
        quantum number of each column from its first non-null element
        (qn(left row) - Div(first basis operator)); groups in order of first
        appearance, a later column inserted at the start of its group."""
        groups: List[List] = []  # [qn, count]
        order: List[int] = []
        for y in range(m.cols):
            col_qn = None
            for x in range(m.rows):
                e = m(x, y)
                if e is None:
                    continue
                q = qn_sub(lvb.qns[lvb.sector_of(x)[0]], op_div(label_op[e.op_labels()[0]], pb_out))
                if col_qn is None:
                    col_qn = q
                    offset = 0
                    for g in groups:
                        if g[0] == q:
                            g[1] += 1
                            order.insert(offset, y)
                            break
                        offset += g[1]
                    else:
                        groups.append([q, 1])
                        order.insert(offset, y)
                elif q != col_qn:
                    raise ValueError("column mixes right-bond quantum numbers")
            if col_qn is None:
                raise ValueError("empty column in an MPO matrix")
        m.transpose_cols(order)
        return order, Index.make([(g[0], g[1]) for g in groups], OUT)

    def gen(self, compress: bool = True) -> List[BlockTensorData]:
        """``Gen`` (mpogen_impl.h:285-322): the MPO tensors.  The columns of
        site i are sorted by right-bond quantum number and the rows of site
        i + 1 follow the same order."""
        mats = self.mat_repr(compress)
        self.bond_dims = [m.cols for m in mats]
        label_coef = self.coef_labels.hub
        label_op = self.op_labels.hub
        triv_in = Index.make([(self.zero, 1)], IN)
        triv_out = Index.make([(self.zero, 1)], OUT)
        mpo = []
        order, rvb = None, None
        for i in range(self.N):
            pb_out = self.sites[i]
            m = mats[i]
            if i == 0:
                lvb = triv_in
                order, rvb = self._sort_cols_by_qn(m, lvb, pb_out, label_op)
            else:
                m.transpose_rows(order)
                lvb = rvb.inverse()
                if i == self.N - 1:
                    rvb = triv_out
                else:
                    order, rvb = self._sort_cols_by_qn(m, lvb, pb_out, label_op)
            W = BlockTensorData([lvb, pb_out.inverse(), pb_out, rvb], {}, self.dtype)
            for x in range(m.rows):
                for y in range(m.cols):
                    e = m(x, y)
                    if e is None:
                        continue
                    op = e.realize(label_coef, label_op)
                    for a, o in np.argwhere(op != 0):
                        W.set_elem((x, int(a), int(o), y), op[a, o])
            mpo.append(W)
        return mpo
