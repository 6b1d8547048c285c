"""Host-side block-sparse tensor container (data only, no arithmetic).

This is the interchange format between the model builders, the C-ABI
(upload/download of block data) and the test oracle.  It restates the
``QLTensor<Elem, QN>`` storage model that qlmps relies on (the tensor type
itself lives in QuantumLiquids/TensorToolkit, which is not vendored):

* an ``Index`` is an ordered list of quantum-number sectors ``(qn, dim)`` plus a
  direction, OUT (+1) or IN (-1)
  (``tests/test_algorithm/test_two_site_update_finite_vmps.cc:64-69``:
  ``IndexT({QNSctT(qn, 1), ...}, TenIndexDirType::OUT)``; ``InverseIndex``
  flips the direction);
* a tensor stores dense blocks keyed by one sector id per index; a block may
  exist only if ``sum_i dir_i * qn(sector_i) == div`` (the divergence), with
  OUT counting +1 and IN -1.  This sign convention is the one under which the
  reference's MPS / MPO constructors come out divergence-free
  (``one_dim_tn/mps/finite_mps/finite_mps_init.h:213-266`` and
  ``one_dim_tn/mpo/mpogen/mpogen_impl.h:373-381``);
* blocks are created only where data is written (sparse beyond the symmetry
  constraint), exactly like the element-setting code in the reference tests.

Quantum numbers are tuples of ints: ``(Sz,)`` for U(1), ``(N, Sz)`` or
``(Nup, Ndn)`` for U(1)xU(1).  Block data are C-ordered (row-major) numpy arrays
whose shape is the tuple of sector dimensions.  Blocks are always enumerated in
lexicographic order of their sector-id tuples; that order defines the packed
buffer layout used on the device.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

import numpy as np

OUT = 1
IN = -1

QN = Tuple[int, ...]


def qn_add(a: QN, b: QN) -> QN:
    return tuple(x + y for x, y in zip(a, b))


def qn_sub(a: QN, b: QN) -> QN:
    return tuple(x - y for x, y in zip(a, b))


def qn_scale(a: QN, s: int) -> QN:
    return tuple(s * x for x in a)


@dataclass(frozen=True)
class Index:
    """Ordered QN sectors plus direction (OUT=+1, IN=-1)."""

    qns: Tuple[QN, ...]
    dims: Tuple[int, ...]
    dir: int

    def __post_init__(self):
        if len(self.qns) != len(self.dims):
            raise ValueError("qns and dims differ in length")
        if self.dir not in (IN, OUT):
            raise ValueError("dir must be IN (-1) or OUT (+1)")

    @staticmethod
    def make(sectors: Sequence[Tuple[Sequence[int], int]], dir: int) -> "Index":
        return Index(tuple(tuple(int(v) for v in q) for q, _ in sectors),
                     tuple(int(d) for _, d in sectors), dir)

    @property
    def nsec(self) -> int:
        return len(self.qns)

    @property
    def dim(self) -> int:
        return int(sum(self.dims))

    @property
    def nq(self) -> int:
        return len(self.qns[0]) if self.qns else 0

    def inverse(self) -> "Index":
        return Index(self.qns, self.dims, -self.dir)

    def offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.dims)]).astype(np.int64)

    def sector_of(self, coor: int) -> Tuple[int, int]:
        """(sector id, position inside the sector) of an actual coordinate."""
        off = 0
        for s, d in enumerate(self.dims):
            if coor < off + d:
                return s, coor - off
            off += d
        raise IndexError(coor)

    def find_qn(self, qn: QN) -> int:
        for s, q in enumerate(self.qns):
            if q == qn:
                return s
        return -1


@dataclass
class BlockTensorData:
    """Block-sparse tensor: indexes + {sector-id tuple: dense C-ordered block}."""

    indexes: List[Index]
    blocks: Dict[Tuple[int, ...], np.ndarray] = field(default_factory=dict)
    dtype: type = np.float64

    @property
    def rank(self) -> int:
        return len(self.indexes)

    @property
    def nq(self) -> int:
        return self.indexes[0].nq

    def block_qn_sum(self, coords: Tuple[int, ...]) -> QN:
        acc = tuple(0 for _ in range(self.nq))
        for ind, s in zip(self.indexes, coords):
            acc = qn_add(acc, qn_scale(ind.qns[s], ind.dir))
        return acc

    def div(self) -> QN:
        keys = self.sorted_keys()
        if not keys:
            return tuple(0 for _ in range(self.nq))
        d = self.block_qn_sum(keys[0])
        for k in keys[1:]:
            if self.block_qn_sum(k) != d:
                raise ValueError("blocks with different divergences")
        return d

    def block_shape(self, coords: Tuple[int, ...]) -> Tuple[int, ...]:
        return tuple(ind.dims[s] for ind, s in zip(self.indexes, coords))

    def sorted_keys(self) -> List[Tuple[int, ...]]:
        return sorted(self.blocks.keys())

    def size(self) -> int:
        return int(sum(b.size for b in self.blocks.values()))

    def copy(self) -> "BlockTensorData":
        return BlockTensorData(list(self.indexes),
                               {k: v.copy() for k, v in self.blocks.items()},
                               self.dtype)

    # element access in actual (dense) coordinates, creating blocks on write
    def set_elem(self, coors: Sequence[int], value) -> None:
        key, inner = [], []
        for ind, c in zip(self.indexes, coors):
            s, p = ind.sector_of(int(c))
            key.append(s)
            inner.append(p)
        key = tuple(key)
        if key not in self.blocks:
            self.blocks[key] = np.zeros(self.block_shape(key), dtype=self.dtype)
        self.blocks[key][tuple(inner)] = value

    def get_elem(self, coors: Sequence[int]):
        key, inner = [], []
        for ind, c in zip(self.indexes, coors):
            s, p = ind.sector_of(int(c))
            key.append(s)
            inner.append(p)
        blk = self.blocks.get(tuple(key))
        return self.dtype(0) if blk is None else blk[tuple(inner)]

    def to_dense(self) -> np.ndarray:
        shape = tuple(ind.dim for ind in self.indexes)
        out = np.zeros(shape, dtype=self.dtype)
        offs = [ind.offsets() for ind in self.indexes]
        for key, blk in self.blocks.items():
            sl = tuple(slice(o[s], o[s] + d) for o, s, d in
                       zip(offs, key, blk.shape))
            out[sl] = blk
        return out

    def packed(self) -> np.ndarray:
        """All blocks concatenated in sorted-key order (the device layout)."""
        keys = self.sorted_keys()
        if not keys:
            return np.zeros(0, dtype=self.dtype)
        return np.concatenate([self.blocks[k].ravel() for k in keys]).astype(
            self.dtype, copy=False)

    def norm(self) -> float:
        return float(np.sqrt(sum(np.vdot(b, b).real for b in self.blocks.values())))


def from_packed(indexes: List[Index], keys: Sequence[Tuple[int, ...]],
                data: np.ndarray, dtype=np.float64) -> BlockTensorData:
    t = BlockTensorData(list(indexes), {}, dtype)
    off = 0
    for k in keys:
        shp = t.block_shape(tuple(k))
        n = int(np.prod(shp)) if shp else 1
        t.blocks[tuple(int(v) for v in k)] = np.array(
            data[off:off + n], dtype=dtype).reshape(shp)
        off += n
    return t
