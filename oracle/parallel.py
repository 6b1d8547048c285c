"""The oracle's two-site matvec spread over host processes.

Test and baseline infrastructure: this is the timed CPU baseline and the
checker's parallel form, never a product code path.

The left environment's bra sectors partition the matvec.  Restricting L to
some of its bra sectors restricts every later step (x W1, x W2, x R) to the
output blocks of those sectors.  So one task per bra sector does disjoint
work, and the union of the tasks' blocks is the whole H_eff * psi.  This is
how the reference's tensor library spreads a contraction over host threads:
block pairs on OpenMP threads, one BLAS call each
(``lanczos_vmps_solver_impl.h:273-287``).

``ParallelMatvec``: workers are forked once the problem is built, so they
share it copy-on-write.  Fork only from a process that has not initialised
CUDA, and load numpy with single-threaded BLAS (``OPENBLAS_NUM_THREADS=1``),
so that N workers use N cores.  Tasks are handed out heaviest sector first
(dynamic scheduling).

``SpawnedMatvec``: the same tasks on spawned workers, for a process that
already holds a CUDA context (a GPU test): the environments reach the workers
once through a file, each state vector through one file per matvec.  It is
called like the oracle's matvec, so it can drive the oracle's Lanczos.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import pickle
import time
from typing import Dict, Optional, Sequence, Tuple

_EFF = None
_PSI = None
_PSI_KEY = None

SERIAL_BLAS = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")


def _task(sectors: Sequence[int]):
    from oracle import blocksparse as bs
    from oracle import krylov
    L = _EFF[0]
    keep = set(sectors)
    Ls = bs.T(list(L.indexes), {k: v for k, v in L.blocks.items() if k[0] in keep}, L.dtype)
    bs.FLOPS[0] = 0.0
    out = krylov.eff_ham_mul_two_site_state([Ls] + list(_EFF[1:]), _PSI)
    return bs.FLOPS[0], out.blocks


class ParallelMatvec:
    """A pool of forked workers holding one (eff_ham, psi) problem."""

    def __init__(self, eff, psi, workers: int):
        global _EFF, _PSI
        _EFF, _PSI = list(eff), psi
        self.workers = max(1, int(workers))
        weight: Dict[int, int] = {}
        for k, v in eff[0].blocks.items():
            weight[k[0]] = weight.get(k[0], 0) + v.size
        self.sectors = sorted(weight, key=lambda s: (-weight[s], s))
        self.indexes = list(psi.indexes)
        self.dtype = psi.dtype
        self.pool = mp.get_context("fork").Pool(self.workers)

    def run(self, sectors: Optional[Sequence[int]] = None) -> Tuple[float, Dict, float]:
        """One matvec over the given bra sectors (all by default): (flops,
        output blocks, wall seconds)."""
        todo = [s for s in self.sectors if sectors is None or s in set(sectors)]
        t0 = time.perf_counter()
        flops, blocks = 0.0, {}
        for f, b in self.pool.imap_unordered(_task, [[s] for s in todo]):
            flops += f
            blocks.update(b)
        return flops, blocks, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def _load_eff(path):
    global _EFF
    with open(path, "rb") as f:
        _EFF = pickle.load(f)


def _task_file(args):
    global _PSI, _PSI_KEY
    path, key, sectors = args
    if _PSI_KEY != key:
        with open(path, "rb") as f:
            _PSI = pickle.load(f)
        _PSI_KEY = key
    return _task(sectors)[1]


def _sector_order(eff):
    weight: Dict[int, int] = {}
    for k, v in eff[0].blocks.items():
        weight[k[0]] = weight.get(k[0], 0) + v.size
    return sorted(weight, key=lambda s: (-weight[s], s))


class SpawnedMatvec:
    """``matvec(eff_ham, state)`` of the oracle over a spawned pool holding
    ``eff`` (its ``eff_ham`` argument is ignored: the pool's is used)."""

    def __init__(self, eff, workers: int, tmpdir: str):
        import numpy as np
        self.tmpdir = tmpdir
        self.dtype0 = eff[0].dtype
        self.sectors = _sector_order(eff)
        path = os.path.join(tmpdir, "oracle_eff.pkl")
        with open(path, "wb") as f:
            pickle.dump(list(eff), f, protocol=pickle.HIGHEST_PROTOCOL)
        saved = {k: os.environ.get(k) for k in SERIAL_BLAS}
        os.environ.update({k: "1" for k in SERIAL_BLAS})
        try:
            self.pool = mp.get_context("spawn").Pool(max(1, int(workers)), initializer=_load_eff,
                                                     initargs=(path,))
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        self.calls = 0
        self._np = np

    def __call__(self, eff_ham, state):
        from oracle import blocksparse as bs
        self.calls += 1
        path = os.path.join(self.tmpdir, f"oracle_psi{self.calls % 2}.pkl")
        with open(path, "wb") as f:
            pickle.dump(state, f, protocol=pickle.HIGHEST_PROTOCOL)
        blocks = {}
        for b in self.pool.imap_unordered(_task_file, [(path, self.calls, [s])
                                                       for s in self.sectors]):
            blocks.update(b)
        # blocks in key order: the result does not depend on task completion order
        return bs.T(list(state.indexes), {k: blocks[k] for k in sorted(blocks)},
                    self._np.result_type(self.dtype0, state.dtype))

    def close(self):
        self.pool.close()
        self.pool.join()
