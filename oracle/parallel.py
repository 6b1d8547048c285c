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

Workers are forked once the problem is built, so they share it
copy-on-write.  Fork only from a process that has not initialised CUDA, and
load numpy with single-threaded BLAS (``OPENBLAS_NUM_THREADS=1``), so that N
workers use N cores.  Tasks are handed out heaviest sector first
(dynamic scheduling).
"""
from __future__ import annotations

import multiprocessing as mp
import time
from typing import Dict, Optional, Sequence, Tuple

_EFF = None
_PSI = None


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
