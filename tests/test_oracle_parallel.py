"""The sector-parallel oracle matvec (``oracle.parallel``, the timed CPU
baseline) against the serial oracle matvec: the same blocks, bit for bit
(each output block is computed by one task with the same arithmetic)."""
import numpy as np
import pytest

from oracle import krylov
from oracle.parallel import ParallelMatvec
from systems import hubbard_system, two_site_problem


@pytest.mark.parametrize("workers", [1, 3])
def test_parallel_matvec_equals_serial(workers):
    mpo, mps = hubbard_system(Lx=3, Ly=2, D=40, seed=1)
    eff, psi = two_site_problem(mpo, mps, 2)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    pm = ParallelMatvec(eff, psi, workers)
    try:
        flops, blocks, _ = pm.run()
        assert flops > 0
        assert set(blocks) == set(ref.blocks)
        for k, v in ref.blocks.items():
            assert np.array_equal(blocks[k], v)
        # a subset of bra sectors gives exactly those sectors' output blocks
        part = pm.sectors[: max(1, len(pm.sectors) // 2)]
        _, sub, _ = pm.run(part)
        assert set(sub) == {k for k in ref.blocks if k[0] in set(part)}
    finally:
        pm.close()


def test_spawned_matvec_equals_serial(tmp_path):
    from oracle.parallel import SpawnedMatvec
    mpo, mps = hubbard_system(Lx=3, Ly=2, D=40, seed=1)
    eff, psi = two_site_problem(mpo, mps, 2)
    ref = krylov.eff_ham_mul_two_site_state(eff, psi)
    sm = SpawnedMatvec(eff, 2, str(tmp_path))
    try:
        for _ in range(2):  # a second call reads a fresh state file
            out = sm(eff, psi)
            assert set(out.blocks) == set(ref.blocks)
            for k, v in ref.blocks.items():
                assert np.array_equal(out.blocks[k], v)
        # it drives the oracle's Lanczos like the serial matvec (block order,
        # hence the summation order of the vector operations, may differ)
        p = krylov.LanczosParams(1e-12, 60)
        a = krylov.lanczos_solver(eff, psi.copy(), krylov.eff_ham_mul_two_site_state, p)
        b = krylov.lanczos_solver(eff, psi.copy(), sm, p)
        assert abs(a.gs_eng - b.gs_eng) <= 1e-10 * abs(a.gs_eng)
    finally:
        sm.close()
