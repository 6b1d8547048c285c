"""The TDVP oracle pinned on the CPU by the reference's free-fermion test
(tests/test_algorithm/test_two_site_finite_tdvp.cc:103-150): the ground-state
energy of the N=6 open chain to 1e-12 and the single-particle Green's
function after a c^dag insertion at the centre against its closed form
(1e-10) over the first steps of dt = 0.01."""
import numpy as np

from oracle import tdvp as otdvp
from oracle import vmps as ovmps
from oracle.krylov import LanczosParams
from systems import act_operator, apply_dense, free_fermion_green, mps_dense, op_tensor
from ultradmrg_gb300 import models as M

GOLD_E0 = -3.4939592074349334893668128643185  # test_two_site_finite_tdvp.cc:125


def ground_state(N=6):
    mpo, pb, ops = M.free_fermion_chain_mpo(N, dtype=np.complex128)
    mps = M.direct_product_mps([pb] * N, [i % 2 for i in range(N)], dtype=np.complex128)
    p = ovmps.FiniteVMPSSweepParams(8, 1, 16, 1e-12, LanczosParams(1e-13, 200))
    e0 = ovmps.two_site_finite_vmps(mps, mpo, p)
    return e0, mps, mpo, pb, ops


def test_oracle_free_fermion_dynamics():
    N, site0, dt, steps = 6, 3, 0.01, 5
    e0, gs, mpo, pb, ops = ground_state(N)
    assert abs(e0 - GOLD_E0) <= 1e-12
    gs_v = mps_dense(gs)
    cdag, f, c = (op_tensor(ops[k], pb) for k in ("cdag", "f", "c"))
    psi = act_operator(gs, cdag, f, site0)
    p = otdvp.TDVPParams(dt, 10, 16, 1e-10, LanczosParams(1e-12, 40))
    for step in range(1, steps + 1):
        psi = otdvp.two_site_finite_tdvp(psi, mpo, p, 1)
        v = mps_dense(psi)
        t = step * dt
        for x2 in range(N):
            g = np.vdot(gs_v, apply_dense(v, ops["c"].mat, x2, ops["f"].mat))
            g *= np.exp(1j * e0 * t)
            assert abs(g - free_fermion_green(t, N, site0, x2)) <= 1e-10, (step, x2)
