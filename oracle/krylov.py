"""Krylov solvers and effective-Hamiltonian matvecs (oracle restatement).

* ``lanczos_solver``          <- ``algorithm/vmps/lanczos_vmps_solver_impl.h:114-248``
* ``eff_ham_mul_two_site_state`` <- ``lanczos_vmps_solver_impl.h:250-289``
* ``eff_ham_mul_single_site_state`` <- ``lanczos_vmps_solver_impl.h:291-304``
* ``tridiag_gs_solver``       <- ``lanczos_vmps_solver_impl.h:306-355`` (LAPACK ?stev)
* ``lanczos_expmv_solver``    <- ``algorithm/tdvp/lanczos_expmv_solver_impl.h:70-184``
* ``tridiag_expme1_solver``   <- ``lanczos_expmv_solver_impl.h:199-240``
* ``distance``                <- ``lanczos_expmv_solver_impl.h:253-269``
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg as sla

from . import blocksparse as bs


@dataclass
class LanczosParams:
    """``LanczosParams`` (``algorithm/lanczos_params.h:27-46``)."""

    error: float = 1.0e-7
    max_iterations: int = 200


@dataclass
class LanczosRes:
    iters: int
    gs_eng: float
    gs_vec: bs.T


def eff_ham_mul_two_site_state(eff_ham, state):
    """H_eff * psi with the four cyclic contractions of the reference."""
    L, W1, W2, R = eff_ham
    t1 = bs.contract(L, state, [2], [0])
    t2 = bs.contract_cyclic(t1, W1, 1, 0, 2)
    t3 = bs.contract_cyclic(t2, W2, 4, 0, 2)
    return bs.contract_cyclic(t3, R, 4, 1, 2)


def eff_ham_mul_single_site_state(eff_ham, state):
    L, W, R = eff_ham
    res = bs.contract(L, state, [2], [0])
    tmp = bs.contract_cyclic(res, W, 1, 0, 2)
    return bs.contract_cyclic(tmp, R, 3, 1, 2)


def tridiag_gs_solver(a, b, n, jobz):
    """Lowest eigenpair of the n x n tridiagonal (a, b) via LAPACK ?stev."""
    d = np.array(a[:n], dtype=np.float64)
    e = np.array(b[:n - 1], dtype=np.float64)
    if jobz == 'N':
        w = sla.eigh_tridiagonal(d, e, eigvals_only=True, lapack_driver='stev')
        return float(w[0]), None
    w, z = sla.eigh_tridiagonal(d, e, lapack_driver='stev')
    return float(w[0]), np.array(z[:, 0])


def lanczos_solver(eff_ham, init_state, matvec, params: LanczosParams) -> LanczosRes:
    """Ground state of H_eff by plain Lanczos (three-term recurrence, no
    reorthogonalisation, all bases kept)."""
    eff_dim = init_state.size()
    maxit = params.max_iterations
    bases = [None] * maxit
    a = np.zeros(maxit)
    b = np.zeros(maxit)
    N = np.zeros(maxit)
    bs.normalize(init_state)
    bases[0] = init_state
    last = matvec(eff_ham, bases[0])
    a[0] = np.real(bs.inner(bases[0], last))
    N[0] = 0.0
    m = 0
    energy0 = a[0]
    while True:
        m += 1
        gamma = last
        if m == 1:
            bs.linear_combine([-a[m - 1]], [bases[m - 1]], 1.0, gamma)
        else:
            bs.linear_combine([-a[m - 1], -np.sqrt(N[m - 1])],
                              [bases[m - 1], bases[m - 2]], 1.0, gamma)
        norm_gamma = bs.normalize(gamma)
        if norm_gamma == 0.0:
            if m == 1:
                return LanczosRes(m, energy0, bases[0].copy())
            eigval, eigvec = tridiag_gs_solver(a, b, m, 'V')
            gs = bs.T(list(bases[0].indexes), {}, bases[0].dtype)
            bs.linear_combine(list(eigvec), bases[:m], 0.0, gs)
            return LanczosRes(m, energy0, gs)
        N[m] = norm_gamma * norm_gamma
        b[m - 1] = norm_gamma
        bases[m] = gamma
        last = matvec(eff_ham, bases[m])
        a[m] = np.real(bs.inner(bases[m], last))
        eigval, _ = tridiag_gs_solver(a, b, m + 1, 'N')
        energy0_new = eigval
        if ((energy0 - energy0_new) < params.error or m == eff_dim
                or m == maxit - 1):
            eigval, eigvec = tridiag_gs_solver(a, b, m + 1, 'V')
            energy0 = energy0_new
            gs = bs.T(list(bases[0].indexes), {}, bases[0].dtype)
            bs.linear_combine(list(eigvec), bases[:m + 1], 0.0, gs)
            return LanczosRes(m + 1, energy0, gs)
        energy0 = energy0_new


def tridiag_expme1_solver(a, b, n, step_length):
    """exp(-i * step * A) e_1 for the n x n tridiagonal A = (a, b)."""
    d = np.array(a[:n], dtype=np.float64)
    e = np.array(b[:n - 1], dtype=np.float64)
    w, z = sla.eigh_tridiagonal(d, e, lapack_driver='stev')
    tmp = np.exp(-1j * step_length * w) * z[0, :]
    return z @ tmp


def distance(v1, v2):
    return float(np.linalg.norm(np.asarray(v2) - np.asarray(v1)))


@dataclass
class ExpmvRes:
    iters: int
    expmv: bs.T


def lanczos_expmv_solver(eff_ham, init_state, matvec, step_length,
                         params: LanczosParams) -> ExpmvRes:
    eff_dim = init_state.size()
    maxit = params.max_iterations
    bases = [None] * maxit
    a = np.zeros(maxit)
    b = np.zeros(maxit)
    initial_norm = bs.normalize(init_state)
    bases[0] = init_state
    last = matvec(eff_ham, bases[0])
    a[0] = np.real(bs.inner(bases[0], last))
    m = 0
    last_coef = np.zeros(maxit, dtype=np.complex128)
    while True:
        m += 1
        gamma = last
        if m == 1:
            bs.linear_combine([-a[m - 1]], [bases[m - 1]], 1.0, gamma)
        else:
            bs.linear_combine([-a[m - 1], -b[m - 2]], [bases[m - 1], bases[m - 2]],
                              1.0, gamma)
        norm_gamma = bs.normalize(gamma)
        if norm_gamma == 0.0:
            if m == 1:
                phase = np.exp(-1j * step_length * a[0])
                return ExpmvRes(m, bs.scale(bases[0], initial_norm * phase))
            coef = tridiag_expme1_solver(a, b, m, step_length) * initial_norm
            out = bs.T(list(bases[0].indexes), {}, np.complex128)
            bs.linear_combine(list(coef), bases[:m], 0.0, out)
            return ExpmvRes(m, out)
        b[m - 1] = norm_gamma
        bases[m] = gamma
        last = matvec(eff_ham, bases[m])
        a[m] = np.real(bs.inner(bases[m], last))
        coef = tridiag_expme1_solver(a, b, m + 1, step_length)
        dist = distance(last_coef[:m + 1], coef)
        if dist < params.error or m == eff_dim or m == maxit - 1:
            coef = coef * initial_norm
            out = bs.T(list(bases[0].indexes), {}, np.complex128)
            bs.linear_combine(list(coef), bases[:m + 1], 0.0, out)
            return ExpmvRes(m + 1, out)
        last_coef = np.zeros(maxit, dtype=np.complex128)
        last_coef[:m + 1] = coef
