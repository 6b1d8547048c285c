"""CPU FP64 oracle for the two-site DMRG/TDVP local update.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``ultradmrg_gb300``) may
import this package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use it, and only as the checker.

It restates, in numpy, the qlmps call sequence of the hot path (Lanczos,
effective-Hamiltonian matvec, environment update, truncated block SVD, the
two-site sweep drivers) over a block-sparse tensor model.  The arithmetic of
the reference lives in QuantumLiquids/TensorToolkit (``qlten``), which is not
vendored and not pinned by the reference; its semantics are restated from the
call sites (each function cites the file:line it follows).

Parity pins: the golden ground-state energies and the dense-ED / known-answer
checks of the reference's own tests (see ``tests/test_oracle_golden.py``).
Sizes beyond those tests are not pinned by the reference.
"""
