"""Synthetic benchmark workloads with the shapes of the reference's configs.

There is no public dataset for this path; the reference benchmark builds its
inputs deterministically (``benchmark/ultradmrg_hubbard2d.cpp``).  Here a
workload is: the model's MPO, a seeded random MPS in mixed-canonical form
around the centre bond whose bond sectors follow a Gaussian Schmidt-weight
model (``models.bond_sectors``, ``models.random_canonical_mps``), and the
two-site problem at the centre bond (environments from the MPS by
environment updates, at the physical scale of a DMRG run).  The MPOs come
from the restated reference generator (``mpogen``, ``builder="reference"``):
the reference's bond dimensions, sector order and channel order.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import models as M


@dataclass(frozen=True)
class Workload:
    name: str
    model: str
    Lx: int
    Ly: int
    D: int
    seed: int
    sigma: float
    U: float = 8.0
    t: float = 1.0
    electrons: int = 0
    builder: str = "reference"  # MPO generator (models._generator)

    @property
    def N(self):
        return self.Lx * self.Ly

    @property
    def centre(self):
        return self.N // 2 - 1


WORKLOADS = {
    # Hubbard 4x16 cylinder, 1/8 doping (56 electrons, Sz=0), U(1)xU(1), D=2000
    "hubbard4x16_D2000": Workload("hubbard4x16_D2000", "hubbard", 16, 4, 2000, 1, 2.0,
                                  electrons=56),
    # Hubbard 4x8 cylinder, 1/8 doping (28 electrons, Sz=0), D=1000
    "hubbard4x8_D1000": Workload("hubbard4x8_D1000", "hubbard", 8, 4, 1000, 1, 2.0,
                                 electrons=28),
    # S=1/2 Heisenberg chain L=32, Sz=0, D=256
    "heisenberg32_D256": Workload("heisenberg32_D256", "heisenberg", 32, 1, 256, 0, 2.0),
    # small case for profiling and tests
    "hubbard4x8_D256": Workload("hubbard4x8_D256", "hubbard", 8, 4, 256, 1, 2.0, electrons=28),
}


def build_host(w: Workload):
    """(mpo, mps) as host block tensors."""
    if w.model == "hubbard":
        mpo, pb = M.hubbard_cylinder_mpo(w.Lx, w.Ly, t=w.t, U=w.U, builder=w.builder)
        div = (w.electrons, 0)
    else:
        mpo, pb = M.heisenberg_chain_mpo(w.N, builder=w.builder)
        div = (0,)
    mps = M.random_canonical_mps([pb] * w.N, div, w.D, w.centre, seed=w.seed, sigma=w.sigma)
    return mpo, mps
