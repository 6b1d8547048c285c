"""Training data and training of the learned rank predictor.

Samples come from the sweeps themselves: every two-site update records, for
each sector of its bond, the features of that sector at the bond's previous
visit and the number of states the truncation keeps now.  Sweeps follow the
reference benchmark's pattern of a growing bond-dimension schedule
(``benchmark/ultradmrg_hubbard2d.cpp:227-248``) on Hubbard cylinders
(``benchmark/ultradmrg_hubbard2d.cpp:149-181``) with the hole placement of
``:212-225``.

``python -m ultradmrg_gb300.rank_training --out FILE`` regenerates the
shipped weights (``rank_model_hubbard.npz``) on one GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np

from . import api
from . import models as M

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "rank_model_hubbard.npz")


@dataclass(frozen=True)
class Stage:
    """One call of the sweep driver: ``sweeps`` sweeps at bond dimension D."""

    D: int
    sweeps: int


@dataclass(frozen=True)
class Chain:
    """A Hubbard cylinder at a filling (holes placed as in the reference)."""

    Lx: int
    Ly: int
    U: float
    holes: int

    @property
    def N(self):
        return self.Lx * self.Ly

    def build(self):
        mpo, pb = M.hubbard_cylinder_mpo(self.Lx, self.Ly, t=1.0, U=self.U)
        labels = M.hubbard_cylinder_holes(self.N, self.holes)
        return mpo, pb, labels


def sweep_schedule(ctx, chain: Chain, schedule: Sequence[Stage], *, model=None, record=False,
                   svd_mode=0, trunc_err=1e-8, lanczos_error=1e-9, precision=api.PREC_MIXED,
                   oversample=8, lanczos_max_iterations=100, svd_audit=False):
    """Runs the schedule from the product state; returns (e0, log, X, Y)
    with the per-site logs and recorded samples of all stages."""
    mpo, pb, labels = chain.build()
    mps0 = M.direct_product_mps([pb] * chain.N, labels)
    dmps = [api.DeviceTensor.from_data(ctx, t) for t in mps0]
    dmpo = [api.DeviceTensor.from_data(ctx, t) for t in mpo]
    if model is not None:
        model.forget()
    logs, xs, ys = [], [], []
    e0 = 0.0
    for st in schedule:
        p = api.FiniteVMPSSweepParams(st.sweeps, 1, st.D, trunc_err, lanczos_error,
                                      lanczos_max_iterations, precision, svd_mode, oversample,
                                      svd_audit)
        if model is None:
            e0, log = api.two_site_finite_vmps(ctx, dmps, dmpo, p)
            x = y = None
        else:
            e0, log, x, y = api.two_site_finite_vmps_learned(ctx, dmps, dmpo, p, model, record)
        logs += [dict(r, stage_D=st.D) for r in log]
        if record and x is not None:
            xs.append(x)
            ys.append(y)
    X = np.concatenate(xs) if xs else np.zeros((0, 0), np.float32)
    Y = np.concatenate(ys) if ys else np.zeros(0, np.float32)
    return e0, logs, X, Y


# Training chains: 4x8 and 4x16 cylinders, U in {4, 8, 12}, doping 1/8 and 1/16.
TRAIN_CHAINS = [Chain(8, 4, U, h) for U in (4.0, 8.0, 12.0) for h in (4, 2)] + \
               [Chain(16, 4, U, h) for U in (4.0, 8.0, 12.0) for h in (8, 4)]
TRAIN_SCHEDULE_4x8 = [Stage(64, 1), Stage(128, 1), Stage(256, 1), Stage(512, 1), Stage(1000, 2)]
TRAIN_SCHEDULE_4x16 = [Stage(100, 1), Stage(250, 1), Stage(500, 1), Stage(1000, 1),
                       Stage(2000, 1)]


def collect(ctx, chains: Sequence[Chain], schedule_of, **kw) -> Tuple[np.ndarray, np.ndarray]:
    """Recorded samples of all chains (an untrained model only records)."""
    rec = api.RankModel(ctx, seed=0)
    xs, ys = [], []
    for ch in chains:
        t0 = time.time()
        _, _, X, Y = sweep_schedule(ctx, ch, schedule_of(ch), model=rec, record=True, **kw)
        xs.append(X)
        ys.append(Y)
        print(f"collected {len(Y)} samples from {ch} in {time.time() - t0:.1f} s",
              file=sys.stderr, flush=True)
    rec.close()
    return np.concatenate(xs), np.concatenate(ys)


def train(ctx, X, Y, *, epochs=400, batch=256, lr=2e-3, seed=0, model_seed=7):
    """A fresh model trained on (X, Y) by the device kernels."""
    m = api.RankModel(ctx, seed=model_seed)
    loss = m.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return m, loss


def save(model, path, meta=None):
    np.savez(path, params=model.params, meta=json.dumps(meta or {}))


def load(ctx, path=WEIGHTS):
    d = np.load(path)
    m = api.RankModel(ctx, seed=0)
    m.params = d["params"]
    return m


def main(argv: List[str] | None = None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=2048)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--small", action="store_true", help="4x8 chains only")
    a = ap.parse_args(argv)
    ctx = api.Context(0)
    chains = [c for c in TRAIN_CHAINS if not a.small or c.Lx == 8]
    t0 = time.time()
    X, Y = collect(ctx, chains,
                   lambda c: TRAIN_SCHEDULE_4x8 if c.Lx == 8 else TRAIN_SCHEDULE_4x16,
                   svd_mode=0)
    t1 = time.time()
    m, loss = train(ctx, X, Y, epochs=a.epochs, batch=a.batch, lr=a.lr)
    t2 = time.time()
    # the rule without the network (kept count of the previous visit), same samples
    base = float(np.mean((10.0 * X[:, -3] - Y) ** 2))
    meta = dict(samples=int(len(Y)), chains=[c.__dict__ for c in chains], loss=loss,
                previous_kept_rule_mse=base, epochs=a.epochs, batch=a.batch, lr=a.lr,
                collect_seconds=t1 - t0, train_seconds=t2 - t1)
    save(m, a.out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
