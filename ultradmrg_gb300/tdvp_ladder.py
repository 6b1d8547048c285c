"""Two-site TDVP on the two-leg S = 1/2 Heisenberg ladder after a local S+
quench: the mixed-precision Krylov matvec against the FP64 one.

``python -m ultradmrg_gb300.tdvp_ladder [--Lx 32] [--D 512] [--steps 40]
[--dt 0.05] [--krylov 20] [--every 10] [--forms fp64,mixed] [--out f.json]``

* The lattice is a 2 x Lx ladder with J_leg = J_rung = 1 and U(1) Sz, with
  sites x*2 + y.  The MPO comes from the restated reference generator.
* The ground state comes from device two-site VMPS (FP64).  It starts from
  a seeded random Sz = 0 product state (seed 2) and the bond dimension grows
  to D (``--gs-schedule``).
* The quench applies S+ on the centre site (``ActOperatorOnMps``, on the
  host).  It uses the operator table of the reference's spin tests, where
  S+ sets element {0, 1}.  Under ``ActOperatorOnMps``'s convention
  A'[o] = sum_i O[i, o] A[i] that element takes basis state 0 to state 1,
  so the total Sz label moves by -1 in this basis.  The ladder's singlet
  ground state is spin-flip symmetric, so both directions give the same
  dynamics.
* The evolution runs ``--steps`` TDVP steps of dt in each form, from the same
  quenched state: Krylov exp(-i dt H) with at most ``--krylov`` vectors,
  Dmax = D, truncation 1e-10.
* The report gives the wall seconds of each form (total and per step) and
  the nvidia-smi clocks sampled while it ran.
  Every ``--every`` steps it also gives the largest difference of the local
  <Sz_i> between the forms, and 1 - |<psi_fp64|psi_mixed>| / (|psi_fp64|
  |psi_mixed|) (device measurements, ``ultradmrg_gb300.measure``).

Prints one JSON object (also written to ``--out``).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api, measure as dm, models as M
from .clocks import ClockSampler


def ladder_problem(Lx: int, dtype=np.complex128):
    N = 2 * Lx
    mpo, pb = M.heisenberg_chain_mpo(N, dtype=dtype, pairs=M.heisenberg_ladder_pairs(Lx, 2),
                                     builder="reference")
    _, ops = M.spin_half_site(dtype)
    return N, mpo, pb, ops


def ground_state(ctx, mpo, pb, N, schedule, seed=2):
    """Device VMPS from a random Sz = 0 product state; schedule = [(sweeps, D)]."""
    mps = [api.DeviceTensor.from_data(ctx, t)
           for t in M.direct_product_mps([pb] * N, M.random_sz0_labels(N, seed))]
    dmpo = [api.DeviceTensor.from_data(ctx, w) for w in mpo]
    e0 = None
    for sweeps, D in schedule:
        e0, _ = api.two_site_finite_vmps(ctx, mps, dmpo, api.FiniteVMPSSweepParams(
            sweeps, min(D, 8), D, 1e-10, 1e-9, 100))
    host = [t.to_data() for t in mps]
    for t in mps + dmpo:
        t.close()
    return e0, host


def overlap_error(b, ket, bra):
    """1 - |<bra|ket>| / (|bra| |ket|) by CalPsi1OpPsi2 with the identity."""
    eye = np.eye(b.info(ket[0])[0][1].dim)
    kb = dm.cal_psi1_op_psi2(b, ket, bra, eye)[0]
    kk = dm.cal_psi1_op_psi2(b, ket, ket, eye)[0]
    bb = dm.cal_psi1_op_psi2(b, bra, bra, eye)[0]
    return float(1.0 - abs(kb) / np.sqrt(abs(kk) * abs(bb)))


def run(ctx, Lx=32, D=512, steps=40, dt=0.05, krylov=20, every=10, forms=("fp64", "mixed"),
        gs_schedule="2:64,2:128,2:256,2:512"):
    """The benchmark on an open context.  Returns (report, {form: host MPS
    after the evolution}, the quenched host MPS, the complex host MPO)."""
    forms = [f for f in forms if f]
    prec = {"fp64": api.PREC_FP64, "mixed": api.PREC_MIXED}
    N, mpo, pb, ops = ladder_problem(Lx, np.float64)
    schedule = [(int(s), min(int(d), D)) for s, d in
                (x.split(":") for x in gs_schedule.split(","))]
    t0 = time.perf_counter()
    e0, gs = ground_state(ctx, mpo, pb, N, schedule)
    gs_sec = time.perf_counter() - t0
    centre = N // 2
    quenched = M.act_operator_on_mps(gs, ops["sp"], None, centre)
    _, mpo_c, _, _ = ladder_problem(Lx, np.complex128)
    dmpo = [api.DeviceTensor.from_data(ctx, w) for w in mpo_c]
    states = {f: [api.DeviceTensor.from_data(ctx, t.copy()) for t in quenched] for f in forms}
    backend = dm.device_backend(ctx)
    out = {"config": {"lattice": f"2x{Lx} Heisenberg ladder", "sites": N, "D": D,
                      "dt": dt, "steps": steps, "krylov": krylov, "quench": "S+",
                      "quench_site": centre, "seed": 2, "gs_schedule": schedule},
           "ground_state": {"energy": e0, "seconds": gs_sec},
           "forms": {f: {"seconds": 0.0, "updates": 0} for f in forms}, "checkpoints": []}
    clocks = {f: [] for f in forms}
    done = 0
    while done < steps:
        n = min(every, steps - done)
        for f in forms:
            p = api.TDVPEvolveParams(dt, n, 1, D, 1e-10, 1e-10, krylov, precision=prec[f])
            ctx.sync()
            with ClockSampler(0) as clk:
                t1 = time.perf_counter()
                log = api.two_site_finite_tdvp(ctx, states[f], dmpo, p)
                ctx.sync()
                out["forms"][f]["seconds"] += time.perf_counter() - t1
            clocks[f].append(clk.summary())
            out["forms"][f]["updates"] += len(log)
            out["forms"][f]["D_max"] = max(r["D"] for r in log)
        done += n
        cp = {"step": done, "time": done * dt}
        sz = {}
        for f in forms:
            m = dm.MPSMeasurer(backend, states[f])
            sz[f] = np.array([r.avg for r in dm.measure_one_site_op(m, ops["sz"].mat.astype(
                np.complex128))])
            m.close()
            cp[f"sz_{f}_centre"] = complex(sz[f][centre]).real
        if "fp64" in forms and "mixed" in forms:
            cp["max_abs_dSz"] = float(np.abs(sz["mixed"] - sz["fp64"]).max())
            cp["overlap_err"] = overlap_error(backend, states["mixed"], states["fp64"])
        out["checkpoints"].append(cp)
    for f in forms:
        out["forms"][f]["seconds_per_step"] = out["forms"][f]["seconds"] / steps
        cs = [c for c in clocks[f] if c["samples"]]
        out["forms"][f]["clocks"] = {
            "sm_mhz_min_of_medians": min((c["sm_mhz"] for c in cs), default=None),
            "sm_max_mhz": max((c["sm_max_mhz"] for c in cs), default=None),
            "reasons": sorted({r for c in cs for r in c["reasons"]}),
            "samples": sum(c["samples"] for c in cs)}
    if "fp64" in forms and "mixed" in forms:
        out["speedup_mixed_vs_fp64"] = (out["forms"]["fp64"]["seconds"] /
                                        out["forms"]["mixed"]["seconds"])
    final = {f: [t.to_data() for t in states[f]] for f in forms}
    for f in forms:
        for t in states[f]:
            t.close()
    for t in dmpo:
        t.close()
    return out, final, quenched, mpo_c


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--Lx", type=int, default=32)
    ap.add_argument("--D", type=int, default=512)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--krylov", type=int, default=20)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--forms", default="fp64,mixed")
    ap.add_argument("--gs-schedule", default="2:64,2:128,2:256,2:512",
                    help="ground-state sweeps:D pairs (D capped at --D)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    ctx = api.Context(0)
    out, _, _, _ = run(ctx, a.Lx, a.D, a.steps, a.dt, a.krylov, a.every, a.forms.split(","),
                       a.gs_schedule)
    line = json.dumps(out)
    print(line)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(line + "\n")
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
