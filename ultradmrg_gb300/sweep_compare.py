"""Two-site sweep of the Hubbard 4x16 cylinder at D = 2000 in three forms.

The reference benchmark (``benchmark/ultradmrg_hubbard2d.cpp:227-253``) grows
the bond dimension over calls of the sweep driver (D = 10, 100, 1000, 2000)
from the product state with one hole every N/8 sites, then times a sweep at
D = 2000.  Here a shorter schedule prepares the D = 2000 state (mixed
precision, exact SVD, the rank model recording each bond's spectrum), and one
full sweep is timed from that same state in each form:

* ``fp64_exact``: plain FP64 block GEMMs in Lanczos, exact block SVD;
* ``mixed_exact``: split-BF16 tensor-core matvec, exact block SVD;
* ``mixed_learned``: split-BF16 matvec, randomized SVD sized by the learned
  rank model (exact SVD on a miss; optional audit by the exact SVD);
* ``mixed_learned_rule``: the same with the cost rule (the exact SVD when
  the predicted sketch exceeds a fraction of the sector dimensions).

``--centre-update`` instead runs, from the prepared state, a right sweep of
mixed-precision two-site updates (exact SVD) up to the centre bond and
reports the centre update (seconds: total, Lanczos, matvec plan, SVD,
environment); that update alone is bracketed as the CUDA profiler's
collection range, so ``ncu --profile-from-start off`` records just its
kernels.

A form name may end in ``@<tol>`` (e.g. ``mixed_exact@1e-11``): that form's
Lanczos runs to that tolerance instead of ``--lanczos-error``.  With
``--sweeps k`` each form runs k sweeps (``sweep_seconds`` is per sweep,
``sweep_energies`` the energy at the end of each).  Each form is
compared with the FP64 form of the same tolerance (``fp64_exact`` with the
same suffix) when it is in the list.

``python -m ultradmrg_gb300.sweep_compare [--out FILE]`` prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api
from . import models as M
from .clocks import ClockSampler
from . import rank_training as RT


def _upload(ctx, tensors):
    return [api.DeviceTensor.from_data(ctx, t) for t in tensors]


def prepare(ctx, Lx=16, Ly=4, schedule="10:2,100:2,500:2,1000:2,2000:1", lanczos_error=1e-9,
            weights=RT.WEIGHTS):
    """The Hubbard cylinder (t=1, U=8, one hole every N/8 sites) grown over the
    schedule ``D:sweeps,...`` (mixed precision, exact SVD, the rank model
    recording each bond's spectrum).  Returns (host MPO, device MPO, host
    state, rank model, per-stage log, seconds)."""
    N = Lx * Ly
    mpo, pb = M.hubbard_cylinder_mpo(Lx, Ly, t=1.0, U=8.0, builder="reference")
    labels = M.hubbard_cylinder_holes(N, 8)
    dmpo = _upload(ctx, mpo)
    dmps = _upload(ctx, M.direct_product_mps([pb] * N, labels))
    model = RT.load(ctx, weights)
    t0 = time.perf_counter()
    prep = []
    for item in schedule.split(","):
        D, sw = (int(v) for v in item.split(":"))
        p = api.FiniteVMPSSweepParams(sw, D, D, 1e-8, lanczos_error, 100,
                                      precision=api.PREC_MIXED)
        e0, log, _, _ = api.two_site_finite_vmps_learned(ctx, dmps, dmpo, p, model, False)
        prep.append(dict(D=D, sweeps=sw, e0=e0, max_trunc_err=max(r["trunc_err"] for r in log)))
    sec = time.perf_counter() - t0
    state = [t.to_data() for t in dmps]
    for t in dmps:
        t.close()
    return mpo, dmpo, state, model, prep, sec


def centre_update(ctx, mpo, dmpo, state, D=2000):
    """The right sweep of mixed two-site updates from the prepared state up to
    the centre bond; returns the centre update's timings and log."""
    N = len(state)
    centre = N // 2 - 1
    p = api.FiniteVMPSSweepParams(1, D, D, 1e-8, 1e-9, 100, precision=api.PREC_MIXED)
    mps = _upload(ctx, state)
    # right environments of the (right-canonical) prepared state: renvs[k]
    # covers the last k sites
    renvs = [api.DeviceTensor.from_data(ctx, api.trivial_env_data(state[N - 1], mpo[N - 1], "r"))]
    for i in range(N - 1, 1, -1):
        renvs.append(api.update_site_renvs(ctx, renvs[-1], mps[i], dmpo[i]))
    L = api.DeviceTensor.from_data(ctx, api.trivial_env_data(state[0], mpo[0], "l"))
    out = {}
    for l in range(centre + 1):
        if l == centre:
            ctx.profiler_range(True)
        t0 = time.perf_counter()
        a, b, e, log = api.two_site_update(ctx, L, renvs[N - l - 2], mps[l], mps[l + 1],
                                           dmpo[l], dmpo[l + 1], p, "r")
        ctx.sync()
        sec = time.perf_counter() - t0
        if l == centre:
            ctx.profiler_range(False)
            out = dict(bond=l, seconds=sec, **{k: log[k] for k in (
                "lancz_sec", "plan_sec", "svd_sec", "env_sec", "iters", "D", "trunc_err", "e0")})
        mps[l].close()
        mps[l + 1].close()
        mps[l], mps[l + 1] = a, b
        L.close()
        L = e
    for t in mps + renvs + [L]:
        t.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--Lx", type=int, default=16)
    ap.add_argument("--Ly", type=int, default=4)
    ap.add_argument("--D", type=int, default=2000)
    ap.add_argument("--schedule", default="10:2,100:2,500:2,1000:2,2000:1")
    ap.add_argument("--weights", default=RT.WEIGHTS)
    ap.add_argument("--forms", default="fp64_exact,mixed_exact,mixed_learned")
    ap.add_argument("--audit", action="store_true")
    ap.add_argument("--lanczos-error", type=float, default=1e-9)
    ap.add_argument("--sweeps", type=int, default=1, help="sweeps of each timed form")
    ap.add_argument("--max-fraction", type=float, default=0.1,
                    help="sketch fraction above which the learned form runs the exact SVD "
                         "(form mixed_learned_rule)")
    ap.add_argument("--centre-update", action="store_true",
                    help="time (and mark for the profiler) the centre bond's update instead")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    ctx = api.Context(0)
    N = a.Lx * a.Ly
    mpo, dmpo, state, model, prep, prep_sec = prepare(ctx, a.Lx, a.Ly, a.schedule,
                                                      a.lanczos_error, a.weights)
    out = dict(workload=f"hubbard{a.Ly}x{a.Lx}", D=a.D, sites=N, preparation=prep,
               preparation_seconds=prep_sec, forms={})
    if a.centre_update:
        out.pop("forms")
        out["centre_update"] = centre_update(ctx, mpo, dmpo, state, a.D)
        print(json.dumps(out), flush=True)
        if a.out:
            with open(a.out, "w") as fh:
                json.dump(out, fh, indent=1)
        return
    forms = a.forms.split(",")
    if a.audit and "mixed_learned" in forms:
        forms.append("mixed_learned_audit")  # untimed: the exact SVD judges every truncation
    for form in forms:
        base, _, tol = form.partition("@")
        lerr = float(tol) if tol else a.lanczos_error
        prec = api.PREC_FP64 if base.startswith("fp64") else api.PREC_MIXED
        mode = 2 if "learned" in base else 0
        p = api.FiniteVMPSSweepParams(a.sweeps, a.D, a.D, 1e-8, lerr, 100, precision=prec,
                                      svd_mode=mode, svd_audit=base.endswith("audit"),
                                      svd_sketch_max_fraction=(a.max_fraction
                                                               if base.endswith("rule") else 1.0))
        if mode == 2:  # a model carrying the bond history of the prepared state
            hist = api.RankModel(ctx, 0)
            hist.params = model.params
            hist.copy_history_from(model)
        mps = _upload(ctx, state)
        ctx.sync()
        with ClockSampler(0) as clk:
            t1 = time.perf_counter()
            if mode == 2:
                e0, log, _, _ = api.two_site_finite_vmps_learned(ctx, mps, dmpo, p, hist, False)
            else:
                e0, log = api.two_site_finite_vmps(ctx, mps, dmpo, p)
            ctx.sync()
            sec = time.perf_counter() - t1
        per = 2 * (N - 2)  # updates per sweep
        f = dict(sweep_seconds=sec / a.sweeps, e0=e0, clocks=clk.summary(),
                 sweep_energies=[log[(k + 1) * per - 1]["e0"] for k in range(a.sweeps)],
                 lanczos_seconds=sum(r["lancz_sec"] for r in log),
                 svd_seconds=sum(r["svd_sec"] for r in log),
                 env_seconds=sum(r["env_sec"] for r in log),
                 lanczos_iters=int(sum(r["iters"] for r in log)),
                 max_trunc_err=max(r["trunc_err"] for r in log),
                 svd_grow_rounds=int(sum(r["svd_grow_rounds"] for r in log)),
                 svd_slowest=[(r["site"], round(r["svd_sec"], 4)) for r in
                              sorted(log, key=lambda r: -r["svd_sec"])[:5]],
                 energies=[r["e0"] for r in log], trunc_errs=[r["trunc_err"] for r in log])
        if p.svd_audit:
            aud = [r for r in log if r["svd_audit_err"] >= 0]
            f["audit"] = dict(updates=len(aud),
                              max_trunc_err_diff=max((r["svd_audit_err"] for r in aud),
                                                     default=0.0),
                              kept_state_diffs=int(sum(r["svd_audit_kept_diff"] for r in aud)))
        out["forms"][form] = f
        for t in mps:
            t.close()
    for k, f in out["forms"].items():
        _, at, tol = k.partition("@")
        ref = out["forms"].get("fp64_exact" + at + tol)
        if ref is None:
            continue
        f["speedup_vs_fp64_exact"] = ref["sweep_seconds"] / f["sweep_seconds"]
        f["rel_dE_vs_fp64_exact"] = abs(f["e0"] - ref["e0"]) / abs(ref["e0"])
        f["max_site_rel_dE_vs_fp64_exact"] = float(np.max(
            np.abs(np.array(f["energies"]) - np.array(ref["energies"])) /
            np.abs(np.array(ref["energies"]))))
        f["max_trunc_err_diff_vs_fp64_exact"] = float(np.max(
            np.abs(np.array(f["trunc_errs"]) - np.array(ref["trunc_errs"]))))
    # FP64 against itself at two tolerances: the sweep's own sensitivity
    tight = [k for k in out["forms"] if k.startswith("fp64_exact@")]
    if "fp64_exact" in out["forms"] and tight:
        r0, r1 = out["forms"]["fp64_exact"], out["forms"][tight[0]]
        out["fp64_tolerance_sensitivity"] = dict(
            forms=["fp64_exact", tight[0]],
            rel_dE=abs(r0["e0"] - r1["e0"]) / abs(r1["e0"]),
            max_site_rel_dE=float(np.max(np.abs(np.array(r0["energies"]) -
                                                np.array(r1["energies"])) /
                                         np.abs(np.array(r1["energies"])))))
    for f in out["forms"].values():
        f.pop("energies")
        f.pop("trunc_errs")
    s = json.dumps(out)
    print(s)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(s + "\n")


if __name__ == "__main__":
    main()
