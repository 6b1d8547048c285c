"""Times the pieces of one two-site update at the centre bond of a workload.

``python -m ultradmrg_gb300.centre_probe svd|lanczos|update|sweep_state [--workload NAME]``

* ``svd``: the exact truncated SVD of the converged two-site state, split to
  the left and to the right (``D`` kept states), twice each;
* ``lanczos``: matvec plan construction (mixed and FP64), the FP64 matvec, and
  the mixed-precision Lanczos solve (1e-9, at most 100 iterations), twice;
* ``update``: all of the above;
* ``sweep_state``: the Hubbard 4x16 cylinder grown to D = 2000 as in
  ``sweep_compare`` (a converged state rather than the synthetic one), then
  a right sweep of two-site updates (mixed precision, exact SVD) up to the
  centre bond, whose update is reported with its log (Lanczos, SVD and
  environment seconds).

Prints one JSON object (seconds); ``launches_before`` lines give the number of
kernels this library launched before the timed part, for a profiler's skip
count.  Except for ``sweep_state``, the state is the seeded synthetic MPS of
the workload (its QN-sector model and bond dimension), environments from
device environment updates.
"""
from __future__ import annotations

import argparse
import json
import time

from . import api
from .workloads import WORKLOADS, build_host


def _problem(ctx, w):
    mpo, mps = build_host(w)
    l = w.centre
    L, R = api.build_envs(ctx, mpo, mps, l, normalize=False)
    A1 = api.DeviceTensor.from_data(ctx, mps[l])
    A2 = api.DeviceTensor.from_data(ctx, mps[l + 1])
    psi = api.contract(ctx, A1, A2, [2], [0])
    W1 = api.DeviceTensor.from_data(ctx, mpo[l])
    W2 = api.DeviceTensor.from_data(ctx, mpo[l + 1])
    return [L, W1, W2, R], psi, tuple(mps[l].div())


def _timed(ctx, f):
    ctx.sync()
    t0 = time.perf_counter()
    r = f()
    ctx.sync()
    return time.perf_counter() - t0, r


def probe_lanczos(ctx, eh, psi, out):
    for prec, name in ((api.PREC_MIXED, "mixed"), (api.PREC_FP64, "fp64")):
        for rep in range(2):
            out[f"plan_{name}_{rep}"], _ = _timed(ctx, lambda: api.MatvecPlan(ctx, eh, psi, prec))
    x = api.MatvecPlan(ctx, eh, psi, api.PREC_FP64)
    y, z = x.embed(psi), x.embed(psi)
    for rep in range(3):
        out[f"fp64_matvec_{rep}"], _ = _timed(ctx, lambda: x.apply(y, z))
    print("launches_before lanczos", ctx.launches(), flush=True)
    for rep in range(2):
        sec, r = _timed(ctx, lambda: api.lanczos_solver(ctx, eh, psi, 1e-9, 100,
                                                        precision=api.PREC_MIXED))
        out[f"lanczos_{rep}"] = sec
        out[f"lanczos_{rep}_iters"] = r.iters
        out[f"lanczos_{rep}_matvec_seconds"] = r.matvec_seconds
    return r.gs_vec


def probe_svd(ctx, g, ldiv, D, out):
    g.scale_(1.0 / g.norm())
    print("launches_before svd", ctx.launches(), flush=True)
    for rep in range(2):
        for mode, name in ((api.SVD_SPLIT_LEFT, "left"), (api.SVD_SPLIT_RIGHT, "right")):
            sec, (u, s, vt, err, kept) = _timed(
                ctx, lambda: api.svd(ctx, g, 2, ldiv, 1e-8, D, D, mode))
            out[f"svd_exact_{name}_{rep}"] = sec
            out["svd_D"] = kept
            for t in (u, s, vt):
                t.close()


def probe_sweep_state(ctx, out):
    from .sweep_compare import prepare
    mpo, dmpo, state, _, _, prep_sec = prepare(ctx)
    out["preparation_seconds"] = prep_sec
    N = len(state)
    centre = N // 2 - 1
    p = api.FiniteVMPSSweepParams(1, 2000, 2000, 1e-8, 1e-9, 100, precision=api.PREC_MIXED)
    mps = [api.DeviceTensor.from_data(ctx, t) for t in state]
    # right environments of the (right-canonical) prepared state
    renvs = [api.DeviceTensor.from_data(ctx, api.trivial_env_data(state[N - 1], mpo[N - 1], "r"))]
    for i in range(N - 1, 1, -1):  # renvs[k]: the last k sites
        renvs.append(api.update_site_renvs(ctx, renvs[-1], mps[i], dmpo[i]))
    L = api.DeviceTensor.from_data(ctx, api.trivial_env_data(state[0], mpo[0], "l"))
    # a right sweep up to the centre bond moves the canonical centre there
    t0 = time.perf_counter()
    for l in range(centre + 1):
        if l == centre:
            print("launches_before update", ctx.launches(), flush=True)
        sec, (a, b, e, log) = _timed(ctx, lambda: api.two_site_update(
            ctx, L, renvs[N - l - 2], mps[l], mps[l + 1], dmpo[l], dmpo[l + 1], p, "r"))
        mps[l].close()
        mps[l + 1].close()
        mps[l], mps[l + 1] = a, b
        L.close()
        L = e
        if l == centre:
            out["update_centre"] = dict(bond=l, seconds=sec, **{k: log[k] for k in (
                "lancz_sec", "svd_sec", "env_sec", "iters", "D", "trunc_err", "e0")})
    out["right_sweep_to_centre_seconds"] = time.perf_counter() - t0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["svd", "lanczos", "update", "sweep_state"])
    ap.add_argument("--workload", default="hubbard4x16_D2000")
    a = ap.parse_args(argv)
    ctx = api.Context(0)
    if a.what == "sweep_state":
        out = dict(workload="hubbard4x16 grown to D=2000")
        probe_sweep_state(ctx, out)
        print(json.dumps(out), flush=True)
        return
    w = WORKLOADS[a.workload]
    eh, psi, ldiv = _problem(ctx, w)
    out = dict(workload=a.workload, bond=w.centre)
    if a.what in ("lanczos", "update"):
        g = probe_lanczos(ctx, eh, psi, out)
    else:
        g = api.lanczos_solver(ctx, eh, psi, 1e-9, 40, precision=api.PREC_MIXED).gs_vec
    if a.what in ("svd", "update"):
        probe_svd(ctx, g, ldiv, w.D, out)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
