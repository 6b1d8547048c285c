#!/usr/bin/env python
"""Benchmark of the two-site DMRG hot path: H_eff * psi (L.W.W.R.psi) over
U(1)xU(1) block-sparse tensors, the matvec inside Lanczos.

One step = one matvec at the centre bond of the workload (default: Hubbard
4x16 cylinder, 1/8 doping, D=2000; synthetic seeded inputs, see
``ultradmrg_gb300/workloads.py``).  ``value`` is matvec TFLOP/s with the
inputs resident in HBM (device time, CUDA events on the library's stream,
L2 flushed before every step); ``e2e`` is the same metric through the C ABI
with host buffers (pinned host -> device copy of psi, matvec, device -> host
copy of the result, every step).  FLOPs are algorithmic: sum of 2*M*N*K over
the block-pair GEMMs of the schedule.

The metric's other half, sweep seconds, comes from the sweep leg
(``sweep_leg``): the same cylinder grown to a near-converged D = 2000 state,
then one timed two-site sweep in the plain FP64 form, the mixed form and the
mixed form with learned truncation (keys ``sweep_*`` and ``sweep``, with the
clocks sampled during each sweep).

``--impl reference`` times the CPU FP64 oracle on the same workload: one
forked process per host core, each running the numpy matvec with
single-threaded OpenBLAS on some of the left environment's bra sectors, the
way the reference's tensor library spreads block pairs over threads.  The
reference's own C++ path cannot be built here (its tensor library is not
vendored).  The GPU arm's ``cpu_baseline`` runs that arm in a CPU-only
subprocess.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from ultradmrg_gb300.clocks import ClockSampler  # noqa: E402

METRIC = ("two-site matvec TFLOP/s (H_eff*psi, U(1)xU(1) block-sparse; algorithmic FLOPs; "
          "mixed split-BF16 tensor-core form, plain FP64 reported beside)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: 2000 mixed matvecs (~1.4 s with the L2 flushes, so the 200 ms
    # clock sampler takes several readings inside the timed region); 20 for
    # the reference arm, whose steps are whole CPU matvecs
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hubbard4x16_D2000")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--matvec-only", action="store_true",
                    help="time the mixed matvec only (profiling runs): no FP64 form, "
                         "Lanczos, local updates, sweeps, e2e or CPU baseline")
    ap.add_argument("--no-sweep", action="store_true",
                    help="leave out the sweep leg (profiling runs of the matvec and updates)")
    ap.add_argument("--sweep-schedule", default="10:2,100:2,500:2,1000:2,2000:2",
                    help="D:sweeps,... that grows the Hubbard 4x16 state before the timed sweeps")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20 if args.impl == "reference" else 2000
    return args


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def ncu_traffic(workload, kernel):
    """DRAM bytes (read + write) per launch of `kernel` on `workload` from the
    committed ncu capture summary (profiles/ncu_traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            t = json.load(f)
        return t[workload][kernel]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


# ---------------------------------------------------------------------------
# CPU side (oracle) -- the cpu_baseline leg and the reference arm
# ---------------------------------------------------------------------------

def cpu_problem(w):
    """Host inputs of the workload built with the oracle's environment updates."""
    from oracle import blocksparse as bs
    from oracle import vmps as ovmps
    from ultradmrg_gb300.workloads import build_host

    mpo, mps = build_host(w)
    l = w.centre
    N = w.N
    L = ovmps.trivial_lenv(mps[0], mpo[0])
    for i in range(l):
        L = ovmps.update_site_lenvs(L, mps[i], mpo[i])
    R = ovmps.trivial_renv(mps[N - 1], mpo[N - 1])
    for i in range(N - 1, l + 1, -1):
        R = ovmps.update_site_renvs(R, mps[i], mpo[i])
    psi = bs.contract(mps[l], mps[l + 1], [2], [0])
    return [L, mpo[l], mpo[l + 1], R], psi


def cpu_matvec_sample(eff, psi, budget_s):
    """Time the oracle matvec; if one full matvec exceeds the budget, time it on
    a subset of the left environment's bra sectors (a proportional sample)."""
    from oracle import blocksparse as bs
    from oracle import krylov

    L = eff[0]
    bra = sorted({k[0] for k in L.blocks})
    frac = 1.0
    for _ in range(6):
        keep = set(bra[::max(1, int(round(1 / frac)))]) if frac < 1 else set(bra)
        Ls = bs.T(list(L.indexes), {k: v for k, v in L.blocks.items() if k[0] in keep}, L.dtype)
        bs.FLOPS[0] = 0.0
        t0 = time.perf_counter()
        krylov.eff_ham_mul_two_site_state([Ls] + list(eff[1:]), psi)
        dt = time.perf_counter() - t0
        if dt <= budget_s or frac < 0.02:
            return bs.FLOPS[0], dt, len(keep), len(bra)
        frac = frac * max(0.05, budget_s / dt * 0.8)
    return bs.FLOPS[0], dt, len(keep), len(bra)


def cpu_baseline(args, w):
    """The reference arm (the oracle on all host cores) run as a CPU-only
    subprocess: its workers fork from a process without a CUDA context.
    Falls back to one in-process oracle matvec when that run fails."""
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env.update({k: "1" for k in SERIAL_BLAS})
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", w.name, "--steps", "3", "--warmup", "1",
           "--cpu-budget", str(args.cpu_budget)]
    why = ""
    try:
        r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300)
        if r.returncode == 0:
            ref = json.loads(r.stdout.strip().splitlines()[-1])
            cb = ref["cpu_baseline"]
            cb["sample"] += f"; {ref['steps']} timed matvecs, {ref['ms_per_step']:.0f} ms each"
            return cb
        why = (r.stderr.strip().splitlines() or ["exit %d" % r.returncode])[-1]
    except Exception as e:  # noqa: BLE001 - any failure of the subprocess
        why = repr(e)
    eff, hpsi = cpu_problem(w)
    cf, ct, kept, nbra = cpu_matvec_sample(eff, hpsi, args.cpu_budget)
    return {"value": cf / ct / 1e12, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
            "sample": f"one oracle matvec (numpy/OpenBLAS FP64, one process) over {kept}/{nbra} "
                      f"bra sectors of the left environment, {ct:.1f} s (the parallel run "
                      f"failed: {why[:160]})"}


def krylov_graph_probe(api, ctx, ops, psi, prec, reps=2):
    """Wall seconds of one Lanczos solve (1e-10, at most 120 steps; matvec plan
    included) with each Krylov step replayed as a CUDA graph and with its
    kernels launched directly, the faster of `reps` runs each."""
    out = {}
    for graph in (False, True):
        ctx.set_krylov_graph(graph)
        best, res = None, None
        for _ in range(reps):
            ctx.sync()
            t0 = time.perf_counter()
            r = api.lanczos_solver(ctx, ops, psi, 1e-10, 120, precision=prec)
            dt = time.perf_counter() - t0
            res = (r.iters, r.gs_eng)
            r.gs_vec.close()
            best = dt if best is None else min(best, dt)
        out[graph] = (best, res)
    ctx.set_krylov_graph(True)
    (tg, rg), (td, rd) = out[True], out[False]
    return {"graph_sec": tg, "direct_sec": td, "iters": rg[0],
            "us_per_step_graph": tg / rg[0] * 1e6, "us_per_step_direct": td / rd[0] * 1e6,
            "identical": rg == rd}


def sweep_leg(api, ctx, local, schedule):
    """The other half of the metric: one full two-site sweep (right then left,
    as ``TwoSiteFiniteVMPSSweep``) of the Hubbard 4x16 cylinder (t=1, U=8, 56
    electrons, U(1)xU(1)) at D = 2000, truncation 1e-8, Lanczos (1e-9, 100),
    timed in each form from one prepared near-converged state: the reference
    benchmark grows D over calls of the sweep driver and times a sweep at
    D = 2000 (``benchmark/ultradmrg_hubbard2d.cpp:227-252``).  The state is
    grown by ``schedule`` in the mixed form (exact SVD; the rank model records
    each bond's spectra for the learned form).  Forms: plain FP64 block GEMMs +
    exact SVD; split-BF16 tensor-core matvec + exact SVD; the same with the
    learned truncation (randomized SVD sized by the rank model where the
    predicted sketch is below a tenth of the sector, exact SVD elsewhere).
    nvidia-smi clocks are sampled during each sweep."""
    import numpy as np
    from ultradmrg_gb300 import sweep_compare as SC
    t0 = time.perf_counter()
    _, dmpo, state, model, prep, _ = SC.prepare(ctx, 16, 4, schedule, 1e-9)
    prep_s = time.perf_counter() - t0
    N = len(state)
    forms, logs = {}, {}
    for name, prec, mode, frac in (("fp64_exact", api.PREC_FP64, 0, 1.0),
                                   ("mixed_exact", api.PREC_MIXED, 0, 1.0),
                                   ("mixed_learned", api.PREC_MIXED, 2, 0.1)):
        p = api.FiniteVMPSSweepParams(1, 2000, 2000, 1e-8, 1e-9, 100, precision=prec,
                                      svd_mode=mode, svd_sketch_max_fraction=frac)
        mps = [api.DeviceTensor.from_data(ctx, t) for t in state]
        hist = None
        if mode == 2:  # a model carrying the bond history of the prepared state
            hist = api.RankModel(ctx, 0)
            hist.params = model.params
            hist.copy_history_from(model)
        ctx.sync()
        with ClockSampler(local) as clk:
            t1 = time.perf_counter()
            if hist is not None:
                e0, log, _, _ = api.two_site_finite_vmps_learned(ctx, mps, dmpo, p, hist, False)
            else:
                e0, log = api.two_site_finite_vmps(ctx, mps, dmpo, p)
            ctx.sync()
            sec = time.perf_counter() - t1
        forms[name] = {
            "sweep_s": sec, "e0": e0,
            "lanczos_s": sum(r["lancz_sec"] for r in log),
            "svd_s": sum(r["svd_sec"] for r in log),
            "env_s": sum(r["env_sec"] for r in log),
            "plan_s": sum(r["plan_sec"] for r in log),
            "lanczos_iters": int(sum(r["iters"] for r in log)),
            "updates": len(log), "max_trunc_err": max(r["trunc_err"] for r in log),
            "svd_grow_rounds": int(sum(r["svd_grow_rounds"] for r in log)),
            "clocks": clk.summary()}
        logs[name] = log
        for t in mps:
            t.close()
        if hist is not None:
            hist.close()
    ref = forms["fp64_exact"]
    e_ref = np.array([r["e0"] for r in logs["fp64_exact"]])
    t_ref = np.array([r["trunc_err"] for r in logs["fp64_exact"]])
    for name in ("mixed_exact", "mixed_learned"):
        f = forms[name]
        f["speedup_vs_fp64"] = ref["sweep_s"] / f["sweep_s"]
        f["rel_dE_vs_fp64"] = abs(f["e0"] - ref["e0"]) / abs(ref["e0"])
        e = np.array([r["e0"] for r in logs[name]])
        t = np.array([r["trunc_err"] for r in logs[name]])
        f["max_site_rel_dE_vs_fp64"] = float(np.max(np.abs(e - e_ref) / np.abs(e_ref)))
        f["max_trunc_err_diff_vs_fp64"] = float(np.max(np.abs(t - t_ref)))
    for t in dmpo:
        t.close()
    model.close()
    return {"workload": "hubbard4x16 cylinder, D=2000, trunc 1e-8, Lanczos (1e-9, 100)",
            "sites": N, "preparation": prep, "preparation_s": prep_s, "schedule": schedule,
            "forms": forms}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


SERIAL_BLAS = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    # one BLAS thread per worker process; set before numpy is loaded
    for k in SERIAL_BLAS:
        os.environ.setdefault(k, "1")
    from oracle.parallel import ParallelMatvec
    from ultradmrg_gb300.workloads import WORKLOADS

    w = WORKLOADS[args.workload]
    eff, psi = cpu_problem(w)
    cores = cpu_threads()
    pm = ParallelMatvec(eff, psi, cores)
    nbra = len(pm.sectors)
    # size each step so that warm-up + steps stay within about two minutes:
    # a full matvec when it fits, else a proportional sample of bra sectors
    per_step = max(0.05, min(args.cpu_budget, 120.0 / max(1, args.steps + args.warmup)))
    _, _, full = pm.run()
    sectors = pm.sectors
    if full > per_step:
        stride = max(1, int(round(full / per_step)))
        sectors = sorted(pm.sectors)[::stride]
    times, flops = [], 0.0
    for i in range(args.warmup + args.steps):
        f, _, dt = pm.run(sectors)
        if i >= args.warmup:
            times.append(dt)
            flops = f
    pm.close()
    kept = len(sectors)
    tot = sum(times)
    val = flops * len(times) / tot / 1e12
    sample = (f"oracle matvec (numpy FP64) over {kept}/{nbra} bra sectors of the left "
              f"environment of {w.name}, one task per sector on {cores} forked processes "
              f"with single-threaded OpenBLAS")
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random MPS, sector model)",
        "config": {"workload": w.name, "D": w.D, "sites": w.N, "bond": w.centre,
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args):
    import numpy as np

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("gloo")
    from ultradmrg_gb300 import api, build
    from ultradmrg_gb300.workloads import WORKLOADS, build_host

    if rank == 0 or ws == 1:
        build.build()
    if ws > 1:
        tdist.barrier()
    w = WORKLOADS[args.workload]
    ctx = api.Context(local)
    mpo, mps = build_host(w)
    l = w.centre
    L, R = api.build_envs(ctx, mpo, mps, l, normalize=False)
    A1 = api.DeviceTensor.from_data(ctx, mps[l])
    A2 = api.DeviceTensor.from_data(ctx, mps[l + 1])
    psi = api.contract(ctx, A1, A2, [2], [0])
    W1 = api.DeviceTensor.from_data(ctx, mpo[l])
    W2 = api.DeviceTensor.from_data(ctx, mpo[l + 1])
    ops = [L, W1, W2, R]
    t0 = time.perf_counter()
    plan = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_MIXED)  # tile autotuner runs here
    plan_s = time.perf_counter() - t0
    tiles = plan.tiles()
    plan64 = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_FP64)
    info = plan.info()
    x = plan.embed(psi)
    y = plan.embed(psi)
    y64 = plan.embed(psi)
    xp, yp = x.device_ptr(), y.device_ptr()
    flops = info["flops"]
    nbytes = info["psi_size"] * 8

    def step():
        plan.apply_ptr(xp, yp)

    def timed(fn, steps, slot0, ring=100):
        # event pairs in a ring of `ring` slots, read back every `ring` steps
        total = 0.0
        for c0 in range(0, steps, ring):
            cn = min(ring, steps - c0)
            for i in range(cn):
                ctx.flush_l2()
                ctx.event(slot0 + 2 * i)
                fn()
                ctx.event(slot0 + 2 * i + 1)
            ctx.sync()
            total += sum(ctx.elapsed_ms(slot0 + 2 * i, slot0 + 2 * i + 1) for i in range(cn))
        return total / steps / 1e3

    for _ in range(args.warmup):
        ctx.flush_l2()
        step()
    ctx.sync()
    if ws > 1:
        tdist.barrier()
    l0 = ctx.launches()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        t_step = timed(step, args.steps, 0)
        wall = time.perf_counter() - wall0
    launches = ctx.launches() - l0
    if ws > 1:
        import torch
        tt = torch.tensor([t_step], dtype=torch.float64)
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        t_step = float(tt.item())
    value = ws * flops / t_step / 1e12
    if args.matvec_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": t_step * 1e3, "higher_is_better": True,
                              "config": {"workload": w.name, "matvec_only": True},
                              "gpu_launches": launches}))
        if ws > 1:
            tdist.barrier()
            tdist.destroy_process_group()
        return 0

    # plain FP64 form on the same inputs (fewer steps: it is ~100x slower)
    y64p = y64.device_ptr()
    plan64.apply_ptr(xp, y64p)
    t64 = timed(lambda: plan64.apply_ptr(xp, y64p), max(2, min(args.steps, 5)), 200)
    ym, yd = y.download_packed(), y64.download_packed()
    mixed_err = float(np.linalg.norm(ym - yd) / max(np.linalg.norm(yd), 1e-300))
    # the mixed solver's FP64-accurate anchor matvec (one per local solve):
    # double-word FP32 block GEMMs against the FP64 pipe's
    plan.apply_anchor_ptr(xp, yp)
    t_anchor = timed(lambda: plan.apply_anchor_ptr(xp, yp), max(2, min(args.steps, 5)), 200)
    ya = y.download_packed()
    anchor = {"double_word_ms": t_anchor * 1e3, "fp64_pipe_ms": t64 * 1e3,
              "speedup": t64 / t_anchor,
              "rel_err_vs_fp64_pipe": float(np.linalg.norm(ya - yd) /
                                            max(np.linalg.norm(yd), 1e-300))}
    # per-stage device times (dominant kernel roofline): the median of five
    # matvecs, each after an L2 flush like the timed steps
    samples = []
    for _ in range(5):
        ctx.flush_l2()
        ms_s, fl_mx = plan.stage_times(xp, yp)
        samples.append(ms_s)
    ms_mx = [float(np.median([s_[i] for s_ in samples])) for i in range(4)]
    ms_64, fl_64 = plan64.stage_times(xp, y64p)
    # the tile autotuner's choice against the fixed tile shapes (one matvec per
    # stage, best of three; the plan of each shape built here)
    tune = {"choice_bn1_bn3": list(tiles[:2]), "tuned": tiles[2],
            "plan_seconds_with_trials": plan_s}
    for bn in (64, 128):
        ctx.set_tc_tiles(bn, bn)
        pf = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_MIXED)
        ctx.set_tc_tiles(0, 0)
        best = None
        for _ in range(3):
            ms_f, _ = pf.stage_times(xp, yp)
            best = ms_f if best is None else [min(u, v) for u, v in zip(best, ms_f)]
        tune[f"fixed_{bn}_stage_ms"] = best
        tune[f"fixed_{bn}_ms"] = sum(best)
        del pf
    best = None
    for _ in range(3):
        ms_t, _ = plan.stage_times(xp, yp)
        best = ms_t if best is None else [min(u, v) for u, v in zip(best, ms_t)]
    tune["tuned_stage_ms"] = best
    tune["tuned_ms"] = sum(best)
    tune["trials_run"], tune["classes"] = ctx.tc_tuning()
    # the grouped FP64 / double-word GEMMs' tile policy: the tuned plans'
    # choice against both fixed policies (FP64 matvec, double-word anchor)
    gemm = {"choice_fp64_plan": plan64.gemm_policy(), "choice_mixed_plan": plan.gemm_policy()}
    for pol in (0, 1):
        ctx.set_gemm_tiles(pol)
        pf64 = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_FP64)
        pfmx = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_MIXED)
        ctx.set_gemm_tiles(-1)
        gemm[f"policy{pol}_fp64_matvec_ms"] = timed(
            lambda: pf64.apply_ptr(xp, y64p), 3, 200) * 1e3
        gemm[f"policy{pol}_anchor_ms"] = timed(lambda: pfmx.apply_anchor_ptr(xp, yp), 3, 200) * 1e3
        del pf64, pfmx
    gemm["trials_run"], gemm["classes"] = ctx.gemm_tuning()
    tune["fp64_gemm_tiles"] = gemm
    # host planning of a warm plan (tile choices cached): wall time and the
    # plan's own build phases (host tables on host threads), median of three
    builds = []
    for _ in range(3):
        t0 = time.perf_counter()
        pw = api.MatvecPlan(ctx, ops, psi, precision=api.PREC_MIXED)
        builds.append((time.perf_counter() - t0, pw.build_times()))
        del pw
    builds.sort(key=lambda b_: b_[0])
    plan_build = {"first_plan_ms_with_trials": plan_s * 1e3,
                  "warm_plan_ms": builds[1][0] * 1e3,
                  "warm_phases_ms": {k: v * 1e3 for k, v in builds[1][1].items()},
                  "first_phases_ms": {k: v * 1e3 for k, v in plan.build_times().items()}}
    # Lanczos energies of both forms from the same start vector, to convergence
    lz = {}
    for name, prec in (("mixed", api.PREC_MIXED), ("fp64", api.PREC_FP64)):
        r = api.lanczos_solver(ctx, ops, psi, 1e-10, 120, precision=prec)
        lz[name] = (r.gs_eng, r.iters, r.matvec_seconds / max(r.matvecs, 1))
        r.gs_vec.close()
    # Krylov steps as CUDA graph replays against direct launches: this
    # workload (mixed) and the L = 32 Heisenberg chain at D = 256 (short steps)
    kg = {f"{w.name}_mixed": krylov_graph_probe(api, ctx, ops, psi, api.PREC_MIXED)}
    sw = WORKLOADS["heisenberg32_D256"]
    smpo, smps = build_host(sw)
    sL, sR = api.build_envs(ctx, smpo, smps, sw.centre, normalize=False)
    sA1 = api.DeviceTensor.from_data(ctx, smps[sw.centre])
    sA2 = api.DeviceTensor.from_data(ctx, smps[sw.centre + 1])
    spsi = api.contract(ctx, sA1, sA2, [2], [0])
    sW1 = api.DeviceTensor.from_data(ctx, smpo[sw.centre])
    sW2 = api.DeviceTensor.from_data(ctx, smpo[sw.centre + 1])
    for prec, tag in ((api.PREC_FP64, "fp64"), (api.PREC_MIXED, "mixed")):
        kg[f"{sw.name}_{tag}"] = krylov_graph_probe(api, ctx, [sL, sW1, sW2, sR], spsi, prec)
    for t in (sL, sR, sA1, sA2, spsi, sW1, sW2):
        t.close()
    # HBM rates of the Lanczos vector kernels on vectors of this workload's
    # Krylov structure size, at three step counts (device-timed, best of four)
    kvec = {"n": info["psi_size"], "hbm_peak_gbs": measured_peaks().get("hbm_gbs", 6800.0)}
    for s_ in (10, 35, 70):
        pr = ctx.krylov_step_probe(info["psi_size"], s_)
        row = {}
        for k_, t_ in pr["ms"].items():
            b_ = pr["bytes"][k_]
            row[k_] = {"ms": t_, "gbs": b_ / (t_ * 1e-3) / 1e9 if b_ > 0 and t_ > 0 else None}
        row["second_pass_ran"] = pr["second_pass_ran"]
        kvec[f"step{s_}"] = row
    # one full local update at the centre bond (Lanczos to 1e-9 as the reference
    # benchmark, truncated SVD to D, environment update) in three forms: plain
    # FP64 + exact SVD, mixed + exact SVD, mixed + randomized SVD sized from the
    # bond's current sector dimensions (certified against the exact selection)
    site = {}
    A1d, A2d = api.DeviceTensor.from_data(ctx, mps[l]), api.DeviceTensor.from_data(ctx, mps[l + 1])
    for name, prec, svd in (("fp64_exact", api.PREC_FP64, 0), ("mixed_exact", api.PREC_MIXED, 0),
                            ("mixed_rsvd", api.PREC_MIXED, 1)):
        sp = api.FiniteVMPSSweepParams(1, w.D, w.D, 1e-8, 1e-9, 100, precision=prec, svd_mode=svd)
        ctx.sync()
        t0 = time.perf_counter()
        na, nb, ne, lg = api.two_site_update(ctx, L, R, A1d, A2d, W1, W2, sp, "r")
        lg["wall_sec"] = time.perf_counter() - t0
        site[name] = lg
        for t in (na, nb, ne):
            t.close()

    # exact truncated SVD against the randomized one with a tight sketch (each
    # sector sized to the exact SVD's kept count, the best a rank predictor can
    # do) on the centre ground state, truncated to D and to D/4
    svd_cmp = {}
    g = api.lanczos_solver(ctx, ops, psi, 1e-9, 100, precision=api.PREC_MIXED).gs_vec
    g.scale_(1.0 / g.norm())
    ldiv = tuple(mps[l].div())
    for dmax in (w.D, w.D // 4):
        best = {}
        for rep in range(2):
            ctx.sync()
            t0 = time.perf_counter()
            u, sv, vt, err, dk = api.svd(ctx, g, 2, ldiv, 1e-8, dmax, dmax, api.SVD_SPLIT_LEFT)
            ctx.sync()
            best["exact_sec"] = min(best.get("exact_sec", 1e9), time.perf_counter() - t0)
            bond = u.to_data().indexes[2]
            sketch = [(q, d) for q, d in zip(bond.qns, bond.dims)]
            for t in (u, sv, vt):
                t.close()
            ctx.sync()
            t0 = time.perf_counter()
            r = api.svd_randomized(ctx, g, 2, ldiv, 1e-8, dmax, dmax, sketch, api.SVD_SPLIT_LEFT)
            ctx.sync()
            best["sketch_sec"] = min(best.get("sketch_sec", 1e9), time.perf_counter() - t0)
            best.update(D=dk, trunc_err_exact=err, trunc_err_sketch=r[3], regrow_rounds=r[5])
            for t in r[:3]:
                t.close()
        best["exact_over_sketch"] = best["exact_sec"] / best["sketch_sec"]
        svd_cmp[f"Dmax={dmax}"] = best
    g.close()

    sweep = None
    if not args.no_sweep:
        for t in (A1d, A2d):
            t.close()
        sweep = sweep_leg(api, ctx, local, args.sweep_schedule)

    # e2e through the C ABI with host buffers
    try:
        import torch
        hx = torch.empty(info["psi_size"], dtype=torch.float64, pin_memory=True)
        hy = torch.empty(info["psi_size"], dtype=torch.float64, pin_memory=True)
        hxp, hyp = hx.data_ptr(), hy.data_ptr()
    except Exception:  # noqa: BLE001 - pinned memory unavailable
        hx = np.zeros(info["psi_size"])
        hy = np.zeros(info["psi_size"])
        hxp, hyp = hx.ctypes.data, hy.ctypes.data
    import ctypes
    from ultradmrg_gb300 import _lib
    x.download_packed()  # warm the path
    _lib.call("udmrg_tensor_download", x.h, ctypes.cast(hxp, _lib.c_double_p))  # psi -> host
    host_mapped_default = ctx.host_mapped()
    for _ in range(2):
        plan.apply_host_ptr(hxp, hyp)
    e0 = time.perf_counter()
    for _ in range(args.steps):  # one C-ABI call per step: copy in, matvec, copy out
        plan.apply_host_ptr(hxp, hyp)
    e2e_t = (time.perf_counter() - e0) / args.steps
    step()  # the device-buffer product of the same input: the host result must equal it
    e2e_same = bool(np.array_equal(y.download_packed(),
                                   hy.numpy() if hasattr(hy, "numpy") else hy))
    # the same call with each host-buffer mode (copies, input read in place,
    # input and output in place); the line's e2e uses the context's default
    e2e_modes = {}
    want = y.download_packed()
    for mode in (0, 1, 2):
        ctx.set_host_mapped(mode)
        for _ in range(2):
            plan.apply_host_ptr(hxp, hyp)
        nrep = min(args.steps, 500)
        e0 = time.perf_counter()
        for _ in range(nrep):
            plan.apply_host_ptr(hxp, hyp)
        tm = (time.perf_counter() - e0) / nrep
        same = bool(np.array_equal(want, hy.numpy() if hasattr(hy, "numpy") else hy))
        e2e_modes[str(mode)] = {"tflops": flops / tm / 1e12, "ms": tm * 1e3, "matches": same}
    ctx.set_host_mapped(host_mapped_default)
    if ws > 1:
        tt = torch.tensor([e2e_t], dtype=torch.float64)
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        e2e_t = float(tt.item())
    e2e_val = ws * flops / e2e_t / 1e12

    fp64_peak = ctx.fp64_peak_tflops()
    peaks = measured_peaks()
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    # dominant kernel: the longest of the stages of one mixed matvec.  Every
    # stage moves its operands through HBM (split-BF16 images, FP32 T1, FP64
    # psi and result): achieved = its algorithmic bytes (plan.stage_bytes)
    # over its event-timed duration, against the measured copy bandwidth; the
    # tensor-core work it issued (six split products) is reported beside
    dom = max(range(4), key=lambda i: ms_mx[i])
    stage_names = ["pack_kernel (psi split-BF16 images)", "tc_gemm_kernel (GEMM L.psi)",
                   "mpo_chunk_kernel (MPO step)",
                   "tc_mpo_gemm_kernel (MPO step fused into GEMM .R)"]
    byts = plan.stage_bytes()
    hbm = peaks.get("hbm_gbs", 6800.0)
    roof = {"bound": "hbm", "achieved": byts[dom] / (ms_mx[dom] / 1e3) / 1e9, "peak": hbm,
            "unit": "GB/s", "algorithmic_bytes": byts[dom],
            "peak_source": ("hbm_gbs of MEASURED_PEAKS.json, of measured" if "hbm_gbs" in peaks
                            else "fallback 6.8 TB/s")}
    if fl_mx[dom] > 0:
        roof["issued_tensor_tflops"] = fl_mx[dom] / (ms_mx[dom] / 1e3) / 1e12
        roof["issued_tensor_frac"] = roof["issued_tensor_tflops"] / bf16_peak
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["kernel"] = stage_names[dom]
    roof["traffic"] = ncu_traffic(w.name, stage_names[dom].split()[0])
    roof["stage_ms"] = {"psi_pack": ms_mx[0], "gemm_L_psi": ms_mx[1], "mpo_step": ms_mx[2],
                        "gemm_R_with_mpo_step": ms_mx[3]}
    roof["stage_gbs"] = [b / (t / 1e3) / 1e9 if t > 0 else 0.0 for b, t in zip(byts, ms_mx)]
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3 split products, f32 accumulate (f64 Krylov vectors)",
        "data": "synthetic (seeded random MPS with a Gaussian QN-sector model; environments "
                "by device environment updates)",
        "config": {"workload": w.name, "D": w.D, "sites": w.N, "bond": l,
                   "psi_elements": info["psi_size"], "mpo_bond_dim": mpo[l].indexes[3].dim,
                   "form": "mixed (tcgen05 split-BF16 block GEMMs)",
                   "tc_tiles_bn1_bn3": list(tiles[:2]),
                   "parallelism": "replicas only" if ws > 1 else "single GPU",
                   "l2": "flushed (512 MB write) before every timed step",
                   "plan_seconds": plan_s},
        "gpu_launches": launches,
        "e2e": {"value": e2e_val, "unit": "TFLOP/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "matches_device_result": e2e_same,
                "host_mapped": host_mapped_default, "by_host_mapped": e2e_modes},
        "roofline": roof,
        "plain_fp64": {"value": flops / t64 / 1e12, "unit": "TFLOP/s", "ms_per_step": t64 * 1e3,
                       "roofline": {"bound": "fp64", "peak": fp64_peak,
                                    "frac": flops / t64 / 1e12 / fp64_peak,
                                    "peak_source": "library DFMA probe (no FP64 entry in "
                                                   "MEASURED_PEAKS.json)"},
                       "stage_ms": ms_64},
        "speedup_mixed_vs_fp64": t64 / t_step,
        "anchor_matvec": anchor,
        "accuracy": {"matvec_rel_err_mixed_vs_fp64": mixed_err,
                     "lanczos_E_mixed": lz["mixed"][0], "lanczos_E_fp64": lz["fp64"][0],
                     "lanczos_iters": [lz["mixed"][1], lz["fp64"][1]],
                     "lanczos_rel_dE": abs(lz["mixed"][0] - lz["fp64"][0]) / abs(lz["fp64"][0])},
        "krylov_graph": kg,
        "krylov_vector_ops": kvec,
        "tile_autotuner": tune,
        "plan_build": plan_build,
        "centre_site_update": {
            k: {kk: v[kk] for kk in ("wall_sec", "lancz_sec", "svd_sec", "env_sec", "iters", "D",
                                     "trunc_err", "e0", "svd_grow_rounds")}
            for k, v in site.items()},
        "centre_site_update_speedup": {
            k: site["fp64_exact"]["wall_sec"] / site[k]["wall_sec"]
            for k in ("mixed_exact", "mixed_rsvd")},
        "svd_exact_vs_tight_sketch": svd_cmp,
        "centre_site_update_rel_dE": {
            k: abs(site[k]["e0"] - site["fp64_exact"]["e0"]) / abs(site["fp64_exact"]["e0"])
            for k in ("mixed_exact", "mixed_rsvd")},
        "clocks": clk.summary(),
        "wall_seconds_timed": wall,
    }
    if sweep is not None:
        fs = sweep["forms"]
        line["sweep_fp64_s"] = fs["fp64_exact"]["sweep_s"]
        line["sweep_mixed_s"] = fs["mixed_exact"]["sweep_s"]
        line["sweep_mixed_learned_s"] = fs["mixed_learned"]["sweep_s"]
        line["sweep_speedup_mixed_vs_fp64"] = fs["mixed_exact"]["speedup_vs_fp64"]
        line["sweep_speedup_mixed_learned_vs_fp64"] = fs["mixed_learned"]["speedup_vs_fp64"]
        line["sweep_rel_dE_mixed_vs_fp64"] = fs["mixed_exact"]["rel_dE_vs_fp64"]
        line["sweep_max_trunc_err_diff_mixed_vs_fp64"] = fs["mixed_exact"][
            "max_trunc_err_diff_vs_fp64"]
        line["sweep"] = sweep
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, w)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        tdist.barrier()
        tdist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
