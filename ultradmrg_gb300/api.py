"""Python mirror of the qlmps-facing API, over the C ABI.

Names and argument meaning follow the reference's entry points for the
two-site path (``LanczosSolver``, ``eff_ham_mul_two_site_state``,
``UpdateSiteLenvs/Renvs``, ``SVD``, ``TwoSiteFiniteVMPS``); the numerics run
in ``libudmrg_gb300.so`` on the GPU.  Host data are
:class:`~ultradmrg_gb300.tensor_data.BlockTensorData` objects.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import call
from .tensor_data import BlockTensorData, Index, from_packed

F64, C128 = 0, 1


class Context:
    """One GPU, one stream (``udmrg_ctx``)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        call("udmrg_ctx_create", device, C.byref(h))
        self.h = h

    def sync(self):
        call("udmrg_ctx_sync", self.h)

    def launches(self) -> int:
        v = C.c_uint64()
        call("udmrg_ctx_launches", self.h, C.byref(v))
        return int(v.value)

    def set_tc_tiles(self, bn1: int = 0, bn3: int = 0):
        """B-tile rows of the mixed matvec's two tcgen05 GEMMs (64 or 128), or
        0, 0 for the autotuner (the default)."""
        call("udmrg_ctx_set_tc_tiles", self.h, bn1, bn3)

    def tc_tuning(self):
        """(timed trials run, shape classes decided) of the tile autotuner."""
        t, c = C.c_int64(), C.c_int64()
        call("udmrg_ctx_tc_tuning", self.h, C.byref(t), C.byref(c))
        return t.value, c.value

    def set_gemm_tiles(self, policy: int = -1):
        """Tile policy of a matvec plan's FP64-accurate grouped GEMMs: 0 least
        padding, 1 fewer 32 x 32 tiles, -1 the autotuner (default)."""
        call("udmrg_ctx_set_gemm_tiles", self.h, int(policy))

    def gemm_tuning(self):
        """(timed trials run, shape classes decided) of the GEMM tile tuner."""
        t, c = C.c_int64(), C.c_int64()
        call("udmrg_ctx_gemm_tuning", self.h, C.byref(t), C.byref(c))
        return t.value, c.value

    def set_anchor_dw(self, dw: bool):
        """The mixed solver's FP64-accurate anchor matvec in double-word FP32
        arithmetic (default) or on the FP64 pipe."""
        call("udmrg_ctx_set_anchor_dw", self.h, 1 if dw else 0)

    def set_host_mapped(self, mode: int):
        """MatvecPlan.apply_host_ptr with page-locked, device-mapped host
        buffers (a mixed-precision plan): 0 copies both ways, 1 reads the
        input in place, 2 also writes the output in place."""
        call("udmrg_ctx_set_host_mapped", self.h, int(mode))

    def host_mapped(self) -> int:
        """The host-buffer mode of apply_host_ptr (see set_host_mapped)."""
        v = C.c_int()
        call("udmrg_ctx_host_mapped", self.h, C.byref(v))
        return v.value

    def profiler_range(self, start: bool):
        """Start or stop the CUDA profiler's collection after this context's
        work so far (for a profiler run with collection off at start)."""
        call("udmrg_ctx_profiler_range", self.h, 1 if start else 0)

    def set_krylov_graph(self, enable: bool):
        """Krylov steps as one CUDA graph replay each (default) or direct launches."""
        call("udmrg_ctx_set_krylov_graph", self.h, 1 if enable else 0)

    def event(self, slot: int):
        call("udmrg_ctx_event_record", self.h, slot)

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_float()
        call("udmrg_ctx_event_elapsed", self.h, a, b, C.byref(v))
        return float(v.value)

    def flush_l2(self, nbytes: int = 512 << 20):
        call("udmrg_ctx_flush_l2", self.h, int(nbytes))

    def fp64_peak_tflops(self) -> float:
        v = C.c_double()
        call("udmrg_probe_fp64_tflops", self.h, C.byref(v))
        return float(v.value)

    def krylov_step_probe(self, n: int, step: int) -> dict:
        """Device times and HBM bytes of one Krylov step's vector kernels at
        `step` on random vectors of n doubles."""
        ms, by, ran = (C.c_double * 5)(), (C.c_double * 5)(), C.c_int()
        call("udmrg_probe_krylov_step", self.h, int(n), int(step), ms, by, C.byref(ran))
        names = ("normalise", "alpha", "update", "reorth_pass1", "reorth_pass2")
        return {"ms": dict(zip(names, list(ms))), "bytes": dict(zip(names, list(by))),
                "second_pass_ran": bool(ran.value)}

    def close(self):
        if self.h:
            call("udmrg_ctx_destroy", self.h)
            self.h = None

    def __del__(self):
        if _lib.SHUTDOWN[0]:
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_lib.c_int32_p)


def _i64(a):
    a = np.ascontiguousarray(a, dtype=np.int64)
    return a, a.ctypes.data_as(_lib.c_int64_p)


class DeviceTensor:
    """Block-sparse tensor resident on the GPU (``udmrg_tensor``)."""

    def __init__(self, ctx: Context, handle: C.c_void_p):
        self.ctx = ctx
        self.h = handle

    @staticmethod
    def from_data(ctx: Context, t: BlockTensorData, dtype=None) -> "DeviceTensor":
        dtype = np.dtype(dtype or t.dtype)
        cplx = dtype == np.complex128
        nq = t.nq
        nsec, qns, dims, dirs = [], [], [], []
        for ind in t.indexes:
            nsec.append(ind.nsec)
            for q, d in zip(ind.qns, ind.dims):
                qns.extend(q)
                dims.append(d)
            dirs.append(ind.dir)
        keys = t.sorted_keys()
        a_nsec, p_nsec = _i32(nsec)
        a_qns, p_qns = _i32(qns if qns else [0])
        a_dims, p_dims = _i64(dims if dims else [1])
        a_dirs, p_dirs = _i32(dirs)
        a_keys, p_keys = _i32(np.array(keys, dtype=np.int32).ravel() if keys else [0])
        h = C.c_void_p()
        call("udmrg_tensor_create", ctx.h, C128 if cplx else F64, nq, t.rank, p_nsec, p_qns,
             p_dims, p_dirs, len(keys), p_keys, C.byref(h))
        dt = DeviceTensor(ctx, h)
        data = t.packed().astype(np.complex128 if cplx else np.float64)
        dt.upload_packed(data)
        return dt

    # --- metadata ---------------------------------------------------------
    def info(self):
        dt, nq, r = C.c_int(), C.c_int(), C.c_int()
        nb, sz = C.c_int64(), C.c_int64()
        call("udmrg_tensor_info", self.h, C.byref(dt), C.byref(nq), C.byref(r), C.byref(nb),
             C.byref(sz))
        return dict(dtype=dt.value, nq=nq.value, rank=r.value, nblocks=nb.value, size=sz.value)

    @property
    def is_complex(self):
        return self.info()["dtype"] == C128

    def indexes(self) -> List[Index]:
        inf = self.info()
        out = []
        for ax in range(inf["rank"]):
            ns, dr = C.c_int32(), C.c_int32()
            call("udmrg_tensor_index", self.h, ax, C.byref(ns), None, None, C.byref(dr))
            qns = np.zeros(max(ns.value * inf["nq"], 1), np.int32)
            dims = np.zeros(max(ns.value, 1), np.int64)
            call("udmrg_tensor_index", self.h, ax, None, qns.ctypes.data_as(_lib.c_int32_p),
                 dims.ctypes.data_as(_lib.c_int64_p), None)
            q = qns[:ns.value * inf["nq"]].reshape(ns.value, inf["nq"])
            out.append(Index(tuple(tuple(int(v) for v in row) for row in q),
                             tuple(int(d) for d in dims[:ns.value]), int(dr.value)))
        return out

    def keys(self):
        inf = self.info()
        k = np.zeros(max(inf["nblocks"] * inf["rank"], 1), np.int32)
        call("udmrg_tensor_keys", self.h, k.ctypes.data_as(_lib.c_int32_p))
        return [tuple(int(v) for v in row) for row in
                k[:inf["nblocks"] * inf["rank"]].reshape(inf["nblocks"], inf["rank"])]

    def upload_packed(self, data: np.ndarray):
        buf = np.ascontiguousarray(data)
        if buf.dtype == np.complex128:
            buf = buf.view(np.float64)
        call("udmrg_tensor_upload", self.h, buf.ctypes.data_as(_lib.c_double_p))

    def download_packed(self) -> np.ndarray:
        inf = self.info()
        n = inf["size"] * (2 if inf["dtype"] == C128 else 1)
        buf = np.zeros(max(n, 1), np.float64)
        call("udmrg_tensor_download", self.h, buf.ctypes.data_as(_lib.c_double_p))
        buf = buf[:n]
        return buf.view(np.complex128) if inf["dtype"] == C128 else buf

    def to_data(self) -> BlockTensorData:
        dtype = np.complex128 if self.is_complex else np.float64
        return from_packed(self.indexes(), self.keys(), self.download_packed(), dtype)

    def norm(self) -> float:
        v = C.c_double()
        call("udmrg_tensor_norm", self.ctx.h, self.h, C.byref(v))
        return float(v.value)

    def scale_(self, alpha: float) -> "DeviceTensor":
        call("udmrg_tensor_scale", self.ctx.h, self.h, float(alpha))
        return self

    def device_ptr(self) -> int:
        p = _lib.c_double_p()
        call("udmrg_tensor_device_ptr", self.h, C.byref(p))
        return C.cast(p, C.c_void_p).value or 0

    def close(self):
        if self.h:
            call("udmrg_tensor_destroy", self.h)
            self.h = None

    def __del__(self):
        if _lib.SHUTDOWN[0]:
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def _handles(ts: Sequence[DeviceTensor]):
    arr = (C.c_void_p * len(ts))(*[t.h.value if isinstance(t.h, C.c_void_p) else t.h for t in ts])
    return arr


def _new(ctx, h):
    return DeviceTensor(ctx, h)


# --- block-sparse operations ---------------------------------------------------

def contract(ctx, a: DeviceTensor, b: DeviceTensor, axes_a, axes_b) -> DeviceTensor:
    xa, pa = _i32(axes_a)
    xb, pb = _i32(axes_b)
    h = C.c_void_p()
    call("udmrg_contract", ctx.h, a.h, b.h, len(axes_a), pa, pb, C.byref(h))
    return _new(ctx, h)


def contract_cyclic(ctx, a, b, a_start, b_start, n) -> DeviceTensor:
    h = C.c_void_p()
    call("udmrg_contract_cyclic", ctx.h, a.h, b.h, a_start, b_start, n, C.byref(h))
    return _new(ctx, h)


def dag(ctx, a) -> DeviceTensor:
    h = C.c_void_p()
    call("udmrg_dag", ctx.h, a.h, C.byref(h))
    return _new(ctx, h)


# --- hot path ------------------------------------------------------------------

def eff_ham_mul_two_site_state(ctx, eff_ham: Sequence[DeviceTensor], state: DeviceTensor):
    h = C.c_void_p()
    call("udmrg_eff_ham_mul_two_site_state", ctx.h, _handles(eff_ham), state.h, C.byref(h))
    return _new(ctx, h)


@dataclass
class LanczosResult:
    iters: int
    gs_eng: float
    gs_vec: DeviceTensor
    matvec_seconds: float
    matvecs: int
    ritz_eng: float = 0.0
    fp64_matvecs: int = 0


PREC_FP64, PREC_MIXED = 0, 1


def lanczos_solver(ctx, eff_ham, init_state, error=1e-7, max_iterations=200,
                   precision=PREC_FP64) -> LanczosResult:
    p = _lib.LanczosParams(error, max_iterations, precision)
    r = _lib.LanczosRes()
    call("udmrg_lanczos_solver", ctx.h, _handles(eff_ham), init_state.h, C.byref(p), C.byref(r))
    return LanczosResult(int(r.iters), float(r.gs_eng), _new(ctx, C.c_void_p(r.gs_vec)),
                         float(r.matvec_seconds), int(r.matvecs), float(r.ritz_eng),
                         int(r.fp64_matvecs))


def eff_ham_mul_single_site_state(ctx, eff_ham: Sequence[DeviceTensor], state: DeviceTensor):
    """``eff_ham_mul_single_site_state`` (eff_ham = [L, W, R]) on the device."""
    h = C.c_void_p()
    call("udmrg_eff_ham_mul_single_site_state", ctx.h, _handles(eff_ham), state.h, C.byref(h))
    return _new(ctx, h)


def lanczos_expmv_solver(ctx, eff_ham, init_state, step, error=1e-10, max_iterations=20,
                         precision=PREC_FP64):
    p = _lib.LanczosParams(error, max_iterations, precision)
    it = C.c_int64()
    h = C.c_void_p()
    call("udmrg_lanczos_expmv_solver", ctx.h, _handles(eff_ham), init_state.h, step, C.byref(p),
         C.byref(it), C.byref(h))
    return int(it.value), _new(ctx, h)


def update_site_lenvs(ctx, lenv, mps_ten, mpo_ten) -> DeviceTensor:
    h = C.c_void_p()
    call("udmrg_update_site_lenvs", ctx.h, lenv.h, mps_ten.h, mpo_ten.h, C.byref(h))
    return _new(ctx, h)


def update_site_renvs(ctx, renv, mps_ten, mpo_ten) -> DeviceTensor:
    h = C.c_void_p()
    call("udmrg_update_site_renvs", ctx.h, renv.h, mps_ten.h, mpo_ten.h, C.byref(h))
    return _new(ctx, h)


SVD_FULL, SVD_SPLIT_LEFT, SVD_SPLIT_RIGHT = 0, 1, 2


def svd(ctx, t, ldims, ldiv, trunc_err, Dmin, Dmax, mode=SVD_FULL):
    xd, pd = _i32(list(ldiv))
    u, s, vt = C.c_void_p(), C.c_void_p(), C.c_void_p()
    err, D = C.c_double(), C.c_int64()
    call("udmrg_svd", ctx.h, t.h, ldims, pd, trunc_err, Dmin, Dmax, mode, C.byref(u), C.byref(s),
         C.byref(vt), C.byref(err), C.byref(D))
    return _new(ctx, u), _new(ctx, s), _new(ctx, vt), float(err.value), int(D.value)


def svd_randomized(ctx, t, ldims, ldiv, trunc_err, Dmin, Dmax, sketch, mode=SVD_FULL,
                   oversample=8, power_iters=4, seed=1):
    """Sector-wise randomized SVD; ``sketch`` = [(bond QN tuple, sketch size), ...]."""
    xd, pd = _i32(list(ldiv))
    qns = [v for q, _ in sketch for v in q] or [0]
    xq, pq = _i32(qns)
    xs, ps = _i64([k for _, k in sketch] or [0])
    u, s, vt = C.c_void_p(), C.c_void_p(), C.c_void_p()
    err, D, gr = C.c_double(), C.c_int64(), C.c_int64()
    call("udmrg_svd_randomized", ctx.h, t.h, ldims, pd, trunc_err, Dmin, Dmax, mode,
         len(sketch), pq, ps, oversample, power_iters, seed, C.byref(u), C.byref(s),
         C.byref(vt), C.byref(err), C.byref(D), C.byref(gr))
    return (_new(ctx, u), _new(ctx, s), _new(ctx, vt), float(err.value), int(D.value),
            int(gr.value))


@dataclass
class FiniteVMPSSweepParams:
    """``FiniteVMPSSweepParams`` (sweeps, Dmin, Dmax, trunc_err, Lanczos params)."""

    sweeps: int
    Dmin: int
    Dmax: int
    trunc_err: float
    lanczos_error: float = 1e-7
    lanczos_max_iterations: int = 200
    precision: int = 0  # matvec precision: 0 FP64, 1 mixed (split-BF16 tensor cores)
    svd_mode: int = 0  # 0 exact, 1 randomized (previous sector dims), 2 randomized (learned)
    svd_oversample: int = 8
    svd_audit: bool = False  # exact SVD judges every randomized one (untimed)
    svd_sketch_max_fraction: float = 1.0  # randomized SVD only below this sketch fraction


def _sweep_params(params: FiniteVMPSSweepParams):
    return _lib.SweepParams(params.sweeps, params.Dmin, params.Dmax, params.trunc_err,
                            _lib.LanczosParams(params.lanczos_error,
                                               params.lanczos_max_iterations, params.precision),
                            params.svd_mode, params.svd_oversample, int(params.svd_audit),
                            params.svd_sketch_max_fraction)


def _log_rows(log, n):
    rows = []
    for i in range(n):
        L = log[i]
        rows.append(dict(site=L.site, e0=L.e0, trunc_err=L.trunc_err, D=L.D, iters=L.iters,
                         ee=L.ee, lancz_sec=L.lancz_sec, svd_sec=L.svd_sec, env_sec=L.env_sec,
                         tot_sec=L.tot_sec, matvec_flops=L.matvec_flops,
                         svd_sketch_total=L.svd_sketch_total,
                         svd_grow_rounds=L.svd_grow_rounds, svd_audit_err=L.svd_audit_err,
                         svd_audit_kept_diff=L.svd_audit_kept_diff, plan_sec=L.plan_sec))
    return rows


def two_site_finite_vmps_noise(ctx, mps: List[DeviceTensor], mpo: List[DeviceTensor],
                               params: FiniteVMPSSweepParams, noises: Sequence[float],
                               noise_decrease=0.95, noise_increase=1.02, max_noise=1.0,
                               alpha=0.3):
    """``TwoSiteFiniteVMPSWithNoise``: updates ``mps`` in place (centre at site 0
    on entry), returns (e0, per-site log, noise applied at each update)."""
    N = len(mps)
    sp = _sweep_params(params)
    arr = (C.c_double * max(1, len(noises)))(*noises)
    npar = _lib.NoiseParams(C.cast(arr, _lib.c_double_p), len(noises), noise_decrease,
                            noise_increase, max_noise, alpha)
    cap = 2 * N * max(params.sweeps, 1)
    log = (_lib.SiteLog * cap)()
    nlog_arr = (C.c_double * cap)()
    e0 = C.c_double()
    nlog = C.c_int64()
    call("udmrg_two_site_finite_vmps_noise", ctx.h, N, _handles(mps), _handles(mpo), C.byref(sp),
         C.byref(npar), C.byref(e0), log, cap, C.byref(nlog), nlog_arr)
    n = min(cap, nlog.value)
    return float(e0.value), _log_rows(log, n), [float(nlog_arr[i]) for i in range(n)]


def two_site_finite_vmps(ctx, mps: List[DeviceTensor], mpo: List[DeviceTensor],
                         params: FiniteVMPSSweepParams):
    """``TwoSiteFiniteVMPS``: updates ``mps`` in place, returns (e0, per-site log)."""
    N = len(mps)
    sp = _sweep_params(params)
    cap = 2 * N * max(params.sweeps, 1)
    log = (_lib.SiteLog * cap)()
    e0 = C.c_double()
    nlog = C.c_int64()
    call("udmrg_two_site_finite_vmps", ctx.h, N, _handles(mps), _handles(mpo), C.byref(sp),
         C.byref(e0), log, cap, C.byref(nlog))
    return float(e0.value), _log_rows(log, min(cap, nlog.value))


class RankModel:
    """The learned rank predictor (``udmrg_rank_model``): a 68-128-1 ReLU MLP
    mapping a bond sector's previous spectrum to log2(1 + kept states) there."""

    def __init__(self, ctx, seed: int = 0):
        n_in, n_hid, n_par = C.c_int(), C.c_int(), C.c_int()
        call("udmrg_rank_model_sizes", C.byref(n_in), C.byref(n_hid), C.byref(n_par))
        self.n_in, self.n_hidden, self.n_params = n_in.value, n_hid.value, n_par.value
        h = C.c_void_p()
        call("udmrg_rank_model_create", ctx.h, int(seed), C.byref(h))
        self.ctx, self.h = ctx, h

    @staticmethod
    def _f32(a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        return a, a.ctypes.data_as(_lib.c_float_p)

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        call("udmrg_rank_model_get_params", self.h, out.ctypes.data_as(_lib.c_float_p))
        return out

    @params.setter
    def params(self, p):
        p, pp = self._f32(p)
        if p.size != self.n_params:
            raise ValueError(f"rank model: expected {self.n_params} parameters, got {p.size}")
        call("udmrg_rank_model_set_params", self.h, pp)

    def predict(self, x) -> np.ndarray:
        x, xp = self._f32(x)
        n = x.shape[0]
        y = np.empty(n, np.float32)
        call("udmrg_rank_model_predict", self.h, n, xp, y.ctypes.data_as(_lib.c_float_p))
        return y

    def loss_grad(self, x, t):
        x, xp = self._f32(x)
        t, tp = self._f32(t)
        loss = C.c_float()
        g = np.empty(self.n_params, np.float32)
        call("udmrg_rank_model_loss_grad", self.h, x.shape[0], xp, tp, C.byref(loss),
             g.ctypes.data_as(_lib.c_float_p))
        return float(loss.value), g

    def train(self, x, t, epochs=200, batch=256, lr=1e-3, seed=0) -> float:
        x, xp = self._f32(x)
        t, tp = self._f32(t)
        loss = C.c_float()
        call("udmrg_rank_model_train", self.h, x.shape[0], xp, tp, int(epochs), int(batch),
             float(lr), int(seed), C.byref(loss))
        return float(loss.value)

    def forget(self):
        """Drop the bond history of the last chain swept with this model."""
        call("udmrg_rank_model_forget", self.h)

    def copy_history_from(self, other: "RankModel"):
        """Take a copy of another model's bond history."""
        call("udmrg_rank_model_copy_history", self.h, other.h)

    def close(self):
        if self.h:
            call("udmrg_rank_model_destroy", self.h)
            self.h = None

    def __del__(self):
        if _lib.SHUTDOWN[0]:
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def two_site_finite_vmps_learned(ctx, mps: List[DeviceTensor], mpo: List[DeviceTensor],
                                 params: FiniteVMPSSweepParams,
                                 model: Optional[RankModel] = None, record: bool = False,
                                 cap: int = 1 << 16):
    """``TwoSiteFiniteVMPS`` with learned truncation.  With ``svd_mode == 2``
    the sketch size of every bond sector comes from ``model``; with ``record``
    the sweep also returns training samples (features, log2(1 + kept)).
    The model keeps each bond's last spectrum across calls (a schedule of
    sweeps with growing Dmax); ``record`` needs a model (it may be untrained).
    Returns (e0, per-site log, x, y)."""
    N = len(mps)
    sp = _sweep_params(params)
    lcap = 2 * N * max(params.sweeps, 1)
    log = (_lib.SiteLog * lcap)()
    e0 = C.c_double()
    nlog = C.c_int64()
    n_in = C.c_int()
    call("udmrg_rank_model_sizes", C.byref(n_in), None, None)
    xs = np.zeros((cap if record else 0, n_in.value), np.float32)
    ys = np.zeros(cap if record else 0, np.float32)
    ns = C.c_int64()
    call("udmrg_two_site_finite_vmps_learned", ctx.h, N, _handles(mps), _handles(mpo),
         C.byref(sp), model.h if model is not None else None, int(record),
         xs.ctypes.data_as(_lib.c_float_p) if record else None,
         ys.ctypes.data_as(_lib.c_float_p) if record else None, cap if record else 0,
         C.byref(ns), C.byref(e0), log, lcap, C.byref(nlog))
    n = min(ns.value, xs.shape[0])
    return float(e0.value), _log_rows(log, min(lcap, nlog.value)), xs[:n], ys[:n]


def finite_dmrg(ctx, mps: List[DeviceTensor], mat_repr, params: FiniteVMPSSweepParams):
    """``FiniteDMRG(mps, mat_repr_mpo, sweep_params)``: ``mat_repr`` is a
    MatReprMPO as returned by ``models.mat_repr_mpo`` (per site rows, cols and
    the (x, y, operator tensor) elements).  Updates ``mps`` in place; returns
    (e0, per-site log)."""
    N = len(mps)
    keep, sites = [], (_lib.MatReprSite * N)()
    for i, (rows, cols, elems) in enumerate(mat_repr):
        ops = [DeviceTensor.from_data(ctx, t) for _, _, t in elems]
        xs = np.array([x for x, _, _ in elems], np.int64)
        ys = np.array([y for _, y, _ in elems], np.int64)
        hs = _handles(ops)
        keep += [ops, xs, ys, hs]
        sites[i] = _lib.MatReprSite(rows, cols, len(elems), xs.ctypes.data_as(_lib.c_int64_p),
                                    ys.ctypes.data_as(_lib.c_int64_p), hs)
    sp = _sweep_params(params)
    cap = 2 * N * max(params.sweeps, 1)
    log = (_lib.SiteLog * cap)()
    e0, nlog = C.c_double(), C.c_int64()
    call("udmrg_finite_dmrg", ctx.h, N, _handles(mps), sites, C.byref(sp), C.byref(e0), log, cap,
         C.byref(nlog))
    return float(e0.value), _log_rows(log, min(cap, nlog.value))


@dataclass
class TDVPEvolveParams:
    """The time-stepping part of ``TDVPEvolveParams`` (tdvp_evolve_params.h:20-85)."""

    tau: float
    steps: int
    Dmin: int
    Dmax: int
    trunc_err: float
    lanczos_error: float = 1e-10
    lanczos_max_iterations: int = 20
    precision: int = 0  # two-site Krylov matvec: 0 FP64, 1 mixed (split-BF16 tensor cores)


def two_site_finite_tdvp(ctx, mps: List[DeviceTensor], mpo: List[DeviceTensor],
                         params: TDVPEvolveParams):
    """``TwoSiteFiniteTDVP`` time stepping: right-canonicalises ``mps`` (centre
    at site 0), then ``params.steps`` sweeps; ``mps`` is updated in place
    (complex).  Returns the per-update log."""
    N = len(mps)
    tp = _lib.TdvpParams(params.tau, params.steps, params.Dmin, params.Dmax, params.trunc_err,
                         _lib.LanczosParams(params.lanczos_error, params.lanczos_max_iterations,
                                            params.precision))
    cap = max(1, params.steps) * (4 * N)
    log = (_lib.TdvpLog * cap)()
    nlog = C.c_int64()
    call("udmrg_two_site_finite_tdvp", ctx.h, N, _handles(mps), _handles(mpo), C.byref(tp), log,
         cap, C.byref(nlog))
    rows = []
    for i in range(min(cap, nlog.value)):
        L = log[i]
        rows.append(dict(step=L.step, site=L.site, kind=L.kind, trunc_err=L.trunc_err, D=L.D,
                         iters=L.iters, ee=L.ee, lancz_sec=L.lancz_sec, tot_sec=L.tot_sec))
    return rows


def trivial_env_data(mps_ten: BlockTensorData, mpo_ten: BlockTensorData, side: str):
    """The 1x1x1 boundary environment of ``InitEnvs``
    (``two_site_update_finite_vmps_impl.h:157-186``): (mps bond, inverse MPO
    bond, inverse mps bond) with element 1."""
    if side == "l":
        i0, iw = mps_ten.indexes[0], mpo_ten.indexes[0].inverse()
    else:
        i0, iw = mps_ten.indexes[2], mpo_ten.indexes[3].inverse()
    t = BlockTensorData([i0, iw, i0.inverse()], {}, np.result_type(mps_ten.dtype, mpo_ten.dtype))
    t.set_elem((0, 0, 0), 1.0)
    return t


def build_envs(ctx, mpo: Sequence[BlockTensorData], mps: Sequence[BlockTensorData], l: int,
               normalize: bool = True):
    """Left environment of sites [0, l) and right environment of sites (l+1, N)
    by device environment updates (each one normalised when ``normalize``)."""
    N = len(mps)
    L = DeviceTensor.from_data(ctx, trivial_env_data(mps[0], mpo[0], "l"))
    for i in range(l):
        nxt = update_site_lenvs(ctx, L, DeviceTensor.from_data(ctx, mps[i]),
                                DeviceTensor.from_data(ctx, mpo[i]))
        L.close()
        L = nxt
        if normalize:
            L.scale_(1.0 / max(L.norm(), 1e-300))
    R = DeviceTensor.from_data(ctx, trivial_env_data(mps[N - 1], mpo[N - 1], "r"))
    for i in range(N - 1, l + 1, -1):
        nxt = update_site_renvs(ctx, R, DeviceTensor.from_data(ctx, mps[i]),
                                DeviceTensor.from_data(ctx, mpo[i]))
        R.close()
        R = nxt
        if normalize:
            R.scale_(1.0 / max(R.norm(), 1e-300))
    return L, R


def two_site_update(ctx, lenv, renv, mps_l, mps_r, mpo_l, mpo_r,
                    params: FiniteVMPSSweepParams, dir: str = "r"):
    """``TwoSiteFiniteVMPSUpdate`` on one bond: (new_l, new_r, new_env, log)."""
    sp = _sweep_params(params)
    sp.sweeps = 1
    a, b, e = C.c_void_p(), C.c_void_p(), C.c_void_p()
    lg = _lib.SiteLog()
    call("udmrg_two_site_update", ctx.h, lenv.h, renv.h, mps_l.h, mps_r.h, mpo_l.h, mpo_r.h,
         C.byref(sp), dir.encode(), C.byref(a), C.byref(b), C.byref(e), C.byref(lg))
    log = _log_rows([lg], 1)[0]
    return _new(ctx, a), _new(ctx, b), _new(ctx, e), log


class MatvecPlan:
    """Reusable H_eff * psi on device buffers (``udmrg_matvec_plan``)."""

    def __init__(self, ctx, eff_ham, psi_struct, precision=PREC_FP64):
        self.ctx = ctx
        h = C.c_void_p()
        call("udmrg_matvec_plan_create_ex", ctx.h, _handles(eff_ham), psi_struct.h, precision,
             C.byref(h))
        self.h = h

    def info(self):
        f, n, w = C.c_double(), C.c_int64(), C.c_int64()
        call("udmrg_matvec_plan_info", self.h, C.byref(f), C.byref(n), C.byref(w))
        return dict(flops=f.value, psi_size=n.value, workspace_bytes=w.value)

    def embed(self, t: DeviceTensor) -> DeviceTensor:
        h = C.c_void_p()
        call("udmrg_matvec_plan_embed", self.h, t.h, C.byref(h))
        return _new(self.ctx, h)

    def apply_ptr(self, d_in: int, d_out: int):
        call("udmrg_matvec_plan_apply", self.h, C.cast(C.c_void_p(d_in), _lib.c_double_p),
             C.cast(C.c_void_p(d_out), _lib.c_double_p))

    def apply(self, x: DeviceTensor, y: DeviceTensor):
        self.apply_ptr(x.device_ptr(), y.device_ptr())

    def apply_host_ptr(self, h_in: int, h_out: int):
        """H_eff * psi with host buffers (addresses of packed FP64 arrays)."""
        call("udmrg_matvec_plan_apply_host", self.h, C.cast(C.c_void_p(h_in), _lib.c_double_p),
             C.cast(C.c_void_p(h_out), _lib.c_double_p))

    def apply_anchor_ptr(self, d_in: int, d_out: int):
        call("udmrg_matvec_plan_apply_anchor", self.h,
             C.cast(C.c_void_p(d_in), _lib.c_double_p), C.cast(C.c_void_p(d_out), _lib.c_double_p))

    def apply_anchor(self, x: DeviceTensor, y: DeviceTensor):
        """The mixed solver's FP64-accurate anchor product (FP64 pipe or
        double-word FP32, per ``Context.set_anchor_dw``)."""
        self.apply_anchor_ptr(x.device_ptr(), y.device_ptr())

    def stage_times(self, d_in: int, d_out: int):
        """(ms[4], flops[4]) of one matvec, CUDA events between the stages."""
        ms = (C.c_double * 4)()
        fl = (C.c_double * 4)()
        call("udmrg_matvec_plan_stage_times", self.h, C.cast(C.c_void_p(d_in), _lib.c_double_p),
             C.cast(C.c_void_p(d_out), _lib.c_double_p), ms, fl)
        return list(ms), list(fl)

    def tiles(self):
        """Mixed form: (bn1, bn3, chosen by the autotuner)."""
        a, b, t = C.c_int(), C.c_int(), C.c_int()
        call("udmrg_matvec_plan_tiles", self.h, C.byref(a), C.byref(b), C.byref(t))
        return a.value, b.value, bool(t.value)

    def gemm_policy(self) -> int:
        """Tile policy of the plan's FP64-accurate grouped GEMMs (0 or 1)."""
        v = C.c_int()
        call("udmrg_matvec_plan_gemm_policy", self.h, C.byref(v))
        return v.value

    PLAN_PHASES = ("closure", "host_tables", "uploads", "mixed_tables",
                   "mixed_device", "tile_tuning")

    def build_times(self) -> dict:
        """Host seconds of the plan's construction, by phase."""
        v = (C.c_double * 6)()
        call("udmrg_matvec_plan_build_times", self.h, v)
        return dict(zip(self.PLAN_PHASES, list(v)))

    def set_fused(self, enable: bool):
        """Mixed form: MPO step inside the .R GEMM's producers or as its own
        kernel (the default; bit-identical results)."""
        call("udmrg_matvec_plan_set_fused", self.h, 1 if enable else 0)

    def stage_bytes(self):
        """Algorithmic HBM bytes of the mixed form's memory-bound stages."""
        b = (C.c_double * 4)()
        call("udmrg_matvec_plan_stage_bytes", self.h, b)
        return list(b)

    def close(self):
        if self.h:
            call("udmrg_matvec_plan_destroy", self.h)
            self.h = None

    def __del__(self):
        if _lib.SHUTDOWN[0]:
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass
