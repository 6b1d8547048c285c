"""ctypes binding of ``include/ultradmrg_gb300.h`` (the C ABI).

The library is the in-tree ``libudmrg_gb300.so``; there is no fallback: if it
is missing or does not load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libudmrg_gb300.so")

c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)
c_void_pp = C.POINTER(C.c_void_p)


class LanczosParams(C.Structure):
    _fields_ = [("error", C.c_double), ("max_iterations", C.c_int64),
                ("matvec_precision", C.c_int64)]


class LanczosRes(C.Structure):
    _fields_ = [("iters", C.c_int64), ("gs_eng", C.c_double), ("gs_vec", C.c_void_p),
                ("matvec_seconds", C.c_double), ("matvecs", C.c_int64),
                ("ritz_eng", C.c_double), ("fp64_matvecs", C.c_int64)]


class SweepParams(C.Structure):
    _fields_ = [("sweeps", C.c_int64), ("Dmin", C.c_int64), ("Dmax", C.c_int64),
                ("trunc_err", C.c_double), ("lancz_params", LanczosParams),
                ("svd_mode", C.c_int64), ("svd_oversample", C.c_int64),
                ("svd_audit", C.c_int64), ("svd_sketch_max_fraction", C.c_double)]


class NoiseParams(C.Structure):
    _fields_ = [("noises", c_double_p), ("n_noises", C.c_int64), ("noise_decrease", C.c_double),
                ("noise_increase", C.c_double), ("max_noise", C.c_double), ("alpha", C.c_double)]


class SiteLog(C.Structure):
    _fields_ = [("site", C.c_int64), ("e0", C.c_double), ("trunc_err", C.c_double),
                ("D", C.c_int64), ("iters", C.c_int64), ("ee", C.c_double),
                ("lancz_sec", C.c_double), ("svd_sec", C.c_double), ("env_sec", C.c_double),
                ("tot_sec", C.c_double), ("matvec_flops", C.c_double),
                ("svd_sketch_total", C.c_int64), ("svd_grow_rounds", C.c_int64),
                ("svd_audit_err", C.c_double), ("svd_audit_kept_diff", C.c_int64),
                ("plan_sec", C.c_double)]


class TdvpParams(C.Structure):
    _fields_ = [("tau", C.c_double), ("steps", C.c_int64), ("Dmin", C.c_int64),
                ("Dmax", C.c_int64), ("trunc_err", C.c_double), ("lancz_params", LanczosParams)]


class TdvpLog(C.Structure):
    _fields_ = [("step", C.c_int64), ("site", C.c_int64), ("kind", C.c_int64),
                ("trunc_err", C.c_double), ("D", C.c_int64), ("iters", C.c_int64),
                ("ee", C.c_double), ("lancz_sec", C.c_double), ("tot_sec", C.c_double)]


class MatReprSite(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("nnz", C.c_int64),
                ("x", c_int64_p), ("y", c_int64_p), ("ops", c_void_pp)]


# name -> argtypes (all return int status)
SIGNATURES = {
    "udmrg_ctx_create": [C.c_int, c_void_pp],
    "udmrg_ctx_destroy": [C.c_void_p],
    "udmrg_ctx_sync": [C.c_void_p],
    "udmrg_ctx_launches": [C.c_void_p, C.POINTER(C.c_uint64)],
    "udmrg_ctx_set_krylov_graph": [C.c_void_p, C.c_int],
    "udmrg_ctx_set_tc_tiles": [C.c_void_p, C.c_int, C.c_int],
    "udmrg_ctx_tc_tuning": [C.c_void_p, c_int64_p, c_int64_p],
    "udmrg_ctx_profiler_range": [C.c_void_p, C.c_int],
    "udmrg_ctx_set_gemm_tiles": [C.c_void_p, C.c_int],
    "udmrg_ctx_gemm_tuning": [C.c_void_p, c_int64_p, c_int64_p],
    "udmrg_ctx_set_anchor_dw": [C.c_void_p, C.c_int],
    "udmrg_ctx_set_host_mapped": [C.c_void_p, C.c_int],
    "udmrg_ctx_host_mapped": [C.c_void_p, C.POINTER(C.c_int)],
    "udmrg_tensor_create": [C.c_void_p, C.c_int, C.c_int, C.c_int, c_int32_p, c_int32_p,
                            c_int64_p, c_int32_p, C.c_int64, c_int32_p, c_void_pp],
    "udmrg_tensor_destroy": [C.c_void_p],
    "udmrg_tensor_info": [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                          C.POINTER(C.c_int), c_int64_p, c_int64_p],
    "udmrg_tensor_index": [C.c_void_p, C.c_int, c_int32_p, c_int32_p, c_int64_p, c_int32_p],
    "udmrg_tensor_keys": [C.c_void_p, c_int32_p],
    "udmrg_tensor_upload": [C.c_void_p, c_double_p],
    "udmrg_tensor_download": [C.c_void_p, c_double_p],
    "udmrg_tensor_device_ptr": [C.c_void_p, C.POINTER(c_double_p)],
    "udmrg_tensor_norm": [C.c_void_p, C.c_void_p, c_double_p],
    "udmrg_tensor_scale": [C.c_void_p, C.c_void_p, C.c_double],
    "udmrg_contract": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, c_int32_p, c_int32_p,
                       c_void_pp],
    "udmrg_contract_cyclic": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                              c_void_pp],
    "udmrg_dag": [C.c_void_p, C.c_void_p, c_void_pp],
    "udmrg_eff_ham_mul_two_site_state": [C.c_void_p, c_void_pp, C.c_void_p, c_void_pp],
    "udmrg_eff_ham_mul_single_site_state": [C.c_void_p, c_void_pp, C.c_void_p, c_void_pp],
    "udmrg_finite_dmrg": [C.c_void_p, C.c_int64, c_void_pp, C.POINTER(MatReprSite),
                          C.POINTER(SweepParams), c_double_p, C.POINTER(SiteLog), C.c_int64,
                          c_int64_p],
    "udmrg_two_site_finite_tdvp": [C.c_void_p, C.c_int64, c_void_pp, c_void_pp,
                                   C.POINTER(TdvpParams), C.POINTER(TdvpLog), C.c_int64,
                                   c_int64_p],
    "udmrg_lanczos_solver": [C.c_void_p, c_void_pp, C.c_void_p, C.POINTER(LanczosParams),
                             C.POINTER(LanczosRes)],
    "udmrg_lanczos_expmv_solver": [C.c_void_p, c_void_pp, C.c_void_p, C.c_double,
                                   C.POINTER(LanczosParams), c_int64_p, c_void_pp],
    "udmrg_update_site_lenvs": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, c_void_pp],
    "udmrg_update_site_renvs": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, c_void_pp],
    "udmrg_svd": [C.c_void_p, C.c_void_p, C.c_int, c_int32_p, C.c_double, C.c_int64, C.c_int64,
                  C.c_int, c_void_pp, c_void_pp, c_void_pp, c_double_p, c_int64_p],
    "udmrg_svd_randomized": [C.c_void_p, C.c_void_p, C.c_int, c_int32_p, C.c_double, C.c_int64,
                             C.c_int64, C.c_int, C.c_int64, c_int32_p, c_int64_p, C.c_int64,
                             C.c_int, C.c_uint64, c_void_pp, c_void_pp, c_void_pp, c_double_p,
                             c_int64_p, c_int64_p],
    "udmrg_two_site_update": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.POINTER(SweepParams), C.c_char,
                              c_void_pp, c_void_pp, c_void_pp, C.POINTER(SiteLog)],
    "udmrg_two_site_finite_vmps": [C.c_void_p, C.c_int64, c_void_pp, c_void_pp,
                                   C.POINTER(SweepParams), c_double_p, C.POINTER(SiteLog),
                                   C.c_int64, c_int64_p],
    "udmrg_two_site_finite_vmps_learned": [C.c_void_p, C.c_int64, c_void_pp, c_void_pp,
                                           C.POINTER(SweepParams), C.c_void_p, C.c_int,
                                           c_float_p, c_float_p, C.c_int64, c_int64_p,
                                           c_double_p, C.POINTER(SiteLog), C.c_int64,
                                           c_int64_p],
    "udmrg_two_site_finite_vmps_noise": [C.c_void_p, C.c_int64, c_void_pp, c_void_pp,
                                         C.POINTER(SweepParams), C.POINTER(NoiseParams),
                                         c_double_p, C.POINTER(SiteLog), C.c_int64, c_int64_p,
                                         c_double_p],
    "udmrg_rank_model_sizes": [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "udmrg_rank_model_create": [C.c_void_p, C.c_uint64, c_void_pp],
    "udmrg_rank_model_destroy": [C.c_void_p],
    "udmrg_rank_model_forget": [C.c_void_p],
    "udmrg_rank_model_copy_history": [C.c_void_p, C.c_void_p],
    "udmrg_rank_model_get_params": [C.c_void_p, c_float_p],
    "udmrg_rank_model_set_params": [C.c_void_p, c_float_p],
    "udmrg_rank_model_predict": [C.c_void_p, C.c_int64, c_float_p, c_float_p],
    "udmrg_rank_model_loss_grad": [C.c_void_p, C.c_int64, c_float_p, c_float_p, c_float_p,
                                   c_float_p],
    "udmrg_rank_model_train": [C.c_void_p, C.c_int64, c_float_p, c_float_p, C.c_int, C.c_int,
                               C.c_float, C.c_uint64, c_float_p],
    "udmrg_matvec_plan_create": [C.c_void_p, c_void_pp, C.c_void_p, c_void_pp],
    "udmrg_matvec_plan_create_ex": [C.c_void_p, c_void_pp, C.c_void_p, C.c_int, c_void_pp],
    "udmrg_matvec_plan_info": [C.c_void_p, c_double_p, c_int64_p, c_int64_p],
    "udmrg_matvec_plan_embed": [C.c_void_p, C.c_void_p, c_void_pp],
    "udmrg_matvec_plan_apply": [C.c_void_p, c_double_p, c_double_p],
    "udmrg_matvec_plan_apply_anchor": [C.c_void_p, c_double_p, c_double_p],
    "udmrg_matvec_plan_apply_host": [C.c_void_p, c_double_p, c_double_p],
    "udmrg_matvec_plan_destroy": [C.c_void_p],
    "udmrg_matvec_plan_stage_times": [C.c_void_p, c_double_p, c_double_p, c_double_p,
                                      c_double_p],
    "udmrg_matvec_plan_stage_bytes": [C.c_void_p, c_double_p],
    "udmrg_matvec_plan_set_fused": [C.c_void_p, C.c_int],
    "udmrg_matvec_plan_tiles": [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int)],
    "udmrg_matvec_plan_gemm_policy": [C.c_void_p, C.POINTER(C.c_int)],
    "udmrg_matvec_plan_build_times": [C.c_void_p, c_double_p],
    "udmrg_probe_fp64_tflops": [C.c_void_p, c_double_p],
    "udmrg_probe_krylov_step": [C.c_void_p, C.c_int64, C.c_int, c_double_p, c_double_p,
                                C.POINTER(C.c_int)],
    "udmrg_ctx_event_record": [C.c_void_p, C.c_int],
    "udmrg_ctx_event_elapsed": [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float)],
    "udmrg_ctx_flush_l2": [C.c_void_p, C.c_int64],
    "udmrg_norm_noalloc": [c_double_p, C.c_int64, c_double_p, C.c_void_p],
    "udmrg_selftest_sym_eig": [C.c_void_p, C.c_int64, c_int32_p, c_double_p, c_int32_p,
                               c_double_p, c_double_p],
    "udmrg_selftest_tc_gemm": [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, c_double_p,
                               c_double_p, c_double_p],
}

_lib = None

# Set at interpreter exit: handle finalizers then skip their device frees (the
# process is ending; the driver reclaims the memory), so no CUDA call runs in
# an arbitrary finalisation order.
SHUTDOWN = [False]


def _at_exit():
    SHUTDOWN[0] = True


import atexit  # noqa: E402

atexit.register(_at_exit)


class UdmrgError(RuntimeError):
    pass


def lib():
    """Load the library (once) and declare every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise UdmrgError(f"{LIB_PATH} is missing: build it with ultradmrg_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.udmrg_last_error.argtypes = []
    L.udmrg_last_error.restype = C.c_char_p
    _lib = L
    return L


def check(status: int, what: str = ""):
    if status != 0:
        msg = lib().udmrg_last_error().decode(errors="replace")
        raise UdmrgError(f"{what} failed (status {status}): {msg}")


def call(name: str, *args):
    check(getattr(lib(), name)(*args), name)
