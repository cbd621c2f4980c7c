"""ctypes binding of libgpuklu (the C ABI declared in include/gpuklu.h).

The library is built in-tree by ``rustspice_gb300.build``. There is no CPU
fallback: every numeric entry point runs on the GPU, and creating a solver
without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double
_lib = None

# Status codes (gpuklu.h)
OK, ANALYZE_FAILED, FACTOR_FAILED, SOLVE_FAILED, SINGULAR, ILL_CONDITIONED, \
    INVALID_MATRIX, DEVICE_TIMEOUT, NONFINITE, CUDA_ERROR = range(10)
PIVOT_REFERENCE, PIVOT_EXACT = 0, 1
# Solver kinds (gpuklu_set_solver_kind), by the oracle's / reference's names
KINDS = {"nativeklu": 0, "sparselu": 1, "sparselubtf": 2, "dense": 3}
AC_MAX_N = 4096  # GPUKLU_AC_MAX_N

# Every symbol the header declares; a test checks the library exports them.
SYMBOLS = [
    "gpuklu_create", "gpuklu_destroy", "gpuklu_prepare", "gpuklu_analyze", "gpuklu_factor",
    "gpuklu_solve", "gpuklu_reset_pattern", "gpuklu_name", "gpuklu_set_parallel_threads",
    "gpuklu_set_pivot_mode", "gpuklu_set_solver_kind", "gpuklu_set_repivot", "gpuklu_repivot_count",
    "gpuklu_set_spin_limit", "gpuklu_set_stop_on_nonfinite", "gpuklu_get_stats", "gpuklu_last_error", "gpuklu_pivot_pass_count", "gpuklu_factor_device",
    "gpuklu_solve_device", "gpuklu_tsolve", "gpuklu_stream", "gpuklu_compile_devices",
    "gpuklu_circuit_free", "gpuklu_circuit_dims", "gpuklu_circuit_pattern",
    "gpuklu_circuit_set_params", "gpuklu_stamp", "gpuklu_newton_dc", "gpuklu_dc_sweep", "gpuklu_batch_create",
    "gpuklu_batch_destroy", "gpuklu_batch_run", "gpuklu_batch_results",
    "gpuklu_batch_update_inputs", "gpuklu_batch_last_error", "gpuklu_batch_info",
    "gpuklu_batch_stream", "gpuklu_batch_work", "gpuklu_batch_phase_ms", "gpuklu_batch_set_schedule", "gpuklu_batch_autotune", "gpuklu_ac_sweep", "gpuklu_tran_create", "gpuklu_tran_forward", "gpuklu_atran_create", "gpuklu_atran_run",
    "gpuklu_tran_backward", "gpuklu_bbd_create", "gpuklu_bbd_destroy", "gpuklu_bbd_last_error",
    "gpuklu_bbd_info", "gpuklu_bbd_perm", "gpuklu_bbd_factor", "gpuklu_bbd_solve", "gpuklu_bbd_newton_dc", "gpuklu_fp64_peak_tflops", "gpuklu_fp64_mma_peak_tflops", "gpuklu_dense_lu_nopivot", "gpuklu_solve_device_noalloc", "gpuklu_dc_backward", "gpuklu_plan_build", "gpuklu_plan_array", "gpuklu_plan_free", "gpuklu_plan_steps", "gpuklu_plan_solve_steps", "gpuklu_btf_info",
]


class Stats(C.Structure):
    _fields_ = [("factor_count", _I64), ("refactor_count", _I64), ("nnz_l", _I64),
                ("nnz_u", _I64), ("nblocks", _I64), ("noffdiag", _I64), ("pivot_swaps", _I64),
                ("refactor_flops", _I64), ("rcond", _D)]


class NewtonConfig(C.Structure):
    _fields_ = [("max_iters", _I64), ("abs_tol", _D), ("rel_tol", _D), ("gmin", _D),
                ("gmin_steps", _I64), ("source_steps", _I64), ("damping", _D),
                ("damping_min", _D)]


def lib_path() -> str:
    from . import build
    return build.LIB


def lib(build_if_missing: bool = True):
    """Loads libgpuklu.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libgpuklu not built: {path}")
        from . import build
        build.build()
    L = C.CDLL(path)
    sig = {
        "gpuklu_create": (_P, [_I64]),
        "gpuklu_destroy": (None, [_P]),
        "gpuklu_prepare": (None, [_P, _I64]),
        "gpuklu_analyze": (C.c_int, [_P, _P, _I64, _P, _I64]),
        "gpuklu_factor": (C.c_int, [_P, _P, _I64, _P, _I64, _P]),
        "gpuklu_solve": (C.c_int, [_P, _P, _I64]),
        "gpuklu_reset_pattern": (None, [_P]),
        "gpuklu_name": (C.c_char_p, [_P]),
        "gpuklu_set_parallel_threads": (None, [_P, C.c_size_t]),
        "gpuklu_set_pivot_mode": (C.c_int, [_P, C.c_int]),
        "gpuklu_set_repivot": (C.c_int, [_P, C.c_int]),
        "gpuklu_set_solver_kind": (C.c_int, [_P, C.c_int]),
        "gpuklu_repivot_count": (_I64, [_P]),
        "gpuklu_set_spin_limit": (C.c_int, [_P, C.c_uint32]),
        "gpuklu_set_stop_on_nonfinite": (C.c_int, [_P, C.c_int]),
        "gpuklu_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
        "gpuklu_last_error": (C.c_char_p, [_P]),
        "gpuklu_pivot_pass_count": (_I64, [_P]),
        "gpuklu_factor_device": (C.c_int, [_P, _P]),
        "gpuklu_solve_device": (C.c_int, [_P, _P]),
        "gpuklu_tsolve": (C.c_int, [_P, _P, _I64]),
        "gpuklu_stream": (_P, [_P]),
        "gpuklu_compile_devices": (_P, [_I64, _I64, _P, _P, _P, C.c_int]),
        "gpuklu_circuit_free": (None, [_P]),
        "gpuklu_circuit_dims": (C.c_int, [_P, _P, _P]),
        "gpuklu_circuit_pattern": (C.c_int, [_P, _P, _P]),
        "gpuklu_circuit_set_params": (C.c_int, [_P, _P]),
        "gpuklu_stamp": (C.c_int, [_P, _P, _P, _I64, _D, _D, _D, _P, _D, _P, _P]),
        "gpuklu_newton_dc": (C.c_int, [_P, _P, C.POINTER(NewtonConfig), _P, _P, _I64, _P, _P,
                                       _P, _P]),
        "gpuklu_dc_sweep": (C.c_int, [_P, _P, C.POINTER(NewtonConfig), _I64, _P, _I64, _P,
                                      _I64, C.c_int, _P, _I64, _P, _P, _P, _P]),
        "gpuklu_batch_create": (_P, [_I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _I64]),
        "gpuklu_batch_destroy": (None, [_P]),
        "gpuklu_batch_run": (C.c_int, [_P, C.POINTER(NewtonConfig)]),
        "gpuklu_batch_results": (C.c_int, [_P, _P, _P, _P, _P, _P]),
        "gpuklu_batch_update_inputs": (C.c_int, [_P, _P, _P]),
        "gpuklu_batch_last_error": (C.c_char_p, [_P]),
        "gpuklu_batch_info": (C.c_int, [_P, _P]),
        "gpuklu_batch_stream": (_P, [_P]),
        "gpuklu_batch_work": (C.c_int, [_P, _P, _P]),
        "gpuklu_batch_phase_ms": (C.c_int, [_P, _P]),
        "gpuklu_batch_set_schedule": (C.c_int, [_P, C.c_int, C.c_int]),
        "gpuklu_batch_autotune": (C.c_int, [_P, C.POINTER(NewtonConfig), _P, _P]),
        "gpuklu_ac_sweep": (C.c_int, [_P, _P, _P, _I64, _P, _I64, _P, _P, _P]),
        "gpuklu_tran_create": (_P, [_I64, _P, _P, _P, _P, _P, _P, _P, _I64, _D, _I64, _I64, _P,
                                    _D]),
        "gpuklu_tran_forward": (C.c_int, [_P, _P, _P, _P, _P, _P]),
        "gpuklu_atran_create": (_P, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I64,
                                     _P]),
        "gpuklu_atran_run": (C.c_int, [_P, C.POINTER(NewtonConfig), _D, _D, _D, _D, _D, _D, _D,
                                       _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
        "gpuklu_tran_backward": (C.c_int, [_P, _P, _P, _P]),
        "gpuklu_bbd_create": (_P, [_I64, _P, _I64, _P, _I64, _P, _I64]),
        "gpuklu_bbd_destroy": (None, [_P]),
        "gpuklu_bbd_last_error": (C.c_char_p, [_P]),
        "gpuklu_bbd_info": (C.c_int, [_P, _P]),
        "gpuklu_bbd_perm": (C.c_int, [_P, _P]),
        "gpuklu_bbd_factor": (C.c_int, [_P, _P]),
        "gpuklu_bbd_solve": (C.c_int, [_P, _P, _I64]),
        "gpuklu_bbd_newton_dc": (C.c_int, [_P, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
        "gpuklu_fp64_peak_tflops": (_D, []),
        "gpuklu_fp64_mma_peak_tflops": (_D, []),
        "gpuklu_dense_lu_nopivot": (C.c_int, [_P, _I64, C.c_int, _P]),
        "gpuklu_solve_device_noalloc": (C.c_int, [_P, _P, _P]),
        "gpuklu_dc_backward": (C.c_int, [_P, _P, _P, _I64, _P, _D, _P, _P]),
        "gpuklu_plan_build": (_P, [_I64, _P, _P, C.c_int, C.c_int, _P]),
        "gpuklu_plan_array": (_I64, [_P, C.c_char_p, _P, _I64]),
        "gpuklu_plan_free": (None, [_P]),
        "gpuklu_plan_steps": (_I64, [_P, C.c_int32, C.c_int32, _P, _I64, _P, _I64]),
        "gpuklu_plan_solve_steps": (_I64, [_P, _P, _I64, _P, _I64]),
        "gpuklu_btf_info": (C.c_int, [_I64, _P, _P, _P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def i64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def newton_config(max_iters=100, abs_tol=1e-6, rel_tol=1e-3, gmin=1e-12, gmin_steps=0,
                  source_steps=0, damping=1.0, damping_min=0.1) -> NewtonConfig:
    """NewtonConfig from the engine's option names (engine.rs:987-999)."""
    return NewtonConfig(max_iters, abs_tol, rel_tol, gmin, gmin_steps, source_steps, damping,
                        damping_min)


def step_program(n, ap, ai, nc, ndv, pivot_mode=PIVOT_REFERENCE, row_perm=None,
                 kind="nativeklu"):
    """The batched warp kernel's step program for a pattern's plan
    (gpuklu_plan_steps): (ops[nops, 2] int32, step_ptr[nsteps + 1] int32),
    or None when the region exceeds 16-bit offsets."""
    L = lib()
    ap, ai = i64(ap), i64(ai)
    rp = i32(row_perm) if row_perm is not None else None
    h = L.gpuklu_plan_build(n, ptr(ap), ptr(ai), pivot_mode, KINDS[kind],
                            ptr(rp) if rp is not None else None)
    if not h:
        raise ValueError("plan build failed")
    try:
        r = L.gpuklu_plan_steps(h, nc, ndv, None, 0, None, 0)
        nops, nsp = r >> 32, r & 0xffffffff
        if nsp == 0:
            return None
        ops = np.zeros(2 * nops, np.int32)
        sp = np.zeros(nsp, np.int32)
        L.gpuklu_plan_steps(h, nc, ndv, ptr(ops), len(ops), ptr(sp), len(sp))
        return ops.reshape(nops, 2), sp
    finally:
        L.gpuklu_plan_free(h)


def solve_step_program(n, ap, ai, pivot_mode=PIVOT_REFERENCE, row_perm=None,
                       kind="nativeklu"):
    """The single-system solve's step program for a pattern's plan
    (gpuklu_plan_solve_steps): (ops[nops, 4] int32, step_ptr[nsteps + 1]), or
    None when the solution exceeds one block's shared memory."""
    L = lib()
    ap, ai = i64(ap), i64(ai)
    rp = i32(row_perm) if row_perm is not None else None
    h = L.gpuklu_plan_build(n, ptr(ap), ptr(ai), pivot_mode, KINDS[kind],
                            ptr(rp) if rp is not None else None)
    if not h:
        raise ValueError("plan build failed")
    try:
        r = L.gpuklu_plan_solve_steps(h, None, 0, None, 0)
        nops, nsp = r >> 32, r & 0xffffffff
        if nsp == 0:
            return None
        ops = np.zeros(4 * nops, np.int32)
        sp = np.zeros(nsp, np.int32)
        L.gpuklu_plan_solve_steps(h, ptr(ops), len(ops), ptr(sp), len(sp))
        return ops.reshape(nops, 4), sp
    finally:
        L.gpuklu_plan_free(h)


class Plan:
    """Host-side symbolic plan (no device needed)."""

    NAMES = ["col_ptr", "dslot", "slot_row", "upd_ptr", "upd_dst", "amap_ptr", "amap_idx",
             "offd_ptr", "offd_col", "offd_raw", "in_pos", "out_pos", "block_ptr", "col_single",
             "pcol_ptr", "pcol_raw", "pcol_q", "pos_block", "raw_slot", "row_perm",
             "lrow_ptr", "lrow_col", "lrow_slot", "urow_ptr", "urow_col", "urow_slot",
             "cs_chunk", "cs_op", "cs_grp", "cs_gchunk", "cs_gop", "task", "ttask"]

    def __init__(self, n, ap, ai, pivot_mode=PIVOT_REFERENCE, row_perm=None, kind="nativeklu"):
        L = lib()
        ap, ai = i64(ap), i64(ai)
        rp = i32(row_perm) if row_perm is not None else None
        h = L.gpuklu_plan_build(n, ptr(ap), ptr(ai), pivot_mode, KINDS[kind],
                                ptr(rp) if rp is not None else None)
        if not h:
            raise ValueError("plan build failed")
        try:
            def get(name):
                m = L.gpuklu_plan_array(h, name.encode(), None, 0)
                out = np.zeros(max(m, 1), np.int64)
                L.gpuklu_plan_array(h, name.encode(), ptr(out), m)
                return out[:m]
            info = get("info")
            self.n, self.nslots, self.nblocks, self.nnz_l, self.nnz_u, self.noffdiag, \
                self.offd_lower, self.swaps = (int(v) for v in info)
            for nm in self.NAMES:
                setattr(self, nm, get(nm))
        finally:
            L.gpuklu_plan_free(h)
