"""ctypes binding of libmkf_gb300.so (the C ABI declared in include/mkf_gb300.h).

The CUDA library is the only compute path: if it is missing this module raises
instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmkf_gb300.so")

P = C.c_void_p
I = C.c_int
U32 = C.c_uint32
U64 = C.c_uint64
I64 = C.c_int64
F = C.c_float
FP = C.POINTER(C.c_float)

MKF_OK = 0
ERRORS = {1: "MKF_ERR_ARG", 2: "MKF_ERR_CUDA", 3: "MKF_ERR_NONPD", 4: "MKF_ERR_NAN",
          5: "MKF_ERR_TIMEOUT", 6: "MKF_ERR_NOMEM", 7: "MKF_ERR_STATE"}
ST_FALLBACK, ST_NAN, ST_NONPD, ST_TRUNC = 1, 2, 4, 8


class MkfError(RuntimeError):
    pass


class BpfModels(C.Structure):
    _fields_ = [("n_models", I), ("d", I), ("K", I), ("J", I),
                ("a", P), ("mu", P), ("Lq", P), ("S0c", P), ("pi", P), ("Bm", P), ("mm", P),
                ("fx", F), ("fy", F), ("cx", F), ("cy", F)]


class MixModelDesc(C.Structure):
    _fields_ = [("d", I), ("K", I), ("J", I), ("pi", P), ("S0", P),
                ("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double)]


class BpfTrack(C.Structure):
    _fields_ = [("n_particles", C.c_int32), ("n_frames", C.c_int32), ("frame_base", C.c_int64),
                ("seed", C.c_uint64), ("track_id", C.c_uint32), ("model_index", C.c_int32),
                ("kappa", F), ("p_detect", F), ("sigma_px", F)]


# name -> (restype, argtypes); every symbol declared in include/mkf_gb300.h
SIGNATURES = {
    "mkf_version": (C.c_char_p, []),
    "mkf_last_error": (C.c_char_p, []),
    "mkf_philox_block": (I, [U64, U32, U32, U32, U32, P]),
    "mkf_draw_particles": (I, [U64, U32, U32, I, I, P, P, P]),
    "mkf_resample_f64": (I, [P, I, I, U32, P, P, P]),
    "mkf_resample_f32": (I, [P, I, I, U32, P, P, P]),
    "mkf_resample_f32_noalloc": (I, [P, I, I, U32, P, P, P]),
    "mkf_bpf_create": (I, [C.POINTER(BpfModels), C.POINTER(BpfTrack), C.POINTER(P)]),
    "mkf_bpf_reset": (I, [P, P]),
    "mkf_bpf_update": (I, [P, U32, P, P, P, P, P, P]),
    "mkf_bpf_set_debug": (I, [P, I]),
    "mkf_bpf_read_debug": (I, [P, P, P, P, P, P]),
    "mkf_bpf_status": (I, [P, C.POINTER(I)]),
    "mkf_bpf_destroy": (I, [P]),
    "mkf_bpf_graph_create": (I, [P, I, P, P, P, P, P, C.POINTER(P)]),
    "mkf_bpf_graph_launch": (I, [P, U32, P]),
    "mkf_bpf_graph_destroy": (I, [P]),
    "mkf_bpf_batch_create": (I, [C.POINTER(BpfModels), I, P, I64, C.POINTER(P)]),
    "mkf_bpf_batch_set_tuning": (I, [P, I, I]),
    "mkf_bpf_batch_set_variant": (I, [P, I]),
    "mkf_bpf_batch_run": (I, [P, P, P, P, P, P, P, P]),
    "mkf_bpf_batch_run_host": (I, [P, P, P, I64, P, P, P, P, P]),
    "mkf_bpf_batch_set_debug": (I, [P, I, P, P]),
    "mkf_bpf_batch_last_grid": (I, [P, C.POINTER(I)]),
    "mkf_bpf_batch_destroy": (I, [P]),
    "mkf_likelihood_blur": (I, [P, I, I, I, P, I, P]),
    "mkf_pdaf_propose_image": (I, [P, P, U32, P, P, I, I, I, I, I, C.c_double, C.c_double, P, P, P, P, P, P, P]),
    "mkf_pose_decode": (I, [P, I, I, I, P, P, P, P, P, P, P]),
    "mkf_pose2d_record": (I, [P, P, I, I, P, P]),
    "mkf_pf2d_create": (I, [I, I, I, I, P, P, P, I, I, U64, U32, C.POINTER(P)]),
    "mkf_pf2d_update": (I, [P, U32, P, P]),
    "mkf_pf2d_estimate": (I, [P, P, P]),
    "mkf_pf2d_read": (I, [P, P, P, P, P, P]),
    "mkf_pf2d_draws": (I, [U64, U32, U32, I, I, P, P, P]),
    "mkf_pf2d_destroy": (I, [P]),
    "mkf_rbpf_create": (I, [I, I, I, I, I, U64, U32, C.POINTER(P)]),
    "mkf_rbpf_load_gaussian": (I, [P, I, P, P, P, P, I, C.c_double, C.c_double]),
    "mkf_rbpf_set_component": (I, [P, I, P, P, P, P, P, C.c_double, P, P]),
    "mkf_rbpf_set_pinhole": (I, [P, P, P, C.c_double, C.c_double, C.c_double, C.c_double]),
    "mkf_rbpf_set_hand_decode": (I, [P, P, P, I]),
    "mkf_rbpf_reset": (I, [P, P, P]),
    "mkf_rbpf_update": (I, [P, U32, P, C.c_uint, P]),
    "mkf_rbpf_update_u": (I, [P, P, C.c_uint, U32, U32, P]),
    "mkf_rbpf_estimate": (I, [P, P, P]),
    "mkf_rbpf_read": (I, [P, P, P, P, P, P, P, P]),
    "mkf_rbpf_write": (I, [P, P, P, P]),
    "mkf_rbpf_status": (I, [P, C.POINTER(I)]),
    "mkf_rbpf_destroy": (I, [P]),
    "mkf_pdaf_associate": (I, [P, P, U32, P, P, I, C.c_double, C.c_double, P, P, P, P, P]),
    "mkf_mixkf_create": (I, [C.POINTER(MixModelDesc), I, P, P, P, P, P, P, I64, C.POINTER(P)]),
    "mkf_mixkf_set_theta": (I, [P, P]),
    "mkf_mixkf_set_theta_device": (I, [P, P, P]),
    "mkf_mixkf_theta_size": (I, [P]),
    "mkf_mixkf_forward": (I, [P, P, P, P, P, P]),
    "mkf_mixkf_backward": (I, [P, P, P, P, P]),
    "mkf_mixkf_set_checkpoint_stride": (I, [P, I]),
    "mkf_mixkf_checkpoint_stride": (I, [P]),
    "mkf_mixkf_status": (I, [P, C.POINTER(I)]),
    "mkf_mixkf_destroy": (I, [P]),
    "mkf_adam_step": (I, [P, P, P, P, P, I, I, C.c_double, C.c_double, C.c_double, C.c_double, I, P]),
}

_lib = None


def lib():
    """Load libmkf_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MkfError("libmkf_gb300.so is missing: run mkfbodytracker_pdaf_gb300.build.build() "
                           "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what=""):
    if status != MKF_OK:
        msg = lib().mkf_last_error().decode(errors="replace")
        raise MkfError("%s: %s %s" % (what, ERRORS.get(status, status), msg))
    return status


def exported_symbols():
    return list(SIGNATURES)
