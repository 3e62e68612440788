"""ctypes binding of libkite_gb300.so: the kite C API (include/kite.h), the engine C ABI
(include/kite_cuda.h), the integer-NTT engine (include/kite_ntt.h) and the PRST-compatible proof
API (include/kite_proof.h).

The library is the product; this module only declares its prototypes.  Loading fails loudly
when the library has not been built: there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkite_gb300.so")

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i64p = C.POINTER(C.c_int64)
dp = C.POINTER(C.c_double)
vp = C.c_void_p


class KiteOpts(C.Structure):
    _fields_ = [("backend", C.c_int), ("fft_len", C.c_uint32), ("threads", C.c_uint32),
                ("plan_order", C.c_uint32)]


PROGRESS_FN = C.CFUNCTYPE(None, vp, C.c_uint64, C.c_uint64, C.c_double)
POINT_FN = C.CFUNCTYPE(C.c_int, vp, C.c_uint32, C.c_uint64, u64p)
CONFIRM_FN = C.CFUNCTYPE(None, vp, C.c_int)


class KitePrpOpts(C.Structure):
    _fields_ = [("fft", KiteOpts), ("gerbicz_block", C.c_uint32), ("gerbicz_blocks", C.c_uint32),
                ("max_roundoff", C.c_double), ("checkpoint", C.c_char_p),
                ("checkpoint_secs", C.c_double), ("checkpoint_unverified", C.c_char_p),
                ("unverified_secs", C.c_double), ("progress", PROGRESS_FN),
                ("progress_arg", vp), ("inject_fault_at", C.c_uint64), ("points", u32p),
                ("npoints", C.c_uint32), ("on_point", POINT_FN), ("point_arg", vp),
                ("abort_flag", C.POINTER(C.c_int))]


class KitePrpResult(C.Structure):
    _fields_ = [("res64", C.c_uint64), ("is_prp", C.c_int), ("fft_len", C.c_uint32),
                ("maxerr", C.c_double), ("gerbicz_errors", C.c_uint32),
                ("roundoff_retries", C.c_uint32), ("resumed", C.c_int),
                ("resumed_at", C.c_uint64), ("seconds", C.c_double)]


class PpGiant(C.Structure):
    """pp_giant (include/kite_proof.h): little-endian 32-bit words, no leading zeros."""
    _fields_ = [("w", u32p), ("len", C.c_int32)]


class KiteLlrOpts(C.Structure):
    _fields_ = [("fft", KiteOpts), ("max_roundoff", C.c_double), ("checkpoint", C.c_char_p),
                ("checkpoint_secs", C.c_double), ("progress", PROGRESS_FN),
                ("on_confirm", CONFIRM_FN), ("progress_arg", vp),
                ("abort_flag", C.POINTER(C.c_int)), ("inject_fault_at", C.c_uint64),
                ("inject_fault_runs", C.c_uint32), ("inject_roundoff_at", C.c_uint64),
                ("inject_roundoff_ladder", C.c_int)]


class KiteLlrResult(C.Structure):
    _fields_ = [("is_prime", C.c_int), ("factor", C.c_uint64), ("res64", C.c_uint64),
                ("P", C.c_uint32), ("fft_len", C.c_uint32), ("maxerr", C.c_double),
                ("roundoff_retries", C.c_uint32), ("confirm_runs", C.c_uint32),
                ("resumed", C.c_int), ("resumed_at", C.c_uint64), ("seconds", C.c_double)]


class KcTestResult(C.Structure):
    _fields_ = [("kind", C.c_int), ("rc", C.c_int), ("k", C.c_uint64), ("n", C.c_uint64),
                ("res64", C.c_uint64), ("is_prp", C.c_int), ("fft_len", C.c_uint32),
                ("maxerr", C.c_double), ("gerbicz_errors", C.c_uint32),
                ("roundoff_retries", C.c_uint32), ("squarings", C.c_uint64),
                ("seconds", C.c_double), ("P", C.c_uint32), ("factor", C.c_uint64),
                ("iter", C.c_uint64), ("position", C.c_uint64)]


KITE_BACKEND_CUDA = 5
KITE_BACKEND_CUDA_NTT = 6
PP_TYPE_VALUE, PP_TYPE_PRODUCT, PP_TYPE_CERT = 1, 3, 4
PP_ABORTED = -2
KC_TEST_FERMAT = 0
KC_TEST_LLR = 1

# name -> (restype, argtypes); every symbol declared in include/kite.h and include/kite_cuda.h
PROTOTYPES = {
    # include/kite.h
    "kite_ctx_new": (vp, [C.c_uint64, C.c_uint64, C.c_int32, C.POINTER(KiteOpts)]),
    "kite_ctx_free": (None, [vp]),
    "kite_fft_len": (C.c_uint32, [vp]),
    "kite_backend_name": (C.c_char_p, [vp]),
    "kite_num_new": (vp, [vp]),
    "kite_num_free": (None, [vp, vp]),
    "kite_copy": (None, [vp, vp, vp]),
    "kite_set_u64": (None, [vp, vp, C.c_uint64]),
    "kite_square": (None, [vp, vp]),
    "kite_square_n": (None, [vp, vp, C.c_uint64]),
    "kite_mul": (None, [vp, vp, vp]),
    "kite_mul_small": (None, [vp, vp, C.c_int64]),
    "kite_add": (None, [vp, vp, vp]),
    "kite_sub": (None, [vp, vp, vp]),
    "kite_max_roundoff": (C.c_double, [vp]),
    "kite_reset_roundoff": (None, [vp]),
    "kite_set_roundoff_check": (None, [vp, C.c_uint32]),
    "kite_limbs": (C.c_size_t, [vp]),
    "kite_get_limbs": (None, [vp, vp, u64p]),
    "kite_set_limbs": (None, [vp, vp, u64p]),
    "kite_res64": (C.c_uint64, [vp, vp]),
    "kite_prp": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(KitePrpOpts),
                           C.POINTER(KitePrpResult)]),
    "kite_llr": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(KiteLlrOpts),
                           C.POINTER(KiteLlrResult)]),
    "kite_llr_choose_P": (C.c_int, [C.c_uint64, C.c_uint64, u32p, u64p]),
    "kite_llr_checkpoint_iter": (C.c_int, [C.c_char_p, C.c_uint64, C.c_uint64, u64p,
                                           C.POINTER(C.c_int)]),
    "kite_prp_checkpoint_iter": (C.c_int, [C.c_char_p, C.c_uint64, C.c_uint64, C.c_uint32, u64p]),
    "kite_debug_corrupt": (None, [vp, vp]),
    "kite_ctx_error": (C.c_int, [vp]),
    "kite_ctx_sync": (C.c_int, [vp]),
    # include/kite_cuda.h
    "kc_engine_new": (vp, [C.c_uint64, C.c_uint64, C.c_uint32, u8p, dp, dp, C.c_uint32,
                           C.c_uint64, C.c_uint32, C.c_uint64, C.c_int]),
    "kc_engine_free": (None, [vp]),
    "kc_num_doubles": (C.c_size_t, [vp]),
    "kc_num_alloc": (vp, [vp]),
    "kc_num_free": (None, [vp, vp]),
    "kc_from_digits": (C.c_int, [vp, vp, i64p]),
    "kc_to_digits": (C.c_int, [vp, vp, i64p]),
    "kc_square": (C.c_int, [vp, vp, C.c_uint64]),
    "kc_square_add": (C.c_int, [vp, vp, C.c_uint64, C.c_int64]),
    "kc_mul": (C.c_int, [vp, vp, vp]),
    "kc_copy": (C.c_int, [vp, vp, vp]),
    "kc_add": (C.c_int, [vp, vp, vp]),
    "kc_sub": (C.c_int, [vp, vp, vp]),
    "kc_equal": (C.c_int, [vp, vp, vp]),
    "kc_maxerr": (C.c_double, [vp]),
    "kc_reset_maxerr": (None, [vp]),
    "kc_set_roundoff_check": (None, [vp, C.c_uint32]),
    "kc_error": (C.c_int, [vp]),
    "kc_sync": (C.c_int, [vp]),
    "kc_stream": (vp, [vp]),
    "kc_shape": (None, [vp, u32p, u32p]),
    "kc_group_width": (C.c_int, [vp]),
    "kc_engine_wait_selftest": (C.c_int, [vp, C.c_uint64]),
    "kc_square_noalloc": (C.c_int, [vp, vp, vp]),
    "kc_batch_new": (vp, [C.c_int, C.c_uint32, C.c_uint32, C.c_size_t]),
    "kc_batch_free": (None, [vp]),
    "kc_batch_add_fermat": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32]),
    "kc_batch_add_llr": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_uint32]),
    "kc_batch_step": (C.c_int, [vp, C.c_uint32, dp]),
    "kc_batch_result": (C.c_int, [vp, C.c_int, C.POINTER(KcTestResult)]),
    "kc_batch_release": (None, [vp, C.c_int]),
    "kc_batch_active": (C.c_int, [vp]),
    "kc_batch_bytes_in_use": (C.c_size_t, [vp]),
    "kc_batch_budget": (C.c_size_t, [vp]),
    "kc_batch_error": (C.c_int, [vp]),
    "kc_batch_error_string": (C.c_char_p, [vp]),
    "kc_fp64_peak": (C.c_double, [C.c_int]),
    "kc_fp64_probe_rate": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "kc_batch_profile": (C.c_int, [vp, C.c_uint32, dp, dp]),
    "kc_batch_profile_steps": (C.c_int, [vp, C.c_uint32, dp, dp]),
    "kc_batch_read": (C.c_int, [vp, C.c_int, u64p]),
    "kc_batch_checkpoint": (C.c_int, [vp, C.c_int, C.c_char_p]),
    "kc_batch_last_transfer": (None, [vp, u64p, u64p]),
    "kc_batch_debug_corrupt": (C.c_int, [vp, C.c_int]),
    "kc_batch_stagger_checks": (None, [vp, C.c_int]),
    "kc_set_fft_shape": (C.c_int, [C.c_uint32, C.c_uint32]),
    "kc_set_fft_time": (None, [C.c_uint32, C.c_double]),
    "kc_fft_shape_candidates": (C.c_int, [C.c_uint32, u32p, u32p, C.c_int]),
    "kc_fft_shape": (C.c_int, [C.c_uint32, u32p, u32p]),
    "kc_set_latency_shape": (C.c_int, [C.c_uint32, C.c_uint32, C.c_int]),
    "kc_tuning_load": (C.c_int, [C.c_char_p]),
    "kc_roundoff_probe": (C.c_double, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64]),
    "kc_layout": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, u8p, dp, dp, u64p]),
    "kc_digits_to_limbs": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, i64p, u64p]),
    "kc_limbs_to_digits": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, u64p, i64p]),
    "kc_carry_digits": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, i64p]),
    "kc_choose_fft_len": (C.c_uint32, [C.c_uint64, C.c_uint64]),
    # the integer-NTT engine (include/kite_ntt.h)
    "kn_engine_new": (vp, [C.c_uint64, C.c_uint64, C.c_int]),
    "kn_engine_free": (None, [vp]),
    "kn_num_words": (C.c_uint32, [vp]),
    "kn_word_bits": (C.c_uint32, [vp]),
    "kn_transform_len": (C.c_uint32, [vp]),
    "kn_num_alloc": (vp, [vp]),
    "kn_num_free": (None, [vp, vp]),
    "kn_limbs": (C.c_size_t, [vp]),
    "kn_set_limbs": (C.c_int, [vp, vp, u64p]),
    "kn_get_limbs": (C.c_int, [vp, vp, u64p]),
    "kn_square": (C.c_int, [vp, vp, C.c_uint64]),
    "kn_square_add": (C.c_int, [vp, vp, C.c_uint64, C.c_int64]),
    "kn_mul": (C.c_int, [vp, vp, vp]),
    "kn_copy": (C.c_int, [vp, vp, vp]),
    "kn_error": (C.c_int, [vp]),
    "kn_sync": (C.c_int, [vp]),
    "kn_layout": (C.c_int, [C.c_uint64, C.c_uint64, u32p, u32p, u32p, u32p]),
    "kn_limbs_to_words": (C.c_int, [C.c_uint64, C.c_uint64, u64p, u64p]),
    "kn_words_to_limbs": (C.c_int, [C.c_uint64, C.c_uint64, u64p, u64p]),
    "kn_group_new": (vp, [C.c_int]),
    "kn_group_free": (None, [vp]),
    "kn_group_add": (C.c_int, [vp, vp, vp]),
    "kn_group_square": (C.c_int, [vp, C.c_uint64, C.POINTER(C.c_float)]),
    "kn_groups_square": (C.c_int, [C.POINTER(vp), C.c_int, C.c_uint64, C.POINTER(C.c_float)]),
    "kn_group_mul": (C.c_int, [vp, C.POINTER(vp), C.POINTER(C.c_float)]),
    "kn_group_error": (C.c_int, [vp]),
    # PRST-compatible proofs (include/kite_proof.h)
    "pp_giant_free": (None, [C.POINTER(PpGiant)]),
    "pp_fingerprint": (C.c_uint32, [C.c_uint64, C.c_uint64]),
    "pp_unique_fingerprint": (C.c_uint32, [C.c_uint32, C.c_char_p]),
    "pp_proof_fingerprint": (C.c_uint32, [C.c_uint64, C.c_uint64, C.c_uint32]),
    "pp_write": (C.c_int, [C.c_char_p, C.c_int, C.c_uint32, C.c_int32, C.POINTER(PpGiant), C.c_int]),
    "pp_read": (C.c_int, [C.c_char_p, C.c_int, C.c_uint32, C.POINTER(C.c_int32), C.POINTER(PpGiant),
                          C.c_int]),
    "pp_points": (C.c_int, [C.c_uint32, C.c_int, u32p]),
    "pp_from_num": (None, [vp, vp, C.POINTER(PpGiant)]),
    "pp_to_num": (None, [vp, vp, C.POINTER(PpGiant)]),
    "pp_res64": (C.c_uint64, [C.POINTER(PpGiant)]),
    "pp_save_products": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, C.c_char_p, C.c_int,
                                   C.POINTER(C.c_int), u64p]),
    "pp_build_cert": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, C.c_char_p, C.c_int,
                                u64p]),
    "pp_verify_cert": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_char_p, u64p, u32p]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load the library (once) and declare every prototype; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"{p} is missing: build it with ahnum_gb300.build.build_library() "
                "(there is no fallback implementation)")
        lib = C.CDLL(p)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def missing_symbols(lib) -> list[str]:
    return [n for n in PROTOTYPES if not hasattr(lib, n)]
