"""ctypes binding of libfocss_gpu.so (the C ABI in include/focss_gpu.h).

The library is the only compute path: if it is missing or cannot find a GPU,
calls raise.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfocss_gpu.so")

FOCSS_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "TIMEOUT", 5: "NOT_CONVERGED",
    6: "UNSUPPORTED", 7: "NO_DEVICE",
}

D, I, P, U64, SZ = C.c_double, C.c_int, C.c_void_p, C.c_uint64, C.c_size_t


class FocssError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__("focss status %s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, message))


class CDomain(C.Structure):
    _fields_ = [("modes", I), ("samples", I), ("time_step", D), ("center_frequency", D)]


class CFiber(C.Structure):
    _fields_ = [("alpha", D), ("beta2", D), ("gamma", D), ("length", D), ("wavelength", D), ("kappa", D)]


class CSsfmOpts(C.Structure):
    _fields_ = [("grid", I), ("total_steps", I), ("maximum_phase_shift", D), ("maximum_step_size", D)]


class CAmp(C.Structure):
    _fields_ = [("gain", D), ("noise_factor", D), ("seed", U64), ("counter0", U64), ("before", I), ("after", I)]


# name -> (restype, argtypes); every symbol the header declares is listed here
# (tests check this table against include/*.h).
SIGNATURES = {
    "focss_abi_version": (I, []),
    "focss_status_string": (C.c_char_p, [I]),
    "focss_ctx_create": (I, [I, C.POINTER(P)]),
    "focss_ctx_destroy": (I, [P]),
    "focss_ctx_sync": (I, [P]),
    "focss_ctx_stream": (P, [P]),
    "focss_ctx_last_error": (C.c_char_p, [P]),
    "focss_field_create": (I, [P, C.POINTER(CDomain), I, C.POINTER(P)]),
    "focss_field_destroy": (I, [P]),
    "focss_field_domain": (I, [P, C.POINTER(CDomain), C.POINTER(I)]),
    "focss_field_upload": (I, [P, P, SZ]),
    "focss_field_download": (I, [P, P, SZ]),
    "focss_field_upload_c64": (I, [P, P, SZ]),
    "focss_field_download_c64": (I, [P, P, SZ]),
    "focss_field_copy": (I, [P, P]),
    "focss_field_device_ptr": (P, [P]),
    "focss_field_copy_realizations": (I, [P, I, P, I, I]),
    "focss_field_copy_modes": (I, [P, I, P, I, I]),
    "focss_field_scale": (I, [P, D, D]),
    "focss_field_power": (I, [P, P, P]),
    "focss_field_fft": (I, [P]),
    "focss_field_ifft": (I, [P]),
    "focss_ssfm_run": (I, [P, P, C.POINTER(CFiber), C.POINTER(CSsfmOpts), D, P]),
    "focss_set_row_staging": (I, [P, I]),
    "focss_set_pass_staging": (I, [P, I]),
    "focss_ssfm_run_record": (I, [P, P, C.POINTER(CFiber), C.POINTER(CSsfmOpts), D, I, P, P]),
    "focss_ssfm_run_steps": (I, [P, P, C.POINTER(CFiber), P, P, I, D]),
    "focss_amplifier_apply": (I, [P, P, D, D, U64, U64, I]),
    "focss_forward_propagation": (I, [P, P, C.POINTER(CFiber), C.POINTER(CSsfmOpts), D, D, U64, U64, I]),
    "focss_backward_propagation": (I, [P, P, C.POINTER(CFiber), C.POINTER(CSsfmOpts), D, I]),
    "focss_cd_compensation": (I, [P, P, C.POINTER(CFiber), I]),
    "focss_span_loop": (I, [P, I, C.POINTER(P), C.POINTER(CFiber), C.POINTER(CSsfmOpts), C.POINTER(CAmp), I, D,
                            P]),
    "focss_autotune": (I, [P, I, I, C.POINTER(I), C.POINTER(D)]),
    "focss_set_fft_split": (I, [P, I, I]),
    "focss_qam16_map": (I, [P, P, SZ, P]),
    "focss_upsample": (I, [P, P, I, P]),
    "focss_downsample": (I, [P, P, I, P]),
    "focss_decimate": (I, [P, P, I, P]),
    "focss_rrc_pulse": (I, [P, I, I, D, P]),
    "focss_filter": (I, [P, P, P, I]),
    "focss_rrc_shaping": (I, [P, P, I, D, D, P]),
    "focss_rrc_sampling": (I, [P, P, I, D, D, P]),
    "focss_frequency_shift": (I, [P, P, D]),
    "focss_bandpass": (I, [P, P, D]),
    "focss_wdm_select": (I, [P, P, I, D, P]),
    "focss_wdm_mux": (I, [P, P, D, P]),
    "focss_hard_decision": (I, [P, P, P]),
    "focss_soft_decision": (I, [P, P, D, P]),
    "focss_find_certainty": (I, [P, P, P, P]),
    "focss_certainty_decision": (I, [P, P, D, P]),
    "focss_hd_codes": (I, [P, P, P]),
    "focss_error_counts": (I, [P, P, P, I, P, P]),
    "focss_bit_error_rate": (I, [P, P, P, I, P]),
    "focss_symbol_error_rate": (I, [P, P, P, I, P]),
    "focss_q2_factor": (I, [P, P, P, I, P]),
    "focss_pse_estimate": (I, [P, P, P, I, P]),
    "focss_scalar_estimate": (I, [P, P, P, P]),
    "focss_field_rotate": (I, [P, P, P]),
    "focss_field_scale_each": (I, [P, P, P]),
    "focss_triplet_apply": (I, [P, P, I, I, P, P, P, P]),
    "focss_sino_equalize": (I, [P, P, P, I, I, P, P, P, D, D, P]),
    "focss_sino_num_features": (I, [I, I]),
    "focss_sino_gram": (I, [P, P, P, I, I, D, D, P, P, P]),
    "focss_sino_residual": (I, [P, P, P, I, I, D, D, P, P]),
    "focss_wdm_ppe_residual": (I, [P, P, P, I, I, P, P]),
    "focss_wdm_ppe_num_features": (I, [I, I]),
    "focss_wdm_ppe_gram": (I, [P, P, P, I, I, P, P, P]),
    "focss_wdm_ppe_apply": (I, [P, P, P, P, P, I, P, I, P, D, D, P]),
    "focss_ldbp_create": (I, [P, I, I, I, I, I, I, D, C.POINTER(P)]),
    "focss_ldbp_destroy": (I, [P]),
    "focss_ldbp_num_params": (I, [P]),
    "focss_ldbp_set_params": (I, [P, P, I]),
    "focss_ldbp_get_params": (I, [P, P, P, I]),
    "focss_ldbp_forward": (I, [P, P, P]),
    "focss_ldbp_loss_grad": (I, [P, P, P, P]),
    "focss_ldbp_adam_step": (I, [P, D, D, D, D, D]),
    "focss_cnn_create": (I, [P, I, I, I, I, D, C.POINTER(P)]),
    "focss_cnn_destroy": (I, [P]),
    "focss_cnn_num_params": (I, [P]),
    "focss_cnn_set_triplets": (I, [P, I, P, P]),
    "focss_cnn_set_params": (I, [P, P, I]),
    "focss_cnn_get_params": (I, [P, P, P, I]),
    "focss_cnn_forward": (I, [P, P, P]),
    "focss_cnn_loss_grad": (I, [P, P, P, P]),
    "focss_cnn_adam_step": (I, [P, D, D, D, D]),
    "focss_ssfm_run_noalloc": (I, [P, P, I, I, D, C.POINTER(CFiber), C.POINTER(CSsfmOpts), D, P]),
    "focss_profile_enable": (I, [P, I]),
    "focss_profile_read": (I, [P, P, P, P, P, I]),
    "focss_measure_fp32_fma": (I, [P, P]),
    "focss_launch_count": (C.c_longlong, []),
}

_lib = None
_shutting_down = False


def _mark_shutdown():
    global _shutting_down
    _shutting_down = True


def alive() -> bool:
    """False once interpreter shutdown began: device objects are then left to
    process teardown instead of being freed after the CUDA runtime is gone."""
    return not _shutting_down


def lib():
    """Load libfocss_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FocssError(6, "libfocss_gpu.so is not built (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        import atexit
        atexit.register(_mark_shutdown)
    return _lib


def check(status, ctx=None):
    if status != FOCSS_OK:
        msg = ""
        if ctx:
            raw = lib().focss_ctx_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise FocssError(status, msg)
