"""ctypes binding of ``libgbspec.so`` (C ABI declared in ``include/gbspec.h``).

The library is the only compute path: if it cannot be loaded, every call
raises ``ImportError``; there is no CPU fallback.
"""

import ctypes
import threading
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libgbspec.so"

GBS_OK = 0
GBS_EINVAL = -22
GBS_ENOMEM = -12
GBS_ECUDA = -5
GBS_ENAN = -33
GBS_ETIMEDOUT = -110
GBS_F32 = 0
GBS_F64 = 1
GBS_STEP_CHECK_NAN = 1
GBS_STEP_DEALIASED = 2
GBS_STEP_TEST_STALL = 64

EXPORTED = (
    "gbs_last_error", "gbs_version", "gbs_fft_plan_create",
    "gbs_fft_plan_destroy", "gbs_fft_r2c", "gbs_fft_c2r", "gbs_ns_create",
    "gbs_ns_destroy", "gbs_ns_tendencies", "gbs_ns_step_rk4",
    "gbs_ns_max_velocity", "gbs_cfl_update", "gbs_ns_spatial_means",
    "gbs_ns_spectrum_size", "gbs_ns_spectrum", "gbs_ns_timing",
    "gbs_ns_timing_report", "gbs_fft_c2r_noalloc", "gbs_ns_set_turb_model",
    "gbs_mlp_grad_workspace", "gbs_mlp_forward", "gbs_mlp_forward_bf16", "gbs_mlp_grad",
    "gbs_mlp_adam",
    "gbs_ns_set_forcing", "gbs_spectral_resample", "gbs_products6",
    "gbs_velocity_gradients", "gbs_ens2d_create", "gbs_ens2d_destroy",
    "gbs_ens2d_set_params", "gbs_ens2d_set_tuning", "gbs_ens2d_step", "gbs_ens2d_nan_flag",
    "gbs_ens2d_mixed_create", "gbs_ens2d_mixed_destroy", "gbs_ens2d_mixed_step",
    "gbs_ens2d_mixed_set_tuning",
    "gbs_ns_is_dealiased", "gbs_ns_step", "gbs_ns_set_projection", "gbs_ns_set_phase_shifts",
    "gbs_spectra_sizes", "gbs_spectra", "gbs_forcing_coarse",
    "gbs_ens2d_persistent_step", "gbs_ens2d_persistent_status",
    "gbs_ens2d_persistent_set_chunk",
)
SCHEMES = {"RK4": 0, "Euler": 1, "RK2": 2, "RK2_trapezoid": 3, "Euler_phaseshift": 4,
           "RK2_phaseshift": 5, "RK2_phaseshift_exact": 6, "Euler_phaseshift_random": 7,
           "RK2_phaseshift_random": 8}


class ForcingParams(ctypes.Structure):
    """Mirror of ``gbs_forcing_params``."""

    _fields_ = [
        ("ndim", ctypes.c_int),
        ("nx", ctypes.c_int64), ("ny", ctypes.c_int64), ("nz", ctypes.c_int64),
        ("nc", ctypes.c_int64),
        ("nvar", ctypes.c_int), ("nkeys", ctypes.c_int), ("keys", ctypes.c_int * 8),
        ("type", ctypes.c_int), ("which_root", ctypes.c_int),
        ("forcing_rate", ctypes.c_double),
        ("dtype", ctypes.c_int),
    ]


class NSParams(ctypes.Structure):
    """Mirror of ``gbs_ns_params``."""

    _fields_ = [
        ("ndim", ctypes.c_int),
        ("nx", ctypes.c_int64), ("ny", ctypes.c_int64), ("nz", ctypes.c_int64),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
        ("nu_2", ctypes.c_double), ("nu_4", ctypes.c_double),
        ("nu_8", ctypes.c_double), ("nu_m4", ctypes.c_double),
        ("beta", ctypes.c_double), ("f", ctypes.c_double),
        ("has_f", ctypes.c_int),
        ("kcut_x", ctypes.c_int64), ("kcut_y", ctypes.c_int64),
        ("kcut_z", ctypes.c_int64),
        ("dtype", ctypes.c_int),
        ("strat", ctypes.c_int), ("N", ctypes.c_double), ("bouss", ctypes.c_int),
    ]


class MLPWeights(ctypes.Structure):
    """Mirror of ``gbs_mlp_weights`` (device pointers)."""

    _fields_ = [(name, ctypes.c_void_p) for name in
                ("W1", "W2", "W3", "b1", "b2", "b3", "in_scale", "out_scale")]


_lock = threading.Lock()
_lib = None


def _declare(lib):
    P = ctypes.c_void_p
    PP = ctypes.POINTER(ctypes.c_void_p)
    I64P = ctypes.POINTER(ctypes.c_int64)
    DP = ctypes.POINTER(ctypes.c_double)
    sig = {
        "gbs_last_error": (ctypes.c_char_p, []),
        "gbs_version": (ctypes.c_char_p, []),
        "gbs_fft_plan_create": (ctypes.c_int, [ctypes.c_int, I64P, ctypes.c_int, ctypes.c_int, PP]),
        "gbs_fft_plan_destroy": (ctypes.c_int, [P]),
        "gbs_fft_r2c": (ctypes.c_int, [P, P, P, P]),
        "gbs_fft_c2r": (ctypes.c_int, [P, P, P, ctypes.c_int, P]),
        "gbs_ns_create": (ctypes.c_int, [ctypes.POINTER(NSParams), PP]),
        "gbs_ns_destroy": (ctypes.c_int, [P]),
        "gbs_ns_tendencies": (ctypes.c_int, [P, P, P, P]),
        "gbs_ns_step_rk4": (ctypes.c_int, [P, P, DP, DP, ctypes.c_int, P]),
        "gbs_ns_step": (ctypes.c_int, [P, ctypes.c_int, P, DP, DP, ctypes.c_int, P]),
        "gbs_ns_set_projection": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
        "gbs_ns_set_phase_shifts": (ctypes.c_int, [P, DP, DP]),
        "gbs_ns_max_velocity": (ctypes.c_int, [P, P, DP, P]),
        "gbs_cfl_update": (ctypes.c_double, [ctypes.c_double] * 4),
        "gbs_ns_spatial_means": (ctypes.c_int, [P, P, DP, P]),
        "gbs_ns_spectrum_size": (ctypes.c_int, [P, I64P]),
        "gbs_ns_spectrum": (ctypes.c_int, [P, P, P, P]),
        "gbs_spectra_sizes": (ctypes.c_int, [ctypes.c_int, I64P, ctypes.POINTER(ctypes.c_double),
                                             I64P]),
        "gbs_spectra": (ctypes.c_int, [ctypes.c_int, I64P, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int, P, P, P, P, P, P, P]),
        "gbs_ns_is_dealiased": (ctypes.c_int, [P, P, ctypes.POINTER(ctypes.c_int), P]),
        "gbs_ns_timing": (ctypes.c_int, [P, ctypes.c_int]),
        "gbs_ns_timing_report": (ctypes.c_int, [P, DP, I64P, ctypes.c_int, I64P]),
        "gbs_fft_c2r_noalloc": (ctypes.c_int, [ctypes.c_int, I64P, ctypes.c_int,
                                               ctypes.c_int, P, P, P]),
        "gbs_ns_set_turb_model": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_double,
                                                 ctypes.POINTER(MLPWeights)]),
        "gbs_mlp_grad_workspace": (ctypes.c_int64, [ctypes.c_int64]),
        "gbs_ns_set_forcing": (ctypes.c_int, [P, P]),
        "gbs_forcing_coarse": (ctypes.c_int, [ctypes.POINTER(ForcingParams), P, P, P, P,
                                              ctypes.c_double, ctypes.c_double, P, P, P]),
        "gbs_ens2d_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_double, PP]),
        "gbs_ens2d_destroy": (ctypes.c_int, [P]),
        "gbs_ens2d_set_params": (ctypes.c_int, [P, DP, DP, DP]),
        "gbs_ens2d_set_tuning": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "gbs_ens2d_step": (ctypes.c_int, [P, P, ctypes.c_int, ctypes.c_int, P]),
        "gbs_ens2d_nan_flag": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
        "gbs_ens2d_mixed_create": (ctypes.c_int, [ctypes.POINTER(P), ctypes.c_int,
                                                  ctypes.POINTER(P)]),
        "gbs_ens2d_mixed_destroy": (ctypes.c_int, [P]),
        "gbs_ens2d_mixed_set_tuning": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int,
                                                      ctypes.c_int]),
        "gbs_ens2d_persistent_step": (ctypes.c_int, [P, ctypes.POINTER(P), ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_double,
                                                     ctypes.c_int, P]),
        "gbs_ens2d_persistent_status": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
        "gbs_ens2d_persistent_set_chunk": (ctypes.c_int, [P, ctypes.c_int]),
        "gbs_ens2d_mixed_step": (ctypes.c_int, [P, ctypes.POINTER(P), ctypes.c_int,
                                                ctypes.c_int, P]),
        "gbs_spectral_resample": (ctypes.c_int, [I64P, I64P, ctypes.c_int, DP,
                                                 ctypes.c_double, ctypes.c_int, P, P, P]),
        "gbs_products6": (ctypes.c_int, [P, P, ctypes.c_int64, P, ctypes.c_int, P]),
        "gbs_velocity_gradients": (ctypes.c_int, [I64P, DP, I64P, ctypes.c_int, P, P, P]),
        "gbs_mlp_forward": (ctypes.c_int, [ctypes.POINTER(MLPWeights), P, ctypes.c_int64, P,
                                           ctypes.c_int64, P]),
        "gbs_mlp_forward_bf16": (ctypes.c_int, [ctypes.POINTER(MLPWeights), P, ctypes.c_int64,
                                                P, ctypes.c_int64, P]),
        "gbs_mlp_grad": (ctypes.c_int, [ctypes.POINTER(MLPWeights), P, P, ctypes.c_int64, P,
                                        ctypes.c_int64, ctypes.c_double, P, P, P, P]),
        "gbs_mlp_adam": (ctypes.c_int, [P, P, P, P, ctypes.c_int64, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(MLPWeights), P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load(build_if_missing=True):
    """Return the loaded library (building it in tree once if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists() and build_if_missing:
            from .build import build
            build()
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m fluidsim_gb300.build`"
            )
        lib = ctypes.CDLL(str(LIB_PATH))
        _declare(lib)
        _lib = lib
        return lib


def check(rc, what=""):
    """Map a GBS_E* return code to the exception the reference raises."""
    if rc == GBS_OK:
        return
    msg = _lib.gbs_last_error().decode(errors="replace") if _lib else ""
    text = f"{what}: {msg}" if what else msg
    if rc in (GBS_EINVAL, GBS_ENAN):
        raise ValueError(text)
    if rc == GBS_ENOMEM:
        raise MemoryError(text)
    raise RuntimeError(f"{text} (code {rc})")
