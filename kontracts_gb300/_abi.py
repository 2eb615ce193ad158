"""ctypes mirror of include/kontract_gpu.h (the engine's C ABI).

The structures below must match the header field for field; the CPU tests
check their sizes against the library.
"""
from __future__ import annotations

import ctypes as C
import os

KX_OK = 0
KX_UNKNOWN_ASSET = 1
KX_TIME_OUT_OF_RANGE = 2
KX_STEP_OUT_OF_RANGE = 3
KX_INCONSISTENT_PATH = 4
KX_SERDE = 5
KX_MALFORMED_CONTRACT = 6
KX_UNSUPPORTED = 7
KX_INVALID_ARGUMENT = 8
KX_LSM_MONOMIAL = 0
KX_VR_ANTITHETIC = 1
KX_VR_CONTROL_VARIATE = 2
KX_LSM_LAGUERRE = 1
KX_CUDA_ERROR = 9
KX_DEVICE_TIMEOUT = 10
KX_NO_DEVICE = 11

STATUS_NAMES = {
    0: "Ok", 1: "UnknownAsset", 2: "TimeOutOfRange", 3: "StepOutOfRange",
    4: "InconsistentPath", 5: "Serde", 6: "MalformedContract", 7: "Unsupported",
    8: "InvalidArgument", 9: "CudaError", 10: "DeviceTimeout", 11: "NoDevice",
}

KX_MODEL_GBM = 0
KX_MODEL_HESTON = 1
KX_HESTON_REFERENCE_FLOOR = 0
KX_HESTON_FULL_TRUNCATION = 1
KX_RNG_PHILOX = 0
KX_RNG_SHARED_DRAWS = 1
KX_PREC_FP32 = 0
KX_PREC_FP64 = 1
KX_PREC_FP32_KAHAN = 2


class KxModel(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("heston_scheme", C.c_int32),
        ("s0", C.c_double), ("mu", C.c_double), ("sigma", C.c_double),
        ("v0", C.c_double), ("kappa", C.c_double), ("theta", C.c_double),
        ("sigma_v", C.c_double), ("rho", C.c_double), ("r", C.c_double),
        ("asset", C.c_char_p),
    ]


class KxMcConfig(C.Structure):
    _fields_ = [
        ("n_paths", C.c_uint64), ("seed", C.c_uint64), ("steps_per_year", C.c_uint32),
        ("rng", C.c_int32), ("precision", C.c_int32), ("flags", C.c_int32),
        ("rate", C.c_double),
    ]


class KxPriceResult(C.Structure):
    _fields_ = [
        ("price", C.c_double), ("sample_std", C.c_double), ("std_error", C.c_double),
        ("ci95_low", C.c_double), ("ci95_high", C.c_double), ("n_paths", C.c_uint64),
    ]


class KxBumps(C.Structure):
    _fields_ = [
        ("spot", C.c_double), ("vol", C.c_double), ("rate", C.c_double),
        ("relative", C.c_int32), ("smooth", C.c_int32), ("smoothing_width", C.c_double),
    ]


KX_MAX_ASSETS = 7


class KxMultiGbm(C.Structure):
    _fields_ = [("n_assets", C.c_uint32), ("reserved", C.c_uint32), ("names", C.c_char_p * KX_MAX_ASSETS),
                ("s0", C.c_double * KX_MAX_ASSETS), ("mu", C.c_double * KX_MAX_ASSETS),
                ("sigma", C.c_double * KX_MAX_ASSETS), ("corr", C.c_double * (KX_MAX_ASSETS * KX_MAX_ASSETS))]


KX_MLMC_MAX_LEVELS = 20


class KxMlmcCfg(C.Structure):
    _fields_ = [("n_levels", C.c_uint32), ("cost_per_step", C.c_uint32), ("pilot_paths", C.c_uint64),
                ("target_variance", C.c_double)]


class KxGreeks(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "price", "delta", "gamma", "vega", "rho",
        "price_se", "delta_se", "gamma_se", "vega_se", "rho_se")]


class KxMlmcResult(C.Structure):
    _fields_ = [("price", KxPriceResult), ("n_levels", C.c_uint32), ("reserved", C.c_uint32),
                ("level_means", C.c_double * (KX_MLMC_MAX_LEVELS + 1)),
                ("level_variances", C.c_double * (KX_MLMC_MAX_LEVELS + 1)),
                ("level_costs", C.c_uint64 * (KX_MLMC_MAX_LEVELS + 1)),
                ("level_paths", C.c_uint64 * (KX_MLMC_MAX_LEVELS + 1)),
                ("total_cost", C.c_uint64)]


class KxAdjointCfg(C.Structure):
    _fields_ = [("checkpoint_every", C.c_uint32), ("reserved", C.c_int32),
                ("smoothing_width", C.c_double)]


class KxSens(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "price", "price_se", "d_s0", "d_sigma", "d_r",
        "d_v0", "d_kappa", "d_theta", "d_sigma_v", "d_rho",
        "se_s0", "se_sigma", "se_r", "se_v0", "se_kappa", "se_theta", "se_sigma_v", "se_rho",
        "smoothing_width")]


class KxLaunchStats(C.Structure):
    _fields_ = [
        ("kernel_ms", C.c_double), ("reduce_ms", C.c_double), ("total_ms", C.c_double),
        ("path_steps", C.c_uint64), ("steps_simulated", C.c_uint64),
        ("kernel_launches", C.c_uint32), ("grid_blocks", C.c_uint32),
        ("block_threads", C.c_uint32), ("path_kernel", C.c_uint32),
        ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
    ]


class KxPlanInfo(C.Structure):
    _fields_ = [
        ("n_assets", C.c_uint32), ("n_fixed_dates", C.c_uint32), ("horizon", C.c_double),
        ("needs_fine_grid", C.c_int32), ("n_triggers", C.c_int32), ("n_flows", C.c_int32),
        ("n_accumulators", C.c_int32),
    ]


class KxBookInfo(C.Structure):
    _fields_ = [
        ("n_contracts", C.c_uint32), ("n_groups", C.c_uint32), ("n_paths", C.c_uint64), ("path_steps", C.c_uint64),
        ("tune_ms", C.c_double), ("group_kernel", C.c_uint32 * 4), ("group_minb", C.c_uint32 * 4),
        ("group_item_paths", C.c_uint32 * 4), ("group_contracts", C.c_uint32 * 4),
    ]


KX_BOOK_TUNE = 1
KX_STATS_CHUNK = 16384


class KxChunkStats(C.Structure):
    _fields_ = [("n", C.c_double), ("mean", C.c_double), ("m2", C.c_double)]

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libkontract_gpu.so")

# name -> (restype, argtypes); every symbol the header declares.
_P = C.c_void_p
SIGNATURES = {
    "kx_abi_version": (C.c_int32, []),
    "kx_last_error_message": (C.c_char_p, []),
    "kx_last_error_payload": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "kx_compile": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "kx_program_free": (None, [_P]),
    "kx_program_plan": (C.c_int, [_P, C.POINTER(KxPlanInfo), C.POINTER(C.c_double), C.c_size_t,
                                  C.c_char_p, C.c_size_t]),
    "kx_time_grid": (C.c_int, [_P, C.c_uint32, C.c_int32, C.POINTER(C.c_double), C.c_size_t,
                               C.POINTER(C.c_size_t)]),
    "kx_set_shared_draws": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_uint64,
                                      C.c_uint64]),
    "kx_clear_shared_draws": (C.c_int, []),
    "kx_price": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                           C.POINTER(KxPriceResult), C.POINTER(C.c_double)]),
    "kx_price_fixed_scratch": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                         C.POINTER(KxPriceResult), C.POINTER(C.c_double)]),
    "kx_price_batch_shared": (C.c_int, [C.c_size_t, C.POINTER(_P), C.POINTER(KxModel),
                                        C.POINTER(KxMcConfig), C.POINTER(KxPriceResult)]),
    "kx_price_batch_sens": (C.c_int, [C.c_size_t, C.POINTER(_P), C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                      C.POINTER(KxPriceResult), C.POINTER(KxSens)]),
    "kx_price_portfolio": (C.c_int, [C.c_size_t, C.POINTER(_P), C.POINTER(KxModel),
                                     C.POINTER(KxMcConfig), C.POINTER(KxPriceResult),
                                     C.POINTER(KxSens)]),
    "kx_greeks_bump": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                 C.POINTER(KxBumps), C.POINTER(KxGreeks)]),
    "kx_greek_surface": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_double),
                                   C.c_size_t, C.POINTER(KxMcConfig), C.POINTER(KxBumps), C.POINTER(KxGreeks)]),
    "kx_calib_gbm_prices": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_double),
                                      C.c_size_t, C.POINTER(KxMcConfig), C.POINTER(C.c_double)]),
    "kx_calib_heston_objective": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_double), C.c_size_t,
                                            C.POINTER(C.c_double), C.c_size_t, C.POINTER(KxMcConfig),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "kx_price_mlmc": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig), C.POINTER(KxMlmcCfg),
                                C.POINTER(KxMlmcResult)]),
    "kx_mlmc_level_variance": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig), C.c_uint32, C.c_uint64,
                                         C.POINTER(C.c_double)]),
    "kx_mlmc_optimal_allocation": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_size_t, C.c_double,
                                             C.POINTER(C.c_uint64)]),
    "kx_price_multi": (C.c_int, [_P, C.POINTER(KxMultiGbm), C.POINTER(KxMcConfig), C.POINTER(KxPriceResult),
                                 C.POINTER(C.c_double)]),
    "kx_greeks_adjoint": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                    C.POINTER(KxAdjointCfg), C.POINTER(KxSens)]),
    "kx_price_american_lsm": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                        C.POINTER(C.c_double), C.c_size_t, C.c_int32,
                                        C.POINTER(KxPriceResult)]),
    "kx_price_american_lsm_basis": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                              C.POINTER(C.c_double), C.c_size_t, C.c_int32, C.c_int32,
                                              C.POINTER(KxPriceResult)]),
    "kx_price_american_lsm_paths": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                              C.POINTER(C.c_double), C.c_size_t, C.c_int32, C.c_int32,
                                              C.POINTER(KxPriceResult), C.POINTER(C.c_double)]),
    "kx_price_american_lsm_batch": (C.c_int, [C.c_size_t, C.POINTER(_P), C.POINTER(KxModel),
                                              C.POINTER(KxMcConfig), C.POINTER(C.POINTER(C.c_double)),
                                              C.POINTER(C.c_size_t), C.c_int32, C.c_int32,
                                              C.POINTER(KxPriceResult)]),
    "kx_measure_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
    "kx_price_chunks": (C.c_int, [_P, C.POINTER(KxModel), C.POINTER(KxMcConfig), C.c_uint64,
                                  C.POINTER(KxChunkStats), C.c_size_t, C.POINTER(C.c_size_t)]),
    "kx_merge_chunks": (C.c_int, [C.POINTER(KxChunkStats), C.c_size_t, C.POINTER(KxPriceResult)]),
    "kx_chunk_moments": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_uint32,
                                   C.POINTER(KxChunkStats)]),
    "kx_book_create": (C.c_int, [C.c_size_t, C.POINTER(_P), C.POINTER(KxModel), C.POINTER(KxMcConfig),
                                 C.c_uint32, C.POINTER(_P)]),
    "kx_book_price": (C.c_int, [_P, C.POINTER(KxPriceResult)]),
    "kx_book_set_models": (C.c_int, [_P, C.POINTER(KxModel)]),
    "kx_book_get_info": (C.c_int, [_P, C.POINTER(KxBookInfo)]),
    "kx_book_free": (None, [_P]),
    "kx_last_launch_stats": (C.c_int, [C.POINTER(KxLaunchStats)]),
    "kx_device_info": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
}

_lib = None


def load(path: str | None = None):
    """Load the engine's shared library (built by __graft_entry__.build()).

    Raises OSError if it is missing: there is no fallback implementation.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"kontract GPU engine not built: {p} is missing "
                      "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
