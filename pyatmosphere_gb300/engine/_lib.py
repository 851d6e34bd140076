"""ctypes binding of libatm.so (include/atm.h).

The library is built in-tree by ``pyatmosphere_gb300.build``.  There is no
fallback: if the library is missing or fails to load, every engine call
raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(_HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libatm.so")
SELFTEST_PATH = os.path.join(LIB_DIR, "libatm_selftest.so")

ABI_VERSION = 3
MAX_PUPILS = 8
FLAG_SIMT_GEMM = 1
FLAG_TC_GEMM = 2
FLAG_TC_CPASYNC = 4
FLAG_STEP_MEASURES = 8
FLAG_TC_N256 = 16
FLAG_TC_N128 = 32
FLAG_TILED = 64
FLAG_ROWMAJOR = 128
FLAG_FFT_SCREENS = 256
ERR_TIMEOUT = -5
ERR_NONFINITE = -6
STEP_SLOTS = 8
SOURCE_GAUSSIAN = 0
SOURCE_PLANE = 1

# per-realisation output slots (ATM_OUT_*)
OUT_ETA_TOTAL = 0
OUT_MEAN_X = 1
OUT_MEAN_Y = 2
OUT_MEAN_X2 = 3
OUT_MEAN_XY = 4
OUT_MEAN_Y2 = 5
OUT_MEAN_X2_R = 6
OUT_I_CENTER = 7
OUT_PUPIL0 = 8

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_float_p = ctypes.POINTER(ctypes.c_float)


class AtmChannelDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("resolution", ctypes.c_int32),
        ("delta", ctypes.c_double),
        ("source_kind", ctypes.c_int32),
        ("wvl", ctypes.c_double),
        ("w0", ctypes.c_double),
        ("F0", ctypes.c_double),
        ("n_screens", ctypes.c_int32),
        ("positions", _c_double_p),
        ("length", ctypes.c_double),
        ("losses_db", ctypes.c_double),
        ("path_output_loss", ctypes.c_int32),
        ("points", ctypes.c_int32),
        ("f_base", _c_float_p),
        ("shift_x", ctypes.c_double),
        ("shift_y", ctypes.c_double),
        ("n_pupils", ctypes.c_int32),
        ("pupil_radius", _c_double_p),
        ("pupil_shift_x", _c_double_p),
        ("pupil_shift_y", _c_double_p),
        ("n_tracked", ctypes.c_int32),
        ("tracked_radius", _c_double_p),
        ("batch", ctypes.c_int32),
        ("cheb_cut", ctypes.c_double),
        ("col_tile", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


class AtmPlanInfo(ctypes.Structure):
    _fields_ = [
        ("n_out", ctypes.c_int32),
        ("low_annuli", ctypes.c_int32),
        ("cheb_terms", ctypes.c_int32),
        ("gemm_k", ctypes.c_int32),
        ("workspace_bytes", ctypes.c_int64),
        ("launches_per_run", ctypes.c_int32),
        ("row_parts", ctypes.c_int32),
        ("col_tile", ctypes.c_int32),
        ("row_variant", ctypes.c_int32),
        ("col_variant", ctypes.c_int32),
        ("tuned", ctypes.c_int32),
        ("gemm_form", ctypes.c_int32),
        ("tiled", ctypes.c_int32),
    ]


# every exported entry point: name -> (restype, argtypes)
SIGNATURES = {
    "atm_abi_version": (ctypes.c_int, []),
    "atm_last_error": (ctypes.c_char_p, []),
    "atm_plan_create": (ctypes.c_int, [ctypes.POINTER(AtmChannelDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "atm_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "atm_plan_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AtmPlanInfo)]),
    "atm_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p]),
    "atm_screen": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p]),
    "atm_vacuum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                  ctypes.c_void_p]),
    "atm_measures": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    "atm_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "atm_structure_function": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    "atm_plan_set_variants": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "atm_profile_begin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "atm_profile_end": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "atm_fma_probe": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                     ctypes.c_void_p]),
    "atm_fft_screen": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "atm_plan_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AtmChannelDesc)]),
    "atm_channel_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AtmChannelDesc),
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "atm_channel_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "atm_run_channel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "atm_run_fft": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]),
    "atm_draw_spectra": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "atm_channel_draw_spectra": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                                ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "atm_mlp_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                      ctypes.POINTER(ctypes.c_void_p)]),
    "atm_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "atm_mlp_num_params": (ctypes.c_int64, [ctypes.c_void_p]),
    "atm_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "atm_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    "atm_mlp_loss": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_mlp_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "atm_mlp_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_int32, ctypes.c_void_p]),
    "atm_mlp_infer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]),
    "atm_mlp_set_infer_form": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "atm_mlp_infer_form": (ctypes.c_int, [ctypes.c_void_p]),
    "atm_mlp_check": (ctypes.c_int, [ctypes.c_void_p]),
    "atm_tc_gemm_test": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_void_p,
                                        ctypes.c_int32, ctypes.c_void_p]),
    "atm_vacuum_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "atm_plan_check": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "atm_set_wait_budget": (ctypes.c_int, [ctypes.c_uint64]),
}

KIND_NAMES = ["screen_prep", "screen_table", "screen_gemm", "row_pass", "col_pass", "finalize", "tracked",
              "screen_eval"]

_lock = threading.Lock()
_lib = None


class EngineError(RuntimeError):
    """A libatm call failed; ``code`` is its ATM_ERR_* status."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


def load(path: str = LIB_PATH):
    """Loads libatm.so once; raises EngineError if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise EngineError(
                f"{path} is not built; run `python -m pyatmosphere_gb300.build` "
                "(or __graft_entry__.build()).  The engine has no CPU fallback.")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.atm_abi_version() != ABI_VERSION:
            raise EngineError(f"libatm ABI {lib.atm_abi_version()} != {ABI_VERSION}")
        _lib = lib
        return lib


def check(rc: int):
    if rc != 0:
        msg = load().atm_last_error().decode(errors="replace")
        raise EngineError(f"libatm error {rc}: {msg}", rc)


def load_selftest(path: str = SELFTEST_PATH):
    if not os.path.exists(path):
        raise EngineError(f"{path} is not built; run `python -m pyatmosphere_gb300.build`")
    lib = ctypes.CDLL(path)
    lib.atm_selftest_fft.restype = ctypes.c_int
    lib.atm_selftest_fft.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.atm_selftest_fft_twrec.restype = ctypes.c_int
    lib.atm_selftest_fft_twrec.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.atm_selftest_fft_twreg.restype = ctypes.c_int
    lib.atm_selftest_fft_twreg.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.atm_selftest_wfft.restype = ctypes.c_int
    lib.atm_selftest_wfft.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.atm_selftest_bessel.restype = ctypes.c_int
    lib.atm_selftest_bessel.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    lib.atm_selftest_turns.restype = ctypes.c_int
    lib.atm_selftest_turns.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    return lib
