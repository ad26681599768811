"""ctypes binding of the fastsht_gb300 C ABI (include/fastsht.h).

The shared library is built in-tree by ``fastsht_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

FSHT_OK = 0
FSHT_EINVAL = -1
FSHT_ENOMEM = -2
FSHT_ECUDA = -3
FSHT_ETIMEOUT = -4
FSHT_EUNSUPPORTED = -5
FSHT_ERANGE = -6
FSHT_PREC_FP64 = 0
FSHT_PREC_SPLIT = 1
FSHT_FLAG_POL = 1
FSHT_FLAG_ITER = 2
FSHT_FLAG_TABLES_ONLY = 4
FSHT_JOB_T2ALM, FSHT_JOB_ALM2T, FSHT_JOB_QU2EB, FSHT_JOB_EB2QU = 0, 1, 2, 3


class FshtJob(C.Structure):
    _fields_ = [("nside", C.c_int), ("lmax", C.c_int), ("nmaps", C.c_int), ("kind", C.c_int),
                ("precision", C.c_int), ("in0", C.c_void_p), ("in1", C.c_void_p),
                ("out0", C.c_void_p), ("out1", C.c_void_p)]

KCAT_NAMES = ["ring_fft_fwd", "ring_fft_inv", "legendre_analysis", "legendre_synthesis",
              "fourier_residual", "split_slice", "other", "split_lambda"]
KCAT_COUNT = 8

_vp = C.c_void_p
_i = C.c_int
_sz = C.c_size_t

# name -> argtypes (all return int)
SIGNATURES = {
    "fsht_plan_create": [_i, _i, _i, _i, _i, _sz, _vp, C.POINTER(_vp)],
    "fsht_plan_destroy": [_vp],
    "fsht_plan_set_stream": [_vp, _vp],
    "fsht_plan_info": [_vp, C.POINTER(_sz), C.POINTER(_i)],
    "fsht_plan_ring_skip": [_vp, C.POINTER(_i)],
    "fsht_t2alm": [_vp, _vp, _vp, _i, _i, _i],
    "fsht_t2alm_host": [_vp, _vp, _vp, _vp, _vp, _i, _i, _i],
    "fsht_plan_set_host_read": [_vp, _i],
    "fsht_alm2t": [_vp, _vp, _vp, _i],
    "fsht_t2alm_noalloc": [_i, _i, _vp, _vp, _i, _vp],
    "fsht_qu2eb": [_vp, _vp, _vp, _vp, _vp, _i, _i],
    "fsht_qu2e": [_vp, _vp, _vp, _vp, _i],
    "fsht_qu2b": [_vp, _vp, _vp, _vp, _i],
    "fsht_eb2qu": [_vp, _vp, _vp, _vp, _vp, _i],
    "fsht_convert_alm_healpy": [_vp, _vp, _vp, _i],
    "fsht_alm2cl": [_vp, _vp, _vp, _i, _i, _i, _vp],
    "fsht_alm_filter": [_vp, _vp, _i, _i, _vp],
    "fsht_alm_norm": [_vp, _vp, _vp, _vp, C.c_double, _i, _i, _vp],
    "fsht_cl2alm": [_vp, _i, _i, _i, _i, C.c_ulonglong, _vp, _vp, _vp, _vp],
    "fsht_convert_alm_healpy_inv": [_vp, _vp, _vp, _i],
    "fsht_plan_sync": [_vp],
    "fsht_plan_check": [_vp],
    "fsht_selftest_wait_timeout": [_vp],
    "fsht_host_alloc": [_sz, C.POINTER(_vp)],
    "fsht_host_free": [_vp],
    "fsht_host_mapped": [_vp, _sz, C.POINTER(_i)],
    "fsht_run_stage": [_vp, _i, _vp, _vp, _i],
    "fsht_profile_enable": [_vp, _i],
    "fsht_profile_read": [_vp, _i, C.POINTER(_i), C.POINTER(C.c_double)],
    "fsht_measure_fp64_peak": [C.POINTER(C.c_double)],
    "fsht_measure_fp32_peak": [C.POINTER(C.c_double)],
    "fsht_measure_dmma_peak": [C.POINTER(C.c_double)],
    "fsht_measure_umma_rate": [C.c_int, C.POINTER(C.c_double)],
    "fsht_last_error": [C.c_char_p, _sz],
    "fsht_batch_create": [C.c_void_p, _i, _i, _sz, _i, _vp, C.POINTER(_vp)],
    "fsht_batch_run": [_vp],
    "fsht_batch_sync": [_vp],
    "fsht_batch_info": [_vp, C.POINTER(_i), C.POINTER(_i)],
    "fsht_batch_plan_tuning": [_vp, _i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i),
                               C.POINTER(_i)],
    "fsht_batch_destroy": [_vp],
    "fsht_plan_autotune": [_vp, _i],
    "fsht_job_workspace": [_vp, _vp, _i, C.POINTER(_sz)],
    "fsht_run_job": [_vp, _vp, _vp, _sz, _vp],
    "fsht_plan_tuning": [_vp, C.POINTER(_i), C.POINTER(_i)],
    "fsht_plan_set_contraction": [_vp, _i, _i, _i],
    "fsht_plan_contraction": [_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)],
}

_lib = None
_lock = threading.Lock()


class FshtError(RuntimeError):
    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func} failed with status {code}: {msg}")
        self.code = code


def lib_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = False):
    """Loads (once) and returns the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not path.exists():
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(
                    f"fastsht_gb300 CUDA library not built ({path} missing); run "
                    "`python -m fastsht_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(str(path))
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _i
        _lib = lib
        return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(2048)
    lib.fsht_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def call(name: str, *args) -> int:
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != FSHT_OK:
        msg = last_error()
        if rc == FSHT_EINVAL:
            raise ValueError(f"{name}: {msg}")
        raise FshtError(rc, name, msg)
    return rc
