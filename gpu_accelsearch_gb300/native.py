"""ctypes binding of libaccelsearch.so (include/accelsearch.h).

This is the only way the package reaches the GPU: there is no CPU or
library fallback.  :func:`lib` raises if the shared library is missing or
fails to load.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libaccelsearch.so")

ACCEL_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "candidate capacity exceeded", -5: "unsupported shape", -6: "over HBM budget"}


class AccelError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("zmax", C.c_int), ("numharm", C.c_int), ("fftlen", C.c_int),
                ("uselen", C.c_int), ("whiten_initbuf", C.c_int), ("whiten_maxbuf", C.c_int),
                ("sigma", C.c_double), ("numindep", C.c_double), ("template_fp16", C.c_int),
                ("chunk_segments", C.c_int), ("cand_capacity", C.c_longlong),
                ("device", C.c_int), ("exact_rsqrt", C.c_int), ("short_transforms", C.c_int),
                ("reserved", C.c_int * 5)]


class Harmonic(C.Structure):
    _fields_ = [("harmnum", C.c_int), ("maxharm", C.c_int), ("zmax", C.c_int),
                ("numzs", C.c_int), ("fftlen", C.c_int), ("halfwidth", C.c_int),
                ("zlo", C.c_int), ("plane_width", C.c_int)]


class Candidate(C.Structure):
    _fields_ = [("trial", C.c_int), ("step", C.c_int), ("r", C.c_double), ("z", C.c_double),
                ("numharm", C.c_int), ("power", C.c_float), ("sigma", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("max_active", C.c_int), ("fftlen", C.c_int),
                ("numharm", C.c_int), ("sigma", C.c_double), ("chunk_segments", C.c_int),
                ("device", C.c_int), ("max_wait_s", C.c_double), ("max_chunk_segments", C.c_int),
                ("reserved", C.c_int * 5)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong),
                ("completed", C.c_longlong), ("queued", C.c_longlong), ("active", C.c_longlong),
                ("bytes_in_use", C.c_double), ("cells", C.c_longlong), ("gpu_ms", C.c_double),
                ("admit_ms", C.c_double), ("group_ms", C.c_double), ("gap_ms", C.c_double),
                ("idle_ms", C.c_double), ("wait_ms", C.c_double), ("launch_ms", C.c_double),
                ("prep_gpu_ms", C.c_double),
                ("groups", C.c_longlong),
                ("group_segments", C.c_longlong)]


class Tuning(C.Structure):
    _fields_ = [("chunk_segments", C.c_int), ("plane_split", C.c_int), ("fused_sum", C.c_int),
                ("hsum_rowwise", C.c_int), ("serial_sum", C.c_int), ("hsum_pipelined", C.c_int),
                ("graph", C.c_int), ("hsum_tile_rows", C.c_int), ("persistent", C.c_int),
                ("hsum_row_copies", C.c_int), ("wait_test", C.c_int)]


class Optimized(C.Structure):
    _fields_ = [("cand", Candidate), ("r_grid", C.c_double), ("z_grid", C.c_double),
                ("harm_power", C.c_float * 16), ("f", C.c_double), ("fdot", C.c_double),
                ("period", C.c_double), ("pdot", C.c_double)]


class FilterbankInfo(C.Structure):
    _fields_ = [("nchans", C.c_int), ("nbits", C.c_int), ("nifs", C.c_int), ("nsamples", C.c_longlong),
                ("tsamp", C.c_double), ("fch1", C.c_double), ("foff", C.c_double),
                ("tstart", C.c_double), ("source_name", C.c_char * 80), ("header_bytes", C.c_int),
                ("is_signed", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("launches", C.c_longlong), ("kind_launches", C.c_longlong * 7),
                ("kind_ms", C.c_double * 7), ("segments", C.c_longlong),
                ("cells", C.c_longlong), ("search_ms", C.c_double), ("searches", C.c_longlong),
                ("graph_launches", C.c_longlong), ("graph_builds", C.c_longlong)]


KINDS = ["prep", "plane", "hsum", "whiten", "rfft", "fund", "step"]

_vp, _ll, _llp = C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)
SIGNATURES = {
    "accel_version": (C.c_char_p, []),
    "accel_last_error": (C.c_char_p, []),
    "accel_config_init": (None, [C.POINTER(Config)]),
    "accel_create": (C.c_int, [C.POINTER(Config), C.POINTER(_vp)]),
    "accel_destroy": (C.c_int, [_vp]),
    "accel_set_stream": (C.c_int, [_vp, _vp]),
    "accel_synchronize": (C.c_int, [_vp]),
    "accel_profile": (C.c_int, [_vp, C.c_int]),
    "accel_get_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "accel_reset_stats": (C.c_int, [_vp]),
    "accel_get_tuning": (C.c_int, [_vp, C.POINTER(Tuning)]),
    "accel_set_tuning": (C.c_int, [_vp, C.POINTER(Tuning)]),
    "accel_num_harmonics": (C.c_int, [_vp]),
    "accel_num_stages": (C.c_int, [_vp]),
    "accel_uselen": (C.c_int, [_vp]),
    "accel_harmonic_info": (C.c_int, [_vp, C.c_int, C.POINTER(Harmonic)]),
    "accel_get_power_cuts": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "accel_set_power_cuts": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "accel_first_bin": (_ll, [_ll, C.c_double]),
    "accel_power_cut": (C.c_double, [C.c_double, C.c_int, C.c_double]),
    "accel_sigma_of_power": (C.c_double, [C.c_double, C.c_int, C.c_double]),
    "accel_step_count": (_ll, [_vp, _ll, C.c_double]),
    "accel_step_harmonic": (C.c_int, [_ll, C.c_int, C.c_int, C.c_int, C.c_int, _llp]),
    "accel_harmonic_indices": (C.c_int, [_ll, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    "accel_autotune": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_int), C.c_int, C.c_int,
                                 C.POINTER(Config), C.POINTER(Tuning), C.POINTER(C.c_double)]),
    "accel_search": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), _llp, C.POINTER(C.c_double),
                               C.c_int, _llp]),
    "accel_search_spectra": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), _llp, _llp, _llp]),
    "accel_candidates": (C.c_int, [_vp, C.POINTER(Candidate), _ll, _llp]),
    "accel_sift_candidates": (C.c_int, [C.POINTER(Candidate), C.c_longlong, C.c_double, C.c_int,
                                        C.c_double, C.POINTER(Candidate), C.c_longlong,
                                        C.POINTER(C.c_longlong)]),
    "accel_optimize_candidates": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(C.c_longlong),
                                            C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                            C.POINTER(Candidate), C.c_longlong,
                                            C.c_int, C.POINTER(Optimized)]),
    "accel_trial_spectrum": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(C.c_longlong)]),
    "accel_whiten": (C.c_int, [_vp, _vp, _ll]),
    "accel_whiten_blocks": (C.c_int, [_ll, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      _ll, _llp]),
    "accel_rfft": (C.c_int, [_vp, _vp, _ll, _vp]),
    "accel_prepare_segments": (C.c_int, [_vp, _vp, _ll, _llp, C.c_int, _vp]),
    "accel_power_planes": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "accel_sum_harmonics": (C.c_int, [_vp, _vp, _llp, C.c_int, _vp, _llp]),
    "accel_layout": (C.c_int, [_vp, _llp, _llp, _llp, _llp, C.POINTER(C.c_int)]),
    "accel_bank_spectra": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "accel_whiten_noalloc": (C.c_int, [_vp, _ll, C.c_int, C.c_int, _vp]),
    "accel_server_config_init": (None, [C.POINTER(ServerConfig)]),
    "accel_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "accel_server_destroy": (C.c_int, [_vp]),
    "accel_server_submit": (C.c_int, [_vp, _vp, _ll, C.c_double, C.c_int, _llp]),
    "accel_server_wait": (C.c_int, [_vp, _ll, C.c_double, C.POINTER(C.c_int)]),
    "accel_server_result": (C.c_int, [_vp, _ll, C.POINTER(Candidate), _ll, _llp,
                                      C.POINTER(C.c_double)]),
    "accel_server_release": (C.c_int, [_vp, _ll]),
    "accel_server_get_stats": (C.c_int, [_vp, C.POINTER(ServerStats)]),
    "accel_server_timing": (C.c_int, [_vp, _ll, C.POINTER(C.c_double)]),
    "accel_dedisperse_delays": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
    "accel_dedisperse": (C.c_int, [_vp, C.c_int, _ll, C.POINTER(C.c_int), C.c_int, _vp, _ll, _vp]),
    "accel_read_filterbank": (C.c_int, [C.c_char_p, C.POINTER(FilterbankInfo),
                                        C.POINTER(C.POINTER(C.c_float))]),
    "accel_free_host": (None, [_vp]),
}

_lib = None


def lib():
    """Load libaccelsearch.so (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run __graft_entry__.build() or "
                               "python -m gpu_accelsearch_gb300.build")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != ACCEL_OK:
        raise AccelError(rc, lib().accel_last_error().decode())
    return rc


def exported_symbols():
    """Names declared in include/accelsearch.h that the library must export."""
    return sorted(SIGNATURES)
