"""ctypes binding of the drop-in layer (include/bpd_compat.h): the reference
pipeline API -- createSubharmonicInfo, deredden, generate_harmonics_ffdot,
generate_harmonic_ffdot_data, perform_fft_harmonics, perform_convolution,
perform_inversefft, generate_fundamental_powers, perform_harmonic_summing,
search_ffdot_powers -- with the reference's names and structs."""
from __future__ import annotations

import ctypes as C

from . import native as N

_c64p = C.c_void_p


class SubharmonicInfo(C.Structure):
    _fields_ = [("maxHarmonic", C.c_ushort), ("currentHarmonic", C.c_ushort), ("zmax", C.c_int),
                ("totalKernelsTemplates", C.c_ushort), ("kernelFFTLength", C.c_int),
                ("z", C.POINTER(C.c_int)), ("kernelHalfWidth", C.POINTER(C.c_ushort)),
                ("kernels_data", C.c_void_p)]


class FfdotInfo(C.Structure):
    _fields_ = [("currentHarmonic", C.c_ushort), ("maxHarmonic", C.c_ushort), ("numrs", C.c_int),
                ("numzs", C.c_int), ("rlo", C.c_int), ("zlo", C.c_int), ("rhi", C.c_double),
                ("fftlen", C.c_int)]


class Candidates(C.Structure):
    _fields_ = [("power", C.c_float), ("sigma", C.c_float), ("numharm", C.c_int), ("r", C.c_double),
                ("z", C.c_double), ("pows", C.c_void_p), ("hirs", C.c_void_p), ("hizs", C.c_void_p),
                ("derivs", C.c_void_p)]


_us, _lp = C.c_ushort, C.POINTER(C.c_long)
SIGNATURES = {
    "accel_compat_set_uselen": (None, [C.c_int]),
    "accel_compat_get_uselen": (C.c_int, []),
    "accel_compat_status": (C.c_int, []),
    "createSubharmonicInfo": (C.POINTER(SubharmonicInfo), [C.c_int, C.c_int]),
    "readData": (C.c_long, [C.c_char_p, C.POINTER(C.POINTER(C.c_float))]),
    "freeData": (None, [C.POINTER(C.c_float)]),
    "freeSubharmonicInfo": (None, [C.POINTER(SubharmonicInfo), C.c_int]),
    "calc_required_z": (C.c_int, [C.c_double, C.c_double]),
    "calc_required_r": (C.c_double, [C.c_double, C.c_double]),
    "index_from_r": (C.c_int, [C.c_double, C.c_double]),
    "index_from_z": (C.c_int, [C.c_double, C.c_double]),
    "getTotalHarmonics": (C.c_int, [C.c_int]),
    "realToComplexFFT": (C.c_uint, [C.POINTER(C.c_float), C.c_long, C.POINTER(C.c_void_p), C.c_int]),
    "complexToComplexFFT": (C.c_uint, [_c64p, C.c_uint, C.POINTER(C.c_void_p), C.c_int]),
    "inverseComplexToComplexFFT": (C.c_uint, [_c64p, C.c_uint, C.POINTER(C.c_void_p), C.c_int]),
    "deredden": (None, [_c64p, C.c_uint]),
    "generate_harmonics_ffdot": (None, [_us, _us, C.POINTER(SubharmonicInfo), C.c_double, C.c_double,
                                        C.c_double, C.POINTER(FfdotInfo), C.POINTER(_us)]),
    "generate_harmonic_ffdot_data": (None, [_us, C.c_long, C.POINTER(FfdotInfo), C.POINTER(_us), _lp,
                                            _c64p, C.c_long, C.c_long, _c64p]),
    "perform_fft_harmonics": (None, [_us, _c64p, _lp, _c64p]),
    "perform_convolution": (None, [_us, _c64p, C.POINTER(FfdotInfo), C.POINTER(SubharmonicInfo), _lp,
                                   _c64p, _lp]),
    "perform_inversefft": (None, [_us, _c64p, _lp, _c64p]),
    "generate_fundamental_powers": (None, [_us, _c64p, _lp, C.POINTER(FfdotInfo),
                                           C.POINTER(SubharmonicInfo), C.c_void_p]),
    "perform_harmonic_summing": (None, [_us, _c64p, _lp, C.POINTER(FfdotInfo),
                                        C.POINTER(SubharmonicInfo), C.c_void_p, C.c_int,
                                        C.POINTER(_us), C.POINTER(_us), C.c_int]),
    "initialize_cuda_plans": (None, [_us, C.POINTER(SubharmonicInfo)]),
    "free_cuda_plans": (None, [_us]),
    "convolveSignal": (None, [C.c_int, C.c_int, _c64p, _c64p, C.c_int, _c64p]),
    "generatePowers": (None, [C.c_int, C.c_int, C.c_int, _c64p, C.c_float, C.c_void_p]),
    "addPowers": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _c64p,
                         C.c_float, C.c_void_p, C.c_int]),
    "search_ffdot_powers_n": (C.POINTER(Candidates), [C.POINTER(FfdotInfo), C.c_int, C.c_float,
                                                      C.c_longlong, _lp]),
    "search_ffdot_powers": (C.POINTER(Candidates), [C.POINTER(FfdotInfo), C.c_int, C.c_float,
                                                    C.c_longlong, C.POINTER(Candidates)]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = N.lib()
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check():
    rc = lib().accel_compat_status()
    if rc != 0:
        raise N.AccelError(rc, lib().accel_last_error().decode())
