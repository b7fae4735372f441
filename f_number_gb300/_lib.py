"""ctypes binding of the C ABI in include/fnum.h (libfnum.so, built in-tree).

The library is required: there is no CPU fallback for the beamformer.  If
libfnum.so is missing every call raises ``LibraryNotBuilt``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfnum.so")

EXPORTS = (
    "fnum_abi_version", "fnum_status_string", "fnum_status_id", "fnum_device_count", "fnum_band",
    "fnum_f_number_values", "fnum_window_value", "fnum_das_pw", "fnum_das_sa", "fnum_pw_plan_create",
    "fnum_sa_plan_create", "fnum_plan_execute", "fnum_plan_execute_dft", "fnum_plan_execute_beamform",
    "fnum_plan_info_get", "fnum_plan_f_numbers", "fnum_plan_destroy", "fnum_diag_fp32_peak",
    "fnum_das_pw_noalloc", "fnum_bmode", "fnum_plan_autotune", "fnum_batch_create", "fnum_batch_execute",
    "fnum_batch_frame_times", "fnum_batch_destroy", "fnum_pw_plan_set_sound_speed", "fnum_pw_sharpness_grad",
    "fnum_plan_m_signal", "fnum_plan_set_kernel_variant", "fnum_diag_mma_f16_peak", "fnum_host_cache_info",
    "fnum_plan_spectra", "fnum_pw_adjoint", "fnum_plan_set_spectra", "fnum_das_pw_sharpness_grad",
    "fnum_batch_info", "fnum_plan_set_shape",
)

ABI_VERSION = 4   # FNUM_ABI_VERSION of include/fnum.h

# status codes (fnum_status)
OK = 0
ERR_NO_DEVICE = 1
ERR_ARGUMENT = 18
ERR_INTERNAL = 21
ERR_NOALLOC_TOO_LARGE = 24
ERR_M_ELEMENTS = 25

# window ids, normalisations, F-number kinds, flags (fnum.h)
WINDOW_BOXCAR, WINDOW_HANN, WINDOW_TUKEY, WINDOW_TRIANGULAR = 0, 1, 2, 4
NORM_OFF, NORM_ON, NORM_WINDOWED = 0, 1, 2
F_DEFAULT, F_CONSTANT, F_ANGLE_LB, F_DISTANCE_CONSTANT, F_DISTANCE_NONE, F_DIRECTIVITY, F_SZABO = range(7)
OBLIQUITY_RIGID, OBLIQUITY_SOFT = 0, 1
FLAG_COMPOUND, FLAG_PLAIN_KERNEL, FLAG_SAFT_INTENDED, FLAG_M_SEMANTICS = 0x1, 0x2, 0x4, 0x8

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


class Window(C.Structure):
    _fields_ = [("id", C.c_int), ("parameter", C.c_double)]


class FNumber(C.Structure):
    _fields_ = [("kind", C.c_int), ("obliquity", C.c_int), ("p", C.c_double * 3)]


class PWDesc(C.Structure):
    _fields_ = [
        ("positions_x", _dp), ("n_x", C.c_int),
        ("positions_z", _dp), ("n_z", C.c_int),
        ("n_samples", C.c_int), ("n_elements", C.c_int),
        ("f_s", C.c_double),
        ("element_width", C.c_double), ("element_pitch", C.c_double),
        ("c_0", C.c_double),
        ("f_bounds", _dp),
        ("index_t0", C.c_double),
        ("window", Window),
        ("f_number", FNumber),
        ("f_number_values", _dp), ("n_f_number_values", C.c_int),
        ("normalization", C.c_int),
        ("device", C.c_int),
        ("normalization_window", Window),
    ]


class SADesc(C.Structure):
    _fields_ = [
        ("positions_x", _dp), ("n_x", C.c_int),
        ("positions_z", _dp), ("n_z", C.c_int),
        ("n_samples", C.c_int), ("n_elements", C.c_int),
        ("f_s", C.c_double),
        ("element_width", C.c_double), ("element_pitch", C.c_double),
        ("c_0", C.c_double),
        ("f_bounds", _dp),
        ("index_t0", C.c_double),
        ("window_tx", Window), ("window_rx", Window),
        ("f_number_tx", FNumber), ("f_number_rx", FNumber),
        ("f_number_tx_values", _dp), ("f_number_rx_values", _dp), ("n_f_number_values", C.c_int),
        ("normalization_tx", C.c_int), ("normalization_rx", C.c_int),
        ("device", C.c_int),
    ]


class PlanInfo(C.Structure):
    _fields_ = [
        ("N_dft", C.c_int), ("k_lb", C.c_int), ("k_ub", C.c_int), ("n_bins", C.c_int),
        ("n_x", C.c_int), ("n_z", C.c_int), ("n_elements", C.c_int), ("n_angles", C.c_int), ("n_samples", C.c_int),
        ("f_monotone", C.c_int),
        ("terms", C.c_longlong), ("active_terms", C.c_longlong), ("zero_weight_bins", C.c_longlong),
        ("scratch_bytes", C.c_longlong),
        ("scale", C.c_double),
        ("executed_terms", C.c_longlong),
        ("kernel_variant", C.c_int), ("grid", C.c_int), ("blocks_per_sm", C.c_int), ("bin_chunk", C.c_int),
    ]


class LibraryNotBuilt(RuntimeError):
    pass


class FNumError(RuntimeError):
    """Error raised with the reference's identifier, e.g.
    ``gpu_bf_das_pw_rf:InvalidFrequencyBounds`` or ``das_pw:NoWindow``."""

    def __init__(self, identifier: str, message: str, status: int | None = None):
        super().__init__("%s: %s" % (identifier, message))
        self.identifier = identifier
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryNotBuilt("libfnum.so is not built: run `python -c \"import __graft_entry__ as g; g.build()\"` "
                              "(or python f_number_gb300/build.py)")
    L = C.CDLL(LIB_PATH)
    L.fnum_abi_version.restype = C.c_int
    L.fnum_status_string.restype = C.c_char_p
    L.fnum_status_string.argtypes = [C.c_int]
    L.fnum_status_id.restype = C.c_char_p
    L.fnum_status_id.argtypes = [C.c_int, C.c_int]
    L.fnum_device_count.restype = C.c_int
    L.fnum_band.restype = C.c_int
    L.fnum_band.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp,
                            C.c_double, _ip, _ip, _ip]
    L.fnum_f_number_values.restype = C.c_int
    L.fnum_f_number_values.argtypes = [C.POINTER(FNumber), _dp, C.c_int, _dp]
    L.fnum_window_value.restype = C.c_double
    L.fnum_window_value.argtypes = [Window, C.c_double, C.c_double]
    L.fnum_das_pw.restype = C.c_int
    L.fnum_das_pw.argtypes = [C.POINTER(PWDesc), _dp, C.c_int, _dp, C.c_int, _fp, _fp, _fp]
    L.fnum_das_sa.restype = C.c_int
    L.fnum_das_sa.argtypes = [C.POINTER(SADesc), _dp, C.c_int, _fp, _fp, _fp, _fp]
    L.fnum_pw_plan_create.restype = C.c_int
    L.fnum_pw_plan_create.argtypes = [C.POINTER(PWDesc), _dp, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.fnum_sa_plan_create.restype = C.c_int
    L.fnum_sa_plan_create.argtypes = [C.POINTER(SADesc), C.c_int, C.POINTER(C.c_void_p)]
    L.fnum_plan_execute.restype = C.c_int
    L.fnum_plan_execute.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.fnum_plan_execute_dft.restype = C.c_int
    L.fnum_plan_execute_dft.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.fnum_plan_execute_beamform.restype = C.c_int
    L.fnum_plan_execute_beamform.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.fnum_plan_info_get.restype = C.c_int
    L.fnum_plan_info_get.argtypes = [C.c_void_p, C.POINTER(PlanInfo)]
    L.fnum_plan_f_numbers.restype = C.c_int
    L.fnum_plan_f_numbers.argtypes = [C.c_void_p, _dp]
    L.fnum_plan_destroy.restype = C.c_int
    L.fnum_plan_destroy.argtypes = [C.c_void_p]
    L.fnum_diag_fp32_peak.restype = C.c_int
    L.fnum_diag_fp32_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.fnum_diag_mma_f16_peak.restype = C.c_int
    L.fnum_diag_mma_f16_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.fnum_das_pw_noalloc.restype = C.c_int
    L.fnum_das_pw_noalloc.argtypes = [C.POINTER(PWDesc), _dp, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    L.fnum_plan_autotune.restype = C.c_int
    L.fnum_plan_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _ip, _fp]
    L.fnum_plan_set_kernel_variant.restype = C.c_int
    L.fnum_plan_set_kernel_variant.argtypes = [C.c_void_p, C.c_int]
    L.fnum_batch_create.restype = C.c_int
    L.fnum_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p), _ip,
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int,
                                    C.POINTER(C.c_void_p)]
    L.fnum_batch_execute.restype = C.c_int
    L.fnum_batch_execute.argtypes = [C.c_void_p, C.c_void_p]
    L.fnum_batch_frame_times.restype = C.c_int
    L.fnum_batch_frame_times.argtypes = [C.c_void_p, _fp]
    L.fnum_plan_set_shape.restype = C.c_int
    L.fnum_plan_set_shape.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.fnum_batch_info.restype = C.c_int
    L.fnum_batch_info.argtypes = [C.c_void_p, _ip, _ip]
    L.fnum_batch_destroy.restype = C.c_int
    L.fnum_batch_destroy.argtypes = [C.c_void_p]
    L.fnum_pw_plan_set_sound_speed.restype = C.c_int
    L.fnum_pw_plan_set_sound_speed.argtypes = [C.c_void_p, C.c_double]
    L.fnum_pw_sharpness_grad.restype = C.c_int
    L.fnum_pw_sharpness_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, _dp, C.c_void_p, C.c_void_p]
    L.fnum_plan_m_signal.restype = C.c_int
    L.fnum_plan_m_signal.argtypes = [C.c_void_p, _dp, _ip]
    L.fnum_das_pw_sharpness_grad.restype = C.c_int
    L.fnum_das_pw_sharpness_grad.argtypes = [C.POINTER(PWDesc), _dp, C.c_int, _dp, _dp, _dp, _fp, _fp]
    L.fnum_pw_adjoint.restype = C.c_int
    L.fnum_pw_adjoint.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, _dp, C.c_void_p]
    L.fnum_plan_set_spectra.restype = C.c_int
    L.fnum_plan_set_spectra.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.fnum_plan_spectra.restype = C.c_int
    L.fnum_plan_spectra.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.fnum_host_cache_info.restype = C.c_int
    L.fnum_host_cache_info.argtypes = [C.c_int, C.POINTER(C.c_longlong), _ip]
    L.fnum_bmode.restype = C.c_int
    L.fnum_bmode.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    if L.fnum_abi_version() != ABI_VERSION:
        raise LibraryNotBuilt("libfnum.so ABI version mismatch")
    _lib = L
    return L


def check(status: int, saft: bool = False):
    if status != OK:
        L = lib()
        raise FNumError(L.fnum_status_id(status, int(saft)).decode(), L.fnum_status_string(status).decode(), status)


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def fptr(a):
    return a.ctypes.data_as(_fp) if a is not None else None
