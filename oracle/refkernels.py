"""ctypes wrapper of oracle/_ref/libref_harness.so: the reference's own CUDA
kernels (compiled from the f_number sources) run with the MEX host sequence.

TEST INFRASTRUCTURE ONLY: generates the golden vectors that pin the oracle
(tests/golden/make_ref_golden.py) and times the reference GPU algorithm.
F-number tables are the oracle's restatement of the MATLAB classes (the MEX
obtains them from MATLAB through mexCallMATLAB).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from . import fnum_oracle as O

_L = None
_d, _f = C.POINTER(C.c_double), C.POINTER(C.c_float)


def available():
    return os.path.exists(_build.HARNESS) and os.path.exists(_build.FATBIN)


def lib():
    global _L
    if _L is None:
        _L = C.CDLL(_build.HARNESS)
        _L.ref_error.restype = C.c_char_p
        _L.ref_load.argtypes = [C.c_char_p]
        _L.ref_das_pw.argtypes = [_d, C.c_int, _d, C.c_int, _d, C.c_int, C.c_int] + [C.c_double] * 8 + [
            C.c_int, C.c_double, _d, C.c_int, C.c_int, _f, _f, _f, _f]
        _L.ref_das_sa.argtypes = [_d, C.c_int, _d, C.c_int, _d, C.c_int, C.c_int] + [C.c_double] * 7 + [
            C.c_int, C.c_double, C.c_int, C.c_double, _d, _d, C.c_int, C.c_int, C.c_int, _f, _f, _f, _f, _f]
        if _L.ref_load(_build.FATBIN.encode()) != 0:
            raise RuntimeError(_L.ref_error().decode())
    return _L


def _p(a, t=_d):
    return a.ctypes.data_as(t)


def das_pw(px, pz, data_rf, f_s, angle, width, pitch, c, f_bounds=None, t0=0.0, window=("boxcar", 0.0),
           F_number=None, normalization="on"):
    """Reference GPU algorithm for one angle.  data_rf [N_t, N_el] (MATLAB
    orientation).  Returns (image [N_z, N_x] complex64, weights, kernel ms)."""
    px = np.ascontiguousarray(px, dtype=np.float64)
    pz = np.ascontiguousarray(pz, dtype=np.float64)
    rf = np.ascontiguousarray(np.asarray(data_rf, dtype=np.float64).T)       # [E][T]
    E, T = rf.shape
    band = O.band_mex(pz, T, E, f_s, width, pitch, c, f_bounds, t0)
    F = np.ascontiguousarray(O._resolve_F(F_number, band, pitch, f_s, c, ("angle_lb", 70.0, 1.5, 10.0)))
    f_const = int(isinstance(F_number, dict) and F_number.get("kind") == "constant")
    f_lb, f_ub = (O.DBL_MIN, f_s / 2.0) if f_bounds is None else f_bounds
    re = np.zeros(px.size * pz.size, np.float32)
    im = np.zeros_like(re)
    w = np.zeros_like(re)
    ms = C.c_float(0)
    st = lib().ref_das_pw(_p(px), px.size, _p(pz), pz.size, _p(rf), T, E, f_s, angle, width, pitch, c, f_lb, f_ub,
                          t0, O.WINDOW_IDS[window[0]], float(window[1]), _p(F), f_const,
                          int(normalization != "off"), _p(re, _f), _p(im, _f), _p(w, _f), C.byref(ms))
    if st != 0:
        raise RuntimeError(lib().ref_error().decode())
    img = (re + 1j * im).reshape(px.size, pz.size).T
    return img.astype(np.complex64), w.reshape(px.size, pz.size).T, ms.value


def das_sa(px, pz, data_rf, f_s, width, pitch, c, f_bounds=None, t0=0.0, window_tx=("boxcar", 0.0),
           window_rx=("boxcar", 0.0), F_tx=None, F_rx=None, norm_tx="on", norm_rx="on"):
    """Reference GPU SAFT.  data_rf [N_t, N_rx, N_tx]."""
    px = np.ascontiguousarray(px, dtype=np.float64)
    pz = np.ascontiguousarray(pz, dtype=np.float64)
    rf = np.ascontiguousarray(np.transpose(np.asarray(data_rf, dtype=np.float64), (2, 1, 0)))   # [tx][rx][t]
    E, _, T = rf.shape
    band = O.band_mex(pz, T, E, f_s, width, pitch, c, f_bounds, t0)
    dflt = ("angle_lb", 70.0, 1.5, 10.0)
    Ftx = np.ascontiguousarray(O._resolve_F(F_tx, band, pitch, f_s, c, dflt))
    Frx = np.ascontiguousarray(O._resolve_F(F_rx, band, pitch, f_s, c, dflt))
    both_const = int(all(isinstance(f, dict) and f.get("kind") == "constant" for f in (F_tx, F_rx)))
    f_lb, f_ub = (O.DBL_MIN, f_s / 2.0) if f_bounds is None else f_bounds
    n = px.size * pz.size
    re, im, wt, wr = (np.zeros(n, np.float32) for _ in range(4))
    ms = C.c_float(0)
    st = lib().ref_das_sa(_p(px), px.size, _p(pz), pz.size, _p(rf), T, E, f_s, width, pitch, c, f_lb, f_ub, t0,
                          O.WINDOW_IDS[window_tx[0]], float(window_tx[1]), O.WINDOW_IDS[window_rx[0]],
                          float(window_rx[1]), _p(Ftx), _p(Frx), both_const, int(norm_tx != "off"),
                          int(norm_rx != "off"), _p(re, _f), _p(im, _f), _p(wt, _f), _p(wr, _f), C.byref(ms))
    if st != 0:
        raise RuntimeError(lib().ref_error().decode())
    sh = (px.size, pz.size)
    return ((re + 1j * im).reshape(sh).T.astype(np.complex64), wt.reshape(sh).T, wr.reshape(sh).T, ms.value)
