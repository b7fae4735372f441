"""ctypes wrapper of oracle/liboracle.so (the C restatement).

TEST INFRASTRUCTURE ONLY: the checker for parity tests at sampled voxels of
full-size workloads, and the timed CPU restatement of das_pw.m.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import build as _build
from . import fnum_oracle as O

_L = None
_d, _i, _ll = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)


def lib():
    global _L
    if _L is None:
        _L = C.CDLL(_build.build())
        _L.oracle_pw_mex.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, _d, _d, C.c_int, _d, _d, _d, C.c_int, C.c_double,
                                     C.c_int, C.c_int, _i, _i, _d, _d, _ll, C.c_int]
        _L.oracle_pw_m.argtypes = [C.c_int, C.c_int, _i, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, _d, _d, C.c_int, _d, _d, _d, C.c_int, C.c_double, C.c_int, C.c_int,
                                   C.c_double, C.c_int, _i, _i, _d, C.c_int]
        _L.oracle_sa_mex.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, _d, _d, _d, _d, _d, C.c_int, C.c_double, C.c_int,
                                     C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, _i, _i, _d, _d, _d, _ll,
                                     C.c_int]
        _L.oracle_max_threads.restype = C.c_int
    return _L


def _p(a, t=_d):
    return a.ctypes.data_as(t)


WIN_IDS = O.WINDOW_IDS


def pw_mex(px, pz, rf, f_s, angles, width, pitch, c, f_bounds, t0, window, F_number, normalization, ix, iz,
           threads=0):
    """Compounded MEX-semantics image at voxels (ix, iz).  rf: [A, E, T]."""
    px = np.ascontiguousarray(px, dtype=np.float64)
    pz = np.ascontiguousarray(pz, dtype=np.float64)
    rf = np.asarray(rf, dtype=np.float64)
    A, E, T = rf.shape
    band = O.band_mex(pz, T, E, f_s, width, pitch, c, f_bounds, t0)
    F = np.ascontiguousarray(O._resolve_F(F_number, band, pitch, f_s, c, ("angle_lb", 70.0, 1.5, 10.0)))
    X = np.fft.fft(rf, n=band.N_dft, axis=2)[:, :, band.k_lb:band.k_ub + 1]          # [A, E, K]
    Xc = np.ascontiguousarray(X.astype(np.complex128)).view(np.float64)
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    iz = np.ascontiguousarray(iz, dtype=np.int32)
    out = np.zeros(2 * ix.size)
    w = np.zeros(ix.size)
    zb = C.c_longlong(0)
    ang = np.ascontiguousarray(np.atleast_1d(angles), dtype=np.float64)
    lib().oracle_pw_mex(E, band.K, band.k_lb, band.N_dft, pitch, width, f_s, c, t0, _p(px), _p(pz), A, _p(ang),
                        _p(Xc), _p(F), WIN_IDS[window[0]], float(window[1]), int(normalization != "off"), ix.size,
                        _p(ix, _i), _p(iz, _i), _p(out), _p(w), C.byref(zb), threads)
    return out.view(np.complex128), w, {"zero_weight_bins": zb.value, "N_dft": band.N_dft, "k_lb": band.k_lb,
                                         "k_ub": band.k_ub, "F": F}


def pw_m_prepare(pz, rf, f_s, width, pitch, c, f_bounds, F_number):
    """Band, F table and spectra of das_pw.m (das_pw.m:343-384)."""
    pz = np.asarray(pz, dtype=np.float64)
    A, E, T = rf.shape
    M = (E - 1) / 2.0
    ctr = np.arange(-M, M + 1) * pitch
    if f_bounds is None:
        f_bounds = (O.EPS, f_s / 2.0)
    N_pad = int(math.ceil((math.sqrt((ctr[-1] - ctr[0]) ** 2 + pz[0] ** 2) - pz[0]) * f_s / c))
    N = T + N_pad + 1 - ((T + N_pad) % 2)
    ks = np.arange(int(math.ceil(f_bounds[0] * N / f_s)), int(math.floor(f_bounds[1] * N / f_s)) + 1)
    F0 = O.f_number_values(F_number, pitch * f_s * ks / N / c)
    return N, ks, F0


def pw_m(px, pz, rf, f_s, angles, width, pitch, c, f_bounds, t0, window, F_number, normalization, ix, iz,
         threads=0, fwindow=("tukey", 0.2)):
    """das_pw.m CPU-semantics image (summed over angles) at voxels (ix, iz)."""
    px = np.ascontiguousarray(px, dtype=np.float64)
    pz = np.ascontiguousarray(pz, dtype=np.float64)
    rf = np.asarray(rf, dtype=np.float64)
    A, E, T = rf.shape
    N, ks, F0 = pw_m_prepare(pz, rf, f_s, width, pitch, c, f_bounds, F_number)
    X = np.fft.fft(rf, n=N, axis=2)[:, :, ks]
    Xc = np.ascontiguousarray(X.astype(np.complex128)).view(np.float64)
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    iz = np.ascontiguousarray(iz, dtype=np.int32)
    ks32 = np.ascontiguousarray(ks, dtype=np.int32)
    out = np.zeros(2 * ix.size)
    ang = np.ascontiguousarray(np.atleast_1d(angles), dtype=np.float64)
    norm = {"off": 0, "on": 1, "windowed": 2}[normalization]
    lib().oracle_pw_m(E, ks.size, _p(ks32, _i), N, pitch, width, f_s, c, t0, _p(px), _p(pz), A, _p(ang), _p(Xc),
                      _p(np.ascontiguousarray(F0)), WIN_IDS[window[0]], float(window[1]), norm,
                      WIN_IDS[fwindow[0]], float(fwindow[1]), ix.size, _p(ix, _i), _p(iz, _i), _p(out), threads)
    return out.view(np.complex128), {"N_dft": N, "ks": ks}


def sa_mex(px, pz, rf, f_s, width, pitch, c, f_bounds, t0, window_tx, window_rx, F_tx, F_rx, norm_tx, norm_rx,
           ix, iz, semantics="reference", threads=0):
    """MEX-semantics SAFT image at voxels.  rf: [Tx, Rx, T]."""
    px = np.ascontiguousarray(px, dtype=np.float64)
    pz = np.ascontiguousarray(pz, dtype=np.float64)
    rf = np.asarray(rf, dtype=np.float64)
    E, _, T = rf.shape
    band = O.band_mex(pz, T, E, f_s, width, pitch, c, f_bounds, t0)
    dflt = ("angle_lb", 70.0, 1.5, 10.0)
    Ftx = np.ascontiguousarray(O._resolve_F(F_tx, band, pitch, f_s, c, dflt))
    Frx = np.ascontiguousarray(O._resolve_F(F_rx, band, pitch, f_s, c, dflt))
    X = np.fft.fft(rf, n=band.N_dft, axis=2)[:, :, band.k_lb:band.k_ub + 1]
    Xc = np.ascontiguousarray(X.astype(np.complex128)).view(np.float64)
    on_t, on_r = norm_tx != "off", norm_rx != "off"
    mode = 0
    if semantics == "reference" and not on_t and not on_r:
        mode = 1
    if semantics == "reference" and not on_t and on_r:
        mode = -1
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    iz = np.ascontiguousarray(iz, dtype=np.int32)
    out = np.zeros(2 * ix.size)
    wt = np.zeros(ix.size)
    wr = np.zeros(ix.size)
    zb = C.c_longlong(0)
    lib().oracle_sa_mex(E, band.K, band.k_lb, band.N_dft, pitch, width, f_s, c, t0, _p(px), _p(pz), _p(Xc), _p(Ftx),
                        _p(Frx), WIN_IDS[window_tx[0]], float(window_tx[1]), WIN_IDS[window_rx[0]],
                        float(window_rx[1]), int(on_t), int(on_r), mode, ix.size, _p(ix, _i), _p(iz, _i), _p(out),
                        _p(wt), _p(wr), C.byref(zb), threads)
    return out.view(np.complex128), wt, wr, {"zero_weight_bins": zb.value, "N_dft": band.N_dft, "k_lb": band.k_lb,
                                             "k_ub": band.k_ub}


def max_threads():
    return lib().oracle_max_threads()
