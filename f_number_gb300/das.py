"""Entry points with the reference's signatures.

* ``das_pw`` / ``das_sa`` follow ``das_pw.m`` / ``das_sa.m``: same positional
  arguments, defaults, validation order and error identifiers
  (``das_pw.m:85-290``, ``das_sa.m:85-277``), then the ``platforms.gpu``
  dispatch (``das_pw.m:296-300``, ``das_sa.m:283-287``).
* ``gpu_bf_das_pw_rf`` / ``gpu_bf_saft_rf`` follow the MEX gateways: their
  argument lists, MEX defaults (boxcar window, ``angle_lb(70, 1.5, 10)``) and
  outputs (image, weights).
* ``PWPlan`` / ``SAPlan`` keep geometry, band tables and scratch resident on
  the device for repeated, stream-ordered execution on device buffers.

Arrays use MATLAB orientation: ``data_RF`` is [N_t, N_el] (PW) or
[N_t, N_rx, N_tx] (SA); images are [N_z, N_x].
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from . import f_numbers as _fn
from . import normalizations as _norm
from . import platforms as _plat
from . import windows as _win
from ._lib import FNumError

EPS = float(np.finfo(np.float64).eps)
DBL_MIN = float(np.finfo(np.float64).tiny)


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def _is_num(x):
    return isinstance(x, (int, float, np.integer, np.floating)) or (
        isinstance(x, np.ndarray) and np.issubdtype(x.dtype, np.number))


def _real_row(x):
    a = np.asarray(x)
    return np.issubdtype(a.dtype, np.number) and not np.iscomplexobj(a) and a.ndim <= 2 and (
        a.ndim < 2 or a.shape[0] == 1)


def _scalar(x):
    a = np.asarray(x)
    return np.issubdtype(a.dtype, np.number) and not np.iscomplexobj(a) and a.size == 1


def _err(ident, msg):
    raise FNumError(ident, msg)


def _f_number_args(F_number, band_p_over_lambda):
    """Native classes go to the library as a spec; any other object with a
    ``compute_values`` method is evaluated here on the band (as the MEX does
    through mexCallMATLAB, ``+cuda/gpu_bf_helper_functions.cu:35-51``)."""
    if F_number is None:
        return _lib.FNumber(_lib.F_DEFAULT, 0, (0.0, 0.0, 0.0)), None
    try:
        return F_number.c_struct(), None
    except (AttributeError, NotImplementedError):
        vals = np.ascontiguousarray(np.asarray(F_number.compute_values(band_p_over_lambda), dtype=np.float64).ravel())
        return _lib.FNumber(_lib.F_DEFAULT, 0, (0.0, 0.0, 0.0)), vals


def _window_struct(w, ident):
    if w is None:
        return _lib.Window(_lib.WINDOW_BOXCAR, 0.0)
    if not isinstance(w, _win.window):
        _err(ident, "Window must be a single object of the class windows.window!")
    return w.c_struct()


def _norm_code(n, ident):
    if n is None:
        return _lib.NORM_ON
    if not isinstance(n, _norm.normalization):
        _err(ident, "Normalization must be a single object of the class normalizations.normalization!")
    return n.code


def band(positions_z, n_samples, n_elements, f_s, element_width, element_pitch, c_0, f_bounds=None, index_t0=0.0):
    """(N_dft, k_lb, k_ub) of the MEX gateways (``gpu_bf_das_pw_rf.cu:522-556``)."""
    pz = np.ascontiguousarray(np.asarray(positions_z, dtype=np.float64).ravel())
    fb = None if f_bounds is None else np.ascontiguousarray(np.asarray(f_bounds, dtype=np.float64).ravel())
    N, lb, ub = _lib.C.c_int(), _lib.C.c_int(), _lib.C.c_int()
    _lib.check(_lib.lib().fnum_band(_lib.dptr(pz), pz.size, int(n_samples), int(n_elements), float(f_s),
                                    float(element_width), float(element_pitch), float(c_0), _lib.dptr(fb),
                                    float(index_t0), _lib.C.byref(N), _lib.C.byref(lb), _lib.C.byref(ub)))
    return N.value, lb.value, ub.value


def _band_pl(pz, nt, ne, f_s, width, pitch, c_0, fb, t0):
    N, k_lb, k_ub = band(pz, nt, ne, f_s, width, pitch, c_0, fb, t0)
    return pitch * np.arange(k_lb, k_ub + 1) * f_s / (N * c_0)


def _band_m(pz, nt, ne, f_s, pitch, c_0, fb):
    """DFT order and band bins of das_pw.m (das_pw.m:340-362): padding from the first
    axial position, aperture in double."""
    M = (ne - 1) / 2.0
    ap = pitch * ((ne - 1) - M) - pitch * (0 - M)
    z0 = float(np.asarray(pz, dtype=np.float64).ravel()[0])
    n_pad = int(math.ceil((math.sqrt(ap * ap + z0 * z0) - z0) * f_s / c_0))
    N = nt + n_pad + 1 - ((nt + n_pad) % 2)
    f_lb, f_ub = (np.finfo(np.float64).eps, f_s / 2.0) if fb is None else (float(fb[0]), float(fb[1]))
    return N, int(math.ceil(f_lb * N / f_s)), int(math.floor(f_ub * N / f_s))


# ---------------------------------------------------------------------------
# MEX gateways
# ---------------------------------------------------------------------------
def gpu_bf_das_pw_rf(positions_x, positions_z, data_RF, f_s, steering_angle, element_width, element_pitch, c_0,
                     f_bounds=None, index_t0=None, window=None, F_number=None, normalization=None, index_gpu=None,
                     verbosity=None, *, compound=True, kernel="fused"):
    """``cuda.gpu_bf_das_pw_rf`` (``+cuda/gpu_bf_das_pw_rf.cu:110``): returns
    (image [N_z, N_x] complex64 scaled by 2/N_dft, weights [N_z, N_x] float32).

    ``steering_angle`` may hold several angles (same geometry, RF stacked along
    a third axis [N_t, N_el, N_angles]); with ``compound`` the images are summed
    into one, else an [N_angles, N_z, N_x] stack is returned.
    ``kernel="plain"`` selects the per-voxel FP32 kernel with the reference's
    arithmetic."""
    ident = "gpu_bf_das_pw_rf"
    px = np.ascontiguousarray(np.asarray(positions_x, dtype=np.float64).ravel())
    pz = np.ascontiguousarray(np.asarray(positions_z, dtype=np.float64).ravel())
    rf = np.asarray(data_RF)
    if rf.ndim not in (2, 3) or np.iscomplexobj(rf):
        _err(ident + ":InvalidRFData", "RF data must be a real-valued matrix of type double!")
    angles = np.ascontiguousarray(np.atleast_1d(np.asarray(steering_angle, dtype=np.float64)).ravel())
    if rf.ndim == 2:
        rf = rf[:, :, None]
    nt, ne, na = rf.shape
    if na != angles.size:
        _err(ident + ":InvalidRFData", "RF data must hold one [N_t x N_el] block per steering angle!")
    # [angle][element][time] memory order
    rf_c = np.ascontiguousarray(np.transpose(rf, (2, 1, 0)), dtype=np.float64)
    fb = None if f_bounds is None or np.size(f_bounds) == 0 else np.ascontiguousarray(
        np.asarray(f_bounds, dtype=np.float64).ravel())
    if fb is not None and fb.size != 2:
        _err(ident + ":InvalidFrequencyBounds", "Frequency bounds must be a real-valued vector with two entries of type double!")
    t0 = 0.0 if index_t0 is None else float(index_t0)
    if verbosity is not None and not (0 <= int(verbosity) < 4):
        _err(ident + ":InvalidVerbosityLevel", "Selected verbosity level does not exist!")
    L = _lib.lib()
    desc = _lib.PWDesc()
    desc.positions_x, desc.n_x = _lib.dptr(px), px.size
    desc.positions_z, desc.n_z = _lib.dptr(pz), pz.size
    desc.n_samples, desc.n_elements = nt, ne
    desc.f_s, desc.element_width, desc.element_pitch, desc.c_0 = float(f_s), float(element_width), \
        float(element_pitch), float(c_0)
    desc.f_bounds = _lib.dptr(fb)
    desc.index_t0 = t0
    desc.window = _window_struct(window, ident + ":InvalidWindow")
    fvals = None
    if F_number is not None and not hasattr(F_number, "compute_values"):
        _err(ident + ":InvalidFNumber", "F-number must be a single object of the class f_numbers.f_number!")
    try:
        pl = _band_pl(pz, nt, ne, f_s, element_width, element_pitch, c_0, fb, t0) if F_number is not None else None
    except FNumError as e:
        raise FNumError(e.identifier, str(e), e.status)
    desc.f_number, fvals = _f_number_args(F_number, pl)
    if fvals is not None:
        desc.f_number_values, desc.n_f_number_values = _lib.dptr(fvals), fvals.size
    desc.normalization = _norm_code(normalization, ident + ":InvalidNormalization")
    desc.device = 0 if index_gpu is None else int(index_gpu)
    flags = (_lib.FLAG_COMPOUND if compound else 0) | (_lib.FLAG_PLAIN_KERNEL if kernel == "plain" else 0)
    n_out = 1 if compound else na
    re = np.empty((n_out, px.size, pz.size), dtype=np.float32)
    im = np.empty_like(re)
    w = np.empty((px.size, pz.size), dtype=np.float32)
    st = L.fnum_das_pw(_lib.C.byref(desc), _lib.dptr(angles), na, _lib.dptr(rf_c), flags, _lib.fptr(re),
                       _lib.fptr(im), _lib.fptr(w))
    _lib.check(st)
    img = (re + 1j * im).astype(np.complex64).transpose(0, 2, 1)
    return (img[0] if n_out == 1 else img), w.T


def gpu_bf_saft_rf(positions_x, positions_z, data_RF, f_s, element_width, element_pitch, c_0, f_bounds=None,
                   index_t0=None, window_tx=None, window_rx=None, F_number_tx=None, F_number_rx=None,
                   normalization_tx=None, normalization_rx=None, index_gpu=None, verbosity=None, *,
                   semantics="reference", kernel="fused"):
    """``cuda.gpu_bf_saft_rf`` (``+cuda/gpu_bf_saft_rf.cu:107``): returns
    (image, weights_tx, weights_rx).  ``semantics="intended"`` divides by the
    sums that are on and always accumulates (the reference keeps only the last
    bin with both normalisations off and returns zeros with only the receive
    normalisation on)."""
    ident = "gpu_bf_saft_rf"
    px = np.ascontiguousarray(np.asarray(positions_x, dtype=np.float64).ravel())
    pz = np.ascontiguousarray(np.asarray(positions_z, dtype=np.float64).ravel())
    rf = np.asarray(data_RF)
    if rf.ndim != 3 or np.iscomplexobj(rf):
        _err(ident + ":InvalidRFData", "RF data must be a real-valued array of type double with 3 dimensions!")
    nt, nrx, ntx = rf.shape
    if nrx != ntx:
        _err(ident + ":InvalidRFData", "Size of RF data must be equal along 2nd and 3rd dimensions!")
    rf_c = np.ascontiguousarray(np.transpose(rf, (2, 1, 0)), dtype=np.float64)  # [tx][rx][t]
    fb = None if f_bounds is None or np.size(f_bounds) == 0 else np.ascontiguousarray(
        np.asarray(f_bounds, dtype=np.float64).ravel())
    t0 = 0.0 if index_t0 is None else float(index_t0)
    L = _lib.lib()
    desc = _lib.SADesc()
    desc.positions_x, desc.n_x = _lib.dptr(px), px.size
    desc.positions_z, desc.n_z = _lib.dptr(pz), pz.size
    desc.n_samples, desc.n_elements = nt, nrx
    desc.f_s, desc.element_width, desc.element_pitch, desc.c_0 = float(f_s), float(element_width), \
        float(element_pitch), float(c_0)
    desc.f_bounds = _lib.dptr(fb)
    desc.index_t0 = t0
    desc.window_tx = _window_struct(window_tx, ident + ":InvalidWindow")
    desc.window_rx = _window_struct(window_rx, ident + ":InvalidWindow")
    pl = None
    if (F_number_tx is not None) or (F_number_rx is not None):
        pl = _band_pl(pz, nt, nrx, f_s, element_width, element_pitch, c_0, fb, t0)
    desc.f_number_tx, ftx = _f_number_args(F_number_tx, pl)
    desc.f_number_rx, frx = _f_number_args(F_number_rx, pl)
    if ftx is not None or frx is not None:
        # a value table replaces both specs: evaluate the native one on the band too
        if ftx is None:
            ftx = (F_number_tx.compute_values(pl) if F_number_tx is not None else
                   _fn.grating.angle_lb(70.0, 1.5, 10.0).compute_values(pl))
        if frx is None:
            frx = (F_number_rx.compute_values(pl) if F_number_rx is not None else
                   _fn.grating.angle_lb(70.0, 1.5, 10.0).compute_values(pl))
        ftx = np.ascontiguousarray(ftx, dtype=np.float64)
        frx = np.ascontiguousarray(frx, dtype=np.float64)
        desc.f_number_tx_values, desc.f_number_rx_values = _lib.dptr(ftx), _lib.dptr(frx)
        desc.n_f_number_values = ftx.size
    desc.normalization_tx = _norm_code(normalization_tx, ident + ":InvalidNormalization")
    desc.normalization_rx = _norm_code(normalization_rx, ident + ":InvalidNormalization")
    desc.device = 0 if index_gpu is None else int(index_gpu)
    flags = (_lib.FLAG_SAFT_INTENDED if semantics == "intended" else 0) | (
        _lib.FLAG_PLAIN_KERNEL if kernel == "plain" else 0)
    re = np.empty((px.size, pz.size), dtype=np.float32)
    im = np.empty_like(re)
    wt = np.empty_like(re)
    wr = np.empty_like(re)
    st = L.fnum_das_sa(_lib.C.byref(desc), _lib.dptr(rf_c), flags, _lib.fptr(re), _lib.fptr(im), _lib.fptr(wt),
                       _lib.fptr(wr))
    _lib.check(st, saft=True)
    return (re + 1j * im).astype(np.complex64).T, wt.T, wr.T


# ---------------------------------------------------------------------------
# das_pw.m / das_sa.m
# ---------------------------------------------------------------------------
def _check_common_m(fn, positions_x, positions_z, f_s):
    if not _real_row(positions_x):
        _err(fn + ":NoNumericAndRealRowVector", "positions_x must be a numeric and real-valued row vector!")
    if not np.all(np.isfinite(np.asarray(positions_x, dtype=np.float64))):
        _err(fn + ":NoFiniteXCoordinates", "positions_x must contain finite x-coordinates!")
    if not _real_row(positions_z):
        _err(fn + ":NoNumericAndRealRowVector", "positions_z must be a numeric and real-valued row vector!")
    pz = np.asarray(positions_z, dtype=np.float64)
    if not (np.all(pz > 0) and np.all(np.isfinite(pz))):
        _err(fn + ":NoPositiveAndFiniteZCoordinates", "positions_z must contain positive and finite z-coordinates!")


def _check_scalar(fn, name, v):
    if not _scalar(v):
        _err(fn + ":NoNumericAndRealScalar", "%s must be a numeric and real-valued scalar!" % name)
    return float(np.asarray(v).ravel()[0])


def _check_tail_m(fn, f_s, f_bounds, index_t0):
    if f_bounds is None or np.size(f_bounds) == 0:
        f_bounds = [EPS, f_s / 2.0]
    if not _real_row(f_bounds):
        _err(fn + ":NoNumericAndRealRowVector", "f_bounds must be a numeric and real-valued row vector!")
    fb = np.asarray(f_bounds, dtype=np.float64).ravel()
    if not (fb.size == 2 and fb[0] > 0 and fb[1] > fb[0] and fb[1] <= f_s / 2):
        _err(fn + ":InvalidFrequencyBounds", "f_bounds must be a strictly monotonic increasing sequence!")
    if index_t0 is None or np.size(index_t0) == 0:
        index_t0 = 0
    t0 = _check_scalar(fn, "index_t0", index_t0)
    if not (t0 >= 0 and t0 == math.floor(t0)):
        _err(fn + ":InvalidTimeIndex", "index_t0 must be a nonnegative integer!")
    return fb, t0


def _check_geometry_m(fn, f_s, element_width, element_pitch, c_0):
    f_s = _check_scalar(fn, "f_s", f_s)
    if not (f_s > 0 and math.isfinite(f_s)):
        _err(fn + ":InvalidSamplingRate", "f_s must be positive and finite!")
    w = _check_scalar(fn, "element_width", element_width)
    if not (w > 0 and math.isfinite(w)):
        _err(fn + ":InvalidElementWidth", "element_width must be positive and finite!")
    p = _check_scalar(fn, "element_pitch", element_pitch)
    if not (p > w and math.isfinite(p)):
        _err(fn + ":InvalidElementPitch", "element_pitch must be larger than element_width and finite!")
    c = _check_scalar(fn, "c_0", c_0)
    if not (c > 0 and math.isfinite(c)):
        _err(fn + ":InvalidSpeedOfSound", "c_0 must be positive and finite!")
    return f_s, w, p, c


def das_pw(positions_x, positions_z, data_RF, f_s, steering_angle, element_width, element_pitch, c_0,
           f_bounds=None, index_t0=None, window=None, F_number=None, normalization=None, platform=None):
    """Fourier-domain DAS for one steered plane wave (``das_pw.m``).

    ``platforms.gpu`` (the default here, ``gpu(0)``) returns the complex image
    [N_z, N_x] of the MEX path (single precision, scaled by 2/N_dft), as
    das_pw.m does.  ``platforms.cpu`` returns what das_pw.m's own loop returns --
    (image, F_number_values, signal) with its semantics (das_pw.m:310-481) --
    computed on GPU 0 by the das_pw.m-semantics kernel: there is no CPU compute
    path.  Defaults follow ``das_pw.m:207-283``."""
    fn = "das_pw"
    _check_common_m(fn, positions_x, positions_z, f_s)
    rf = np.asarray(data_RF)
    if not (np.issubdtype(rf.dtype, np.number) and not np.iscomplexobj(rf) and rf.ndim == 2):
        _err(fn + ":NoNumericAndRealMatrix", "data_RF must be a numeric and real-valued matrix!")
    if not (rf.shape[0] > 1 and rf.shape[1] > 1):
        _err(fn + ":NoSamples", "data_RF must contain at least two temporal and two spatial samples!")
    if not np.all(np.isfinite(rf)):
        _err(fn + ":NoFiniteRFData", "data_RF must contain finite samples!")
    f_s_v = _check_scalar(fn, "f_s", f_s)
    if not (f_s_v > 0 and math.isfinite(f_s_v)):
        _err(fn + ":InvalidSamplingRate", "f_s must be positive and finite!")
    th = _check_scalar(fn, "steering_angle", steering_angle)
    if not (-math.pi / 2 < th < math.pi / 2):
        _err(fn + ":InvalidSteeringAngle",
             "steering_angle must be larger than negative pi over two and smaller than pi over two!")
    f_s_v, w, p, c = _check_geometry_m(fn, f_s, element_width, element_pitch, c_0)
    fb, t0 = _check_tail_m(fn, f_s_v, f_bounds, index_t0)
    if window is None or (isinstance(window, (list, tuple, np.ndarray)) and len(window) == 0):
        window = _win.tukey(0.2)
    if not isinstance(window, _win.window):
        _err(fn + ":NoWindow", "window must be scalar windows.window!")
    if F_number is None:
        F_number = _fn.grating.angle_lb(60.0, 1.5)
    if not isinstance(F_number, _fn.f_number):
        _err(fn + ":NoFNumber", "F_number must be scalar f_numbers.f_number!")
    if normalization is None:
        normalization = _norm.on()
    if not isinstance(normalization, _norm.normalization):
        _err(fn + ":NoNormalization", "normalization must be scalar normalizations.normalization!")
    if platform is None:
        platform = _plat.gpu(0)
    if not isinstance(platform, _plat.platform):
        _err(fn + ":NoPlatform", "platform must be scalar platforms.platform!")
    if not isinstance(platform, _plat.gpu):
        return _das_pw_m(positions_x, positions_z, rf, f_s_v, th, w, p, c, fb, t0, window, F_number, normalization)
    image, _ = gpu_bf_das_pw_rf(positions_x, positions_z, rf, f_s_v, th, w, p, c, fb, t0, window, F_number,
                                normalization, platform.index)
    return image


def _das_pw_m(positions_x, positions_z, rf, f_s, th, width, pitch, c_0, fb, t0, window, F_number, normalization):
    """platforms.cpu of das_pw: the semantics of das_pw.m's own loop (das_pw.m:310-481),
    computed on GPU 0 by the das_pw.m-semantics kernel.  Returns (image [N_z, N_x]
    complex128 as das_pw.m, F_number_values [n_bins, N_z] (capped per depth,
    das_pw.m:371-377), signal (das_pw.m:477-481))."""
    import torch
    px = np.asarray(positions_x, dtype=np.float64).ravel()
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    nt, ne = rf.shape
    plan = PWPlan(px, pz, nt, ne, f_s, [th], width, pitch, c_0, fb, t0, window, F_number, normalization, device=0,
                  compound=True, semantics="m")
    try:
        rf_d = torch.tensor(np.ascontiguousarray(rf.T), dtype=torch.float64, device="cuda:0")
        img = plan.execute(rf_d)
        torch.cuda.synchronize()
        image = img[0].cpu().numpy().T.astype(np.complex128)
        inf = plan.info()
        f = f_s * np.arange(inf["k_lb"], inf["k_ub"] + 1) / inf["N_dft"]
        F0 = plan.f_numbers()
        F = np.minimum(F0[:, None], np.sqrt(f[:, None] * pz[None, :] / (2.88 * c_0)))
        return image, F, plan.m_signal()
    finally:
        plan.close()


def das_sa(positions_x, positions_z, data_RF, f_s, element_width, element_pitch, c_0, f_bounds=None, index_t0=None,
           window_tx=None, window_rx=None, F_number_tx=None, F_number_rx=None, normalization_tx=None,
           normalization_rx=None, platform=None):
    """Fourier-domain DAS for a full synthetic aperture data set (``das_sa.m``);
    data_RF is [N_t, N_rx, N_tx].  Returns (image, weights_tx, weights_rx) of
    the GPU path (``das_sa.m:285``).  The receive parameters default to the
    transmit defaults (``das_sa.m`` defines none for them)."""
    fn = "das_sa"
    _check_common_m(fn, positions_x, positions_z, f_s)
    rf = np.asarray(data_RF)
    if not (np.issubdtype(rf.dtype, np.number) and not np.iscomplexobj(rf) and rf.ndim == 3):
        _err(fn + ":NoNumericAndReal3DArray", "data_RF must be a numeric and real-valued 3d array!")
    if not np.all(np.isfinite(rf)):
        _err(fn + ":NoFiniteRFData", "data_RF must contain finite samples!")
    f_s_v, w, p, c = _check_geometry_m(fn, f_s, element_width, element_pitch, c_0)
    fb, t0 = _check_tail_m(fn, f_s_v, f_bounds, index_t0)
    window_tx = _win.tukey(0.2) if window_tx is None else window_tx
    window_rx = _win.tukey(0.2) if window_rx is None else window_rx
    for wv in (window_tx, window_rx):
        if not isinstance(wv, _win.window):
            _err(fn + ":NoWindow", "window must be scalar windows.window!")
    F_number_tx = _fn.grating.angle_lb(60.0, 1.5) if F_number_tx is None else F_number_tx
    F_number_rx = _fn.grating.angle_lb(60.0, 1.5) if F_number_rx is None else F_number_rx
    for fv in (F_number_tx, F_number_rx):
        if not isinstance(fv, _fn.f_number):
            _err(fn + ":NoFNumber", "F_number must be scalar f_numbers.f_number!")
    normalization_tx = _norm.on() if normalization_tx is None else normalization_tx
    normalization_rx = _norm.on() if normalization_rx is None else normalization_rx
    for nv in (normalization_tx, normalization_rx):
        if not isinstance(nv, _norm.normalization):
            _err(fn + ":NoNormalization", "normalization must be scalar normalizations.normalization!")
    platform = _plat.gpu(0) if platform is None else platform
    if not isinstance(platform, _plat.platform):
        _err(fn + ":NoPlatform", "platform must be scalar platforms.platform!")
    if not isinstance(platform, _plat.gpu):
        _err(fn + ":CPUPathNotProvided",
             "platforms.cpu is the reference's MATLAB implementation; this package provides platforms.gpu")
    return gpu_bf_saft_rf(positions_x, positions_z, rf, f_s_v, w, p, c, fb, t0, window_tx, window_rx, F_number_tx,
                          F_number_rx, normalization_tx, normalization_rx, platform.index)


# ---------------------------------------------------------------------------
# device-resident plans
# ---------------------------------------------------------------------------
class _Plan:
    _ptr = None
    _saft = False

    def info(self) -> dict:
        inf = _lib.PlanInfo()
        _lib.check(_lib.lib().fnum_plan_info_get(self._ptr, _lib.C.byref(inf)), self._saft)
        return {f: getattr(inf, f) for f, _ in _lib.PlanInfo._fields_}

    def f_numbers(self):
        n = self.n_bins * (2 if self._saft else 1)
        out = np.empty(n, dtype=np.float64)
        _lib.check(_lib.lib().fnum_plan_f_numbers(self._ptr, _lib.dptr(out)), self._saft)
        return out

    def close(self):
        if self._ptr is not None:
            _lib.lib().fnum_plan_destroy(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _stream_ptr(stream):
        if stream is None:
            import torch
            stream = torch.cuda.current_stream()
        return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)

    def execute(self, rf, out=None, weights=None, weights_rx=None, stream=None):
        """rf: torch CUDA tensor (float32 or float64), PW [A, E, T] / SA [Tx, Rx, T].
        Returns the image as a complex64 tensor [n_out, N_x, N_z] (scaled)."""
        import torch
        if not rf.is_cuda or not rf.is_contiguous():
            raise ValueError("rf must be a contiguous CUDA tensor")
        if rf.dtype not in (torch.float32, torch.float64):
            raise ValueError("rf must be float32 or float64")
        if out is None:
            out = torch.empty((self.n_out, self.n_x, self.n_z), dtype=torch.complex64, device=rf.device)
        st = _lib.lib().fnum_plan_execute(self._ptr, rf.data_ptr(), int(rf.dtype == torch.float64), out.data_ptr(),
                                          weights.data_ptr() if weights is not None else None,
                                          weights_rx.data_ptr() if weights_rx is not None else None,
                                          self._stream_ptr(stream))
        _lib.check(st, self._saft)
        return out

    def execute_dft(self, rf, stream=None):
        import torch
        _lib.check(_lib.lib().fnum_plan_execute_dft(self._ptr, rf.data_ptr(), int(rf.dtype == torch.float64),
                                                    self._stream_ptr(stream)), self._saft)

    def spectra(self, stream=None):
        """Band spectra of the last execute (fnum_plan_spectra): complex64 tensor,
        plane wave [n_elements, n_bins, n_angles], SAFT [n_tx, n_rx, n_bins]."""
        import torch
        inf = self.info()
        shape = ((inf["n_elements"], inf["n_elements"], inf["n_bins"]) if self._saft else
                 (inf["n_elements"], inf["n_bins"], inf["n_angles"]))
        out = torch.empty(shape, dtype=torch.complex64, device=torch.device("cuda", self.device))
        _lib.check(_lib.lib().fnum_plan_spectra(self._ptr, out.data_ptr(), self._stream_ptr(stream)), self._saft)
        return out

    def execute_beamform(self, out, weights=None, weights_rx=None, stream=None):
        _lib.check(_lib.lib().fnum_plan_execute_beamform(
            self._ptr, out.data_ptr(), weights.data_ptr() if weights is not None else None,
            weights_rx.data_ptr() if weights_rx is not None else None, self._stream_ptr(stream)), self._saft)
        return out

    def autotune(self, rf):
        """Times the fused kernel's variants on this plan's data (fnum_plan_autotune)
        and keeps the fastest.  Returns (variant, beamform ms of the choice)."""
        import torch
        v = _lib.C.c_int(0)
        ms = _lib.C.c_float(0.0)
        _lib.check(_lib.lib().fnum_plan_autotune(self._ptr, rf.data_ptr(), int(rf.dtype == torch.float64),
                                                 _lib.C.byref(v), _lib.C.byref(ms)), self._saft)
        return v.value, ms.value

    def set_shape(self, blocks_per_sm=0, bin_chunk=0):
        """Pins the launch shape of the current variant (fnum_plan_set_shape)."""
        _lib.check(_lib.lib().fnum_plan_set_shape(self._ptr, int(blocks_per_sm), int(bin_chunk)), self._saft)

    def set_kernel_variant(self, variant):
        """Pins the kernel variant (fnum_plan_set_kernel_variant): 0 = default; 1..9 for a
        plane-wave plan; 1 (recurrence kernels) or 2 (tensor cores) for a
        synthetic-aperture plan."""
        _lib.check(_lib.lib().fnum_plan_set_kernel_variant(self._ptr, int(variant)), self._saft)


class PWPlan(_Plan):
    """Plane-wave plan: one or many steering angles with the same geometry."""

    def __init__(self, positions_x, positions_z, n_samples, n_elements, f_s, steering_angles, element_width,
                 element_pitch, c_0, f_bounds=None, index_t0=0.0, window=None, F_number=None, normalization=None,
                 device=0, compound=True, kernel="fused", semantics="mex"):
        """semantics: "mex" (the reference's GPU gateway, the default) or "m" (its CPU
        path das_pw.m: see FNUM_FLAG_M_SEMANTICS; images are not scaled by 2/N_dft)."""
        if semantics not in ("mex", "m"):
            raise ValueError("semantics must be 'mex' or 'm'")
        self.semantics = semantics
        self._px = np.ascontiguousarray(np.asarray(positions_x, dtype=np.float64).ravel())
        self._pz = np.ascontiguousarray(np.asarray(positions_z, dtype=np.float64).ravel())
        self._angles = np.ascontiguousarray(np.atleast_1d(np.asarray(steering_angles, dtype=np.float64)).ravel())
        self._fb = None if f_bounds is None else np.ascontiguousarray(np.asarray(f_bounds, dtype=np.float64).ravel())
        d = _lib.PWDesc()
        d.positions_x, d.n_x = _lib.dptr(self._px), self._px.size
        d.positions_z, d.n_z = _lib.dptr(self._pz), self._pz.size
        d.n_samples, d.n_elements = int(n_samples), int(n_elements)
        d.f_s, d.element_width, d.element_pitch, d.c_0 = float(f_s), float(element_width), float(element_pitch), \
            float(c_0)
        d.f_bounds = _lib.dptr(self._fb)
        d.index_t0 = float(index_t0)
        d.window = _window_struct(window, "gpu_bf_das_pw_rf:InvalidWindow")
        if semantics == "m":
            Nm, klm, kum = _band_m(self._pz, int(n_samples), int(n_elements), f_s, element_pitch, c_0, self._fb)
            pl = element_pitch * np.arange(klm, kum + 1) * f_s / (Nm * c_0) if F_number is not None else None
        else:
            pl = _band_pl(self._pz, n_samples, n_elements, f_s, element_width, element_pitch, c_0, self._fb,
                          index_t0) if F_number is not None else None
        d.f_number, self._fvals = _f_number_args(F_number, pl)
        if self._fvals is not None:
            d.f_number_values, d.n_f_number_values = _lib.dptr(self._fvals), self._fvals.size
        d.normalization = _norm_code(normalization, "gpu_bf_das_pw_rf:InvalidNormalization")
        if isinstance(normalization, _norm.windowed):
            d.normalization_window = normalization.window.c_struct()
        d.device = int(device)
        flags = (_lib.FLAG_COMPOUND if compound else 0) | (_lib.FLAG_PLAIN_KERNEL if kernel == "plain" else 0) | (
            _lib.FLAG_M_SEMANTICS if semantics == "m" else 0)
        ptr = _lib.C.c_void_p()
        _lib.check(_lib.lib().fnum_pw_plan_create(_lib.C.byref(d), _lib.dptr(self._angles), self._angles.size, flags,
                                                  _lib.C.byref(ptr)))
        self._ptr = ptr
        self.device = int(device)
        inf = self.info()
        self.n_x, self.n_z, self.n_bins = inf["n_x"], inf["n_z"], inf["n_bins"]
        self.n_elements, self.n_angles = inf["n_elements"], inf["n_angles"]
        self.n_out = 1 if compound else self._angles.size


def _pw_m_signal(self):
    """das_pw.m's `signal` output after an execute of a plan with semantics="m": the
    inverse DFT (length N_dft) of the focused spectrum of the last voxel processed
    (das_pw.m:477-481), or None when that column has no active bin."""
    inf = self.info()
    spec = np.zeros(2 * self.n_bins, dtype=np.float64)
    has = _lib.C.c_int(0)
    _lib.check(_lib.lib().fnum_plan_m_signal(self._ptr, _lib.dptr(spec), _lib.C.byref(has)))
    if not has.value:
        return None
    full = np.zeros(inf["N_dft"], dtype=np.complex128)
    full[inf["k_lb"]:inf["k_ub"] + 1] = spec[0::2] + 1j * spec[1::2]
    return np.fft.ifft(full, inf["N_dft"])


PWPlan.m_signal = _pw_m_signal


def _pw_set_sound_speed(self, c_0):
    """Re-times the phase tables at sound speed c_0 (fnum_pw_plan_set_sound_speed);
    DFT order, band, F table and apertures stay those of the creation speed."""
    _lib.check(_lib.lib().fnum_pw_plan_set_sound_speed(self._ptr, float(c_0)))


def _pw_sharpness_grad(self, rf, grad_spectra=True, stream=None):
    """Sharpness loss L = -sum|I|^4 / (sum|I|^2)^2 of the compounded image of rf,
    dL/dc, and (optionally) the Wirtinger gradient dL/dX* of the band spectra as
    a complex64 CUDA tensor [n_elements, n_bins, n_angles]
    (fnum_pw_sharpness_grad).  Returns (L, dL/dc, gradient or None)."""
    import torch
    g = None
    if grad_spectra:
        g = torch.empty((self.n_elements, self.n_bins, self.n_angles), dtype=torch.complex64, device=rf.device)
    L = _lib.C.c_double(0.0)
    dc = _lib.C.c_double(0.0)
    _lib.check(_lib.lib().fnum_pw_sharpness_grad(self._ptr, rf.data_ptr(), int(rf.dtype == torch.float64),
                                                 _lib.C.byref(L), _lib.C.byref(dc),
                                                 g.data_ptr() if g is not None else None, self._stream_ptr(stream)))
    return L.value, dc.value, g


def _pw_set_spectra(self, spectra, stream=None):
    """Loads band spectra (complex64 CUDA tensor [n_elements, n_bins, n_angles]) into
    the plan (fnum_plan_set_spectra), for execute_beamform or adjoint."""
    import torch
    if spectra.dtype != torch.complex64 or not spectra.is_cuda or not spectra.is_contiguous():
        raise ValueError("spectra must be a contiguous complex64 CUDA tensor")
    if tuple(spectra.shape) != (self.n_elements, self.n_bins, self.n_angles):
        raise ValueError("spectra must have shape [n_elements, n_bins, n_angles]")
    _lib.check(_lib.lib().fnum_plan_set_spectra(self._ptr, spectra.data_ptr(), self._stream_ptr(stream)))


def _pw_adjoint(self, cotangent, dc=True, stream=None):
    """Adjoint of the compounded beamformer (fnum_pw_adjoint): for G = dL/dI*
    (complex64 CUDA tensor [N_x, N_z]) at the plan's current spectra and sound
    speed, returns (dL/dX* as a complex64 tensor [n_elements, n_bins, n_angles],
    dL/dc or None)."""
    import torch
    cot = cotangent.reshape(self.n_x, self.n_z).to(torch.complex64).contiguous()
    g = torch.empty((self.n_elements, self.n_bins, self.n_angles), dtype=torch.complex64, device=cot.device)
    v = _lib.C.c_double(0.0)
    _lib.check(_lib.lib().fnum_pw_adjoint(self._ptr, cot.data_ptr(), g.data_ptr(), _lib.C.byref(v) if dc else None,
                                          self._stream_ptr(stream)))
    return g, (v.value if dc else None)


PWPlan.set_sound_speed = _pw_set_sound_speed
PWPlan.sharpness_grad = _pw_sharpness_grad
PWPlan.set_spectra = _pw_set_spectra
PWPlan.adjoint = _pw_adjoint


class SAPlan(_Plan):
    """Synthetic-aperture plan."""
    _saft = True

    def __init__(self, positions_x, positions_z, n_samples, n_elements, f_s, element_width, element_pitch, c_0,
                 f_bounds=None, index_t0=0.0, window_tx=None, window_rx=None, F_number_tx=None, F_number_rx=None,
                 normalization_tx=None, normalization_rx=None, device=0, semantics="reference", kernel="fused"):
        self._px = np.ascontiguousarray(np.asarray(positions_x, dtype=np.float64).ravel())
        self._pz = np.ascontiguousarray(np.asarray(positions_z, dtype=np.float64).ravel())
        self._fb = None if f_bounds is None else np.ascontiguousarray(np.asarray(f_bounds, dtype=np.float64).ravel())
        d = _lib.SADesc()
        d.positions_x, d.n_x = _lib.dptr(self._px), self._px.size
        d.positions_z, d.n_z = _lib.dptr(self._pz), self._pz.size
        d.n_samples, d.n_elements = int(n_samples), int(n_elements)
        d.f_s, d.element_width, d.element_pitch, d.c_0 = float(f_s), float(element_width), float(element_pitch), \
            float(c_0)
        d.f_bounds = _lib.dptr(self._fb)
        d.index_t0 = float(index_t0)
        d.window_tx = _window_struct(window_tx, "gpu_bf_saft_rf:InvalidWindow")
        d.window_rx = _window_struct(window_rx, "gpu_bf_saft_rf:InvalidWindow")
        d.f_number_tx, _ = _f_number_args(F_number_tx, None)
        d.f_number_rx, _ = _f_number_args(F_number_rx, None)
        d.normalization_tx = _norm_code(normalization_tx, "gpu_bf_saft_rf:InvalidNormalization")
        d.normalization_rx = _norm_code(normalization_rx, "gpu_bf_saft_rf:InvalidNormalization")
        d.device = int(device)
        flags = (_lib.FLAG_SAFT_INTENDED if semantics == "intended" else 0) | (
            _lib.FLAG_PLAIN_KERNEL if kernel == "plain" else 0)
        ptr = _lib.C.c_void_p()
        _lib.check(_lib.lib().fnum_sa_plan_create(_lib.C.byref(d), flags, _lib.C.byref(ptr)), True)
        self._ptr = ptr
        self.device = int(device)
        inf = self.info()
        self.n_x, self.n_z, self.n_bins = inf["n_x"], inf["n_z"], inf["n_bins"]
        self.n_out = 1


# ---------------------------------------------------------------------------
# post-processing on the device
# ---------------------------------------------------------------------------
def bmode(image, floor_db=float("-inf"), stream=None):
    """B-mode image in dB on the device: 20 log10(|sum_a I_a| / max |sum_a I_a|),
    clamped below at floor_db.  image: complex64 CUDA tensor [n_images, N_x, N_z]
    (per-angle images are compounded coherently first, examples.m:78) or
    [N_x, N_z].  Returns (dB tensor [N_x, N_z] float32, max |I| as a 0-d tensor).
    Replaces the host-side steps of the reference's example script
    (examples.m:88,96)."""
    import torch
    img = image if image.dim() == 3 else image.unsqueeze(0)
    if img.dtype != torch.complex64 or not img.is_cuda:
        raise TypeError("bmode expects a complex64 CUDA tensor")
    img = img.contiguous()
    n_img, nx, nz = img.shape
    db = torch.empty((nx, nz), dtype=torch.float32, device=img.device)
    mx = torch.empty((), dtype=torch.float32, device=img.device)
    st = _Plan._stream_ptr(stream if stream is not None else torch.cuda.current_stream(img.device))
    _lib.check(_lib.lib().fnum_bmode(img.data_ptr(), nx * nz, n_img, float(floor_db), db.data_ptr(), mx.data_ptr(),
                                     st))
    return db, mx


class Batch:
    """Frames of uneven shape in one CUDA graph (fnum_batch_*).  plans: distinct
    plans; rfs / images (and weights, optional): the CUDA tensors each frame
    reads and writes, bound for the batch's life.  n_streams concurrent branches
    share the GPU among small frames."""

    def __init__(self, plans, rfs, images, weights=None, n_streams=4):
        import torch
        n = len(plans)
        if not (len(rfs) == len(images) == n) or (weights is not None and len(weights) != n):
            raise ValueError("plans, rfs, images (and weights) must have the same length")
        self._keep = (list(plans), list(rfs), list(images), list(weights) if weights is not None else None)
        P = (_lib.C.c_void_p * n)(*[p._ptr for p in plans])
        R = (_lib.C.c_void_p * n)(*[r.data_ptr() for r in rfs])
        D = (_lib.C.c_int * n)(*[int(r.dtype == torch.float64) for r in rfs])
        I = (_lib.C.c_void_p * n)(*[im.data_ptr() for im in images])
        W = None if weights is None else (_lib.C.c_void_p * n)(*[w.data_ptr() if w is not None else None
                                                                   for w in weights])
        ptr = _lib.C.c_void_p()
        _lib.check(_lib.lib().fnum_batch_create(P, n, R, D, I, W, None, int(n_streams), _lib.C.byref(ptr)))
        self._ptr = ptr
        self.n = n

    def execute(self, stream=None):
        _lib.check(_lib.lib().fnum_batch_execute(self._ptr, _Plan._stream_ptr(stream)))

    def persistent(self):
        """(frames carried by persistent tensor-core launches, number of such launches)."""
        f, l = _lib.C.c_int(0), _lib.C.c_int(0)
        _lib.check(_lib.lib().fnum_batch_info(self._ptr, _lib.C.byref(f), _lib.C.byref(l)))
        return f.value, l.value

    def frame_times(self):
        """Completion time of each frame in ms from the start of the last execute."""
        out = np.empty(self.n, dtype=np.float32)
        _lib.check(_lib.lib().fnum_batch_frame_times(self._ptr, out.ctypes.data_as(_lib.C.POINTER(_lib.C.c_float))))
        return out

    def close(self):
        if getattr(self, "_ptr", None) is not None:
            _lib.lib().fnum_batch_destroy(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
