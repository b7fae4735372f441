"""FP64 CPU oracle for the Fourier-domain delay-and-sum beamformer of f_number.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``f_number_gb300``) imports
this module; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only
as the checker or the timed CPU restatement of the reference's CPU path.

What it restates (file:line in the f_number project):

* MEX semantics of the CUDA path (``mode="mex"``), the contract the GPU
  library honours:
  - geometry, DFT order and band  ``+cuda/gpu_bf_das_pw_rf.cu:495-556``
    (the zero padding uses ``positions_z[1]``, the *second* axial position,
    ``gpu_bf_das_pw_rf.cu:525``; SAFT ``+cuda/gpu_bf_saft_rf.cu:602-652``)
  - DFT (cuFFT R2C, e^{-j} convention) ``gpu_bf_das_pw_rf.cu:917-925``
  - incident distances ``+cuda/das_kernel_distances_pw.cu:27``,
    ``+cuda/das_kernel_distances_sw.cu:26-28``
  - aperture / window / phase per term ``+cuda/das_kernel_phase_shifts.cu:83-145``,
    ``+cuda/saft_kernel_phase_shifts.cu:41-198``
  - windows ``+cuda/gpu_bf_windows.cu:15-103``
  - GEMV + per-bin normalisation ``gpu_bf_das_pw_rf.cu:1023-1048``,
    ``+cuda/das_kernel_normalization.cu:27-31``; SAFT ``gpu_bf_saft_rf.cu:1144-1201``
  - 2/N_dft scaling ``gpu_bf_das_pw_rf.cu:1113-1122``
* CPU semantics of ``das_pw.m`` (``mode="m"``): ``das_pw.m:310-481``.
* Parameter objects: ``+f_numbers/**``, ``+windows/**``, ``+normalizations/**``.

Parity status: the reference is MATLAB + CUDA MEX code.  Neither MATLAB nor
GNU Octave exists here and the reference ships no tests, golden vectors or
fixtures, so this restatement is pinned by (1) closed-form known answers of
the parameter classes, (2) analytic properties of the beamformer, and (3) the
reference's own CUDA kernels compiled from source and run on the GPU behind a
project-written host driver (``oracle/ref_harness``), where that harness is
available.  Without (3) the oracle is "parity unpinned".

Departures, each a documented contract decision:
* a bin whose apodization sum is zero contributes 0 (the MEX divides 0/0 and
  produces NaN, ``das_kernel_normalization.cu:30-31``); the count of such
  (voxel, bin) pairs is returned in ``info["zero_weight_bins"]``.
* ``fminbnd`` (MATLAB, closed source) is replaced by Brent's published
  minimiser in the Forsythe-Malcolm-Moler ``fmin`` form, TolX = 1e-4.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

FLT_EPSILON = float(np.finfo(np.float32).eps)  # 1.1920929e-07, used as F > FLT_EPSILON
DBL_MIN = float(np.finfo(np.float64).tiny)
EPS = float(np.finfo(np.float64).eps)

# ---------------------------------------------------------------------------
# F-number classes (+f_numbers/**)
# ---------------------------------------------------------------------------


def _deg2rad(deg):
    return (math.pi / 180.0) * deg


def fnum_constant(value, p):
    """``+f_numbers/constant.m:72``: repmat of the value."""
    return np.full(np.shape(p), float(value))


def fnum_distance_constant(distance_deg, F_ub, p):
    """``+f_numbers/+distance/constant.m:90-120`` (fixed angular distance)."""
    p = np.asarray(p, dtype=np.float64)
    rad = _deg2rad(distance_deg)
    sin_d = math.sin(rad)
    opc = 1.0 + math.cos(rad)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv_sin = 1.0 / sin_d if sin_d != 0.0 else math.inf
        ind_lb = p >= 1.0 / opc
        ind_ub = p < inv_sin
        ind_tr = (~ind_lb) & (p >= 0.5)
        ind_pos = ind_lb & ind_ub
        v = np.zeros_like(p)
        pt = p[ind_tr]
        v[ind_tr] = np.sqrt(1.0 / (1.0 / pt - 1.0) ** 2 - 1.0) / 2.0
        t = p[ind_pos] ** 2
        vp = (np.sqrt(2.0 * opc * t - 1.0) + opc * sin_d * t) / (2.0 - 2.0 * sin_d ** 2 * t)
        v[ind_pos] = np.minimum(vp, F_ub)
        v[~ind_ub] = F_ub
    return v


def fnum_angle_lb(angle_lb_deg, F_ub, distance_deg, p):
    """``+f_numbers/+grating/angle_lb.m:44-75`` with ``grating.m:72-75`` bounds."""
    p = np.asarray(p, dtype=np.float64)
    thresh = math.sin(_deg2rad(angle_lb_deg))
    lower = 1.0 / (1.0 + thresh)
    upper = 1.0 / (1.0 / math.sqrt(1.0 + (2.0 * F_ub) ** 2) + thresh)
    rel = (p > lower) & (p < upper)
    imp = p >= upper
    v = np.zeros_like(p)
    pr = p[rel]
    v[rel] = np.sqrt(1.0 / (1.0 / pr - thresh) ** 2 - 1.0) / 2.0
    v[imp] = F_ub
    if distance_deg >= 0:
        v = np.maximum(v, fnum_distance_constant(distance_deg, math.inf, p))
    return v


def _sinc(x):
    """MATLAB ``sinc``: sin(pi x)/(pi x), 1 at 0."""
    if x == 0.0:
        return 1.0
    y = math.pi * x
    return math.sin(y) / y


def fminbnd(f, ax, bx, tol=1e-4):
    """Brent's minimiser on [ax, bx] (Forsythe, Malcolm & Moler, ``fmin``, 1977;
    R. P. Brent, Algorithms for Minimization without Derivatives, 1973, ch. 5).
    Stands in for MATLAB ``fminbnd`` with its default TolX = 1e-4
    (``+f_numbers/+directivity/directivity.m:116``)."""
    c = 0.5 * (3.0 - math.sqrt(5.0))
    sqeps = math.sqrt(EPS)
    a, b = float(ax), float(bx)
    v = a + c * (b - a)
    w = x = v
    e = d = 0.0
    fx = f(x)
    fv = fw = fx
    for _ in range(500):
        xm = 0.5 * (a + b)
        tol1 = sqeps * abs(x) + tol / 3.0
        tol2 = 2.0 * tol1
        if abs(x - xm) <= tol2 - 0.5 * (b - a):
            break
        golden = True
        if abs(e) > tol1:
            r = (x - w) * (fx - fv)
            q = (x - v) * (fx - fw)
            p = (x - v) * q - (x - w) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                p = -p
            q = abs(q)
            r = e
            e = d
            if abs(p) < abs(0.5 * q * r) and p > q * (a - x) and p < q * (b - x):
                d = p / q
                u = x + d
                if (u - a) < tol2 or (b - u) < tol2:
                    d = tol1 if (xm - x) >= 0.0 else -tol1
                golden = False
        if golden:
            e = (a - x) if x >= xm else (b - x)
            d = c * e
        if abs(d) >= tol1:
            u = x + d
        else:
            u = x + (tol1 if d >= 0.0 else -tol1)
        fu = f(u)
        if fu <= fx:
            if u >= x:
                a = x
            else:
                b = x
            v, fv = w, fw
            w, fw = x, fx
            x, fx = u, fu
        else:
            if u < x:
                a = u
            else:
                b = u
            if fu <= fw or w == x:
                v, fv = w, fw
                w, fw = u, fu
            elif fu <= fv or v == x or v == w:
                v, fv = u, fu
    return x


def fnum_directivity(width_over_pitch, obliquity, attenuation_dB, p):
    """``+f_numbers/+directivity/directivity.m:91-120`` with the obliquity
    factors ``+obliquity/rigid.m:62`` (1) and ``+obliquity/soft.m:62`` (cos)."""
    p = np.asarray(p, dtype=np.float64)
    thresh = 10.0 ** (-attenuation_dB / 20.0)
    soft = obliquity == "soft"
    out = np.zeros_like(p)
    for i, pl in enumerate(p.ravel()):
        wl = width_over_pitch * pl

        def f(theta, wl=wl):
            ob = math.cos(theta) if soft else 1.0
            return abs(ob * _sinc(wl * math.sin(theta)) - thresh)

        alpha = fminbnd(f, 0.0, math.pi / 2.0)
        out.flat[i] = 1.0 / (2.0 * math.tan(alpha))
    return out


def fnum_szabo(width_over_pitch, p):
    """``+f_numbers/+directivity/szabo.m:86``: (w/lambda)/1.2."""
    return width_over_pitch * np.asarray(p, dtype=np.float64) / 1.2


def f_number_values(spec, p):
    """Dispatch on a spec dict ``{"kind": ..., ...}`` (same keys as the
    product's parameter objects) -> F per normalised pitch p = pitch/lambda."""
    k = spec["kind"]
    if k == "constant":
        return fnum_constant(spec["value"], p)
    if k == "grating.angle_lb":
        return fnum_angle_lb(spec["angle_lb_deg"], spec["F_number_ub"], spec.get("distance_deg", 10.0), p)
    if k == "distance.constant":
        return fnum_distance_constant(spec["distance_deg"], spec.get("F_number_ub", math.inf), p)
    if k == "distance.none":
        return fnum_distance_constant(0.0, math.inf, p)
    if k == "directivity":
        return fnum_directivity(spec["width_over_pitch"], spec.get("obliquity", "soft"),
                                spec.get("attenuation_dB", 3.0), p)
    if k == "directivity.szabo":
        return fnum_szabo(spec["width_over_pitch"], p)
    raise ValueError(f"unknown F-number kind {k!r}")


# ---------------------------------------------------------------------------
# windows
# ---------------------------------------------------------------------------
# MEX ids (+cuda/gpu_bf_helper_functions.cu:56-97): boxcar 0, hann 1, tukey 2, triangular 4
WINDOW_IDS = {"boxcar": 0, "hann": 1, "tukey": 2, "triangular": 4}


def window_mex(win, l, L):
    """``+cuda/gpu_bf_windows.cu:15-103``: 0 where |l| >= L, else the window
    of l relative to the half-width L.  ``win`` = (name, parameter)."""
    name, par = win
    l = np.asarray(l, dtype=np.float64)
    L = np.asarray(L, dtype=np.float64)
    out = np.zeros(np.broadcast(l, L).shape)
    inside = np.abs(l) < L
    with np.errstate(divide="ignore", invalid="ignore"):
        u = np.where(inside, np.abs(l) / np.where(inside, L, 1.0), 0.0)
    if name == "boxcar":
        val = np.ones_like(u)
    elif name == "hann":
        val = (1.0 + np.cos(math.pi * u)) / 2.0
    elif name == "tukey":
        thr = 1.0 - par
        val = np.where(u <= thr, 1.0, (1.0 + np.cos(math.pi * (u - thr) / par)) / 2.0)
    elif name == "triangular":
        val = 1.0 - u
    else:
        raise ValueError(name)
    out = np.where(inside, val, 0.0)
    return out


def window_m(win, u_abs):
    """MATLAB ``compute_samples_scalar`` on |position / half-width|:
    ``+windows/boxcar.m:62``, ``hann.m:62``, ``tukey.m:101-105``,
    ``triangular.m:62``.  Note hann/triangular carry no cut-off at |u| >= 1."""
    name, par = win
    u = np.abs(np.atleast_1d(np.asarray(u_abs, dtype=np.float64)))
    if np.ndim(u_abs) == 0:
        return window_m(win, u)[0]
    if name == "boxcar":
        return (u < 1).astype(np.float64)
    if name == "hann":
        return (1.0 + np.cos(math.pi * u)) / 2.0
    if name == "tukey":
        fr = 1.0 - par
        s = (u < 1).astype(np.float64)
        taper = (u < 1) & (u > fr)
        s[taper] = (1.0 + np.cos(math.pi * (u[taper] - fr) / par)) / 2.0
        return s
    if name == "triangular":
        return 1.0 - u
    raise ValueError(name)


# ---------------------------------------------------------------------------
# geometry and band (MEX semantics)
# ---------------------------------------------------------------------------


@dataclass
class Band:
    N_dft: int
    k_lb: int
    k_ub: int
    coef: float     # 2 pi f_s / (N c)  rad per bin per metre
    add: float      # 2 pi t0 / N
    M: float
    ctr: np.ndarray
    lb: np.ndarray
    ub: np.ndarray

    @property
    def K(self):
        return self.k_ub - self.k_lb + 1

    @property
    def ks(self):
        return np.arange(self.k_lb, self.k_ub + 1)


def band_mex(positions_z, N_t, N_el, f_s, element_width, element_pitch, c_0, f_bounds, index_t0):
    """``gpu_bf_das_pw_rf.cu:495-556`` (identical in ``gpu_bf_saft_rf.cu:602-652``)."""
    M = (N_el - 1.0) / 2.0
    ctr = element_pitch * (np.arange(N_el) - M)
    lb = ctr - element_width / 2.0
    ub = ctr + element_width / 2.0
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    z1 = pz[1] if pz.size >= 2 else pz[0]      # P1: the MEX reads positions_z[1]
    # float element centres, float difference squared in float (gpu_bf_das_pw_rf.cu:498-507, 525)
    c_f = (element_pitch * (np.arange(N_el) - M)).astype(np.float32)
    ap_f = np.float32(c_f[-1] - c_f[0])
    ap2 = float(np.float32(ap_f * ap_f))
    N_pad = int(math.ceil((math.sqrt(ap2 + z1 * z1) - z1) * f_s / c_0))
    N = N_t + N_pad + 1 - ((N_t + N_pad) % 2)
    f_lb, f_ub = (DBL_MIN, f_s / 2.0) if f_bounds is None else (float(f_bounds[0]), float(f_bounds[1]))
    k_lb = int(math.ceil(f_lb * N / f_s))
    k_ub = int(math.floor(f_ub * N / f_s))
    if not (k_lb > 0 and k_lb <= k_ub and k_ub < N // 2 + 1):
        raise ValueError("InvalidFrequencyBounds")
    coef = 2.0 * math.pi * f_s / (N * c_0)
    add = 2.0 * math.pi * index_t0 / N
    return Band(N, k_lb, k_ub, coef, add, M, ctr, lb, ub)


def pitch_over_lambda(band, element_pitch, f_s, c_0):
    """``gpu_bf_das_pw_rf.cu:568-572``."""
    return element_pitch * band.ks * f_s / (band.N_dft * c_0)


def rf_band_spectra(data_rf, band):
    """X[k, e] = sum_t x_e(t) e^{-j 2 pi k t / N} for the band bins
    (cuFFT R2C convention, ``gpu_bf_das_pw_rf.cu:917-925``).  data_rf is
    [N_t, ...] (time first, MATLAB column-major)."""
    X = np.fft.fft(np.asarray(data_rf, dtype=np.float64), n=band.N_dft, axis=0)
    return X[band.k_lb:band.k_ub + 1]


def _aperture_weights(win, x, z, F, band, N_el, element_pitch):
    """Receive apodization a[k, z, e] for one lateral position x
    (``+cuda/das_kernel_phase_shifts.cu:83-145``).  z: [Z], F: [K]."""
    M, ctr, lb, ub = band.M, band.ctr, band.lb, band.ub
    dx = ctr - x                                   # [E]
    left = dx < 0
    Fk = F[:, None]                                # [K,1]
    zz = z[None, :]                                # [1,Z]
    pos = Fk > FLT_EPSILON
    with np.errstate(divide="ignore", invalid="ignore"):
        w2 = np.where(pos, zz / (2.0 * np.where(pos, Fk, 1.0)), 0.0)
        i_l = np.where(pos, np.maximum(np.ceil(M + (x - w2) / element_pitch), 0), 0).astype(np.int64)
        i_r = np.where(pos, np.minimum(np.floor(M + (x + w2) / element_pitch), N_el - 1), N_el - 1).astype(np.int64)
    L_l = x - lb[np.clip(i_l, 0, N_el - 1)]        # [K,Z]
    L_r = ub[np.clip(i_r, 0, N_el - 1)] - x
    a_l = np.where((i_l < N_el)[..., None], window_mex(win, dx[None, None, :], L_l[..., None]), 0.0)
    a_r = np.where((i_r >= 0)[..., None], window_mex(win, dx[None, None, :], L_r[..., None]), 0.0)
    return np.where(left[None, None, :], a_l, a_r)  # [K,Z,E]


def _phase(band, d):
    """exp(+j k (coef d + add)) for d [..] -> [K, ..]."""
    k = band.ks.reshape((-1,) + (1,) * np.ndim(d))
    return np.exp(1j * k * (band.coef * d + band.add))


# ---------------------------------------------------------------------------
# das_pw, MEX semantics
# ---------------------------------------------------------------------------


def das_pw_mex(positions_x, positions_z, data_rf, f_s, steering_angle, element_width, element_pitch,
               c_0, f_bounds=None, index_t0=0.0, window=("boxcar", 0.0), F_number=None,
               normalization="on", voxels=None):
    """Restates ``cuda.gpu_bf_das_pw_rf`` (``+cuda/gpu_bf_das_pw_rf.cu:110-1178``).

    ``F_number``: spec dict or an array of F values per band bin; default
    ``angle_lb(70, 1.5, 10)`` (``gpu_bf_das_pw_rf.cu:360-365``).
    ``normalization``: "on" | "off" | "windowed" (windowed is parsed but not
    applied by the MEX, ``gpu_bf_das_pw_rf.cu:421-427``).
    ``voxels``: optional (ix, iz) index arrays -> values at those voxels only.

    Returns (image [Z, X] complex128 scaled by 2/N_dft, weights [Z, X] =
    apodization sum of the last band bin, info dict).
    """
    px = np.asarray(positions_x, dtype=np.float64).ravel()
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    rf = np.asarray(data_rf, dtype=np.float64)
    N_t, N_el = rf.shape
    band = band_mex(pz, N_t, N_el, f_s, element_width, element_pitch, c_0, f_bounds, index_t0)
    F = _resolve_F(F_number, band, element_pitch, f_s, c_0, default=("angle_lb", 70.0, 1.5, 10.0))
    X = rf_band_spectra(rf, band)                   # [K, E]
    e_x, e_z = -math.sin(steering_angle), math.cos(steering_angle)
    x_ref = -band.M * element_pitch if e_x >= 0 else band.M * element_pitch
    norm = normalization != "off"
    return _pw_core(px, pz, X, band, F, e_x, e_z, x_ref, window, norm, element_pitch, voxels)


def _resolve_F(F_number, band, element_pitch, f_s, c_0, default):
    if F_number is None:
        _, a, fu, d = default
        F_number = {"kind": "grating.angle_lb", "angle_lb_deg": a, "F_number_ub": fu, "distance_deg": d}
    if isinstance(F_number, dict):
        return f_number_values(F_number, pitch_over_lambda(band, element_pitch, f_s, c_0))
    F = np.asarray(F_number, dtype=np.float64).ravel()
    if F.size == 1:
        F = np.full(band.K, F[0])
    return F


def _pw_core(px, pz, X, band, F, e_x, e_z, x_ref, window, norm, pitch, voxels):
    N_el = X.shape[1]
    N = band.N_dft
    info = {"N_dft": N, "k_lb": band.k_lb, "k_ub": band.k_ub, "zero_weight_bins": 0, "F": F}
    cols = range(px.size) if voxels is None else sorted(set(np.asarray(voxels[0]).tolist()))
    image = np.zeros((pz.size, px.size), dtype=np.complex128)
    weights = np.zeros((pz.size, px.size))
    want = None
    if voxels is not None:
        want = {}
        for ix, iz in zip(np.asarray(voxels[0]).tolist(), np.asarray(voxels[1]).tolist()):
            want.setdefault(ix, set()).add(iz)
    for ix in cols:
        x = px[ix]
        zi = np.arange(pz.size) if want is None else np.array(sorted(want[ix]))
        z = pz[zi]
        d_tx = e_x * (x - x_ref) + e_z * z                       # das_kernel_distances_pw.cu:27
        dx = band.ctr - x
        d = d_tx[:, None] + np.sqrt(dx[None, :] ** 2 + z[:, None] ** 2)   # [Z,E]
        a = _aperture_weights(window, x, z, F, band, N_el, pitch)      # [K,Z,E]
        ph = _phase(band, d)                                             # [K,Z,E]
        S = np.einsum("kze,kze,ke->kz", a, ph, X)                        # GEMV per bin
        W = a.sum(axis=2)                                                # [K,Z]
        if norm:
            zero = W == 0
            info["zero_weight_bins"] += int(zero.sum())
            S = np.where(zero, 0.0, S / np.where(zero, 1.0, W))
        image[zi, ix] = (2.0 / N) * S.sum(axis=0)
        weights[zi, ix] = W[-1]
    return image, weights, info


# ---------------------------------------------------------------------------
# image-sharpness loss of a compounded plane-wave image and its gradients
# (no counterpart in the reference; the forward model is das_pw_mex's)
# ---------------------------------------------------------------------------
def pw_sharpness_grad(positions_x, positions_z, rf, f_s, angles, element_width, element_pitch, c, f_bounds=None,
                      index_t0=0.0, window=("boxcar", 0.0), F_number=None, normalization="on", c_freeze=None):
    """FP64 loss L = -sum|I|^4 / (sum|I|^2)^2 of the compounded MEX-semantics image
    I = sum over angles of das_pw_mex, with the DFT order, band, F table and
    apertures frozen at c_freeze (default c) and the phases at c.
    rf: [A, E, T].  Returns (L, dL/dc, dL/dX* as complex [E, K, A], image [Z, X]).
    dL/dX* is the Wirtinger gradient: dL = 2 Re sum conj(dL/dX*) dX."""
    px = np.asarray(positions_x, dtype=np.float64).ravel()
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    rf = np.asarray(rf, dtype=np.float64)
    A, E, T = rf.shape
    c0 = c if c_freeze is None else c_freeze
    band = band_mex(pz, T, E, f_s, element_width, element_pitch, c0, f_bounds, index_t0)
    F = _resolve_F(F_number, band, element_pitch, f_s, c0, default=("angle_lb", 70.0, 1.5, 10.0))
    N, K = band.N_dft, band.K
    ks = band.ks.astype(np.float64)
    coef = 2.0 * math.pi * f_s / (N * c)               # rad per bin per metre at the trial c
    X = np.stack([rf_band_spectra(rf[a].T, band) for a in range(A)], axis=2)   # [K, E, A]
    norm = normalization != "off"
    cache = []
    image = np.zeros((pz.size, px.size), dtype=np.complex128)
    for ix, x in enumerate(px):
        a_w = _aperture_weights(window, x, pz, F, band, E, element_pitch)       # [K, Z, E]
        W = a_w.sum(axis=2)
        b = a_w / np.where(W == 0, 1.0, W)[..., None] if norm else a_w
        b = np.where((W == 0)[..., None], 0.0, b)
        d_rx = np.sqrt((band.ctr[None, :] - x) ** 2 + pz[:, None] ** 2)      # [Z, E]
        ph, dph = [], []
        for ia, th in enumerate(angles):
            e_x, e_z = -math.sin(th), math.cos(th)
            x_ref = -band.M * element_pitch if e_x >= 0 else band.M * element_pitch
            d = (e_x * (x - x_ref) + e_z * pz)[:, None] + d_rx                 # [Z, E]
            p = np.exp(1j * ks[:, None, None] * (coef * d[None] + band.add))    # [K, Z, E]
            ph.append(p)
            dph.append(p * (1j * ks[:, None, None] * (-coef * d[None] / c)))   # d(phase factor)/dc
            image[:, ix] += (2.0 / N) * np.einsum("kze,kze,ke->z", b, p, X[:, :, ia])
        cache.append((b, ph, dph))
    m2 = np.abs(image) ** 2
    S2, S4 = m2.sum(), (m2 * m2).sum()
    L = -S4 / S2 ** 2
    G = -2.0 * image * (m2 / S2 ** 2 - S4 / S2 ** 3)                            # dL/dI*
    gX = np.zeros((K, E, A), dtype=np.complex128)
    dLdc = 0.0
    for ix in range(px.size):
        b, ph, dph = cache[ix]
        for ia in range(A):
            gX[:, :, ia] += (2.0 / N) * np.einsum("z,kze,kze->ke", G[:, ix], b, np.conj(ph[ia]))
            dI = (2.0 / N) * np.einsum("kze,kze,ke->z", b, dph[ia], X[:, :, ia])
            dLdc += 2.0 * np.real(np.sum(np.conj(G[:, ix]) * dI))
    return L, dLdc, np.transpose(gX, (1, 0, 2)), image


# ---------------------------------------------------------------------------
# das_pw, CPU (.m) semantics
# ---------------------------------------------------------------------------


def das_pw_m(positions_x, positions_z, data_rf, f_s, steering_angle, element_width, element_pitch,
             c_0, f_bounds=None, index_t0=0.0, window=("tukey", 0.2), F_number=None,
             normalization="on", voxels=None):
    """Restates the CPU path of ``das_pw.m:310-481``: N_dft padded with the
    *first* z (``das_pw.m:343``), F capped by sqrt(f z / (2.88 c))
    (``das_pw.m:374-377``), boxcar on the ideal half-width (``das_pw.m:436-441``),
    other windows on the element-edge widths without a cut-off
    (``das_pw.m:449-452``), ``normalizations.windowed`` applied
    (``+normalizations/windowed.m:69-87``), frequencies with an empty index
    range skipped (``das_pw.m:403``), no 2/N scaling (``das_pw.m:384,467``).
    info["F_capped"] is the [K, Z] F-number table actually used
    (``das_pw.m:371-377``); info["signal"] the inverse DFT of the last processed
    voxel's focused spectrum (``das_pw.m:477-481``)."""
    px = np.asarray(positions_x, dtype=np.float64).ravel()
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    rf = np.asarray(data_rf, dtype=np.float64)
    N_t, N_el = rf.shape
    M = (N_el - 1) / 2.0
    ctr = np.arange(-M, M + 1) * element_pitch
    lbs = ctr - element_width / 2.0
    ubs = ctr + element_width / 2.0
    e_x, e_z = -math.sin(steering_angle), math.cos(steering_angle)
    x_ref = np.sign(e_x) * ctr[0]
    if f_bounds is None:
        f_bounds = (EPS, f_s / 2.0)
    N_pad = int(math.ceil((math.sqrt((ctr[-1] - ctr[0]) ** 2 + pz[0] ** 2) - pz[0]) * f_s / c_0))
    N = N_t + N_pad + 1 - ((N_t + N_pad) % 2)
    i_lb = int(math.ceil(f_bounds[0] * N / f_s)) + 1
    i_ub = int(math.floor(f_bounds[1] * N / f_s)) + 1
    ks = np.arange(i_lb, i_ub + 1) - 1                   # 0-based bins
    f = f_s * ks / N
    omega = 2.0 * math.pi * f
    p_l = element_pitch * f / c_0
    if F_number is None:
        F_number = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
    F0 = f_number_values(F_number, p_l) if isinstance(F_number, dict) else np.broadcast_to(
        np.asarray(F_number, dtype=np.float64).ravel(), ks.shape).copy()
    F_ub = np.sqrt(f[:, None] * pz[None, :] / (2.88 * c_0))           # [K, Z]
    Fv = np.minimum(F0[:, None], F_ub)                                 # [K, Z]
    Xf = np.fft.fft(rf, n=N, axis=0)
    Xa = 2.0 * Xf[ks, :]                                               # [K, E]
    with np.errstate(divide="ignore", invalid="ignore"):
        w_des = pz[None, :] / (2.0 * Fv)                               # [K, Z]
    image = np.zeros((pz.size, px.size), dtype=np.complex128)
    want = None
    if voxels is not None:
        want = {}
        for ix, iz in zip(np.asarray(voxels[0]).tolist(), np.asarray(voxels[1]).tolist()):
            want.setdefault(ix, set()).add(iz)
    cols = range(px.size) if want is None else sorted(want)
    norm_kind = normalization if isinstance(normalization, str) else normalization[0]
    for ix in cols:
        x = px[ix]
        dl = ctr - x
        left = dl < 0
        with np.errstate(invalid="ignore"):
            ilb = np.maximum(np.ceil(M + (x - w_des) / element_pitch) + 1, 1)
            iub = np.minimum(np.floor(M + (x + w_des) / element_pitch) + 1, N_el)
        valid = ilb <= iub                                             # [K, Z]
        zs = np.nonzero(valid.any(axis=0))[0]
        if want is not None:
            zs = np.array([z for z in zs if z in want[ix]], dtype=np.int64)
        for iz in zs:
            v = valid[:, iz]
            tof = (e_x * (x - x_ref) + e_z * pz[iz]) / c_0 + index_t0 / f_s \
                + np.sqrt((dl / c_0) ** 2 + (pz[iz] / c_0) ** 2)
            wts = np.exp(1j * omega[v][:, None] * tof[None, :])       # [Kv, E]
            if window[0] == "boxcar":
                ws = window_m(window, dl[None, :] / w_des[v, iz][:, None])
            else:
                wl = x - lbs[ilb[v, iz].astype(np.int64) - 1]
                wr = ubs[iub[v, iz].astype(np.int64) - 1] - x
                ws = np.concatenate([window_m(window, dl[None, left] / wl[:, None]),
                                     window_m(window, dl[None, ~left] / wr[:, None])], axis=1)
            if norm_kind in ("on", "windowed"):
                ws = ws / ws.sum(axis=1, keepdims=True)
                if norm_kind == "windowed":
                    fwin = normalization[1]
                    n_over_two = (ws > 0).sum(axis=0) / 2.0
                    idx = np.arange(ws.shape[0])[:, None]
                    ws = ws * window_m(fwin, (idx - n_over_two[None, :]) / n_over_two[None, :])
            focused = np.sum(ws * wts * Xa[v, :], axis=1)               # [Kv]
            image[iz, ix] = np.sum(focused)
            last = (ks[v], focused)
    # signal of the last voxel processed (das_pw.m:477-481): its focused spectrum at the
    # active bins of a length-N spectrum, inverse DFT
    signal = None
    if want is None and px.size and 'last' in locals():
        spec = np.zeros(N, dtype=np.complex128)
        spec[last[0]] = last[1]
        signal = np.fft.ifft(spec, N)
    return image, {"N_dft": N, "k_lb": int(ks[0]), "k_ub": int(ks[-1]), "F": F0, "F_capped": Fv,
                   "signal": signal}


# ---------------------------------------------------------------------------
# das_sa (SAFT), MEX semantics
# ---------------------------------------------------------------------------


def das_sa_mex(positions_x, positions_z, data_rf, f_s, element_width, element_pitch, c_0,
               f_bounds=None, index_t0=0.0, window_tx=("boxcar", 0.0), window_rx=("boxcar", 0.0),
               F_number_tx=None, F_number_rx=None, normalization_tx="on", normalization_rx="on",
               voxels=None, semantics="reference"):
    """Restates ``cuda.gpu_bf_saft_rf`` (``+cuda/gpu_bf_saft_rf.cu:107-1349``)
    with ``saft_kernel_phase_shifts.cu:41-198`` per term.  data_rf is
    [N_t, N_rx, N_tx] (MATLAB column-major).

    Normalisation combinations (``gpu_bf_saft_rf.cu:1128-1199``):
    semantics="reference" reproduces the MEX: both on -> sum_k S_k/(Wrx Wtx);
    tx on / rx off -> sum_k S_k/Wtx; tx off / rx on -> zero image (never
    accumulated); both off -> only the last bin survives (the per-bin memset
    of the shared buffer).  semantics="intended" divides by whichever sums are
    on and always accumulates.  Constant tx AND rx F-numbers are computed as a
    constant table (the MEX kernel for that case is commented out,
    ``gpu_bf_saft_rf.cu:1095-1101``)."""
    px = np.asarray(positions_x, dtype=np.float64).ravel()
    pz = np.asarray(positions_z, dtype=np.float64).ravel()
    rf = np.asarray(data_rf, dtype=np.float64)
    N_t, N_rx, N_tx = rf.shape
    if N_rx != N_tx:
        raise ValueError("InvalidRFData")
    band = band_mex(pz, N_t, N_rx, f_s, element_width, element_pitch, c_0, f_bounds, index_t0)
    default = ("angle_lb", 70.0, 1.5, 10.0)
    Ftx = _resolve_F(F_number_tx, band, element_pitch, f_s, c_0, default)
    Frx = _resolve_F(F_number_rx, band, element_pitch, f_s, c_0, default)
    X = rf_band_spectra(rf, band)                    # [K, R, T]
    N = band.N_dft
    on_tx = normalization_tx != "off"
    on_rx = normalization_rx != "off"
    info = {"N_dft": N, "k_lb": band.k_lb, "k_ub": band.k_ub, "zero_weight_bins": 0}
    image = np.zeros((pz.size, px.size), dtype=np.complex128)
    w_tx_out = np.zeros((pz.size, px.size))
    w_rx_out = np.zeros((pz.size, px.size))
    if voxels is None:
        vox = [(ix, iz) for ix in range(px.size) for iz in range(pz.size)]
    else:
        vox = list(zip(np.asarray(voxels[0]).tolist(), np.asarray(voxels[1]).tolist()))
    last_only = (semantics == "reference") and not on_tx and not on_rx
    zero_img = (semantics == "reference") and (not on_tx) and on_rx
    for ix, iz in vox:
        x, z = px[ix], pz[iz]
        zz = np.array([z])
        a_tx = _aperture_weights(window_tx, x, zz, Ftx, band, N_tx, element_pitch)[:, 0, :]  # [K,T]
        a_rx = _aperture_weights(window_rx, x, zz, Frx, band, N_rx, element_pitch)[:, 0, :]  # [K,R]
        dist = np.sqrt((band.ctr - x) ** 2 + z * z)                     # [E]
        d = dist[None, :] + dist[:, None]                               # [R,T]
        ph = _phase(band, d)                                            # [K,R,T]
        S = np.einsum("kt,kr,krt,krt->k", a_tx, a_rx, ph, X)
        Wtx = a_tx.sum(axis=1)
        Wrx = a_rx.sum(axis=1)
        den = np.ones_like(Wtx)
        if on_rx:
            den = den * Wrx
        if on_tx:
            den = den * Wtx
        zero = den == 0
        info["zero_weight_bins"] += int(zero.sum())
        Sn = np.where(zero, 0.0, S / np.where(zero, 1.0, den))
        if last_only:
            val = S[-1]
        elif zero_img:
            val = 0.0
        else:
            val = Sn.sum()
        image[iz, ix] = (2.0 / N) * val
        w_tx_out[iz, ix] = Wtx[-1]
        w_rx_out[iz, ix] = Wrx[-1]
    return image, w_tx_out, w_rx_out, info
