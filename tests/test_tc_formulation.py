"""The tensor-core plane-wave formulation, emulated in numpy against the FP64 oracle.

Per band bin k the compounded image gains sum_a t_{v,a}^k G_k(v, a) with
G_k(v, a) = sum_e R_k(v, e) X_k(e, a), R_k = (a_{v,e,k} / W_{v,k}) r_{v,e}^k.  The
kernel forms G_k with fp16 operands, each fp32 value split into hi + lo, as
hi.hi + hi.lo + lo.hi, after scaling the spectra by a power of two below 2^14.
This restates that arithmetic (float32 values, fp16 splits, float64 sums) on a
small case with the oracle's own apertures, windows, phases and spectra, and
checks the image against das_pw_mex's FP64 result.  It isolates the precision of
the operand split from the kernel's recurrences (which the GPU tests cover)."""
import math

import numpy as np
import pytest

from f_number_gb300 import synth
from oracle import fnum_oracle as O


def _split(v):
    hi = v.astype(np.float16)
    lo = (v - hi.astype(np.float32)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64)


def _cmul3(a, b):
    """sum over e of a[..., e] b[e, ...] for complex float32 a, b with fp16 hi/lo
    operands in real form (three products), float64 accumulation."""
    arh, arl = _split(a.real.astype(np.float32))
    aih, ail = _split(a.imag.astype(np.float32))
    brh, brl = _split(b.real.astype(np.float32))
    bih, bil = _split(b.imag.astype(np.float32))

    def mm(xh, xl, yh, yl):
        return xh @ yh + xh @ yl + xl @ yh

    re = mm(arh, arl, brh, brl) - mm(aih, ail, bih, bil)
    im = mm(arh, arl, bih, bil) + mm(aih, ail, brh, brl)
    return re + 1j * im


@pytest.mark.parametrize("window", [("hann", 0.0), ("boxcar", 0.0)])
def test_tensor_core_formulation_matches_fp64(window):
    rng = np.random.default_rng(23)
    ne, nt, fs, c = 24, 512, 20e6, 1540.0
    pitch, width = 0.3048e-3, 0.918 * 0.3048e-3
    arr = synth.LinearArray(ne, pitch, width)
    angles = np.deg2rad([-6.0, 0.0, 6.0])
    px = np.linspace(-2e-3, 2e-3, 9)
    pz = np.linspace(5e-3, 12e-3, 8)
    sc = synth.random_points(rng, 5, (px[0], px[-1]), (pz[0], pz[-1]))
    rf = synth.pw_rf(rng, arr, sc, list(angles), nt, fs, c)                # [A, E, T]
    spec = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
    ref = sum(O.das_pw_mex(px, pz, rf[a].T.astype(np.float64), fs, angles[a], width, pitch, c, (2e6, 7e6), 0.0,
                           window, spec, "on")[0] for a in range(len(angles)))

    band = O.band_mex(pz, nt, ne, fs, width, pitch, c, (2e6, 7e6), 0.0)
    F = O.f_number_values(spec, O.pitch_over_lambda(band, pitch, fs, c))
    X = np.stack([O.rf_band_spectra(rf[a].T.astype(np.float64), band) for a in range(len(angles))], axis=2)  # [K,E,A]
    m = float(np.max(np.abs(np.concatenate([X.real.ravel(), X.imag.ravel()]))))
    sigma = 2.0 ** (14 - math.frexp(m)[1])
    Xs = (X * sigma).astype(np.complex64)
    ks = band.ks.astype(np.float64)
    img = np.zeros((pz.size, px.size), dtype=np.complex128)
    for ix, x in enumerate(px):
        a = O._aperture_weights(window, x, pz, F, band, ne, pitch)                 # [K,Z,E]
        W = a.sum(axis=2)
        b = np.where(W[..., None] > 0, a / np.where(W > 0, W, 1.0)[..., None], 0.0)
        d_rx = np.sqrt((band.ctr - x)[None, :] ** 2 + pz[:, None] ** 2)           # [Z,E]
        img_col = np.zeros(pz.size, dtype=np.complex128)
        for ia, th in enumerate(angles):
            e_x, e_z = -math.sin(th), math.cos(th)
            x_ref = -band.M * pitch if e_x >= 0 else band.M * pitch
            d_tx = e_x * (x - x_ref) + e_z * pz                                     # [Z]
            for kk, k in enumerate(ks):
                R = (b[kk] * np.exp(1j * k * band.coef * d_rx)).astype(np.complex64)           # [Z,E]
                G = _cmul3(R, Xs[kk, :, ia:ia + 1])[:, 0]                                     # [Z]
                img_col += np.exp(1j * k * (band.coef * d_tx + band.add)) * G
        img[:, ix] = img_col * (2.0 / band.N_dft) / sigma
    err = np.linalg.norm(img - ref) / np.linalg.norm(ref)
    assert err < 5e-7, err          # measured 6e-8 (Hann) and 8e-8 (boxcar)
