"""Known answers and analytic properties that pin the FP64 oracle (CPU only).

The reference ships no tests or golden vectors, so the oracle is checked
against closed forms derived from the definitions of the parameter classes,
the band arithmetic of the MEX gateways, and physical properties of the
beamformer.
"""
import math

import numpy as np
import pytest

from f_number_gb300 import synth
from oracle import coracle as CO
from oracle import fnum_oracle as O

ANGLE_LB = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}


# --- F-number classes ---------------------------------------------------------
def test_angle_lb_grating_condition():
    """In its relevant band angle_lb puts the first grating lobe exactly at the
    lower bound: 1/p - 1/sqrt(1 + 4F^2) = sin(angle_lb) (angle_lb.m:56-66)."""
    for alpha in (45.0, 60.0, 70.0):
        s = math.sin(math.radians(alpha))
        lower, upper = 1 / (1 + s), 1 / (1 / math.sqrt(1 + 9.0) + s)
        p = np.linspace(lower + 1e-6, upper - 1e-6, 50)
        F = O.fnum_angle_lb(alpha, 1.5, -1, p)          # no anti-aliasing floor
        lhs = 1 / p - 1 / np.sqrt(1 + 4 * F ** 2)
        np.testing.assert_allclose(lhs, s, rtol=0, atol=1e-12)
        assert np.all(O.fnum_angle_lb(alpha, 1.5, -1, np.array([lower * 0.9])) == 0.0)
        assert np.all(O.fnum_angle_lb(alpha, 1.5, -1, np.array([upper, upper * 1.5])) == 1.5)


def test_distance_constant_branches_meet():
    """distance.constant: 0 below p = 1/2, tan(d)/2 where the transition branch
    meets the main branch at p = 1/(1 + cos d), F_ub beyond 1/sin(d)."""
    for d in (5.0, 10.0, 20.0):
        r = math.radians(d)
        p0 = 1 / (1 + math.cos(r))
        left = O.fnum_distance_constant(d, math.inf, np.array([p0 * (1 - 1e-12)]))[0]
        right = O.fnum_distance_constant(d, math.inf, np.array([p0]))[0]
        assert abs(left - math.tan(r) / 2) < 1e-9
        assert abs(right - math.tan(r) / 2) < 1e-9
        assert O.fnum_distance_constant(d, math.inf, np.array([0.49]))[0] == 0.0
        assert O.fnum_distance_constant(d, 3.0, np.array([1 / math.sin(r) * 1.01]))[0] == 3.0
        assert O.fnum_distance_constant(d, 1.0, np.array([p0 * 1.5]))[0] <= 1.0


def test_angle_lb_takes_max_with_distance():
    p = np.linspace(0.2, 1.5, 200)
    F = O.fnum_angle_lb(60, 1.5, 10, p)
    np.testing.assert_array_equal(F, np.maximum(O.fnum_angle_lb(60, 1.5, -1, p),
                                                 O.fnum_distance_constant(10, math.inf, p)))
    assert np.all(np.diff(F) >= 0)      # monotone over the imaging band


def test_directivity_attenuation_point():
    """perrot / soft / rigid: the returned F = 1/(2 tan a) sits where the element
    directivity falls to -att dB (directivity.m:103-118), within Brent's TolX."""
    p = np.linspace(0.3, 2.0, 12)
    for obl, att in (("soft", 3.0), ("rigid", 3.0), ("soft", 6.0)):
        F = O.fnum_directivity(0.918, obl, att, p)
        a = np.arctan(1 / (2 * F))
        wl = 0.918 * p
        ob = np.cos(a) if obl == "soft" else 1.0
        D = ob * np.sinc(wl * np.sin(a))
        # a crossing exists where the directivity at 90 degrees is below the threshold
        d90 = (0.0 if obl == "soft" else 1.0) * np.sinc(wl)
        has = d90 < 10 ** (-att / 20)
        np.testing.assert_allclose(D[has], 10 ** (-att / 20), atol=5e-4)
        # otherwise the minimiser runs to 90 degrees: F -> 0 (full aperture)
        assert np.all(F[~has] < 1e-3)


def test_fminbnd_quadratic():
    x = O.fminbnd(lambda t: (t - 0.3) ** 2, 0.0, 1.0)
    assert abs(x - 0.3) < 1e-4


def test_szabo_and_constant():
    p = np.array([0.5, 1.0, 2.0])
    np.testing.assert_allclose(O.f_number_values({"kind": "directivity.szabo", "width_over_pitch": 0.918}, p),
                               0.918 * p / 1.2)
    np.testing.assert_array_equal(O.f_number_values({"kind": "constant", "value": 1.7}, p), 1.7)


# --- windows --------------------------------------------------------------------
def test_windows_mex_values():
    L = 2.0
    assert O.window_mex(("hann", 0), 0.0, L) == 1.0
    assert abs(O.window_mex(("hann", 0), 1.0, L) - 0.5) < 1e-15
    assert O.window_mex(("hann", 0), 2.0, L) == 0.0          # |l| >= L -> 0
    assert O.window_mex(("tukey", 0.5), 1.0, L) == 1.0
    assert abs(O.window_mex(("tukey", 0.5), 1.5, L) - 0.5) < 1e-15
    assert O.window_mex(("triangular", 0), -0.5, L) == 0.75
    assert O.window_mex(("boxcar", 0), 1.999, L) == 1.0
    assert O.window_mex(("boxcar", 0), -2.0, L) == 0.0


def test_windows_matlab_no_cutoff():
    """hann.m / triangular.m have no cut-off at |u| >= 1 (das_pw.m uses them on
    elements outside the aperture)."""
    assert abs(O.window_m(("hann", 0), 1.5) - 0.5) < 1e-15
    assert O.window_m(("triangular", 0), 1.5) == -0.5
    assert O.window_m(("tukey", 0.2), 1.2) == 0.0


# --- band -------------------------------------------------------------------------
def test_band_known_answers():
    wl = synth.pw_single_angle(with_rf=False)
    b = O.band_mex(wl.positions_z, 2048, 128, 20e6, wl.array.width, wl.array.pitch, 1540.0, wl.f_bounds, 0)
    assert (b.N_dft, b.k_lb, b.k_ub) == (2489, 281, 840)
    wl2 = synth.cpwc_11_angles(with_rf=False)
    b2 = O.band_mex(wl2.positions_z, 2048, 128, 20e6, wl2.array.width, wl2.array.pitch, 1540.0, wl2.f_bounds, 0)
    assert (b2.N_dft, b2.k_lb, b2.k_ub) == (2491, 250, 871)
    wl3 = synth.saft_128(with_rf=False)
    b3 = O.band_mex(wl3.positions_z, 3072, 128, 40e6, wl3.array.width, wl3.array.pitch, 1540.0, None, 0)
    assert (b3.N_dft, b3.k_lb, b3.k_ub) == (3985, 1, 1992)
    # das_pw.m pads with the first axial position: 2491 for the single-angle grid
    N, ks, _ = CO.pw_m_prepare(wl.positions_z, np.zeros((1, 128, 2048)), 20e6, wl.array.width, wl.array.pitch,
                               1540.0, wl.f_bounds, ANGLE_LB)
    assert N == 2491


def test_band_invalid_bounds():
    with pytest.raises(ValueError):
        O.band_mex(np.array([0.01, 0.02]), 64, 16, 20e6, 1e-4, 2e-4, 1540.0, (9.99e6, 9.995e6), 0)


# --- beamformer properties ------------------------------------------------------------
def _small_pw(seed=0, n_el=32, n_t=512, angles=(0.0,)):
    arr = synth.LinearArray(n_el, 0.3048e-3, 0.918 * 0.3048e-3)
    rng = np.random.default_rng(seed)
    sc = synth.Scatterers(np.array([0.6e-3]), np.array([11e-3]), np.array([1.0]))
    rf = synth.pw_rf(rng, arr, sc, list(angles), n_t, 20e6, 1540.0, snr_db=np.inf)
    return arr, rf


def test_point_scatterer_focus():
    arr, rf = _small_pw()
    px = np.linspace(-0.6e-3, 1.8e-3, 17)
    pz = np.linspace(10e-3, 12e-3, 17)
    img, _, info = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0,
                                ("hann", 0.0), ANGLE_LB, "on")
    iz, ix = np.unravel_index(np.argmax(np.abs(img)), img.shape)
    assert abs(px[ix] - 0.6e-3) <= 0.16e-3 and abs(pz[iz] - 11e-3) <= 0.13e-3
    assert info["zero_weight_bins"] == 0


def test_zero_and_linearity():
    arr, rf = _small_pw()
    rng = np.random.default_rng(5)
    rf2 = rng.standard_normal(rf.shape)
    px = np.linspace(-1e-3, 1e-3, 5)
    pz = np.linspace(9e-3, 12e-3, 4)
    args = (20e6, 0.05, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0, ("tukey", 0.5), ANGLE_LB, "on")
    z0, _, _ = O.das_pw_mex(px, pz, np.zeros_like(rf[0].T), *args)
    assert np.all(z0 == 0)
    a, _, _ = O.das_pw_mex(px, pz, rf[0].T, *args)
    b, _, _ = O.das_pw_mex(px, pz, rf2[0].T, *args)
    c, _, _ = O.das_pw_mex(px, pz, 2.0 * rf[0].T - 3.0 * rf2[0].T, *args)
    np.testing.assert_allclose(c, 2 * a - 3 * b, rtol=0, atol=1e-12 * np.abs(c).max())


def test_m_equals_mex_times_N_when_quirks_neutral():
    """With z[0] == z[1] (same N_dft), a constant F below the depth cap, a Tukey
    window (element-edge widths and a cut-off in both) and normalisation on,
    das_pw.m's image equals N_dft times the MEX image."""
    arr, rf = _small_pw(angles=(0.1,))
    px = np.linspace(-1e-3, 1e-3, 6)
    pz = np.array([10e-3, 10e-3, 11e-3, 12e-3])
    F = {"kind": "constant", "value": 1.0}
    mex, _, info = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.1, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0,
                                ("tukey", 0.5), F, "on")
    m, infom = O.das_pw_m(px, pz, rf[0].T, 20e6, 0.1, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0,
                          ("tukey", 0.5), F, "on")
    assert info["N_dft"] == infom["N_dft"]
    np.testing.assert_allclose(m, info["N_dft"] * mex, rtol=1e-10, atol=1e-10 * np.abs(m).max())


def test_c_oracle_matches_numpy_oracle():
    arr = synth.LinearArray(24, 0.3048e-3, 0.918 * 0.3048e-3)
    rng = np.random.default_rng(3)
    sc = synth.random_points(rng, 4, (-2e-3, 2e-3), (8e-3, 12e-3))
    angs = [-0.1, 0.07]
    rf = synth.pw_rf(rng, arr, sc, angs, 400, 20e6, 1540.0)
    px = np.linspace(-2e-3, 2e-3, 5)
    pz = np.linspace(8e-3, 12e-3, 4)
    ix, iz = [a.ravel() for a in np.meshgrid(np.arange(5), np.arange(4), indexing="ij")]
    for win in (("hann", 0.0), ("boxcar", 0.0)):
        ref = sum(O.das_pw_mex(px, pz, rf[a].T, 20e6, angs[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0, win,
                               ANGLE_LB, "on")[0] for a in range(2))
        out, _, _ = CO.pw_mex(px, pz, rf, 20e6, angs, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0, win, ANGLE_LB,
                              "on", ix, iz, threads=2)
        np.testing.assert_allclose(out, ref[iz, ix], rtol=0, atol=1e-12 * np.abs(ref).max())
        refm = sum(O.das_pw_m(px, pz, rf[a].T, 20e6, angs[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0, win,
                              ANGLE_LB, "on")[0] for a in range(2))
        outm, _ = CO.pw_m(px, pz, rf, 20e6, angs, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0, win, ANGLE_LB,
                          "on", ix, iz, threads=2)
        np.testing.assert_allclose(outm, refm[iz, ix], rtol=0, atol=1e-11 * np.abs(refm).max())


def test_saft_normalisation_semantics():
    arr = synth.LinearArray(10, 0.3e-3, 0.918 * 0.3e-3)
    rng = np.random.default_rng(2)
    sc = synth.random_points(rng, 3, (-1e-3, 1e-3), (3e-3, 6e-3))
    rf = synth.sa_rf(rng, arr, sc, 200, 40e6, 1540.0)
    px = np.linspace(-1e-3, 1e-3, 3)
    pz = np.linspace(3e-3, 6e-3, 3)
    data = np.transpose(rf, (2, 1, 0))
    args = (40e6, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0, ("boxcar", 0), ("hann", 0), ANGLE_LB, ANGLE_LB)
    off_on, _, _, _ = O.das_sa_mex(px, pz, data, *args, "off", "on")
    assert np.all(off_on == 0)               # never accumulated (gpu_bf_saft_rf.cu:1195-1199)
    off_off, _, _, info = O.das_sa_mex(px, pz, data, *args, "off", "off")
    last, _, _, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0,
                                 (info["k_ub"] * 40e6 / info["N_dft"] * 0.9999, 7e6), 0, ("boxcar", 0),
                                 ("hann", 0), ANGLE_LB, ANGLE_LB, "off", "off", semantics="intended")
    assert np.abs(off_off).max() > 0
    on_on, wt, wr, _ = O.das_sa_mex(px, pz, data, *args, "on", "on")
    assert np.all(wt > 0) and np.all(wr > 0)


def test_sharpness_gradient_oracle_matches_finite_differences():
    """The FP64 gradients of the sharpness loss (oracle.pw_sharpness_grad) against
    central differences: h = 1e-3 m/s on c (band, F table and apertures frozen)
    and a random RF direction (dL = 2 Re sum conj(dL/dX*) dX)."""
    from f_number_gb300 import synth
    rng = np.random.default_rng(3)
    arr = synth.LinearArray(16, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = [-0.05, 0.05]
    px, pz = np.linspace(-2e-3, 2e-3, 6), np.linspace(5e-3, 9e-3, 7)
    rf = synth.pw_rf(rng, arr, synth.random_points(rng, 3, (-2e-3, 2e-3), (5e-3, 9e-3)), angles, 384, 20e6, 1540.0)
    F = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
    kw = dict(f_bounds=(2e6, 7e6), index_t0=0.0, window=("hann", 0.0), F_number=F, normalization="on")
    run = lambda r, c: O.pw_sharpness_grad(px, pz, r, 20e6, angles, arr.width, arr.pitch, c, c_freeze=1540.0, **kw)
    L, dLdc, gX, _ = run(rf, 1540.0)
    h = 1e-3
    fd = (run(rf, 1540.0 + h)[0] - run(rf, 1540.0 - h)[0]) / (2 * h)
    assert abs(fd - dLdc) <= 1e-6 * abs(dLdc)
    d_rf = rng.standard_normal(rf.shape)
    band = O.band_mex(pz, 384, 16, 20e6, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0)
    dX = np.stack([O.rf_band_spectra(d_rf[a].T, band) for a in range(2)], axis=2).transpose(1, 0, 2)
    an = 2 * np.real(np.sum(np.conj(gX) * dX))
    eps = 1e-5                                 # relative to the RF's ~0.13 rms (central differences, error ~eps^2)
    fd = (run(rf + eps * d_rf, 1540.0)[0] - run(rf - eps * d_rf, 1540.0)[0]) / (2 * eps)
    assert abs(fd - an) <= 1e-6 * abs(an)


def test_saft_transmit_receive_symmetry_identity():
    """The identity behind the SAFT kernels' symmetric path, in FP64: with equal transmit
    and receive windows, F-numbers and normalisations, beamforming RF' with
    RF'[t][r] = RF[t][r] + RF[r][t] (t < r), RF'[t][t] = RF[t][t], RF'[t][r] = 0 (t > r)
    gives the image of RF (the band DFT is linear and pair (t, r) has the weight and
    phase of (r, t)).  With unequal F-numbers it does not."""
    rng = np.random.default_rng(17)
    ne, nt = 10, 200
    rf = rng.standard_normal((ne, ne, nt))                   # [tx, rx, t], not reciprocal
    sym = np.zeros_like(rf)
    for t in range(ne):
        sym[t, t] = rf[t, t]
        for r in range(t + 1, ne):
            sym[t, r] = rf[t, r] + rf[r, t]
    px = np.linspace(-1e-3, 1e-3, 5)
    pz = np.linspace(3e-3, 6e-3, 4)
    fn = {"kind": "directivity", "width_over_pitch": 0.918, "obliquity": "soft", "attenuation_dB": 3.0}
    other = {"kind": "constant", "value": 1.2}
    for wt, ftx, equal in ((("hann", 0.0), fn, True), (("boxcar", 0.0), fn, True), (("boxcar", 0.0), other, False)):
        a = O.das_sa_mex(px, pz, np.transpose(rf, (2, 1, 0)), 40e6, 0.918 * 0.3e-3, 0.3e-3, 1540.0, (2e6, 9e6), 0.0,
                         wt, wt, ftx, fn, "on", "on")[0]
        b = O.das_sa_mex(px, pz, np.transpose(sym, (2, 1, 0)), 40e6, 0.918 * 0.3e-3, 0.3e-3, 1540.0, (2e6, 9e6), 0.0,
                         wt, wt, ftx, fn, "on", "on")[0]
        rel = np.linalg.norm(a - b) / np.linalg.norm(a)
        if equal:
            assert rel < 1e-12, (wt, rel)
        else:
            assert rel > 1e-3, (wt, rel)
