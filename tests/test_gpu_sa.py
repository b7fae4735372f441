"""Synthetic-aperture parity: the CUDA path (through the C ABI) against the
FP64 oracle, for every normalisation combination of the MEX gateway
(reference semantics) and for the intended semantics.  Tolerances as in
test_gpu_pw.py."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, normalizations, synth, windows
from oracle import coracle as CO
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4
TOL_W = 1e-5
TOL_PLAIN = 2e-3


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def small_sa(seed=0, n_el=16, n_t=384):
    arr = synth.LinearArray(n_el, 0.3e-3, 0.918 * 0.3e-3)
    rng = np.random.default_rng(seed)
    sc = synth.random_points(rng, 4, (-1.5e-3, 1.5e-3), (3e-3, 8e-3))
    rf = synth.sa_rf(rng, arr, sc, n_t, 40e6, 1540.0)          # [tx, rx, t]
    px = np.linspace(-1.5e-3, 1.5e-3, 7)
    pz = np.linspace(3e-3, 8e-3, 6)
    return arr, rf, px, pz


NORMS = {"on": normalizations.on(), "off": normalizations.off()}


@pytest.mark.parametrize("ntx,nrx", [("on", "on"), ("on", "off"), ("off", "on"), ("off", "off")])
@pytest.mark.parametrize("semantics", ["reference", "intended"])
def test_sa_normalisations(gpu, ntx, nrx, semantics):
    arr, rf, px, pz = small_sa()
    data = np.transpose(rf, (2, 1, 0))
    wt, wr = windows.boxcar(), windows.hann()
    fn = f_numbers.directivity.perrot(0.918)
    img, wtx, wrx = das.gpu_bf_saft_rf(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0, wt, wr, fn,
                                       fn, NORMS[ntx], NORMS[nrx], 0, semantics=semantics)
    ref, rwt, rwr, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0, wt.spec(),
                                    wr.spec(), fn.spec(), fn.spec(), ntx, nrx, semantics=semantics)
    if np.all(ref == 0):
        assert np.all(img == 0)
    else:
        assert rel_l2(img, ref) < TOL_L2
    np.testing.assert_allclose(wtx, rwt, rtol=TOL_W)
    np.testing.assert_allclose(wrx, rwr, rtol=TOL_W)


@pytest.mark.parametrize("wt,wr", [(windows.tukey(0.4), windows.triangular()), (windows.hann(), windows.boxcar())],
                         ids=["tukey-tri", "hann-box"])
def test_sa_windows_and_f_numbers(gpu, wt, wr):
    arr, rf, px, pz = small_sa(seed=3)
    data = np.transpose(rf, (2, 1, 0))
    ftx, frx = f_numbers.grating.angle_lb(60, 1.5), f_numbers.constant(1.0)
    img, _, _ = das.gpu_bf_saft_rf(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0, wt, wr, ftx, frx)
    ref, _, _, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0, wt.spec(),
                                wr.spec(), ftx.spec(), frx.spec(), "on", "on")
    assert rel_l2(img, ref) < TOL_L2


def test_sa_plain_kernel(gpu):
    arr, rf, px, pz = small_sa(seed=5, n_el=12)
    data = np.transpose(rf, (2, 1, 0))
    fn = f_numbers.directivity.perrot(0.918)
    img, wt, wr = das.gpu_bf_saft_rf(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0,
                                     windows.boxcar(), windows.boxcar(), fn, fn, kernel="plain")
    ref, rwt, rwr, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0,
                                    ("boxcar", 0.0), ("boxcar", 0.0), fn.spec(), fn.spec(), "on", "on")
    assert rel_l2(img, ref) < TOL_PLAIN
    np.testing.assert_allclose(wt, rwt, rtol=TOL_W)


def test_sa_full_size_sampled(gpu):
    """128 x 128 transmits/receives, 3072 samples at 40 MHz, 400 x 400 grid,
    perrot(0.918) F-number, boxcar windows, 2-7 MHz band."""
    wl = synth.saft_128(seed=0, f_bounds=(2e6, 7e6))
    fn = f_numbers.directivity.perrot(0.918)
    data = np.asfortranarray(np.transpose(wl.rf, (2, 1, 0)))
    img, wt, wr = das.gpu_bf_saft_rf(wl.positions_x, wl.positions_z, data, wl.f_s, wl.array.width, wl.array.pitch,
                                     wl.c, list(wl.f_bounds), 0, windows.boxcar(), windows.boxcar(), fn, fn)
    rng = np.random.default_rng(4)
    ix, iz = rng.integers(0, 400, 24), rng.integers(0, 400, 24)
    ref, rwt, rwr, _ = CO.sa_mex(wl.positions_x, wl.positions_z, wl.rf, wl.f_s, wl.array.width, wl.array.pitch, wl.c,
                                 wl.f_bounds, 0.0, ("boxcar", 0.0), ("boxcar", 0.0), fn.spec(), fn.spec(), "on", "on",
                                 ix, iz)
    assert rel_l2(img[iz, ix], ref) < TOL_L2
    np.testing.assert_allclose(wt[iz, ix], rwt, rtol=TOL_W)


@pytest.mark.parametrize("ntx,nrx", [("on", "on"), ("off", "off"), ("on", "off")])
@pytest.mark.parametrize("ftx_kind", ["same", "other"])
def test_sa_transmit_receive_symmetry(gpu, ntx, nrx, ftx_kind):
    """Boxcar windows with equal F-numbers and normalisations beamform only r >= t from
    X[t][r] + X[r][t]; the RF here is not reciprocal (independent noise per pair), so a
    path that assumed X[t][r] = X[r][t] would fail.  Unequal settings keep all pairs."""
    arr = synth.LinearArray(18, 0.3e-3, 0.918 * 0.3e-3)
    rng = np.random.default_rng(41)
    rf = rng.standard_normal((18, 18, 320))
    px = np.linspace(-2e-3, 2e-3, 9)
    pz = np.linspace(3e-3, 9e-3, 7)
    data = np.transpose(rf, (2, 1, 0))
    fn = f_numbers.directivity.perrot(0.918)
    ftx = fn if ftx_kind == "same" else f_numbers.grating.angle_lb(60, 1.5)
    box = windows.boxcar()
    img, wtx, wrx = das.gpu_bf_saft_rf(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0, box, box,
                                       ftx, fn, NORMS[ntx], NORMS[nrx], 0, semantics="intended")
    ref, rwt, rwr, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0, box.spec(),
                                    box.spec(), ftx.spec(), fn.spec(), ntx, nrx, semantics="intended")
    assert rel_l2(img, ref) < TOL_L2
    np.testing.assert_allclose(wtx, rwt, rtol=TOL_W)
    np.testing.assert_allclose(wrx, rwr, rtol=TOL_W)


@pytest.mark.parametrize("win", [windows.hann(), windows.tukey(0.3), windows.triangular()], ids=["hann", "tukey", "tri"])
def test_sa_symmetry_windowed(gpu, win):
    """Equal non-boxcar windows on both sides: the in-loop kernel with r >= t only."""
    arr = synth.LinearArray(14, 0.3e-3, 0.918 * 0.3e-3)
    rng = np.random.default_rng(43)
    rf = rng.standard_normal((14, 14, 300))
    px = np.linspace(-1.5e-3, 1.5e-3, 8)
    pz = np.linspace(3e-3, 8e-3, 6)
    data = np.transpose(rf, (2, 1, 0))
    fn = f_numbers.directivity.perrot(0.918)
    img, _, _ = das.gpu_bf_saft_rf(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0, win, win, fn, fn)
    ref, _, _, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0, win.spec(),
                                win.spec(), fn.spec(), fn.spec(), "on", "on")
    assert rel_l2(img, ref) < TOL_L2
