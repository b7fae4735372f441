"""The band DFT on the tensor cores (fnum_dft_tc.cu) against the FP64 DFT of the
float32 RF lines, and against FP32 cuFFT (torch.fft, the library the reference
calls, +cuda/gpu_bf_das_pw_rf.cu:917-925) as the measure of FP32 accuracy: the
spectra must be as accurate as the reference's own FP32 transform (bar: 2x its
rel-L2, which is 1.7e-7 to 2.5e-7 here; measured 1.5e-7 to 1.9e-7).  Plane-wave layout [e][k][a] and SAFT
layout [tx][rx][k] are both checked, as are double RF (rounded to float first,
so bit-identical to float RF) and DFT orders that are not multiples of the
64-sample stage or the 128-column tile."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, synth, windows
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n_el,n_t,n_ang", [(64, 1024, 3), (37, 777, 2), (130, 2048, 1)])
def test_pw_band_dft_matches_fp64(gpu, n_el, n_t, n_ang):
    import torch
    rng = np.random.default_rng(n_el)
    arr = synth.LinearArray(n_el, 0.3048e-3, 0.918 * 0.3048e-3)
    sc = synth.random_points(rng, 8, (-5e-3, 5e-3), (5e-3, 25e-3))
    angles = np.linspace(-0.1, 0.1, n_ang)
    rf = synth.pw_rf(rng, arr, sc, list(angles), n_t, 20e6, 1540.0, snr_db=30.0).astype(np.float32)   # [A, E, T]
    px, pz = np.linspace(-3e-3, 3e-3, 5), np.linspace(6e-3, 9e-3, 4)
    plan = das.PWPlan(px, pz, n_t, n_el, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0,
                      windows.hann(), f_numbers.constant(1.5))
    inf = plan.info()
    N, k_lb, K = inf["N_dft"], inf["k_lb"], inf["n_bins"]
    rf_d = torch.tensor(rf, device=gpu)
    plan.execute_dft(rf_d)
    got = plan.spectra().cpu().numpy()                                                  # [E, K, A]
    plan.execute_dft(rf_d.double())
    got_d = plan.spectra().cpu().numpy()
    ref = np.fft.fft(rf.astype(np.float64), N, axis=2)[:, :, k_lb:k_lb + K].transpose(1, 2, 0)
    cufft = torch.fft.fft(rf_d, n=N, dim=2)[:, :, k_lb:k_lb + K].permute(1, 2, 0).cpu().numpy()
    e_ours, e_cufft = _rel(got, ref), _rel(cufft, ref)
    assert e_ours < 2 * e_cufft, (e_ours, e_cufft)
    np.testing.assert_array_equal(got, got_d)
    plan.close()


def test_sa_band_dft_matches_fp64(gpu):
    import torch
    rng = np.random.default_rng(2)
    arr = synth.LinearArray(12, 0.3e-3, 0.918 * 0.3e-3)
    sc = synth.random_points(rng, 4, (-2e-3, 2e-3), (3e-3, 6e-3))
    rf = synth.sa_rf(rng, arr, sc, 500, 40e6, 1540.0).astype(np.float32)                # [tx, rx, t]
    px, pz = np.linspace(-1e-3, 1e-3, 4), np.linspace(3e-3, 5e-3, 3)
    fn = f_numbers.directivity.perrot(0.918)
    plan = das.SAPlan(px, pz, 500, 12, 40e6, arr.width, arr.pitch, 1540.0, None, 0.0, windows.boxcar(),
                      windows.hann(), fn, fn)
    inf = plan.info()
    N, k_lb, K = inf["N_dft"], inf["k_lb"], inf["n_bins"]
    rf_d = torch.tensor(rf, device=gpu)
    plan.execute_dft(rf_d)
    got = plan.spectra().cpu().numpy()                                                  # [tx, rx, K]
    ref = np.fft.fft(rf.astype(np.float64), N, axis=2)[:, :, k_lb:k_lb + K]
    cufft = torch.fft.fft(rf_d, n=N, dim=2)[:, :, k_lb:k_lb + K].cpu().numpy()
    e_ours, e_cufft = _rel(got, ref), _rel(cufft, ref)
    assert e_ours < 2 * e_cufft, (e_ours, e_cufft)
    plan.close()
