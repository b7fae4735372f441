"""Precision of the tensor-core band DFT (f_number_gb300/csrc/fnum_dft_tc.cu),
restated in numpy: each RF line, rounded to float32 and scaled by the power of
two that brings its largest sample below 2^14, and each float32 twiddle of the
FP64 table are split into fp16 hi = rn(v) and lo = rn(v - hi); a band bin is
sum_t hi_x hi_w + hi_x lo_w + lo_x hi_w.  Against the FP64 DFT of the same
float32 line (the reference rounds RF to float before its FP32 cuFFT,
+cuda/gpu_bf_das_pw_rf.cu:787-793) the split alone costs ~1e-7 relative; the
GPU adds its FP32 accumulation, which the GPU test bounds."""
import numpy as np

from f_number_gb300 import synth


def _split(v):
    hi = v.astype(np.float16)
    lo = (v - hi.astype(np.float32)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64)


def band_dft_split(x32, N, k_lb, K):
    m = float(np.max(np.abs(x32)))
    ex = int(np.frexp(m)[1]) if m > 0 else 0
    sc = np.float32(2.0 ** (14 - ex)) if m > 0 else np.float32(1.0)
    xh, xl = _split((x32 * sc).astype(np.float32))
    t = np.arange(x32.size)
    ks = np.arange(k_lb, k_lb + K)
    m_idx = (ks[:, None] * t[None, :]) % N
    tw = np.exp(-2j * np.pi * np.arange(N) / N).astype(np.complex64)          # the float twiddle table
    w = tw[m_idx]
    wrh, wrl = _split(w.real.astype(np.float32))
    wih, wil = _split(w.imag.astype(np.float32))
    re = (wrh * xh).sum(1) + (wrl * xh).sum(1) + (wrh * xl).sum(1)
    im = (wih * xh).sum(1) + (wil * xh).sum(1) + (wih * xl).sum(1)
    return (re + 1j * im) / np.float64(sc)


def test_split_dft_matches_fp64_dft():
    rng = np.random.default_rng(5)
    arr = synth.LinearArray(8, 0.3048e-3, 0.918 * 0.3048e-3)
    sc = synth.merge(synth.random_points(rng, 5, (-5e-3, 5e-3), (5e-3, 25e-3)),
                     synth.random_points(rng, 50, (-5e-3, 5e-3), (5e-3, 25e-3), amp=0.01))
    rf = synth.pw_rf(rng, arr, sc, [0.0], 1024, 20e6, 1540.0, snr_db=40.0)[0].astype(np.float32)
    N, k_lb, K = 1133, 114, 284          # a 2-7 MHz band of an odd DFT order
    worst = 0.0
    for x in rf:
        ref = np.fft.fft(x.astype(np.float64), N)[k_lb:k_lb + K]
        got = band_dft_split(x, N, k_lb, K)
        worst = max(worst, np.linalg.norm(got - ref) / np.linalg.norm(ref))
    assert worst < 2e-7, worst
