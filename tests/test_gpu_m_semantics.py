"""das_pw.m semantics on the GPU (FNUM_FLAG_M_SEMANTICS; das_pw with
platforms.cpu) against the FP64 restatement of das_pw.m's loop
(oracle.das_pw_m): depth-capped F, ideal-width boxcar, windows without a
cut-off, normalizations.windowed along frequency, no 2/N scaling, and the
F_number_values / signal outputs (das_pw.m:371-377, 477-481)."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, normalizations, platforms, synth, windows
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4

PITCH = 0.3048e-3
WINDOWS = [windows.boxcar(), windows.hann(), windows.tukey(0.5), windows.triangular()]
NORMS = [normalizations.on(), normalizations.off(), normalizations.windowed(windows.hann())]
FNUMS = [f_numbers.grating.angle_lb(60.0, 1.5), f_numbers.constant(1.2)]


def _case(seed=21, ne=24, nt=640, angle=0.08):
    rng = np.random.default_rng(seed)
    arr = synth.LinearArray(ne, PITCH, 0.918 * PITCH)
    px = np.linspace(-3e-3, 3e-3, 14)
    pz = np.linspace(5e-3, 12e-3, 18)
    sc = synth.random_points(rng, 4, (-3e-3, 3e-3), (5e-3, 12e-3))
    rf = synth.pw_rf(rng, arr, sc, [angle], nt, 20e6, 1540.0)[0].T        # [T, E]
    return arr, px, pz, rf, angle


def _norm_spec(n):
    if isinstance(n, normalizations.windowed):
        return ("windowed", n.window.spec())
    return n.string()


@pytest.mark.parametrize("win", WINDOWS, ids=lambda w: w.string())
@pytest.mark.parametrize("norm", NORMS, ids=lambda n: n.string())
def test_m_semantics_matches_oracle(gpu, win, norm):
    arr, px, pz, rf, angle = _case()
    for fn in FNUMS:
        img, F, sig = das.das_pw(px, pz, rf, 20e6, angle, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0, win, fn,
                                 norm, platforms.cpu())
        ref, info = O.das_pw_m(px, pz, rf, 20e6, angle, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0, win.spec(),
                               fn.spec(), _norm_spec(norm))
        # normalizations.windowed divides by each element's half-count of bins with a
        # positive weight; where an element has none, MATLAB (and the oracle) give
        # 0 * NaN = NaN.  The GPU must give NaN at the same voxels.
        bad = ~np.isfinite(ref)
        assert np.array_equal(~np.isfinite(img), bad), (fn.string(),)
        if (~bad).any():
            assert np.linalg.norm(img[~bad] - ref[~bad]) / np.linalg.norm(ref[~bad]) < TOL_L2, (fn.string(),)
        np.testing.assert_allclose(F, info["F_capped"], rtol=1e-12)
        assert sig is not None and info["signal"] is not None
        sbad = ~np.isfinite(info["signal"])
        assert np.array_equal(~np.isfinite(sig), sbad)
        if (~sbad).any():
            s_ok, r_ok = sig[~sbad], info["signal"][~sbad]
            assert np.linalg.norm(s_ok - r_ok) / np.linalg.norm(r_ok) < TOL_L2


def test_m_semantics_band_and_scaling(gpu):
    """N_dft comes from positions_z[0] (das_pw.m:343), and the image is N_dft times
    larger than the MEX's in the limit where the other differences vanish: checked
    through the plan's band against the oracle's."""
    arr, px, pz, rf, angle = _case(seed=22)
    plan = das.PWPlan(px, pz, rf.shape[0], arr.n_elements, 20e6, [angle], arr.width, arr.pitch, 1540.0, [2e6, 7e6],
                      0.0, windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5), semantics="m")
    _, info = O.das_pw_m(px, pz, rf, 20e6, angle, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0, ("hann", 0.0),
                         f_numbers.grating.angle_lb(60.0, 1.5).spec(), "on")
    pi = plan.info()
    assert (pi["N_dft"], pi["k_lb"], pi["k_ub"]) == (info["N_dft"], info["k_lb"], info["k_ub"])
    plan.close()


def test_m_semantics_rejects_large_arrays(gpu):
    from f_number_gb300._lib import FNumError
    with pytest.raises(FNumError) as e:
        das.PWPlan(np.zeros(4), np.linspace(5e-3, 6e-3, 4), 256, 300, 20e6, [0.0], 0.28e-3, PITCH, 1540.0,
                   semantics="m")
    assert e.value.identifier.endswith("TooManyElements")
