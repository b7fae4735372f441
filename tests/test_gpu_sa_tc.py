"""The synthetic-aperture tensor-core kernel (variant 2) against the FP64 oracle
and against the per-pair recurrence kernels (variant 1) on the same spectra:
element counts that fill one to four 32-element chunks (and ones that are not a
multiple of 4), every window pair, unequal transmit and receive F-numbers,
normalisation combinations, a time offset, and the variant API."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, normalizations, synth, windows
from f_number_gb300._lib import FNumError
from oracle import coracle as CO
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4      # against the FP64 oracle (as the other parity tests)
TOL_VAR = 2e-5     # tensor cores against the recurrence kernels


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def case(n_el, seed, nx=9, nz=8, n_t=360, x_half=None, z=(3e-3, 9e-3)):
    arr = synth.LinearArray(n_el, 0.3e-3, 0.918 * 0.3e-3)
    rng = np.random.default_rng(seed)
    xh = x_half if x_half is not None else min(2e-3, 0.15e-3 * n_el)
    sc = synth.random_points(rng, 6, (-xh, xh), z)
    rf = synth.sa_rf(rng, arr, sc, n_t, 40e6, 1540.0)           # [tx, rx, t]
    rf = rf + 0.05 * np.abs(rf).max() * rng.standard_normal(rf.shape)
    px = np.linspace(-xh, xh, nx)
    pz = np.linspace(z[0], z[1], nz)
    return arr, rf, px, pz


def run_plan(arr, rf, px, pz, variant, t0=0.0, wt=None, wr=None, ftx=None, frx=None, ntx="on", nrx="on",
             semantics="reference", fb=(2e6, 9e6)):
    import torch
    wt = wt or windows.boxcar()
    wr = wr or windows.boxcar()
    fn = f_numbers.directivity.perrot(0.918)
    norms = {"on": normalizations.on(), "off": normalizations.off()}
    plan = das.SAPlan(px, pz, rf.shape[2], arr.n_elements, 40e6, arr.width, arr.pitch, 1540.0, list(fb), t0, wt, wr,
                      ftx or fn, frx or fn, norms[ntx], norms[nrx], device=0, semantics=semantics)
    try:
        plan.set_kernel_variant(variant)
        x = torch.tensor(rf, dtype=torch.float64, device="cuda").contiguous()
        wtx = torch.empty((plan.n_x, plan.n_z), dtype=torch.float32, device="cuda")
        wrx = torch.empty_like(wtx)
        img = plan.execute(x, weights=wtx, weights_rx=wrx)
        torch.cuda.synchronize()
        info = plan.info()
        out = img[0].cpu().numpy().T, wtx.cpu().numpy().T, wrx.cpu().numpy().T, info
    finally:
        plan.close()
    return out


def oracle(arr, rf, px, pz, t0=0.0, wt=None, wr=None, ftx=None, frx=None, ntx="on", nrx="on", semantics="reference",
           fb=(2e6, 9e6)):
    wt = wt or windows.boxcar()
    wr = wr or windows.boxcar()
    fn = f_numbers.directivity.perrot(0.918)
    data = np.transpose(rf, (2, 1, 0))
    ref, rwt, rwr, _ = O.das_sa_mex(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, fb, t0, wt.spec(), wr.spec(),
                                    (ftx or fn).spec(), (frx or fn).spec(), ntx, nrx, semantics=semantics)
    return ref, rwt, rwr


@pytest.mark.parametrize("n_el", [8, 30, 45, 64, 97])
def test_tc_element_counts(gpu, n_el):
    """One to four 32-element chunks; 30, 45 and 97 are not multiples of 4 (padded planes)."""
    arr, rf, px, pz = case(n_el, seed=n_el)
    img2, wt2, wr2, info = run_plan(arr, rf, px, pz, 2)
    assert info["kernel_variant"] == 2
    img1, _, _, _ = run_plan(arr, rf, px, pz, 1)
    ref, rwt, rwr = oracle(arr, rf, px, pz)
    assert rel_l2(img2, ref) < TOL_L2
    assert rel_l2(img2, img1) < TOL_VAR
    np.testing.assert_allclose(wt2, rwt, rtol=1e-5)
    np.testing.assert_allclose(wr2, rwr, rtol=1e-5)


@pytest.mark.parametrize("wt,wr", [(windows.hann(), windows.hann()), (windows.tukey(0.4), windows.triangular()),
                                   (windows.boxcar(), windows.hann()), (windows.triangular(), windows.boxcar())],
                         ids=["hann-hann", "tukey-tri", "box-hann", "tri-box"])
def test_tc_windows(gpu, wt, wr):
    arr, rf, px, pz = case(40, seed=7)
    img2, _, _, _ = run_plan(arr, rf, px, pz, 2, wt=wt, wr=wr)
    ref, _, _ = oracle(arr, rf, px, pz, wt=wt, wr=wr)
    assert rel_l2(img2, ref) < TOL_L2


@pytest.mark.parametrize("ntx,nrx,semantics", [("on", "off", "reference"), ("on", "off", "intended"),
                                               ("off", "on", "intended"), ("off", "off", "intended")])
def test_tc_normalisations_and_f_numbers(gpu, ntx, nrx, semantics):
    """Unequal transmit and receive F-numbers (the two apertures differ); the
    normalisations that accumulate.  (Reference semantics with tx off keep the
    recurrence kernels: their MEX quirks leave a single bin or a zero image.)"""
    arr, rf, px, pz = case(36, seed=11)
    ftx, frx = f_numbers.grating.angle_lb(60, 1.5), f_numbers.constant(1.2)
    img2, _, _, info = run_plan(arr, rf, px, pz, 2, ftx=ftx, frx=frx, ntx=ntx, nrx=nrx, semantics=semantics)
    ref, _, _ = oracle(arr, rf, px, pz, ftx=ftx, frx=frx, ntx=ntx, nrx=nrx, semantics=semantics)
    assert rel_l2(img2, ref) < TOL_L2


@pytest.mark.parametrize("variant", [1, 2])
def test_time_offset(gpu, variant):
    """index_t0 > 0 adds 2 pi k t0 / N to every pair's phase
    (saft_kernel_phase_shifts.cu:180)."""
    arr, rf, px, pz = case(24, seed=5)
    img, _, _, _ = run_plan(arr, rf, px, pz, variant, t0=17.25)
    ref, _, _ = oracle(arr, rf, px, pz, t0=17.25)
    assert rel_l2(img, ref) < TOL_L2
    ref0, _, _ = oracle(arr, rf, px, pz, t0=0.0)
    assert rel_l2(ref, ref0) > 1e-2   # the offset matters at this size


def test_tc_full_aperture_128(gpu):
    """128 elements, voxels deep enough that every aperture covers the whole array
    (four chunks, N = 256), against the C oracle on sampled voxels."""
    wl = synth.saft_128(seed=2, f_bounds=(2e6, 7e6))
    fn = f_numbers.directivity.perrot(0.918)
    px = np.linspace(-4e-3, 4e-3, 12)
    pz = np.linspace(30e-3, 40e-3, 40)
    arr = wl.array
    img2, wt2, _, info = run_plan(arr, wl.rf, px, pz, 2, fb=wl.f_bounds)
    assert info["kernel_variant"] == 2
    rng = np.random.default_rng(9)
    ix, iz = rng.integers(0, px.size, 20), rng.integers(0, pz.size, 20)
    ref, rwt, _, _ = CO.sa_mex(px, pz, wl.rf, wl.f_s, arr.width, arr.pitch, wl.c, wl.f_bounds, 0.0, ("boxcar", 0.0),
                               ("boxcar", 0.0), fn.spec(), fn.spec(), "on", "on", ix, iz)
    assert rel_l2(img2[iz, ix], ref) < TOL_L2
    np.testing.assert_allclose(wt2[iz, ix], rwt, rtol=1e-5)


def test_variant_api(gpu):
    import torch
    arr, rf, px, pz = case(16, seed=1)
    fn = f_numbers.directivity.perrot(0.918)
    plan = das.SAPlan(px, pz, rf.shape[2], 16, 40e6, arr.width, arr.pitch, 1540.0, [2e6, 9e6], 0.0, windows.boxcar(),
                      windows.boxcar(), fn, fn, normalizations.on(), normalizations.on(), device=0)
    try:
        assert plan.info()["kernel_variant"] == 2          # the default when available
        with pytest.raises(FNumError):
            plan.set_kernel_variant(3)
        x = torch.tensor(rf, dtype=torch.float32, device="cuda").contiguous()
        v, ms = plan.autotune(x)
        assert v in (1, 2) and ms > 0
        assert plan.info()["kernel_variant"] == v
    finally:
        plan.close()
    # more than 128 elements: the tensor-core kernel is not available
    big = synth.LinearArray(132, 0.3e-3, 0.918 * 0.3e-3)
    plan = das.SAPlan(px, pz, 300, 132, 40e6, big.width, big.pitch, 1540.0, [2e6, 9e6], 0.0, windows.boxcar(),
                      windows.boxcar(), fn, fn, normalizations.on(), normalizations.on(), device=0)
    try:
        assert plan.info()["kernel_variant"] == 1
        with pytest.raises(FNumError):
            plan.set_kernel_variant(2)
    finally:
        plan.close()


def test_tc_long_band_tile_ranges(gpu):
    """More than 2048 band bins: the kernel uses each tile's element range for every bin
    (no per-bin table) and must give the same image."""
    arr, rf, px, pz = case(8, seed=21, nx=5, nz=4, n_t=4700)
    img2, _, _, info = run_plan(arr, rf, px, pz, 2, fb=(0.2e6, 19.9e6))
    assert info["kernel_variant"] == 2 and info["n_bins"] > 2048
    img1, _, _, _ = run_plan(arr, rf, px, pz, 1, fb=(0.2e6, 19.9e6))
    ref, _, _ = oracle(arr, rf, px, pz, fb=(0.2e6, 19.9e6))
    assert rel_l2(img2, ref) < TOL_L2
    assert rel_l2(img2, img1) < TOL_VAR
