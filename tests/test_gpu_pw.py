"""Plane-wave parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances: the fused FP32 + double-float-phase kernel must stay within
1e-4 relative L2 of the complex image and 1e-3 dB of the B-mode image
(voxels above -40 dB); weights (apodization sums) within 1e-5 relative.
The plain FP32 kernel uses the reference's per-term arithmetic (__sincosf on
arguments up to ~2.6e3 rad) and is held to 2e-3.
"""
import math

import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, normalizations, synth, windows
from oracle import coracle as CO
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4
TOL_DB = 1e-3
TOL_W = 1e-5
TOL_PLAIN = 2e-3


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def bmode_err(a, b, floor_db=-40.0):
    ref = 20 * np.log10(np.abs(b) / np.abs(b).max())
    got = 20 * np.log10(np.abs(a) / np.abs(b).max())
    m = ref > floor_db
    return float(np.max(np.abs(got[m] - ref[m])))


def small_case(seed=0, n_el=48, n_t=768, angles=(0.0,), n_scat=6):
    arr = synth.LinearArray(n_el, 0.3048e-3, 0.918 * 0.3048e-3)
    rng = np.random.default_rng(seed)
    sc = synth.random_points(rng, n_scat, (-4e-3, 4e-3), (7e-3, 16e-3))
    rf = synth.pw_rf(rng, arr, sc, list(angles), n_t, 20e6, 1540.0, snr_db=30.0)
    px = np.linspace(-4e-3, 4e-3, 14)
    pz = np.linspace(7e-3, 16e-3, 12)
    return arr, rf, px, pz


WINDOWS = [windows.boxcar(), windows.hann(), windows.tukey(0.5), windows.triangular()]
FNUMS = [f_numbers.grating.angle_lb(60, 1.5), f_numbers.constant(1.5), f_numbers.constant(0.0),
         f_numbers.directivity.perrot(0.918), f_numbers.distance.none()]


@pytest.mark.parametrize("win", WINDOWS, ids=lambda w: w.string())
@pytest.mark.parametrize("fn", FNUMS, ids=lambda f: f.string())
def test_fused_matches_oracle(gpu, win, fn):
    arr, rf, px, pz = small_case()
    for norm in (normalizations.on(), normalizations.off()):
        img, w = das.gpu_bf_das_pw_rf(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0,
                                      win, fn, norm, 0)
        ref, wref, info = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                                       win.spec(), fn.spec(), norm.string())
        assert rel_l2(img, ref) < TOL_L2, (norm.string(), rel_l2(img, ref))
        assert bmode_err(img, ref) < TOL_DB
        np.testing.assert_allclose(w, wref, rtol=TOL_W, atol=TOL_W * np.abs(wref).max())


def test_steered_and_time_shift(gpu):
    arr, rf, px, pz = small_case(seed=4, angles=(0.2,))
    for t0 in (0.0, 7.0):
        img, _ = das.gpu_bf_das_pw_rf(px, pz, rf[0].T, 20e6, 0.2, arr.width, arr.pitch, 1540.0, [2.5e6, 6.5e6], t0,
                                      windows.hann(), f_numbers.grating.angle_lb(70, 1.5, 10))
        ref, _, _ = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.2, arr.width, arr.pitch, 1540.0, (2.5e6, 6.5e6), t0,
                                 ("hann", 0.0), {"kind": "grating.angle_lb", "angle_lb_deg": 70.0,
                                                 "F_number_ub": 1.5, "distance_deg": 10.0}, "on")
        assert rel_l2(img, ref) < TOL_L2


def test_mex_defaults(gpu):
    """boxcar window, angle_lb(70, 1.5, 10), normalisation on, full band [DBL_MIN, f_s/2]."""
    arr, rf, px, pz = small_case(seed=7, n_el=32, n_t=400)
    img, w = das.gpu_bf_das_pw_rf(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0)
    ref, wref, info = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0)
    assert info["k_lb"] == 1
    assert rel_l2(img, ref) < TOL_L2
    np.testing.assert_allclose(w, wref, rtol=TOL_W)


def test_compound_and_per_angle(gpu):
    angles = (-0.1, -0.03, 0.04, 0.12)
    arr, rf, px, pz = small_case(seed=2, angles=angles)
    data = np.transpose(rf, (2, 1, 0))                        # [T, E, A]
    win, fn = windows.hann(), f_numbers.grating.angle_lb(60, 1.5)
    refs = [O.das_pw_mex(px, pz, rf[a].T, 20e6, angles[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                         win.spec(), fn.spec(), "on")[0] for a in range(len(angles))]
    comp, _ = das.gpu_bf_das_pw_rf(px, pz, data, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win, fn)
    assert rel_l2(comp, sum(refs)) < TOL_L2
    stack, _ = das.gpu_bf_das_pw_rf(px, pz, data, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win,
                                    fn, compound=False)
    for a in range(len(angles)):
        assert rel_l2(stack[a], refs[a]) < TOL_L2


def test_plain_kernel(gpu):
    angles = (0.0, 0.08)
    arr, rf, px, pz = small_case(seed=3, angles=angles)
    data = np.transpose(rf, (2, 1, 0))
    win, fn = windows.tukey(0.5), f_numbers.grating.angle_lb(60, 1.5)
    ref = sum(O.das_pw_mex(px, pz, rf[a].T, 20e6, angles[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                           win.spec(), fn.spec(), "on")[0] for a in range(2))
    img, w = das.gpu_bf_das_pw_rf(px, pz, data, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win, fn,
                                  kernel="plain")
    fused, wf = das.gpu_bf_das_pw_rf(px, pz, data, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win,
                                     fn)
    assert rel_l2(img, ref) < TOL_PLAIN
    assert rel_l2(fused, ref) < TOL_L2
    np.testing.assert_allclose(w, wf, rtol=1e-5)


def test_edge_cases(gpu):
    arr, rf, px, pz = small_case(seed=9, n_el=32)
    win, fn = windows.hann(), f_numbers.grating.angle_lb(60, 1.5)
    # voxels beside the array: empty apertures at high bins (the MEX returns NaN there)
    pxo = np.linspace(-12e-3, 12e-3, 9)
    img, w = das.gpu_bf_das_pw_rf(pxo, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win, fn)
    ref, wref, info = O.das_pw_mex(pxo, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                                   win.spec(), fn.spec(), "on")
    assert info["zero_weight_bins"] > 0
    assert np.all(np.isfinite(img))
    assert rel_l2(img, ref) < TOL_L2
    np.testing.assert_allclose(w, wref, rtol=TOL_W, atol=1e-6)
    # voxels exactly on element centres, and a single axial position
    centres = arr.centers[10:16]
    for pzz in (pz, pz[:1]):
        img, _ = das.gpu_bf_das_pw_rf(centres, pzz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0,
                                      win, fn)
        ref, _, _ = O.das_pw_mex(centres, pzz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                                 win.spec(), fn.spec(), "on")
        assert rel_l2(img, ref) < TOL_L2


class _Wavy(f_numbers.f_number):
    """A user F-number without a native implementation and with a
    non-monotone table: exercises the general (deactivating) segment path."""

    def compute_values(self, p):
        p = np.asarray(p, dtype=np.float64)
        return 1.0 + 0.8 * np.sin(9.0 * p)

    def spec(self):
        raise NotImplementedError

    def string(self):
        return "wavy"


def test_non_monotone_f_number(gpu):
    arr, rf, px, pz = small_case(seed=11, n_el=40)
    fn = _Wavy()
    img, w = das.gpu_bf_das_pw_rf(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0,
                                  windows.tukey(0.3), fn)
    b = O.band_mex(pz, rf.shape[2], 40, 20e6, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0)
    F = fn.compute_values(O.pitch_over_lambda(b, arr.pitch, 20e6, 1540.0))
    ref, wref, _ = O.das_pw_mex(px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                                ("tukey", 0.3), F, "on")
    assert rel_l2(img, ref) < TOL_L2
    np.testing.assert_allclose(w, wref, rtol=TOL_W)


def test_device_plan_matches_host_api(gpu):
    import torch
    angles = (-0.05, 0.05)
    arr, rf, px, pz = small_case(seed=5, angles=angles)
    win, fn = windows.hann(), f_numbers.grating.angle_lb(60, 1.5)
    plan = das.PWPlan(px, pz, rf.shape[2], arr.n_elements, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6],
                      0.0, win, fn)
    for dt in (torch.float64, torch.float32):
        x = torch.tensor(rf, dtype=dt, device=gpu)
        w = torch.empty(px.size, pz.size, device=gpu)
        out = plan.execute(x, weights=w)
        torch.cuda.synchronize()
        img = out[0].cpu().numpy().T
        ref = sum(O.das_pw_mex(px, pz, rf[a].T, 20e6, angles[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                               win.spec(), fn.spec(), "on")[0] for a in range(2))
        assert rel_l2(img, ref) < TOL_L2
    info = plan.info()
    assert info["active_terms"] > 0 and info["active_terms"] <= info["terms"]
    assert info["f_monotone"] == 1
    np.testing.assert_allclose(plan.f_numbers(), O.f_number_values(
        fn.spec(), O.pitch_over_lambda(O.band_mex(pz, rf.shape[2], arr.n_elements, 20e6, arr.width, arr.pitch,
                                                  1540.0, (2e6, 7e6), 0), arr.pitch, 20e6, 1540.0)))
    plan.close()


def test_abi_error_identifiers(gpu):
    from f_number_gb300 import FNumError
    arr, rf, px, pz = small_case(n_el=16, n_t=256)
    base = (px, pz, rf[0].T, 20e6, 0.0, arr.width, arr.pitch, 1540.0)

    def ident(*extra, **kw):
        with pytest.raises(FNumError) as e:
            das.gpu_bf_das_pw_rf(*base, *extra, **kw)
        return e.value.identifier

    assert ident([9.9999e6, 1.0e7]) == "gpu_bf_das_pw_rf:InvalidFrequencyBounds"
    assert ident([3e6, 2e6]) == "gpu_bf_das_pw_rf:InvalidFrequencyBound"
    assert ident([2e6, 7e6], -1.0) == "gpu_bf_das_pw_rf:InvalidTimeShift"
    # distance.constant(80) is infinite above p/lambda = 1/sin(80 deg) (constant.m:118)
    assert ident([2e6, 7e6], 0, None, f_numbers.distance.constant(80)) == "gpu_bf_das_pw_rf:InvalidFNumber"
    assert ident([2e6, 7e6], 0, None, None, None, 99) == "gpu_bf_das_pw_rf:InvalidCUDADevice"


# --- full-size workloads at sampled voxels (checked by the C oracle) ------------------
def _sample(nx, nz, n, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, nx, n), rng.integers(0, nz, n)


def test_cpwc_full_size_sampled(gpu):
    """11 angles, 128 elements, 2048 samples, 512 x 512 grid, Hann, angle_lb(60, 1.5)."""
    wl = synth.cpwc_11_angles(seed=0)
    win = windows.hann()
    fn = f_numbers.grating.angle_lb(60, 1.5)
    data = np.asfortranarray(np.transpose(wl.rf, (2, 1, 0)))
    img, _ = das.gpu_bf_das_pw_rf(wl.positions_x, wl.positions_z, data, wl.f_s, wl.angles, wl.array.width,
                                  wl.array.pitch, wl.c, list(wl.f_bounds), 0, win, fn)
    ix, iz = _sample(512, 512, 96, 1)
    ref, _, info = CO.pw_mex(wl.positions_x, wl.positions_z, wl.rf, wl.f_s, wl.angles, wl.array.width,
                             wl.array.pitch, wl.c, wl.f_bounds, 0.0, win.spec(), fn.spec(), "on", ix, iz)
    got = img[iz, ix]
    assert rel_l2(got, ref) < TOL_L2
    ph = np.angle(got / ref)
    strong = np.abs(ref) > 0.1 * np.abs(ref).max()
    assert np.max(np.abs(ph[strong])) < 1e-3


def test_single_angle_full_size_sampled(gpu):
    """0 deg, 128 elements, 2048 samples, 256 x 256 grid, Tukey(0.5), 2.25-6.75 MHz."""
    wl = synth.pw_single_angle(seed=0)
    win = windows.tukey(0.5)
    fn = f_numbers.grating.angle_lb(60, 1.5)
    img, w = das.gpu_bf_das_pw_rf(wl.positions_x, wl.positions_z, wl.rf[0].T, wl.f_s, 0.0, wl.array.width,
                                  wl.array.pitch, wl.c, list(wl.f_bounds), 0, win, fn)
    ix, iz = _sample(256, 256, 96, 2)
    ref, wref, _ = CO.pw_mex(wl.positions_x, wl.positions_z, wl.rf, wl.f_s, [0.0], wl.array.width, wl.array.pitch,
                             wl.c, wl.f_bounds, 0.0, win.spec(), fn.spec(), "on", ix, iz)
    assert rel_l2(img[iz, ix], ref) < TOL_L2
    np.testing.assert_allclose(w[iz, ix], wref, rtol=TOL_W)


def test_host_plan_cache_keys_on_values(gpu):
    """The host-buffer gateway keeps its plans by argument values: equal geometry
    in fresh arrays (as MATLAB passes temporaries) reuses the plan; alternating
    between two geometries keeps both."""
    import ctypes as C
    from f_number_gb300 import _lib
    L = _lib.lib()

    def created():
        n = C.c_longlong(0)
        L.fnum_host_cache_info(0, C.byref(n), None)
        return n.value

    arr = synth.LinearArray(32, 0.3048e-3, 0.918 * 0.3048e-3)
    rng = np.random.default_rng(11)
    sc = synth.random_points(rng, 3, (-2e-3, 2e-3), (6e-3, 10e-3))
    rf = synth.pw_rf(rng, arr, sc, [0.0], 400, 20e6, 1540.0)[0].T
    win, fn = windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5)

    def call(nx):
        px = np.linspace(-2e-3, 2e-3, nx)            # a fresh array on every call
        pz = np.linspace(6e-3, 10e-3, 9)
        return das.gpu_bf_das_pw_rf(px, pz, rf.copy(), 20e6, 0.0, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0, win,
                                    fn, normalizations.on(), 0)

    first = call(7)[0]
    n0 = created()
    again = call(7)[0]
    assert created() == n0                      # same values, new arrays: no new plan
    np.testing.assert_array_equal(first, again)
    call(8)
    n1 = created()
    assert n1 == n0 + 1
    call(7)
    call(8)
    assert created() == n1                      # both geometries stay cached
