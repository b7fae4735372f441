"""fnum_das_pw_noalloc -- the plane-wave beamformer for callers that may not
allocate device memory (a real-time acquisition loop that must not block on
the allocator, a host that owns a fixed device pool, a plug-in in a process
whose device memory is someone else's) -- must give the images of the
allocating plan path (fnum_pw_plan_create + fnum_plan_execute) and of the FP64
oracle.  Both are called through the C ABI; the bar is the parity tests' 1e-4
relative L2 and 1e-5 on the weights, on two calls in a row (the static scratch
keeps the first call's contents, so the second call, on a smaller problem of
another shape, checks that everything is reset).

This file is collected last on purpose: if it fails, a run stopped at the
first failure has already run every other test.
"""
import ctypes as C
import math

import numpy as np
import pytest

from f_number_gb300 import _lib, das, f_numbers, synth, windows

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4
TOL_W = 1e-5


def _desc(px, pz, n_samples, n_elements, arr, f_bounds, window, fnum):
    d = _lib.PWDesc()
    d.positions_x, d.n_x = _lib.dptr(px), px.size
    d.positions_z, d.n_z = _lib.dptr(pz), pz.size
    d.n_samples, d.n_elements = n_samples, n_elements
    d.f_s, d.element_width, d.element_pitch, d.c_0 = 20e6, arr.width, arr.pitch, 1540.0
    d.f_bounds = _lib.dptr(f_bounds)
    d.index_t0 = 0.0
    d.window = window.c_struct()
    d.f_number = fnum.c_struct()
    d.normalization = _lib.NORM_ON
    d.device = 0
    return d


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(n_el, nx, nz, n_angles, n_samples, seed):
    arr = synth.LinearArray(n_el, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = np.linspace(-0.08, 0.06, n_angles)
    px = np.ascontiguousarray(np.linspace(-6e-3, 6e-3, nx))
    pz = np.ascontiguousarray(np.linspace(6e-3, 20e-3, nz))
    rng = np.random.default_rng(seed)
    sc = synth.random_points(rng, 6, (-6e-3, 6e-3), (6e-3, 20e-3))
    rf = synth.pw_rf(rng, arr, sc, list(angles), n_samples, 20e6, 1540.0).astype(np.float32)
    return arr, angles, px, pz, rf


def test_no_alloc_matches_plan_path(gpu):
    """Two calls in a row, the second on a smaller problem of another shape (other
    element, angle, sample and voxel counts), so the static scratch holds the
    larger first call's data when the second starts.  Each call is checked
    against the plan path; the second also against the FP64 oracle."""
    import torch
    from oracle import coracle as CO
    L = _lib.lib()
    fb = np.array([2e6, 7e6])
    win, fn = windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5)
    stream = torch.cuda.current_stream()
    for call, (n_el, nx, nz, na, nt, seed) in enumerate(((64, 40, 56, 3, 1024, 3), (48, 24, 30, 5, 768, 4))):
        arr, angles, px, pz, rf_h = _case(n_el, nx, nz, na, nt, seed)
        plan = das.PWPlan(px, pz, nt, n_el, 20e6, angles, arr.width, arr.pitch, 1540.0, fb, 0.0, win, fn,
                          compound=True)
        plan_pa = das.PWPlan(px, pz, nt, n_el, 20e6, angles, arr.width, arr.pitch, 1540.0, fb, 0.0, win, fn,
                             compound=False)
        desc = _desc(px, pz, nt, n_el, arr, fb, win, fn)
        rf = torch.tensor(rf_h, device=gpu)
        ref_w = torch.empty((px.size, pz.size), dtype=torch.float32, device=gpu)
        ref = plan.execute(rf, weights=ref_w, stream=stream)
        img = torch.full((1, px.size, pz.size), float("nan"), dtype=torch.complex64, device=gpu)
        w = torch.full((px.size, pz.size), float("nan"), dtype=torch.float32, device=gpu)
        st = L.fnum_das_pw_noalloc(C.byref(desc), _lib.dptr(angles), angles.size, rf.data_ptr(), _lib.FLAG_COMPOUND,
                                   img.data_ptr(), w.data_ptr(), stream.cuda_stream)
        assert st == _lib.OK, L.fnum_status_string(st)
        torch.cuda.synchronize()
        a, b = img.cpu().numpy()[0], ref.cpu().numpy()[0]
        assert np.all(np.isfinite(a))
        assert _rel_l2(a, b) < TOL_L2, (call, _rel_l2(a, b))
        np.testing.assert_allclose(w.cpu().numpy(), ref_w.cpu().numpy(), rtol=TOL_W)
        if call == 1:
            ix, iz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
            o, _, _ = CO.pw_mex(px, pz, rf_h.astype(np.float64), 20e6, angles, arr.width, arr.pitch, 1540.0,
                                tuple(fb), 0.0, win.spec(), fn.spec(), "on", ix.ravel(), iz.ravel())
            assert _rel_l2(a.ravel(), o) < TOL_L2, _rel_l2(a.ravel(), o)
        # one image per angle
        stack = torch.empty((angles.size, px.size, pz.size), dtype=torch.complex64, device=gpu)
        st = L.fnum_das_pw_noalloc(C.byref(desc), _lib.dptr(angles), angles.size, rf.data_ptr(), 0,
                                   stack.data_ptr(), None, stream.cuda_stream)
        assert st == _lib.OK
        ref_stack = plan_pa.execute(rf, stream=stream)
        torch.cuda.synchronize()
        assert _rel_l2(stack.cpu().numpy(), ref_stack.cpu().numpy()) < TOL_L2
        plan.close()
        plan_pa.close()


def test_no_alloc_checks_arguments_like_the_gateway(gpu):
    """Invalid inputs get the plane-wave gateway's status codes, before any work."""
    import torch
    L = _lib.lib()
    arr, angles, px, pz, rf_h = _case(32, 8, 8, 3, 512, 5)
    fb = np.array([2e6, 7e6])
    rf = torch.tensor(rf_h, device=gpu)
    img = torch.zeros((1, px.size, pz.size), dtype=torch.complex64, device=gpu)
    s = torch.cuda.current_stream().cuda_stream

    def run(desc, ang=angles):
        return L.fnum_das_pw_noalloc(C.byref(desc), _lib.dptr(ang) if ang is not None else None,
                                     0 if ang is None else ang.size, rf.data_ptr(), _lib.FLAG_COMPOUND,
                                     img.data_ptr(), None, s)

    bad_x = px.copy()
    bad_x[3] = np.nan
    d = _desc(bad_x, pz, 512, 32, arr, fb, windows.hann(), f_numbers.constant(1.0))
    assert run(d) == 3                                   # FNUM_ERR_LATERAL_POSITIONS
    bad_z = pz.copy()
    bad_z[0] = np.inf
    assert run(_desc(px, bad_z, 512, 32, arr, fb, windows.hann(), f_numbers.constant(1.0))) == 4
    d = _desc(px, pz, 512, 32, arr, fb, windows.hann(), f_numbers.constant(1.0))
    assert run(d, None) == 7                             # FNUM_ERR_STEERING_ANGLE
    d.f_s = float("inf")
    assert run(d) == 6                                   # FNUM_ERR_SAMPLING_RATE
    torch.cuda.synchronize()


def test_no_alloc_rejects_oversized(gpu):
    """Spectra alone (192 elements x 1246 bins x 40 angles x 8 B = 77 MB) exceed
    the 64 MiB scratch: the call must refuse before touching the device."""
    import torch
    L = _lib.lib()
    arr = synth.LinearArray(192, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = np.linspace(-0.3, 0.3, 40)
    px = np.ascontiguousarray(np.linspace(-5e-3, 5e-3, 8))
    pz = np.ascontiguousarray(np.linspace(5e-3, 10e-3, 8))
    desc = _desc(px, pz, 2048, arr.n_elements, arr, None, windows.boxcar(), f_numbers.constant(1.0))
    rf = torch.zeros((angles.size, arr.n_elements, 2048), dtype=torch.float32, device=gpu)
    img = torch.zeros((1, px.size, pz.size), dtype=torch.complex64, device=gpu)
    st = L.fnum_das_pw_noalloc(C.byref(desc), _lib.dptr(angles), angles.size, rf.data_ptr(), _lib.FLAG_COMPOUND,
                               img.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_NOALLOC_TOO_LARGE
    assert L.fnum_status_id(st, 0) == b"gpu_bf_das_pw_rf:NoAllocScratchTooSmall"
    assert math.isfinite(float(img.abs().sum()))
