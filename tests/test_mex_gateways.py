"""The MEX gateways (f_number_gb300/mex) run under a minimal stand-in for the
MATLAB MEX runtime (tests/mexshim): numeric mxArrays with separate imaginary
planes, parameter objects by class name and properties, mexErrMsgIdAndTxt
identifiers, and mexCallMATLAB for isa and a user class's compute_values.
This executes the gateways' argument handling -- the reference's
+cuda/gpu_bf_das_pw_rf.cu:126-485 and +cuda/gpu_bf_saft_rf.cu:124-592 -- and
checks their outputs against the reference kernels' golden vectors (GPU)."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "mexshim"))
import shim  # noqa: E402
from test_golden_ref import PW, SA, TOL_REF, rel_l2_finite  # noqa: E402


@pytest.mark.parametrize("name", ["gpu_bf_das_pw_rf.cpp", "gpu_bf_saft_rf.cpp", "gpu_bf_das_pw_sharpness_grad.cpp"])
def test_gateway_compiles(name):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "tests", "mexshim"), os.path.join(ROOT, "f_number_gb300", "mex", name)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="module")
def gateways(tmp_path_factory, built_lib):
    d = str(tmp_path_factory.mktemp("mex"))
    return {g: shim.Gateway(shim.build(g, d))
            for g in ("gpu_bf_das_pw_rf", "gpu_bf_saft_rf", "gpu_bf_das_pw_sharpness_grad")}


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_gateways_run_and_report_identifiers(gateways):
    """Without a GPU the gateways raise the reference's NoCUDADevices identifier;
    with one, a call with too few inputs raises :nrhs -- either way the gateway
    code ran and its error reached the caller as a MATLAB identifier."""
    g = gateways["gpu_bf_das_pw_rf"]
    with pytest.raises(shim.MexError) as e:
        g.call(1, [g.array(np.zeros(3))])
    assert e.value.identifier == ("gpu_bf_das_pw_rf:nrhs" if _has_gpu() else "gpu_bf_das_pw_rf:NoCUDADevices")
    s = gateways["gpu_bf_saft_rf"]
    with pytest.raises(shim.MexError) as e:
        s.call(1, [s.array(np.zeros(3))])
    assert e.value.identifier == ("gpu_bf_saft_rf:nrhs" if _has_gpu() else "gpu_bf_saft_rf:NoCUDADevices")


def _pw_args(g, i, F=None, rf=None):
    d, m = PW
    c, a = m["cases"][i], m["array"]
    rf = d["%d_rf" % i].astype(np.float64).T if rf is None else rf                     # [T, E]
    args = [g.array(d["%d_px" % i]), g.array(d["%d_pz" % i]), g.array(rf), g.array(m["f_s"]), g.array(c["angle"]),
            g.array(a["width"]), g.array(a["pitch"]), g.array(m["c"]),
            g.array(c["f_bounds"]) if c["f_bounds"] else g.empty(), g.array(c["t0"]), g.window(c["window"]),
            F if F is not None else (g.f_number(c["F"]) if c["F"] else g.empty()), g.normalization(c["norm"]),
            g.array(0.0)]
    return args


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(PW[1]["cases"])), ids=[c["name"] for c in PW[1]["cases"]])
def test_pw_gateway_matches_reference(gateways, gpu, i):
    g = gateways["gpu_bf_das_pw_rf"]
    d = PW[0]
    (img, cls), (w, wcls) = g.call(2, _pw_args(g, i))
    assert cls == shim.MX_SINGLE and wcls == shim.MX_SINGLE
    assert img.shape == d["%d_image" % i].shape and np.iscomplexobj(img)
    assert rel_l2_finite(img, d["%d_image" % i]) < TOL_REF
    np.testing.assert_allclose(w, d["%d_weights" % i], rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_pw_gateway_errors_and_user_f_number(gateways, gpu):
    g = gateways["gpu_bf_das_pw_rf"]
    d, m = PW
    rf = d["0_rf"].astype(np.float64).T
    cases = [
        (lambda a: a[:7], "gpu_bf_das_pw_rf:nrhs"),
        (lambda a: a[:2] + [g.array(rf * (1 + 1j))] + a[3:], "gpu_bf_das_pw_rf:InvalidRFData"),
        (lambda a: a[:10] + [g.obj("windows.gauss", ("windows.window",))] + a[11:], "gpu_bf_das_pw_rf:InvalidWindow"),
        (lambda a: a[:10] + [g.normalization("on")] + a[11:], "gpu_bf_das_pw_rf:InvalidWindow"),
        (lambda a: a[:8] + [g.array([7e6, 2e6])] + a[9:], "gpu_bf_das_pw_rf:InvalidFrequencyBound"),
        (lambda a: a[:13] + [g.array(3.0)], "gpu_bf_das_pw_rf:InvalidCUDADevice"),
    ]
    for edit, ident in cases:
        args = _pw_args(g, 0)
        use = edit(args)
        for h in args:
            if h not in use:
                g.L.shim_free(h)
        with pytest.raises(shim.MexError) as e:
            g.call(2, use)
        assert e.value.identifier == ident, (ident, e.value)
    # a user-defined F-number class: the gateway asks MATLAB for compute_values
    g.on_matlab_call(lambda name, args: np.full(g.read(args[1])[0].size, 1.2) if name == "compute_values" else None)
    user = g.obj("my.fixed_f_number", ("f_numbers.f_number",))
    (img_u, _), = g.call(1, _pw_args(g, 2, F=user))
    assert "compute_values" in g.calls
    (img_c, _), = g.call(1, _pw_args(g, 2))           # case 2 uses f_numbers.constant(1.2)
    np.testing.assert_array_equal(img_u, img_c)


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(SA[1]["cases"])), ids=[c["name"] for c in SA[1]["cases"]])
def test_sa_gateway_matches_reference(gateways, gpu, i):
    g = gateways["gpu_bf_saft_rf"]
    d, m = SA
    c, a = m["cases"][i], m["array"]
    rf = np.transpose(d["%d_rf" % i].astype(np.float64), (2, 1, 0))                    # [T, Rx, Tx]
    args = [g.array(d["%d_px" % i]), g.array(d["%d_pz" % i]), g.array(rf), g.array(m["f_s"]), g.array(a["width"]),
            g.array(a["pitch"]), g.array(m["c"]), g.array(m["f_bounds"]), g.array(0.0), g.window(c["wt"]),
            g.window(c["wr"]), g.f_number(c["Ft"]), g.f_number(c["Fr"]), g.normalization(c["nt"]),
            g.normalization(c["nr"]), g.array(0.0), g.array(0.0)]
    (img, cls), (wt, _), (wr, _) = g.call(3, args)
    assert cls == shim.MX_SINGLE and np.iscomplexobj(img)
    assert np.all(np.isfinite(img))
    if c["Ft"]["kind"] == "constant" and c["Fr"]["kind"] == "constant":
        return                     # reference: NaN image, zero weights (kernel commented out); here: a constant table
    np.testing.assert_allclose(wt, d["%d_wtx" % i], rtol=1e-5)
    np.testing.assert_allclose(wr, d["%d_wrx" % i], rtol=1e-5)
    if c["nt"] == "off" and c["nr"] == "on":
        assert np.all(img == 0)
    else:
        assert rel_l2_finite(img, d["%d_image" % i]) < TOL_REF


@pytest.mark.gpu
def test_sharpness_gradient_gateway(gateways, gpu):
    """MATLAB's route to the gradients (gpu_bf_das_pw_sharpness_grad): loss, dL/dc
    and dL/dX* [N_bins x N_el x N_angles] equal the device plan's
    fnum_pw_sharpness_grad on the same RF."""
    import torch
    from f_number_gb300 import das, f_numbers, synth, windows
    g = gateways["gpu_bf_das_pw_sharpness_grad"]
    rng = np.random.default_rng(9)
    arr = synth.LinearArray(32, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = np.deg2rad([-5.0, 0.0, 5.0])
    px, pz = np.linspace(-3e-3, 3e-3, 18), np.linspace(6e-3, 13e-3, 20)
    sc = synth.random_points(rng, 5, (-3e-3, 3e-3), (6e-3, 13e-3))
    rf = synth.pw_rf(rng, arr, sc, list(angles), 700, 20e6, 1500.0).astype(np.float32).astype(np.float64)
    spec = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
    args = [g.array(px), g.array(pz), g.array(np.transpose(rf, (2, 1, 0))), g.array(20e6), g.array(angles),
            g.array(arr.width), g.array(arr.pitch), g.array(1520.0), g.array([2e6, 7e6]), g.array(0.0),
            g.window(("hann", 0.0)), g.f_number(spec), g.normalization("on"), g.array(0.0)]
    (L, _), (dc, _), (gX, gcls) = g.call(3, args)
    plan = das.PWPlan(px, pz, 700, 32, 20e6, angles, arr.width, arr.pitch, 1520.0, [2e6, 7e6], 0.0, windows.hann(),
                      f_numbers.grating.angle_lb(60.0, 1.5), compound=True)
    Lp, dcp, gp = plan.sharpness_grad(torch.tensor(rf, device=gpu))
    plan.close()
    assert gcls == shim.MX_SINGLE and gX.shape == (gp.shape[1], 32, 3)
    assert abs(float(L.ravel()[0]) - Lp) <= 1e-6 * abs(Lp)
    assert abs(float(dc.ravel()[0]) - dcp) <= 1e-6 * abs(dcp)
    ref = np.transpose(gp.cpu().numpy(), (1, 0, 2))                                   # [K, E, A]
    # the same kernels on the same data; FP64 atomics may reorder the slice sums
    np.testing.assert_allclose(gX, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
