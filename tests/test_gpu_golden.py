"""The GB300 library (through the C ABI) against golden vectors produced by the
reference's own CUDA kernels.  Bars as in test_golden_ref.py: 2e-4 rel-L2
(the reference's own FP32 error is ~4e-5 here), weights 1e-5; where the
reference returns NaN (empty apertures) the library returns finite values."""
import numpy as np
import pytest

from f_number_gb300 import das
from test_golden_ref import PW, PWM, SA, TOL_REF, rel_l2_finite
import specs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("i", range(len(PW[1]["cases"])), ids=[c["name"] for c in PW[1]["cases"]])
@pytest.mark.parametrize("kernel", ["fused", "plain"])
def test_library_matches_reference_pw(gpu, i, kernel):
    d, m = PW
    c, a = m["cases"][i], m["array"]
    rf = d["%d_rf" % i].astype(np.float64)
    ref, wref = d["%d_image" % i], d["%d_weights" % i]
    img, w = das.gpu_bf_das_pw_rf(d["%d_px" % i], d["%d_pz" % i], rf.T, m["f_s"], c["angle"], a["width"], a["pitch"],
                                  m["c"], c["f_bounds"], c["t0"], specs.window(c["window"]), specs.f_number(c["F"]),
                                  specs.normalization(c["norm"]), 0, kernel=kernel)
    assert rel_l2_finite(img, ref) < TOL_REF
    assert np.all(np.isfinite(img))
    np.testing.assert_allclose(w, wref, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("i", range(len(SA[1]["cases"])), ids=[c["name"] for c in SA[1]["cases"]])
def test_library_matches_reference_sa(gpu, i):
    d, m = SA
    c, a = m["cases"][i], m["array"]
    rf = d["%d_rf" % i].astype(np.float64)
    ref = d["%d_image" % i]
    img, wt, wr = das.gpu_bf_saft_rf(d["%d_px" % i], d["%d_pz" % i], np.transpose(rf, (2, 1, 0)), m["f_s"],
                                     a["width"], a["pitch"], m["c"], m["f_bounds"], 0, specs.window(c["wt"]),
                                     specs.window(c["wr"]), specs.f_number(c["Ft"]), specs.f_number(c["Fr"]),
                                     specs.normalization(c["nt"]), specs.normalization(c["nr"]), 0)
    assert np.all(np.isfinite(img))
    if c["Ft"]["kind"] == "constant" and c["Fr"]["kind"] == "constant":
        return                                   # reference: NaN (kernel commented out); here: constant table
    if c["nt"] == "off" and c["nr"] == "on":
        assert np.all(img == 0)
    else:
        assert rel_l2_finite(img, ref) < TOL_REF
    np.testing.assert_allclose(wt, d["%d_wtx" % i], rtol=1e-5)
    np.testing.assert_allclose(wr, d["%d_wrx" % i], rtol=1e-5)


@pytest.mark.parametrize("i", range(len(PWM[1]["cases"])), ids=[c["name"] for c in PWM[1]["cases"]])
def test_default_kernel_matches_reference_compounded(gpu, i):
    """The default plane-wave path for 3+ angles -- the tensor-core kernel,
    variant 9 -- against compounded images of the reference's own kernels (sum of
    its per-angle gateway calls), through a device plan and through the
    host-buffer gateway with all angles in one call."""
    import torch
    d, m = PWM
    c, a = m["cases"][i], m["array"]
    px, pz = np.array(m["positions_x"]), np.array(m["positions_z"])
    rf = d["%d_rf" % i]                                                           # [A, E, T] float32
    angles = d["%d_angles" % i]
    ref, wref = d["%d_image" % i], d["%d_weights" % i]
    plan = das.PWPlan(px, pz, rf.shape[2], rf.shape[1], m["f_s"], angles, a["width"], a["pitch"], m["c"],
                      c["f_bounds"], c["t0"], specs.window(c["window"]), specs.f_number(c["F"]),
                      specs.normalization(c["norm"]), compound=True)
    w = torch.empty((px.size, pz.size), dtype=torch.float32, device=gpu)
    img = plan.execute(torch.tensor(rf, device=gpu), weights=w)[0].cpu().numpy().T
    assert plan.info()["kernel_variant"] == 9
    plan.close()
    assert rel_l2_finite(img, ref) < TOL_REF, rel_l2_finite(img, ref)
    np.testing.assert_allclose(w.cpu().numpy().T, wref, rtol=1e-5, atol=1e-6)
    img2, w2 = das.gpu_bf_das_pw_rf(px, pz, np.transpose(rf, (2, 1, 0)).astype(np.float64), m["f_s"], angles,
                                    a["width"], a["pitch"], m["c"], c["f_bounds"], c["t0"], specs.window(c["window"]),
                                    specs.f_number(c["F"]), specs.normalization(c["norm"]), 0)
    assert rel_l2_finite(img2, ref) < TOL_REF
    np.testing.assert_allclose(w2, wref, rtol=1e-5, atol=1e-6)
