"""The C ABI library loads, exports every symbol include/fnum.h declares, and
its host-only parts (band, F-number classes, windows, status identifiers,
argument validation) agree with the oracle -- no GPU needed."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import fnum_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fnum.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fnum_[a-z0-9_]+)\s*\(", src)))


def test_exports_match_header(built_lib):
    from f_number_gb300 import _lib
    names = declared_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fnum_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names
    for n in names:
        getattr(built_lib, n)


def test_band_matches_oracle(built_lib):
    from f_number_gb300 import band
    rng = np.random.default_rng(0)
    for _ in range(40):
        ne = int(rng.integers(8, 200))
        nt = int(rng.integers(64, 5000))
        pitch = rng.uniform(0.1e-3, 0.5e-3)
        pz = np.sort(rng.uniform(1e-3, 60e-3, 3))
        fs = float(rng.choice([20e6, 31.25e6, 40e6]))
        fb = (rng.uniform(0.5e6, 3e6), rng.uniform(5e6, fs / 2))
        b = O.band_mex(pz, nt, ne, fs, 0.9 * pitch, pitch, 1540.0, fb, 0)
        assert band(pz, nt, ne, fs, 0.9 * pitch, pitch, 1540.0, fb) == (b.N_dft, b.k_lb, b.k_ub)


def test_f_number_classes_match_oracle(built_lib):
    from f_number_gb300 import f_numbers as F
    p = np.linspace(0.05, 6.0, 301)
    objs = [F.constant(0.0), F.constant(1.7), F.grating.angle_lb(60, 1.5), F.grating.angle_lb(70, 1.5, 10),
            F.grating.angle_lb(45, 3.0, 5), F.distance.constant(10), F.distance.constant(5, 2.5), F.distance.none(),
            F.directivity.perrot(0.918), F.directivity.rigid(0.5), F.directivity.soft(0.7, 6.0),
            F.directivity.szabo(0.918)]
    for o in objs:
        a = o.compute_values(p)
        b = O.f_number_values(o.spec(), p)
        np.testing.assert_array_equal(a, b, err_msg=o.string())


def test_f_number_strings():
    from f_number_gb300 import f_numbers as F
    assert F.grating.angle_lb(60, 1.5).string() == "angle_lb_deg_60.00_F_ub_1.50_distance_deg_10.00"
    assert F.constant(1.2).string() == "constant_1.20"
    assert F.directivity.perrot(0.918).string() == "directivity_soft_fill_91.80_att_3.0_dB"


def test_window_values_match_oracle(built_lib):
    from f_number_gb300 import _lib
    for name, par, wid in (("boxcar", 0.0, 0), ("hann", 0.0, 1), ("tukey", 0.3, 2), ("triangular", 0.0, 4)):
        for l in np.linspace(-2.5, 2.5, 41):
            v = built_lib.fnum_window_value(_lib.Window(wid, par), l, 2.0)
            assert abs(v - float(O.window_mex((name, par), l, 2.0))) < 1e-15


def test_status_identifiers(built_lib):
    assert built_lib.fnum_status_id(12, 0) == b"gpu_bf_das_pw_rf:InvalidFrequencyBounds"
    assert built_lib.fnum_status_id(22, 1) == b"gpu_bf_saft_rf:InvalidTXFNumber"
    assert built_lib.fnum_status_id(19, 0) == b"gpu_bf_error_handling:CUDAError"
    assert built_lib.fnum_status_string(14).startswith(b"Unknown window")


def test_das_pw_argument_errors():
    """das_pw.m:85-290 identifiers, raised before any device call."""
    from f_number_gb300 import FNumError, das_pw, windows
    ok = dict(positions_x=np.linspace(-1e-3, 1e-3, 4), positions_z=np.linspace(5e-3, 6e-3, 3),
              data_RF=np.zeros((64, 8)), f_s=20e6, steering_angle=0.0, element_width=2e-4, element_pitch=3e-4,
              c_0=1540.0)

    def expect(ident, **kw):
        args = dict(ok)
        args.update(kw)
        with pytest.raises(FNumError) as e:
            das_pw(**args)
        assert e.value.identifier == ident

    expect("das_pw:NoFiniteXCoordinates", positions_x=np.array([0.0, np.nan]))
    expect("das_pw:NoPositiveAndFiniteZCoordinates", positions_z=np.array([0.0, 1e-3]))
    expect("das_pw:NoSamples", data_RF=np.zeros((1, 8)))
    expect("das_pw:NoFiniteRFData", data_RF=np.full((64, 8), np.inf))
    expect("das_pw:InvalidSamplingRate", f_s=-1.0)
    expect("das_pw:InvalidSteeringAngle", steering_angle=math.pi / 2)
    expect("das_pw:InvalidElementWidth", element_width=0.0)
    expect("das_pw:InvalidElementPitch", element_pitch=1e-4)
    expect("das_pw:InvalidSpeedOfSound", c_0=0.0)
    expect("das_pw:InvalidFrequencyBounds", f_bounds=[3e6, 2e6])
    expect("das_pw:InvalidTimeIndex", index_t0=1.5)
    expect("das_pw:NoWindow", window="hann")
    expect("das_pw:NoFNumber", F_number=1.5)
    expect("das_pw:NoNormalization", normalization="on")
    from f_number_gb300 import platforms
    import torch
    if not torch.cuda.is_available():
        # platforms.cpu runs das_pw.m's semantics on the GPU: without one, the device check fails
        expect("gpu_bf_das_pw_rf:NoCUDADevices", platform=platforms.cpu())
    with pytest.raises(FNumError) as e:
        windows.tukey(1.0)
    assert e.value.identifier == "tukey:InvalidFractionCosine"


def test_no_device_is_reported(built_lib):
    """Without a GPU the gateway answers NoCUDADevices (gpu_bf_das_pw_rf.cu:117-121)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from f_number_gb300 import FNumError, gpu_bf_das_pw_rf
    with pytest.raises(FNumError) as e:
        gpu_bf_das_pw_rf(np.zeros(3), np.array([1e-3, 2e-3]), np.zeros((64, 8)), 20e6, 0.0, 2e-4, 3e-4, 1540.0)
    assert e.value.identifier == "gpu_bf_das_pw_rf:NoCUDADevices"


def test_variant_and_peak_entry_points_check_arguments(built_lib):
    """fnum_plan_set_kernel_variant and fnum_diag_mma_f16_peak refuse null arguments
    before touching a device."""
    from f_number_gb300 import _lib
    L = _lib.lib()
    assert L.fnum_plan_set_kernel_variant(None, 1) == _lib.ERR_ARGUMENT
    assert L.fnum_diag_mma_f16_peak(0, None) == _lib.ERR_ARGUMENT
    assert L.fnum_diag_fp32_peak(0, None) == _lib.ERR_ARGUMENT
