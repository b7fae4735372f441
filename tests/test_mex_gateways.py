"""The MEX gateways (f_number_gb300/mex) compile against the C ABI and the
MEX C API declarations (tests/mexshim/mex.h); MATLAB itself is not present."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", ["gpu_bf_das_pw_rf.cpp", "gpu_bf_saft_rf.cpp"])
def test_gateway_compiles(name):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "tests", "mexshim"), os.path.join(ROOT, "f_number_gb300", "mex", name)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
