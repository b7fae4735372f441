"""Generates tests/golden/ref_pw.npz and tests/golden/ref_sa.npz: outputs of the
reference's own CUDA kernels (f_number +cuda/*.cu, compiled from source into
oracle/_ref and driven with the MEX host sequence by oracle/refkernels.py) on
small seeded cases.  These golden vectors pin the FP64 oracle and the GB300
library to the reference implementation.

Run on a machine with a GPU after `python -c "import __graft_entry__ as g;
g.build()"` (the fatbin is compiled where the reference sources are mounted):
    python tests/golden/make_ref_golden.py [outdir]
RF is stored as float32: the reference converts RF to float32 before its DFT
(+cuda/gpu_bf_das_pw_rf.cu:787-793), so no information the reference sees is lost.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from f_number_gb300 import synth  # noqa: E402
from oracle import refkernels as R  # noqa: E402

ANGLE60 = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
PERROT = {"kind": "directivity", "width_over_pitch": 0.918, "obliquity": "soft", "attenuation_dB": 3.0}

PW_CASES = [
    dict(name="hann_anglelb60_on", angle=0.1, window=("hann", 0.0), F=ANGLE60, norm="on", f_bounds=(2e6, 7e6),
         t0=0.0, px=(-3e-3, 3e-3)),
    dict(name="tukey_perrot_off", angle=-0.05, window=("tukey", 0.5), F=PERROT, norm="off", f_bounds=(2e6, 7e6),
         t0=0.0, px=(-3e-3, 3e-3)),
    dict(name="boxcar_constantF_on", angle=0.0, window=("boxcar", 0.0), F={"kind": "constant", "value": 1.2},
         norm="on", f_bounds=(2.5e6, 6.5e6), t0=0.0, px=(-3e-3, 3e-3)),
    dict(name="triangular_none_on", angle=0.05, window=("triangular", 0.0), F={"kind": "distance.none"},
         norm="on", f_bounds=(2e6, 7e6), t0=2.0, px=(-3e-3, 3e-3)),
    dict(name="mex_defaults_fullband", angle=-0.15, window=("boxcar", 0.0), F=None, norm="on", f_bounds=None,
         t0=3.0, px=(-3e-3, 3e-3)),
    dict(name="beside_array_hann", angle=0.0, window=("hann", 0.0), F=ANGLE60, norm="on", f_bounds=(2e6, 7e6),
         t0=0.0, px=(-9e-3, 9e-3)),
]

SA_CASES = [
    dict(name="box_hann_perrot_on_on", wt=("boxcar", 0.0), wr=("hann", 0.0), Ft=PERROT, Fr=PERROT, nt="on", nr="on"),
    dict(name="tukey_box_angle_on_off", wt=("tukey", 0.4), wr=("boxcar", 0.0), Ft=ANGLE60, Fr=PERROT, nt="on",
         nr="off"),
    dict(name="box_box_perrot_off_on", wt=("boxcar", 0.0), wr=("boxcar", 0.0), Ft=PERROT, Fr=PERROT, nt="off",
         nr="on"),
    dict(name="box_box_perrot_off_off", wt=("boxcar", 0.0), wr=("boxcar", 0.0), Ft=PERROT, Fr=PERROT, nt="off",
         nr="off"),
    dict(name="constant_both_on_on", wt=("boxcar", 0.0), wr=("boxcar", 0.0), Ft={"kind": "constant", "value": 1.0},
         Fr={"kind": "constant", "value": 1.0}, nt="on", nr="on"),
]


def make_pw():
    arr = synth.LinearArray(24, 0.3048e-3, 0.918 * 0.3048e-3)
    out, meta = {}, []
    for i, c in enumerate(PW_CASES):
        rng = np.random.default_rng(100 + i)
        sc = synth.random_points(rng, 4, (-3e-3, 3e-3), (6e-3, 10e-3))
        rf = synth.pw_rf(rng, arr, sc, [c["angle"]], 384, 20e6, 1540.0, snr_db=30.0)[0].astype(np.float32)
        px = np.linspace(c["px"][0], c["px"][1], 10)
        pz = np.linspace(6e-3, 10e-3, 8)
        img, w, _ = R.das_pw(px, pz, rf.T.astype(np.float64), 20e6, c["angle"], arr.width, arr.pitch, 1540.0,
                             c["f_bounds"], c["t0"], c["window"], c["F"], c["norm"])
        out["%d_rf" % i] = rf
        out["%d_px" % i] = px
        out["%d_pz" % i] = pz
        out["%d_image" % i] = img
        out["%d_weights" % i] = w
        meta.append({k: (list(v) if isinstance(v, tuple) else v) for k, v in c.items()})
    return out, {"array": {"n_elements": 24, "pitch": arr.pitch, "width": arr.width}, "f_s": 20e6, "c": 1540.0,
                 "cases": meta}


def make_sa():
    arr = synth.LinearArray(8, 0.3e-3, 0.918 * 0.3e-3)
    out, meta = {}, []
    for i, c in enumerate(SA_CASES):
        rng = np.random.default_rng(200 + i)
        sc = synth.random_points(rng, 3, (-1e-3, 1e-3), (3e-3, 5e-3))
        rf = synth.sa_rf(rng, arr, sc, 320, 40e6, 1540.0).astype(np.float32)      # [tx, rx, t], 320 samples cover 2 x 5 mm
        px = np.linspace(-1e-3, 1e-3, 5)
        pz = np.linspace(3e-3, 5e-3, 4)
        data = np.transpose(rf, (2, 1, 0)).astype(np.float64)
        img, wt, wr, _ = R.das_sa(px, pz, data, 40e6, arr.width, arr.pitch, 1540.0, (2e6, 9e6), 0.0, c["wt"],
                                  c["wr"], c["Ft"], c["Fr"], c["nt"], c["nr"])
        out["%d_rf" % i] = rf
        out["%d_px" % i] = px
        out["%d_pz" % i] = pz
        out["%d_image" % i] = img
        out["%d_wtx" % i] = wt
        out["%d_wrx" % i] = wr
        meta.append({k: (list(v) if isinstance(v, tuple) else v) for k, v in c.items()})
    return out, {"array": {"n_elements": 8, "pitch": arr.pitch, "width": arr.width}, "f_s": 40e6, "c": 1540.0,
                 "f_bounds": [2e6, 9e6], "cases": meta}


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name, fn in (("ref_pw", make_pw), ("ref_sa", make_sa)):
        arrays, meta = fn()
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **arrays)
        with open(os.path.join(outdir, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1)
        print("wrote", name, len(meta["cases"]), "cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
