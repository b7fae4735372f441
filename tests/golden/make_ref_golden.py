"""Generates tests/golden/ref_pw.npz, ref_pw_multi.npz and ref_sa.npz: outputs of the
reference's own CUDA kernels (f_number +cuda/*.cu, compiled from source into
oracle/_ref and driven with the MEX host sequence by oracle/refkernels.py) on
small seeded cases.  These golden vectors pin the FP64 oracle and the GB300
library to the reference implementation.

Run on a machine with a GPU after `python -c "import __graft_entry__ as g;
g.build()"` (the fatbin is compiled where the reference sources are mounted):
    python tests/golden/make_ref_golden.py [outdir] [--only ref_pw,ref_pw_multi,ref_sa]
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

# Compounded plane waves: the reference's gateway beamforms one angle per call
# (das_pw.m:298, +cuda/gpu_bf_das_pw_rf.cu:110); the golden image of a case is
# the sum of its per-angle reference images, as a CPWC user would form it.
# Three or more angles and 64 elements reach the library's tensor-core kernel.
PW_MULTI_CASES = [
    dict(name="cpwc5_hann_anglelb60_on", angles_deg=(-8.0, -4.0, 0.0, 4.0, 8.0), window=("hann", 0.0), F=ANGLE60,
         norm="on", f_bounds=(2e6, 7e6), t0=0.0),
    dict(name="cpwc7_tukey_perrot_on", angles_deg=(-9.0, -6.0, -3.0, 0.0, 3.0, 6.0, 9.0), window=("tukey", 0.5),
         F=PERROT, norm="on", f_bounds=(2.25e6, 6.75e6), t0=0.0),
    dict(name="cpwc5_boxcar_constantF_off", angles_deg=(-10.0, -5.0, 0.0, 5.0, 10.0), window=("boxcar", 0.0),
         F={"kind": "constant", "value": 1.5}, norm="off", f_bounds=(2e6, 7e6), t0=0.0),
    dict(name="cpwc6_triangular_distconst_on", angles_deg=(-7.5, -4.5, -1.5, 1.5, 4.5, 7.5),
         window=("triangular", 0.0), F={"kind": "distance.constant", "distance_deg": 10.0, "F_number_ub": 3.0},
         norm="on", f_bounds=(2e6, 7e6), t0=1.0),
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


def make_pw_multi():
    arr = synth.LinearArray(64, 0.3048e-3, 0.918 * 0.3048e-3)
    n_t = 640                                     # covers the two-way path to 16 mm depth at 10 deg
    px = np.linspace(-4e-3, 4e-3, 32)
    pz = np.linspace(8e-3, 16e-3, 32)
    out, meta = {}, []
    for i, c in enumerate(PW_MULTI_CASES):
        rng = np.random.default_rng(300 + i)
        angles = np.deg2rad(np.array(c["angles_deg"]))
        sc = synth.merge(synth.random_points(rng, 6, (-4e-3, 4e-3), (9e-3, 15e-3)),
                         synth.random_points(rng, 40, (-4e-3, 4e-3), (9e-3, 15e-3), amp=0.2))
        rf = synth.pw_rf(rng, arr, sc, list(angles), n_t, 20e6, 1540.0, snr_db=30.0).astype(np.float32)  # [A, E, T]
        img = np.zeros((pz.size, px.size), np.complex128)
        wts = None
        for a in range(angles.size):
            ia, w, _ = R.das_pw(px, pz, rf[a].T.astype(np.float64), 20e6, float(angles[a]), arr.width, arr.pitch,
                                1540.0, c["f_bounds"], c["t0"], c["window"], c["F"], c["norm"])
            img += ia
            wts = w if wts is None else wts
        out["%d_rf" % i] = rf
        out["%d_angles" % i] = angles
        out["%d_image" % i] = img.astype(np.complex64)
        out["%d_weights" % i] = wts
        meta.append({k: (list(v) if isinstance(v, tuple) else v) for k, v in c.items()})
    return out, {"array": {"n_elements": 64, "pitch": arr.pitch, "width": arr.width}, "f_s": 20e6, "c": 1540.0,
                 "n_samples": n_t, "positions_x": px.tolist(), "positions_z": pz.tolist(), "cases": meta}


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


def main(outdir, only=None):
    os.makedirs(outdir, exist_ok=True)
    for name, fn in (("ref_pw", make_pw), ("ref_pw_multi", make_pw_multi), ("ref_sa", make_sa)):
        if only and name not in only:
            continue
        arrays, meta = fn()
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **arrays)
        with open(os.path.join(outdir, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1)
        print("wrote", name, len(meta["cases"]), "cases")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only")]
    only = [a.split("=", 1)[1].split(",") for a in sys.argv[1:] if a.startswith("--only=")]
    main(args[0] if args else os.path.dirname(os.path.abspath(__file__)), only[0] if only else None)
