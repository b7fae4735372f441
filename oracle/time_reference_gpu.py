"""Times the reference's own GPU algorithm on the plane-wave bench workload.

ORACLE-SIDE TOOLING: runs the f_number CUDA kernels compiled from source
(oracle/_ref, built by oracle/build.py) through refkernels.py, with the MEX
host sequence of +cuda/gpu_bf_das_pw_rf.cu:
- cuFFT R2C;
- per band bin, das_kernel_phase_shifts writes the voxel x element phase
  matrix, cublasCgemm reduces it against the spectra, and
  das_kernel_normalization divides.

The reference beamforms one steering angle per call (das_pw.m:298), so one
11-angle frame is 11 calls.  The script times `--angles` of them (kernel time
from the harness's CUDA events) and scales to the frame.  It also beamforms
the same angle with this library and prints the relative L2 difference of
the two images.

    python oracle/time_reference_gpu.py [--angles 2] [--grid 512]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--angles", type=int, default=2)
    ap.add_argument("--grid", type=int, default=512)
    args = ap.parse_args()
    from f_number_gb300 import das, f_numbers, synth, windows
    from oracle import refkernels as R
    if not R.available():
        print(json.dumps({"unavailable": "oracle/_ref is not built (needs the f_number sources at build time)"}))
        return
    wl = synth.cpwc_11_angles(seed=0, grid=(args.grid, args.grid))
    F = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}
    idx = [len(wl.angles) // 2 + i for i in range(args.angles)]
    ms, rel = [], []
    for a in idx:
        rf = wl.rf[a].T.astype(np.float64)                                    # [T, E]
        R.das_pw(wl.positions_x, wl.positions_z, rf, wl.f_s, wl.angles[a], wl.array.width, wl.array.pitch, wl.c,
                 tuple(wl.f_bounds), 0.0, ("hann", 0.0), F, "on")                # warm-up (plans, module load)
        img_ref, _, t = R.das_pw(wl.positions_x, wl.positions_z, rf, wl.f_s, wl.angles[a], wl.array.width,
                                 wl.array.pitch, wl.c, tuple(wl.f_bounds), 0.0, ("hann", 0.0), F, "on")
        ms.append(t)
        ours, _ = das.gpu_bf_das_pw_rf(wl.positions_x, wl.positions_z, rf, wl.f_s, wl.angles[a], wl.array.width,
                                       wl.array.pitch, wl.c, list(wl.f_bounds), 0, windows.hann(),
                                       f_numbers.grating.angle_lb(60.0, 1.5), None, 0)
        rel.append(float(np.linalg.norm(ours - img_ref) / np.linalg.norm(ours)))
    per_angle = float(np.mean(ms))
    print(json.dumps({"implementation": "f_number CUDA kernels (phase matrix + cublasCgemm per bin), MEX host "
                      "sequence", "workload": "cpwc_11angles_128el_2048smp_%dx%d_2-7MHz_hann_anglelb60"
                      % (args.grid, args.grid), "angles_timed": len(ms), "ms_per_angle": per_angle,
                      "ms_per_frame_11_angles": 11 * per_angle, "frames_per_s": 1e3 / (11 * per_angle),
                      "rel_l2_reference_vs_this_library": rel}))


if __name__ == "__main__":
    main()
