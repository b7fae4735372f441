"""Benchmark: coherent plane-wave compounding frames/s on the GB300.

Workload (default): 11 plane waves (-10..10 deg, 2 deg steps), 128 elements,
pitch 0.3048 mm, 2048 samples at 20 MHz, 512 x 512 voxels at 0.06 mm,
2-7 MHz band (622 bins), Hann window, angle_lb(60, 1.5) F-number, RF from
the seeded point + speckle + cyst model (synthetic: the reference's phantom
recording is not distributed).  One step = one compounded frame: band DFT of
the 11 x 128 RF lines and the fused beamformer, inputs resident in HBM.

Prints one JSON line.  ``--impl reference`` times the reference's CPU path
(das_pw.m, restated in C with OpenMP under oracle/) on the host cores instead;
on the 11-angle frame it times a bounded random sample of voxels and says so in
its ``extrapolated`` field.  ``--workload pw1`` (single 0 deg plane wave,
256 x 256, Tukey(0.5), 2.25-6.75 MHz) is small enough for both arms to time
complete frames; the headline line carries that comparison as ``cfg1_anchor``.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CPWC frames/s (11 angles, 512x512, 128 el)"
PW1_METRIC = "PW frames/s (1 angle, 256x256, 128 el)"
UNIT = "frames/s"
L2_FLUSH_BYTES = 512 << 20          # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kernel", default="fused", choices=["fused", "plain"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--grid", type=int, default=512, help="voxels per side (512 = the benchmark grid; smaller "
                    "sizes keep the same 0.06 mm spacing, for profiling)")
    ap.add_argument("--workload", default="cpwc", choices=["cpwc", "pw1", "saft", "batch", "adjoint"],
                    help="cpwc (default, the headline); pw1: single 0 deg plane wave, 256 x 256, whole frames "
                    "on both arms; saft: 128 x 128 synthetic aperture, 3072 samples at "
                    "40 MHz, 400 x 400 voxels, directivity F-number, boxcar windows; batch: 64 plane-wave frames "
                    "of uneven shape in one CUDA graph; adjoint: sharpness-loss gradients (dL/dc, dL/dX*) of the cpwc "
                    "geometry with RF simulated at 1500 m/s")
    ap.add_argument("--frames", type=int, default=64, help="batch: frames per batch")
    ap.add_argument("--no-autotune", action="store_true", help="batch: keep each plan's default kernel variant")
    ap.add_argument("--variant", type=int, default=0,
                    help="cpwc / saft: pin the kernel variant (fnum_plan_set_kernel_variant; 0 = the default; "
                    "saft: 1 recurrence kernels, 2 tensor cores)")
    ap.add_argument("--no-accuracy", action="store_true", help="saft: skip the error against the FP64 oracle")
    ap.add_argument("--band", default="full", choices=["full", "2-7"],
                    help="saft band: the gateway default [DBL_MIN, f_s/2] or 2-7 MHz")
    return ap.parse_args()


def workload(grid=512):
    from f_number_gb300 import f_numbers, synth, windows
    wl = synth.cpwc_11_angles(seed=0, grid=(grid, grid))
    return wl, windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5)


def workload_pw1(grid=256):
    from f_number_gb300 import f_numbers, synth, windows
    wl = synth.pw_single_angle(seed=0, grid=(grid, grid))
    return wl, windows.tukey(0.5), f_numbers.grating.angle_lb(60.0, 1.5)


def config_of(wl, kernel):
    g = "%dx%d" % (wl.positions_x.size, wl.positions_z.size)
    if wl.angles.size == 1:
        return {"workload": "pw_1angle_128el_2048smp_%s_2.25-6.75MHz_tukey0.5_anglelb60" % g,
                "n_angles": 1, "n_elements": wl.array.n_elements, "n_samples": wl.n_samples,
                "grid": [int(wl.positions_x.size), int(wl.positions_z.size)], "band_hz": list(wl.f_bounds),
                "kernel": kernel, "l2": "flushed between timed steps (512 MB write)", "data": "synthetic seeded RF"}
    return {"workload": "cpwc_11angles_128el_2048smp_%s_2-7MHz_hann_anglelb60" % g,
            "n_angles": int(wl.angles.size), "n_elements": wl.array.n_elements, "n_samples": wl.n_samples,
            "grid": [int(wl.positions_x.size), int(wl.positions_z.size)], "band_hz": list(wl.f_bounds),
            "kernel": kernel, "l2": "flushed between timed steps (512 MB write)", "data": "synthetic seeded RF"}


# ---------------------------------------------------------------------------
# CPU baseline: das_pw.m restated in C (oracle), bounded sample of voxels
# ---------------------------------------------------------------------------
def cpu_das_pw_m(wl, win, fn, seconds, threads=0):
    """das_pw.m CPU semantics on a bounded random sample of the frame's voxels,
    scaled to the frame (the per-voxel cost is nearly uniform).  Returns
    (frames/s, cpu_baseline dict with an ``extrapolated`` record)."""
    from oracle import coracle as CO
    nx, nz = wl.positions_x.size, wl.positions_z.size
    rng = np.random.default_rng(123)
    n_vox = nx * nz
    th = threads or CO.max_threads()

    def run(n):
        ix = rng.integers(0, nx, n)
        iz = rng.integers(0, nz, n)
        t = time.perf_counter()
        CO.pw_m(wl.positions_x, wl.positions_z, wl.rf, wl.f_s, wl.angles, wl.array.width, wl.array.pitch, wl.c,
                wl.f_bounds, 0.0, win.spec(), fn.spec(), "on", ix, iz, threads=th)
        return time.perf_counter() - t

    n = 2 * th
    t = run(n)
    while t < 0.5:
        n *= 4
        t = run(n)
    n = max(th, int(n * seconds / max(t, 1e-3)))
    t = run(n)
    fps = n / (t * n_vox)
    return fps, {"value": fps, "unit": UNIT, "cores": th, "kind": "port",
                 "sample": "das_pw.m CPU semantics (oracle/fnum_oracle.c) on %d random voxels x %d angles "
                           "(%.1f s incl. FFT), scaled to the %d-voxel frame" % (n, wl.angles.size, t, n_vox),
                 "extrapolated": {"voxels": int(n), "of": int(n_vox), "seconds": t}}


def cpu_whole_frame(wl, win, fn, threads=0):
    """das_pw.m CPU semantics over every voxel of the frame (no extrapolation).
    Returns (frames/s, seconds)."""
    from oracle import coracle as CO
    nx, nz = wl.positions_x.size, wl.positions_z.size
    ix, iz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    th = threads or CO.max_threads()
    t = time.perf_counter()
    CO.pw_m(wl.positions_x, wl.positions_z, wl.rf, wl.f_s, wl.angles, wl.array.width, wl.array.pitch, wl.c,
            wl.f_bounds, 0.0, win.spec(), fn.spec(), "on", ix.ravel(), iz.ravel(), threads=th)
    dt = time.perf_counter() - t
    return 1.0 / dt, dt, th


def accuracy_of(wl, win, fn, img, n_random=192, n_bright=64):
    """Error of a compounded frame (img: [n_x, n_z] complex, scaled like the MEX)
    against the FP64 oracle (MEX semantics, oracle/fnum_oracle.c) on a fixed
    sample of voxels: n_random seeded random ones plus the n_bright brightest
    of the frame.  The RF is the float32 RF the GPU beamformed."""
    from oracle import coracle as CO
    nx, nz = img.shape
    rng = np.random.default_rng(7)
    flat = np.abs(img).ravel()
    pick = np.unique(np.concatenate([rng.choice(nx * nz, n_random, replace=False),
                                     np.argsort(flat)[-n_bright:]]))
    ix, iz = pick // nz, pick % nz
    rf32 = np.asarray(wl.rf, dtype=np.float32).astype(np.float64)
    ref, _, _ = CO.pw_mex(wl.positions_x, wl.positions_z, rf32, wl.f_s, wl.angles, wl.array.width, wl.array.pitch,
                          wl.c, wl.f_bounds, 0.0, win.spec(), fn.spec(), "on", ix, iz)
    got = img[ix, iz].astype(np.complex128)
    thr = flat.max() * 10 ** (-40 / 20)
    hi = np.abs(ref) > thr
    dphi = np.abs(np.angle(got[hi] * np.conj(ref[hi])))
    ddb = np.abs(20 * np.log10(np.abs(got[hi]) / np.abs(ref[hi])))
    return {"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "max_phase_err_rad": float(dphi.max()) if dphi.size else None,
            "max_bmode_db_err": float(ddb.max()) if ddb.size else None,
            "voxels": int(pick.size), "voxels_above_-40dB": int(hi.sum()),
            "against": "FP64 oracle (MEX semantics, oracle/fnum_oracle.c) on the float32 RF of the timed frame",
            "sample": "%d seeded random voxels + the %d brightest of the frame" % (n_random, n_bright),
            "bmode": "20 |log10(|I| / |I_ref|)| on voxels above -40 dB of the frame maximum (a common "
                     "normaliser cancels)"}


def measured_peaks():
    """Measured HBM and bf16 peaks of the GPU (MEASURED_PEAKS.json beside this file), or {}."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def saft_accuracy_of(wl, fn, img, n_random=40, n_bright=16):
    """Error of a SAFT frame (img: [n_x, n_z] complex) against the FP64 oracle (MEX
    semantics, oracle/fnum_oracle.c) on seeded random voxels plus the brightest."""
    from oracle import coracle as CO
    nx, nz = img.shape
    rng = np.random.default_rng(7)
    flat = np.abs(img).ravel()
    pick = np.unique(np.concatenate([rng.choice(nx * nz, n_random, replace=False), np.argsort(flat)[-n_bright:]]))
    ix, iz = pick // nz, pick % nz
    rf32 = np.asarray(wl.rf, dtype=np.float32).astype(np.float64)
    ref, _, _, _ = CO.sa_mex(wl.positions_x, wl.positions_z, rf32, wl.f_s, wl.array.width, wl.array.pitch, wl.c,
                             wl.f_bounds, 0.0, ("boxcar", 0.0), ("boxcar", 0.0), fn.spec(), fn.spec(), "on", "on",
                             ix, iz)
    got = img[ix, iz].astype(np.complex128)
    thr = flat.max() * 10 ** (-40 / 20)
    hi = np.abs(ref) > thr
    dphi = np.abs(np.angle(got[hi] * np.conj(ref[hi])))
    return {"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "max_phase_err_rad": float(dphi.max()) if dphi.size else None,
            "voxels": int(pick.size), "voxels_above_-40dB": int(hi.sum()),
            "against": "FP64 oracle (MEX semantics, oracle/fnum_oracle.c) on the float32 RF of the timed frame",
            "sample": "%d seeded random voxels + the %d brightest of the frame" % (n_random, n_bright)}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def pw_kernel_name(variant, window):
    """Name of the plane-wave fused kernel a plan's variant launches."""
    if variant == 9:
        return "pw_tc_kernel<%s> (mma.sync m16n8k16, fp16 hi/lo operands)" % window
    shapes = {1: (1, 11), 2: (2, 4), 3: (2, 2), 4: (4, 1)}
    ept, na = shapes[(variant - 1) % 4 + 1]
    return "%s<%d,%d,%s>" % ("pw_event_kernel" if variant <= 4 else "pw_fused_kernel", ept, na, window)


def traffic_from_profiles(variant=9):
    """DRAM bytes per launch of the launched kernel at the bench workload (ncu capture),
    None for a variant without a capture."""
    name = {9: "pw_tc_cpwc_512.json", 1: "pw_event_cpwc_512.json"}.get(variant)
    if name is None:
        return None
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except (ValueError, OSError):
            return None
    return None


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pw1 = args.workload == "pw1"
    wl, win, fn = workload_pw1(256 if args.grid == 512 else args.grid) if pw1 else workload(args.grid)
    vals = []
    cb = None
    if pw1:
        # complete frames: every voxel of the 256 x 256 frame, each step
        for _ in range(min(args.warmup, 1)):
            cpu_whole_frame(wl, win, fn)
        secs = []
        for _ in range(args.steps):
            fps, dt, th = cpu_whole_frame(wl, win, fn)
            vals.append(fps)
            secs.append(dt)
        value = float(args.steps / sum(secs))
        cb = {"value": value, "unit": UNIT, "cores": th, "kind": "port",
              "sample": "das_pw.m CPU semantics (oracle/fnum_oracle.c), complete %dx%d frames"
                        % (wl.positions_x.size, wl.positions_z.size)}
        ms_per_step = 1e3 * sum(secs) / args.steps
    else:
        for _ in range(args.warmup if args.warmup < 1 else 1):
            cpu_das_pw_m(wl, win, fn, min(2.0, args.cpu_seconds / 4))
        per = max(2.0, args.cpu_seconds / max(args.steps, 1))
        samples = []
        for _ in range(args.steps):
            fps, cb = cpu_das_pw_m(wl, win, fn, per)
            vals.append(fps)
            samples.append(cb["extrapolated"])
        value = float(np.mean(vals))
        cb["value"] = value
        cb["extrapolated"] = {"voxels": int(sum(x["voxels"] for x in samples)), "of": samples[0]["of"],
                              "seconds": float(sum(x["seconds"] for x in samples)), "steps": len(samples),
                              "note": "each step times a random voxel sample and scales it to the frame"}
        ms_per_step = 1e3 / value
    out = {"impl": "reference", "metric": PW1_METRIC if pw1 else METRIC, "value": value, "unit": UNIT,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config_of(wl, "cpu"), "cpu_baseline": cb,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not pw1:
        out["extrapolated"] = cb["extrapolated"]
    print(json.dumps(out))


def replica_throughput(total_ms, steps, dist=None, device=None):
    """Whole-job frames/s of replicas: each of the world's ranks processed `steps`
    frames of its own, and the job took as long as its slowest rank (max over ranks
    of the timed region).  Returns (frames/s, ms per step of the slowest rank)."""
    world = 1
    if dist is not None:
        import torch
        world = dist.get_world_size()
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return steps * world / (total_ms * 1e-3), total_ms / steps


def run_ours(args):
    import torch
    from f_number_gb300 import _lib, das
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pw1 = args.workload == "pw1"
    wl, win, fn = workload_pw1(256 if args.grid == 512 else args.grid) if pw1 else workload(args.grid)
    plan = das.PWPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.angles,
                      wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0.0, win, fn, device=local,
                      compound=True, kernel=args.kernel)
    if args.variant and args.kernel == "fused":
        plan.set_kernel_variant(args.variant)
    rf = torch.tensor(wl.rf, dtype=torch.float32, device=dev)                 # [A, E, T]
    img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=dev)
    wts = torch.empty((plan.n_x, plan.n_z), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        plan.execute_dft(rf, stream)
        plan.execute_beamform(img, wts, stream=stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    for s in range(args.steps):
        flush.zero_()
        e0, e1, e2 = evs[s]
        e0.record(stream)
        plan.execute_dft(rf, stream)
        e1.record(stream)
        plan.execute_beamform(img, wts, stream=stream)
        e2.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(c) for a, b, c in evs]
    dft_ms = [a.elapsed_time(b) for a, b, c in evs]    # operand split + tcgen05 GEMM
    bf_ms = [b.elapsed_time(c) for a, b, c in evs]
    value, ms_per_step = replica_throughput(float(sum(step_ms)), args.steps, dist, dev)
    info = plan.info()

    # end to end through the public API: pinned host RF (double, MATLAB layout) in, host image out
    e2e = None
    if not args.no_e2e:
        A, E, T = wl.rf.shape
        pinned = torch.empty((A, E, T), dtype=torch.float64, pin_memory=True)
        pinned.numpy()[...] = wl.rf
        host_rf = np.transpose(pinned.numpy(), (2, 1, 0))                     # [T, E, A], Fortran order
        call = lambda: das.gpu_bf_das_pw_rf(wl.positions_x, wl.positions_z, host_rf, wl.f_s, wl.angles,
                                           wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0, win, fn,
                                           None, local, kernel=args.kernel)
        for _ in range(2):
            call()
        n = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(n):
            im, _w = call()
        dt = time.perf_counter() - t0
        e2e = {"value": n / dt, "unit": UNIT, "h2d_bytes_per_step": int(A * E * T * 8),
               "d2h_bytes_per_step": int(plan.n_x * plan.n_z * (8 + 4)),
               "api": "f_number_gb300.gpu_bf_das_pw_rf -> fnum_das_pw (host buffers, pinned RF)"}

    peak = _lib.C.c_double(0.0)
    _lib.check(_lib.lib().fnum_diag_fp32_peak(local, _lib.C.byref(peak)))
    bf_avg_ms = float(np.mean(bf_ms))
    if args.kernel == "plain":
        # the plain kernel keeps no counters; the active-term count is a property of
        # the workload, taken from one untimed run of the fused kernel on the same plan
        fplan = das.PWPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.angles,
                           wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0.0, win, fn, device=local,
                           compound=True, kernel="fused")
        fplan.execute_dft(rf, stream)
        fplan.execute_beamform(img, wts, stream=stream)
        torch.cuda.synchronize()
        finfo = fplan.info()
        fplan.close()
        info = dict(info, active_terms=finfo["active_terms"], executed_terms=info["terms"])
    flops = 8.0 * info["active_terms"]
    achieved = flops / (bf_avg_ms * 1e-3) / 1e12
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value if peak.value else None, "traffic": traffic_from_profiles(info["kernel_variant"]) if args.kernel == "fused" else None,
            "kernel": "pw_plain_kernel" if args.kernel == "plain" else pw_kernel_name(info["kernel_variant"], "hann"),
            "work": "8 FLOP per active voxel x element x bin x angle term "
            "(complex MAC); %d active of %d nominal terms" % (info["active_terms"], info["terms"]),
            "executed_terms": info["executed_terms"],
            "peak_source": "measured FP32 FMA throughput (fnum_diag_fp32_peak); MEASURED_PEAKS.json "
            "holds only HBM and bf16 figures"}
    if args.kernel == "fused" and info["kernel_variant"] == 9:
        # the tensor pipe: three m16n8k16 products per 16 voxels x 8 elements x 4 angles
        mpeak = _lib.C.c_double(0.0)
        _lib.check(_lib.lib().fnum_diag_mma_f16_peak(local, _lib.C.byref(mpeak)))
        na_pass = min(12, len(wl.angles))
        mma_flops = info["executed_terms"] / (16.0 * 8.0 * na_pass) * 3 * 3 * 2 * 16 * 8 * 16  # 3 n-tiles
        roof["tensor"] = {"achieved": mma_flops / (bf_avg_ms * 1e-3) / 1e12, "peak": mpeak.value,
                          "unit": "TFLOP/s", "frac": mma_flops / (bf_avg_ms * 1e-3) / 1e12 / mpeak.value,
                          "work": "mma.sync m16n8k16 instructions issued (3 fp16 products per operand tile)",
                          "peak_source": "measured mma.sync m16n8k16 f16/f32 throughput (fnum_diag_mma_f16_peak)"}
    if rank != 0:
        return
    acc = accuracy_of(wl, win, fn, img[0].cpu().numpy())
    cb, anchor = None, None
    if not args.no_cpu:
        if pw1:
            fps_cpu, dt_cpu, th = cpu_whole_frame(wl, win, fn)
            cb = {"value": fps_cpu, "unit": UNIT, "cores": th, "kind": "port",
                  "sample": "das_pw.m CPU semantics (oracle/fnum_oracle.c), one complete %dx%d frame (%.1f s)"
                            % (wl.positions_x.size, wl.positions_z.size, dt_cpu)}
        else:
            _, cb = cpu_das_pw_m(wl, win, fn, args.cpu_seconds)
            anchor = cfg1_anchor(args, local, dev, flush)
    out = {"metric": PW1_METRIC if pw1 else METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (double-float phase)", "data": "synthetic",
           "config": config_of(wl, args.kernel),
           "gterms_per_s": info["terms"] / (ms_per_step * 1e-3) / 1e9,
           "stage_ms": {"band_dft": float(np.mean(dft_ms)), "beamform": bf_avg_ms},
           "e2e": e2e, "roofline": roof, "cpu_baseline": cb, "clocks": clk, "accuracy": acc,
           # per step: the band DFT (operand split + tcgen05 GEMM) and the beamformer, which adds
           # the scale and fragment kernels for variant 9; no library kernels
           "gpu_launches": args.steps * (5 if (args.kernel == "fused" and info["kernel_variant"] == 9) else 3),
           "library_launches": {}}
    if anchor is not None:
        out["cfg1_anchor"] = anchor
    print(json.dumps(out))
    plan.close()
    if dist:
        dist.destroy_process_group()


def cfg1_anchor(args, local, dev, flush, steps=10, warmup=3):
    """The single-angle 256 x 256 frame (pw1) on both arms with complete frames:
    GPU frames/s (device-timed, L2 flushed; and end to end through the gateway)
    against the das_pw.m CPU semantics over every voxel of the frame."""
    import torch
    from f_number_gb300 import das
    wl, win, fn = workload_pw1()
    plan = das.PWPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.angles,
                      wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0.0, win, fn, device=local,
                      compound=True)
    rf = torch.tensor(wl.rf, dtype=torch.float32, device=dev)
    img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        plan.execute(rf, out=img, stream=stream)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for a, b in evs:
        flush.zero_()
        a.record(stream)
        plan.execute(rf, out=img, stream=stream)
        b.record(stream)
    torch.cuda.synchronize()
    gpu_fps = steps / (sum(a.elapsed_time(b) for a, b in evs) * 1e-3)
    host_rf = np.ascontiguousarray(wl.rf[0].T)                                 # [T, E]
    call = lambda: das.gpu_bf_das_pw_rf(wl.positions_x, wl.positions_z, host_rf, wl.f_s, 0.0, wl.array.width,
                                       wl.array.pitch, wl.c, list(wl.f_bounds), 0, win, fn, None, local)
    for _ in range(2):
        call()
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    e2e_fps = steps / (time.perf_counter() - t0)
    acc = accuracy_of(wl, win, fn, img[0].cpu().numpy())
    variant = plan.info()["kernel_variant"]
    plan.close()
    cpu_fps, cpu_s, th = cpu_whole_frame(wl, win, fn)
    return {"workload": config_of(wl, "fused")["workload"], "gpu_value": gpu_fps, "gpu_e2e": e2e_fps,
            "cpu_value": cpu_fps, "cpu_seconds_per_frame": cpu_s, "cpu_cores": th, "unit": UNIT,
            "ratio_device": gpu_fps / cpu_fps, "ratio_e2e": e2e_fps / cpu_fps, "kernel_variant": variant,
            "accuracy": acc,
            "note": "both arms time complete frames: the GPU over %d steps, the CPU (das_pw.m semantics in C, "
                    "all host threads) over one frame" % steps}


# ---------------------------------------------------------------------------
# synthetic-aperture workload (reported beside the headline; same contract)
# ---------------------------------------------------------------------------
SA_METRIC = "SAFT frames/s (128 tx x 128 rx, 3072 smp, 400x400)"


def saft_workload(band, grid=400):
    from f_number_gb300 import synth
    return synth.saft_128(seed=0, grid=(grid, grid), f_bounds=None if band == "full" else (2e6, 7e6))


def saft_config(wl, kernel, band):
    g = "%dx%d" % (wl.positions_x.size, wl.positions_z.size)
    return {"workload": "saft_128x128_3072smp_40MHz_%s_%s_boxcar_perrot" % (g, "fullband" if band == "full"
                                                                          else "2-7MHz"),
            "n_elements": wl.array.n_elements, "n_samples": wl.n_samples,
            "grid": [int(wl.positions_x.size), int(wl.positions_z.size)], "kernel": kernel,
            "l2": "inputs larger than L2 (201 MB RF, band spectra up to 261 MB)", "data": "synthetic seeded RF"}


def run_saft(args):
    import torch
    from f_number_gb300 import _lib, das, f_numbers, windows
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = saft_workload(args.band, 400 if args.grid == 512 else args.grid)
    fn = f_numbers.directivity.perrot(0.918)
    plan = das.SAPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.array.width,
                      wl.array.pitch, wl.c, wl.f_bounds, 0.0, windows.boxcar(), windows.boxcar(), fn, fn,
                      device=local, kernel=args.kernel)
    if args.variant:
        plan.set_kernel_variant(args.variant)
    rf = torch.tensor(wl.rf, dtype=torch.float32, device=dev)                 # [tx, rx, t]
    img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.execute_dft(rf, stream)
        plan.execute_beamform(img, stream=stream)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for s in range(args.steps):
        e0, e1, e2 = evs[s]
        e0.record(stream)
        plan.execute_dft(rf, stream)
        e1.record(stream)
        plan.execute_beamform(img, stream=stream)
        e2.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(c) for a, b, c in evs]
    bf_ms = float(np.mean([b.elapsed_time(c) for a, b, c in evs]))
    info = plan.info()
    value = args.steps / (sum(step_ms) * 1e-3)
    peak = _lib.C.c_double(0.0)
    _lib.check(_lib.lib().fnum_diag_fp32_peak(local, _lib.C.byref(peak)))
    active = info["active_terms"] if args.kernel == "fused" else info["terms"]
    achieved = 8.0 * active / (bf_ms * 1e-3) / 1e12
    tc = args.kernel == "fused" and info["kernel_variant"] == 2
    fp32 = {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value if peak.value else None,
            "work": "8 FLOP per active voxel x tx x rx x bin term; %d active of %d nominal terms"
            % (info["active_terms"], info["terms"]),
            "peak_source": "measured FP32 FMA throughput (fnum_diag_fp32_peak)"}
    if tc:
        # tcgen05.mma work: per executed voxel x tx x rx x bin term of a tile's element range,
        # 4 real products (real form) x 3 (fp16 hi.lo, lo.hi, hi.hi) x 2 FLOP
        mflops = 24.0 * info["executed_terms"]
        mpk = measured_peaks().get("bf16_tflops")
        tach = mflops / (bf_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": tach, "peak": mpk, "unit": "TFLOP/s",
                "frac": tach / mpk if mpk else None, "traffic": None, "kernel": "sa_tc_kernel<boxcar,boxcar>",
                "work": "24 FLOP per executed term (real-form complex product, three fp16 products); %d executed "
                        "terms (tile element ranges x bins), %d active" % (info["executed_terms"], info["active_terms"]),
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst; fp16 runs at the bf16 rate)",
                "fp32_equivalent": fp32}
    else:
        roof = dict(fp32, traffic=None,
                    kernel="sa_event_kernel<12,boxcar> (boxcar receive window)" if args.kernel == "fused"
                    else "sa_plain_kernel")
    acc = None
    if rank == 0 and not args.no_accuracy:
        acc = saft_accuracy_of(wl, fn, img[0].cpu().numpy())
    if rank != 0:
        return
    out = {"metric": SA_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 (double-float phase)", "data": "synthetic",
           "config": saft_config(wl, args.kernel, args.band),
           "gterms_per_s": info["terms"] / (np.mean(step_ms) * 1e-3) / 1e9,
           "stage_ms": {"band_dft": float(np.mean([a.elapsed_time(b) for a, b, c in evs])), "beamform": bf_ms},
           "roofline": roof, "accuracy": acc, "kernel_variant": info["kernel_variant"], "clocks": clk,
           # per step: the band DFT (operand split + tcgen05 GEMM), then either the spectra scale,
           # the operand planes and the tensor-core beamformer, or the symmetrisation kernel and
           # the recurrence beamformer (or the plain kernel); no library kernels
           "gpu_launches": args.steps * (5 if tc else 4 if args.kernel == "fused" else 3),
           "library_launches": {}}
    print(json.dumps(out))
    plan.close()


# ---------------------------------------------------------------------------
# batched workload: uneven plane-wave frames in one CUDA graph
# ---------------------------------------------------------------------------
BATCH_METRIC = "batched PW frames/s (uneven shapes, one CUDA graph)"


def run_batch(args):
    import torch
    from f_number_gb300 import das, f_numbers, synth, windows
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    frames = synth.batch_64(seed=0, n_frames=args.frames)
    synth_s = time.perf_counter() - t0
    fn = f_numbers.grating.angle_lb(60.0, 1.5)
    plans, rfs, imgs, variants = [], [], [], []
    for wl in frames:
        p = das.PWPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.angles,
                       wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0.0, windows.hann(), fn, device=0,
                       compound=True)
        rf = torch.tensor(wl.rf, dtype=torch.float32, device=dev)
        variants.append(p.autotune(rf)[0] if not args.no_autotune else p.info()["kernel_variant"])
        plans.append(p)
        rfs.append(rf)
        imgs.append(torch.empty((1, p.n_x, p.n_z), dtype=torch.complex64, device=dev))
    stream = torch.cuda.current_stream()
    # stand-alone latency of each frame (band DFT + beamformer), for p50 / p99
    solo = []
    for p, rf, im in zip(plans, rfs, imgs):
        p.execute(rf, out=im, stream=stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        p.execute(rf, out=im, stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        solo.append(a.elapsed_time(b))
    batch = das.Batch(plans, rfs, imgs, n_streams=4)
    n_persist_launches = batch.persistent()[1]
    for _ in range(args.warmup):
        batch.execute(stream)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for s in range(args.steps):
        batch.execute(stream)
        ev[s + 1].record(stream)
    torch.cuda.synchronize()
    done = batch.frame_times()                      # completion within the last batch
    clk = clocks.stop()
    total_ms = ev[0].elapsed_time(ev[-1])
    n = len(plans)
    terms = sum(p.info()["terms"] for p in plans)
    out = {"metric": BATCH_METRIC, "value": n * args.steps / (total_ms * 1e-3), "unit": UNIT, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 (double-float phase)", "data": "synthetic",
           "config": {"workload": "batch_%d_pw_frames_uneven_seed0" % n, "frames": n,
                      "elements": sorted({p.n_elements for p in plans}), "angles": sorted({p.n_angles for p in plans}),
                      "grid_sides": [min(p.n_x for p in plans), max(p.n_x for p in plans)], "n_streams": 4,
                      "autotune": not args.no_autotune, "kernel_variants": variants,
                      "l2": "a batch reads 1.5+ GB of RF and spectra, larger than L2", "rf_synthesis_s": synth_s},
           "gterms_per_s": terms * args.steps / (total_ms * 1e-3) / 1e9,
           "latency_ms": {"standalone_p50": float(np.percentile(solo, 50)),
                          "standalone_p99": float(np.percentile(solo, 99)),
                          "in_batch_completion_p50": float(np.percentile(done, 50)),
                          "in_batch_completion_p99": float(np.percentile(done, 99)),
                          "sum_of_standalone": float(np.sum(solo))},
           "clocks": clk,
           # per frame: the band DFT (two kernels); a compounded tensor-core frame then its
           # scale and fragment kernels, its tiles beamformed by the persistent launches (one
           # per window and pass width); any other frame per beamform launch the kernel (+
           # scale and fragment kernels for the tensor-core variant)
           "gpu_launches": args.steps * (n_persist_launches + sum(
               2 + (2 if (p.n_out == 1 and v == 9) else (1 if p.n_out == 1 else p.n_angles) * (3 if v == 9 else 1))
               for p, v in zip(plans, variants)))}
    print(json.dumps(out))
    batch.close()
    for p in plans:
        p.close()


# ---------------------------------------------------------------------------
# adjoint workload: sharpness-loss gradients of the CPWC frame
# ---------------------------------------------------------------------------
ADJ_METRIC = "sharpness-gradient evaluations/s (CPWC 11 angles, 512x512: loss, dL/dc, dL/dX*)"


def run_adjoint(args):
    import torch
    from f_number_gb300 import das, synth
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    wl, win, fn = workload(args.grid)
    # echoes simulated at 1500 m/s, beamformed at trial speeds (band, F table, apertures frozen at 1540)
    rng = np.random.default_rng(1)
    xr, zr = (-15e-3, 15e-3), (5e-3, 45e-3)
    sc = synth.merge(synth.random_points(rng, 100, xr, zr), synth.speckle_with_cyst(rng, 2000, xr, zr, (0.0, 20e-3),
                                                                                      5e-3))
    rf = torch.tensor(synth.pw_rf(rng, wl.array, sc, wl.angles, wl.n_samples, wl.f_s, 1500.0, snr_db=30.0),
                      dtype=torch.float32, device=dev)
    plan = das.PWPlan(wl.positions_x, wl.positions_z, wl.n_samples, wl.array.n_elements, wl.f_s, wl.angles,
                      wl.array.width, wl.array.pitch, wl.c, list(wl.f_bounds), 0.0, win, fn, device=0, compound=True)
    sweep = {}
    for c in (1450.0, 1500.0, 1550.0):
        plan.set_sound_speed(c)
        L, dc, _ = plan.sharpness_grad(rf, grad_spectra=False)
        sweep["%g" % c] = {"loss": L, "dL_dc": dc}
    plan.set_sound_speed(1500.0)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.sharpness_grad(rf, stream=stream)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan.sharpness_grad(rf, stream=stream)          # synchronises: loss and dL/dc reach the host
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=dev)
    a.record(stream)
    plan.execute(rf, out=img, stream=stream)
    b.record(stream)
    torch.cuda.synchronize()
    fwd_ms = a.elapsed_time(b)
    # the adjoint alone (fnum_pw_adjoint without dL/dc: pw_adjoint_tc_kernel and its scale and finishing
    # kernels), then with dL/dc (adds the derivative forward pass and its reduction), on the frame's spectra
    cot = torch.randn((plan.n_x, plan.n_z), dtype=torch.complex64, device=dev)

    def timed(fn):
        fn()
        ts = []
        for _ in range(3):
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.mean(ts))

    adj_ms = timed(lambda: plan.adjoint(cot, dc=False, stream=stream))
    adj_dc_ms = timed(lambda: plan.adjoint(cot, dc=True, stream=stream))
    info = plan.info()
    from f_number_gb300 import _lib
    peak = _lib.C.c_double(0.0)
    _lib.check(_lib.lib().fnum_diag_fp32_peak(0, _lib.C.byref(peak)))
    # per active voxel x element x bin x angle term the adjoint forms one complex MAC into dL/dX*
    # (8 FLOP); the tensor cores do it, so the FP32 figure is an FP32-equivalent rate
    adj_tflops = 8.0 * info["active_terms"] / (adj_ms * 1e-3) / 1e12
    roof = {"bound": "fp32", "achieved": adj_tflops, "peak": peak.value, "unit": "TFLOP/s",
            "frac": adj_tflops / peak.value if peak.value else None, "traffic": None,
            "kernel": "pw_adjoint_tc_kernel",
            "work": "8 FLOP per active term (one complex MAC into dL/dX*, FP32-equivalent: the products run on "
                    "the tensor cores); %d active terms" % info["active_terms"],
            "peak_source": "measured FP32 FMA throughput (fnum_diag_fp32_peak)"}
    out = {"metric": ADJ_METRIC, "value": args.steps / dt, "unit": "evaluations/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (double-float phase, FP64 reductions)", "data": "synthetic",
           "config": {"workload": "adjoint_cpwc_11angles_128el_2048smp_%dx%d_rf_at_1500" % (args.grid, args.grid),
                      "trial_c": 1500.0, "frozen_at_c": 1540.0},
           "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "adjoint_with_dc_ms": adj_dc_ms,
           "derivative_forward_ms": adj_dc_ms - adj_ms, "roofline": roof, "sweep": sweep, "clocks": clk}
    print(json.dumps(out))
    plan.close()


def main():
    args = parse()
    import __graft_entry__ as g
    g.build()
    if args.workload == "adjoint":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint"}))
            return
        run_adjoint(args)
        return
    if args.workload == "batch":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batch workload has no CPU arm; the CPU "
                              "baseline of the headline is the cpwc workload"}))
            return
        run_batch(args)
    elif args.workload == "saft":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the saft workload has no CPU arm; the CPU "
                              "baseline of the headline is the cpwc workload"}))
            return
        run_saft(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
