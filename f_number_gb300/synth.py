"""Seeded synthetic RF data for the beamformer workloads.

The reference's example data (a CIRS040 phantom recording, ``data_RF.mat``)
is not distributed with the project, so every workload here runs on point
scatterers synthesised from a seed.  Each scatterer of amplitude A at
two-way delay tau contributes A g(t - tau), where g is a Gaussian-modulated
cosine with centre frequency f_c and fractional bandwidth bw (-6 dB):
g(t) = exp(-alpha t^2) cos(2 pi f_c t), alpha = (pi f_c bw)^2 / (4 ln 2), so
the spectrum falls to half amplitude at f_c (1 +- bw/2).

Delays follow the beamformer's own propagation model: for a steered plane
wave (``das_pw.m:323-336``, ``+cuda/gpu_bf_das_pw_rf.cu:513-519``)
tau = (e_x (x_s - x_ref) + e_z z_s + |r_e - r_s|) / c; for a synthetic
aperture (``das_sa.m``) tau = (|r_tx - r_s| + |r_rx - r_s|) / c.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def pulse_alpha(f_c: float, bw: float) -> float:
    return (math.pi * f_c * bw) ** 2 / (4.0 * math.log(2.0))


@dataclass
class LinearArray:
    n_elements: int
    pitch: float
    width: float

    @property
    def centers(self) -> np.ndarray:
        M = (self.n_elements - 1) / 2.0
        return self.pitch * (np.arange(self.n_elements) - M)


@dataclass
class Scatterers:
    x: np.ndarray
    z: np.ndarray
    amp: np.ndarray


def random_points(rng, n, x_range, z_range, amp=1.0):
    x = rng.uniform(x_range[0], x_range[1], n)
    z = rng.uniform(z_range[0], z_range[1], n)
    a = np.full(n, float(amp))
    return Scatterers(x, z, a)


def speckle_with_cyst(rng, n, x_range, z_range, cyst_center, cyst_radius):
    """n scatterers with N(0,1) amplitudes, none inside the circular cyst."""
    xs, zs = [], []
    need = n
    while need > 0:
        x = rng.uniform(x_range[0], x_range[1], 2 * need)
        z = rng.uniform(z_range[0], z_range[1], 2 * need)
        keep = (x - cyst_center[0]) ** 2 + (z - cyst_center[1]) ** 2 > cyst_radius ** 2
        xs.append(x[keep][:need])
        zs.append(z[keep][:need])
        need -= int(min(keep.sum(), need))
    x = np.concatenate(xs)[:n]
    z = np.concatenate(zs)[:n]
    return Scatterers(x, z, rng.standard_normal(n))


def merge(*parts: Scatterers) -> Scatterers:
    return Scatterers(np.concatenate([p.x for p in parts]), np.concatenate([p.z for p in parts]),
                      np.concatenate([p.amp for p in parts]))


def _render(delays: np.ndarray, amps: np.ndarray, n_samples: int, f_s: float, f_c: float,
            bw: float, half_width: int) -> np.ndarray:
    """Sum of pulses: delays [L, S] (s), amps [S] -> rf [L, n_samples]."""
    alpha = pulse_alpha(f_c, bw)
    L, S = delays.shape
    rf = np.zeros((L, n_samples))
    n0 = np.floor(delays * f_s).astype(np.int64)                   # [L, S]
    offs = np.arange(-half_width, half_width + 1)                 # [W]
    idx = n0[..., None] + offs                                     # [L, S, W]
    t = idx / f_s - delays[..., None]
    val = amps[None, :, None] * np.exp(-alpha * t * t) * np.cos(2.0 * math.pi * f_c * t)
    ok = (idx >= 0) & (idx < n_samples)
    rows = np.broadcast_to(np.arange(L)[:, None, None], idx.shape)
    np.add.at(rf, (rows[ok], idx[ok]), val[ok])
    return rf


def _half_width(f_s, f_c, bw):
    alpha = pulse_alpha(f_c, bw)
    return int(math.ceil(math.sqrt(18.0 / alpha) * f_s)) + 1       # exp(-18) ~ 1.5e-8


def add_noise(rng, rf: np.ndarray, snr_db: float) -> np.ndarray:
    p = float(np.mean(rf * rf))
    if p <= 0.0 or not np.isfinite(snr_db):
        return rf
    sigma = math.sqrt(p / (10.0 ** (snr_db / 10.0)))
    return rf + sigma * rng.standard_normal(rf.shape)


def pw_rf(rng, array: LinearArray, scat: Scatterers, angles, n_samples, f_s, c, f_c=5e6, bw=0.6,
          snr_db=30.0, chunk=16):
    """Plane-wave RF, float64 [n_angles, n_elements, n_samples] (element-major:
    the memory order of MATLAB's data_RF(t, e))."""
    ctr = array.centers
    M = (array.n_elements - 1) / 2.0
    hw = _half_width(f_s, f_c, bw)
    out = np.zeros((len(angles), array.n_elements, n_samples))
    for ia, th in enumerate(angles):
        e_x, e_z = -math.sin(th), math.cos(th)
        x_ref = -M * array.pitch if e_x >= 0 else M * array.pitch
        t_in = (e_x * (scat.x - x_ref) + e_z * scat.z) / c          # [S]
        for e0 in range(0, array.n_elements, chunk):
            ce = ctr[e0:e0 + chunk]
            t_sc = np.sqrt((ce[:, None] - scat.x[None, :]) ** 2 + scat.z[None, :] ** 2) / c
            out[ia, e0:e0 + chunk] = _render(t_in[None, :] + t_sc, scat.amp, n_samples, f_s, f_c, bw, hw)
        out[ia] = add_noise(rng, out[ia], snr_db)
    return out


def sa_rf(rng, array: LinearArray, scat: Scatterers, n_samples, f_s, c, f_c=5e6, bw=0.6, snr_db=20.0):
    """Full synthetic-aperture RF, float64 [n_tx, n_rx, n_samples] (the memory
    order of MATLAB's data_RF(t, rx, tx))."""
    ctr = array.centers
    hw = _half_width(f_s, f_c, bw)
    dist = np.sqrt((ctr[:, None] - scat.x[None, :]) ** 2 + scat.z[None, :] ** 2) / c   # [E, S]
    N = array.n_elements
    out = np.zeros((N, N, n_samples))
    for t in range(N):
        out[t] = _render(dist[t][None, :] + dist, scat.amp, n_samples, f_s, f_c, bw, hw)
    return add_noise(rng, out, snr_db)


# ---------------------------------------------------------------------------
# named workloads (sizes and distributions of the benchmark configurations)
# ---------------------------------------------------------------------------


@dataclass
class PWWorkload:
    name: str
    array: LinearArray
    f_s: float
    c: float
    n_samples: int
    angles: np.ndarray
    positions_x: np.ndarray
    positions_z: np.ndarray
    f_bounds: tuple
    window: tuple
    f_number: dict
    rf: np.ndarray = field(repr=False, default=None)       # [A, E, T] float64


def pw_single_angle(seed=0, grid=(256, 256), n_samples=2048, with_rf=True) -> PWWorkload:
    """Single 0 deg plane wave, 128 elements, pitch 0.3048 mm, 20 scatterers
    (x in [-15, 15] mm, z in [5, 45] mm), 30 dB SNR, 2.25-6.75 MHz, Tukey(0.5),
    grating F-number angle_lb(60, 1.5), image grid over the same region."""
    rng = np.random.default_rng(seed)
    pitch = 0.3048e-3
    arr = LinearArray(128, pitch, 0.918 * pitch)
    nx, nz = grid
    wl = PWWorkload("pw_0deg_128el_%dx%d" % (nx, nz), arr, 20e6, 1540.0, n_samples, np.array([0.0]),
                    np.linspace(-15e-3, 15e-3, nx), np.linspace(5e-3, 45e-3, nz), (2.25e6, 6.75e6),
                    ("tukey", 0.5),
                    {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0})
    if with_rf:
        sc = random_points(rng, 20, (-15e-3, 15e-3), (5e-3, 45e-3))
        wl.rf = pw_rf(rng, arr, sc, wl.angles, n_samples, wl.f_s, wl.c, snr_db=30.0)
    return wl


def cpwc_11_angles(seed=0, grid=(512, 512), n_samples=2048, with_rf=True) -> PWWorkload:
    """Coherent plane-wave compounding: 11 angles -10..10 deg in 2 deg steps,
    100 points plus 2000 N(0,1) speckle scatterers around a 10 mm anechoic cyst
    centred at (0, 20) mm, grid x = (-255.5..255.5) 0.06 mm, z = 5 mm + (0..511)
    0.06 mm, 2-7 MHz, Hann window, angle_lb(60, 1.5) F-number."""
    rng = np.random.default_rng(seed)
    pitch = 0.3048e-3
    arr = LinearArray(128, pitch, 0.918 * pitch)
    nx, nz = grid
    dx = 0.06e-3
    px = (np.arange(nx) - (nx - 1) / 2.0) * dx
    pz = 5e-3 + np.arange(nz) * dx
    wl = PWWorkload("cpwc_11ang_128el_%dx%d" % (nx, nz), arr, 20e6, 1540.0, n_samples,
                    np.deg2rad(np.arange(-10, 11, 2, dtype=np.float64)), px, pz, (2e6, 7e6), ("hann", 0.0),
                    {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0})
    if with_rf:
        xr = (-15e-3, 15e-3)
        zr = (5e-3, 45e-3)
        pts = random_points(rng, 100, xr, zr)
        spk = speckle_with_cyst(rng, 2000, xr, zr, (0.0, 20e-3), 5e-3)
        wl.rf = pw_rf(rng, arr, merge(pts, spk), wl.angles, n_samples, wl.f_s, wl.c, snr_db=30.0)
    return wl


@dataclass
class SAWorkload:
    name: str
    array: LinearArray
    f_s: float
    c: float
    n_samples: int
    positions_x: np.ndarray
    positions_z: np.ndarray
    f_bounds: tuple
    window: tuple
    f_number: dict
    rf: np.ndarray = field(repr=False, default=None)       # [T, R, S]


def saft_128(seed=0, grid=(400, 400), n_samples=3072, n_elements=128, f_bounds=None,
             with_rf=True) -> SAWorkload:
    """Full synthetic aperture: 128 single-element transmits x 128 receives,
    pitch 0.3 mm, 40 MHz, 3072 samples, 50 points, 20 dB SNR, grid over
    x in [-19, 19] mm, z in [3, 40] mm, directivity F-number perrot(0.918),
    boxcar windows.  f_bounds None = the MEX default band [DBL_MIN, f_s/2]."""
    rng = np.random.default_rng(seed)
    pitch = 0.3e-3
    arr = LinearArray(n_elements, pitch, 0.918 * pitch)
    nx, nz = grid
    wl = SAWorkload("saft_%dx%d_%dx%d" % (n_elements, n_elements, nx, nz), arr, 40e6, 1540.0, n_samples,
                    np.linspace(-19e-3, 19e-3, nx), np.linspace(3e-3, 40e-3, nz), f_bounds, ("boxcar", 0.0),
                    {"kind": "directivity", "width_over_pitch": 0.918, "obliquity": "soft",
                     "attenuation_dB": 3.0})
    if with_rf:
        sc = random_points(rng, 50, (-19e-3, 19e-3), (3e-3, 40e-3))
        wl.rf = sa_rf(rng, arr, sc, n_samples, wl.f_s, wl.c, snr_db=20.0)
    return wl


def batch_64(seed=0, n_frames=64, with_rf=True, n_points=60, n_speckle=240):
    """Plane-wave frames of uneven shape: per frame, elements from {64, 96, 128,
    192}, angles from {1, 5, 11, 31} (0 deg, or evenly spaced over -10..10 deg),
    samples from {1024, 2048, 4096}, a square grid of 128 .. 768 voxels per side
    at pitch / 5 spacing starting 5 mm deep, 2-7 MHz, Hann window, angle_lb(60,
    1.5).  RF from the seeded point + speckle model with a smaller scatterer
    count than the single-frame workloads (60 points + 240 speckle scatterers),
    so that 64 frames synthesise in seconds; the beamformer's cost does not
    depend on the RF content."""
    rng = np.random.default_rng(seed)
    frames = []
    for f in range(n_frames):
        ne = int(rng.choice([64, 96, 128, 192]))
        na = int(rng.choice([1, 5, 11, 31]))
        nt = int(rng.choice([1024, 2048, 4096]))
        side = int(rng.integers(128, 769))
        pitch = 0.3048e-3
        arr = LinearArray(ne, pitch, 0.918 * pitch)
        dx = pitch / 5.0
        px = (np.arange(side) - (side - 1) / 2.0) * dx
        pz = 5e-3 + np.arange(side) * dx
        angles = np.zeros(1) if na == 1 else np.deg2rad(np.linspace(-10.0, 10.0, na))
        wl = PWWorkload("batch_%02d_%del_%dang_%dsmp_%dx%d" % (f, ne, na, nt, side, side), arr, 20e6, 1540.0, nt,
                        angles, px, pz, (2e6, 7e6), ("hann", 0.0),
                        {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0})
        if with_rf:
            half = 0.5 * ne * pitch
            xr = (-half, half)
            zr = (5e-3, min(5e-3 + nt / 20e6 * 1540.0 / 2.0, 5e-3 + side * dx))
            pts = random_points(rng, n_points, xr, zr)
            spk = random_points(rng, n_speckle, xr, zr)
            spk.amp = rng.standard_normal(n_speckle)
            wl.rf = pw_rf(rng, arr, merge(pts, spk), wl.angles, nt, wl.f_s, wl.c, snr_db=30.0)
        frames.append(wl)
    return frames
