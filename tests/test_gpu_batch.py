"""Batches of uneven frames in one CUDA graph (fnum_batch_*) and the per-plan
kernel autotuner (fnum_plan_autotune).

A frame in a batch runs the same kernels as its plan's stand-alone execute, and
each voxel's arithmetic does not depend on which block or stream processes it,
so batch images must equal the stand-alone images bit for bit.  The autotuner
only regroups elements and angles into passes, which changes the rounding of
the per-group sums: its images stay within 1e-5 relative L2 of the default
variant's, and within the parity bound of the FP64 oracle."""
import numpy as np
import pytest

from f_number_gb300 import _lib, das, f_numbers, synth, windows
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

PITCH = 0.3048e-3
FN = f_numbers.grating.angle_lb(60.0, 1.5)


def _frame(rng, ne, na, nt, side, compound, gpu):
    import torch
    arr = synth.LinearArray(ne, PITCH, 0.918 * PITCH)
    dx = PITCH / 2
    px = (np.arange(side) - (side - 1) / 2.0) * dx
    pz = 6e-3 + np.arange(side) * dx
    angles = np.zeros(1) if na == 1 else np.deg2rad(np.linspace(-8.0, 8.0, na))
    sc = synth.random_points(rng, 6, (px[0], px[-1]), (pz[0], pz[-1]))
    rf = torch.tensor(synth.pw_rf(rng, arr, sc, list(angles), nt, 20e6, 1540.0), dtype=torch.float32, device=gpu)
    plan = das.PWPlan(px, pz, nt, ne, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0, windows.hann(), FN,
                      compound=compound)
    return plan, rf, (arr, px, pz, angles)


SHAPES = [(32, 1, 512, 24, True), (48, 5, 1024, 40, False), (64, 11, 1024, 32, True), (40, 3, 768, 28, True),
          (56, 2, 512, 36, False), (24, 31, 512, 20, True)]


def test_batch_equals_standalone_plans(gpu):
    import torch
    rng = np.random.default_rng(11)
    frames = [_frame(rng, *s, gpu) for s in SHAPES]
    plans = [f[0] for f in frames]
    rfs = [f[1] for f in frames]
    expect, expect_w = [], []
    for p, rf in zip(plans, rfs):
        w = torch.empty((p.n_x, p.n_z), dtype=torch.float32, device=gpu)
        expect.append(p.execute(rf, weights=w).clone())
        expect_w.append(w.clone())
    images = [torch.full_like(e, float("nan")) for e in expect]
    weights = [torch.full_like(w, float("nan")) if i % 2 == 0 else None for i, w in enumerate(expect_w)]
    batch = das.Batch(plans, rfs, images, weights=weights, n_streams=3)
    # the compounded frames with 3+ angles (tensor-core kernel) go to persistent launches,
    # one per pass width: 12-angle passes (11 and 3 angles) and 16-angle passes (31 angles)
    n_tc = sum(1 for p in plans if p.n_out == 1 and p.info()["kernel_variant"] == 9)
    assert n_tc == 3 and batch.persistent() == (n_tc, 2)
    for rep in range(2):                        # the graph is relaunched: same results
        for im in images:
            im.fill_(float("nan"))
        batch.execute()
        torch.cuda.synchronize()
        for i, (im, e) in enumerate(zip(images, expect)):
            assert torch.equal(im, e), (rep, i)
            if weights[i] is not None:
                assert torch.equal(weights[i], expect_w[i])
        t = batch.frame_times()
        assert np.all(np.isfinite(t)) and np.all(t > 0)
    batch.close()
    for p in plans:
        p.close()


def test_batch_rejects_a_plan_twice(gpu):
    import torch
    rng = np.random.default_rng(12)
    plan, rf, _ = _frame(rng, 32, 1, 512, 16, True, gpu)
    im = [torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=gpu) for _ in range(2)]
    with pytest.raises(_lib.FNumError):
        das.Batch([plan, plan], [rf, rf], im)
    plan.close()


@pytest.mark.parametrize("na", [1, 5, 11])
def test_autotune_keeps_results(gpu, na):
    rng = np.random.default_rng(13 + na)
    plan, rf, (arr, px, pz, angles) = _frame(rng, 48, na, 1024, 32, True, gpu)
    ref = plan.execute(rf).cpu().numpy()
    v, ms = plan.autotune(rf)
    assert 1 <= v <= 9 and ms > 0
    assert plan.info()["kernel_variant"] == v
    img = plan.execute(rf).cpu().numpy()
    assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-5
    # against the FP64 oracle (compounded MEX semantics, image [z][x])
    rf_np = rf.cpu().numpy().astype(np.float64)
    o = sum(O.das_pw_mex(px, pz, rf_np[a].T, 20e6, angles[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                         ("hann", 0.0), FN.spec(), "on")[0] for a in range(na))
    got = img[0].T
    assert np.linalg.norm(got - o) / np.linalg.norm(o) < 1e-4
    plan.close()


@pytest.mark.parametrize("win", [windows.boxcar(), windows.hann(), windows.tukey(0.5), windows.triangular()],
                         ids=["boxcar", "hann", "tukey", "triangular"])
def test_boundary_strategies_agree(gpu, win):
    """Variants 1..4 resolve the segment boundaries ahead of the bin loop,
    variants 5..8 inside it, with the same arithmetic: equal images."""
    import torch
    rng = np.random.default_rng(21)
    for ne, na, nt, side in [(48, 11, 1024, 32), (40, 5, 768, 28), (36, 1, 512, 24)]:
        arr = synth.LinearArray(ne, PITCH, 0.918 * PITCH)
        px = (np.arange(side) - (side - 1) / 2.0) * PITCH / 3
        pz = 5e-3 + np.arange(side) * PITCH / 3
        angles = np.zeros(1) if na == 1 else np.deg2rad(np.linspace(-8.0, 8.0, na))
        sc = synth.random_points(rng, 6, (px[0], px[-1]), (pz[0], pz[-1]))
        rf = torch.tensor(synth.pw_rf(rng, arr, sc, list(angles), nt, 20e6, 1540.0), dtype=torch.float32,
                          device=gpu)
        plan = das.PWPlan(px, pz, nt, ne, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0, win, FN)
        for v in range(1, 5):
            plan.set_kernel_variant(v)
            assert plan.info()["kernel_variant"] == v
            a = plan.execute(rf).clone()
            plan.set_kernel_variant(v + 4)
            b = plan.execute(rf)
            assert torch.equal(a, b), (ne, na, v)
        for bad in (-1, 10):
            with pytest.raises(_lib.FNumError):
                plan.set_kernel_variant(bad)
        plan.set_kernel_variant(0)
        plan.close()


@pytest.mark.parametrize("win", [windows.boxcar(), windows.hann(), windows.tukey(0.5), windows.triangular()],
                         ids=["boxcar", "hann", "tukey", "triangular"])
def test_tensor_core_variant(gpu, win):
    """Variant 9 (mma.sync with fp16 hi/lo operands) against variant 1 and the FP64 oracle.
    Passes of 16 angles (4 mma n-tiles) where they take fewer passes than 12: 13, 31 and 49
    angles (1, 2 and 4 passes); 36 angles runs three passes of 12."""
    import torch
    rng = np.random.default_rng(31)
    for ne, na, nt, side in [(48, 11, 1024, 40), (45, 13, 768, 36), (36, 5, 512, 24), (29, 1, 512, 20),
                             (24, 31, 512, 20), (20, 49, 384, 14), (16, 36, 384, 14)]:
        arr = synth.LinearArray(ne, PITCH, 0.918 * PITCH)
        px = (np.arange(side) - (side - 1) / 2.0) * PITCH / 3
        pz = 5e-3 + np.arange(side + 3) * PITCH / 3
        angles = np.zeros(1) if na == 1 else np.deg2rad(np.linspace(-8.0, 8.0, na))
        sc = synth.random_points(rng, 6, (px[0], px[-1]), (pz[0], pz[-1]))
        rf_np = synth.pw_rf(rng, arr, sc, list(angles), nt, 20e6, 1540.0)
        rf = torch.tensor(rf_np, dtype=torch.float32, device=gpu)
        plan = das.PWPlan(px, pz, nt, ne, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0, win, FN)
        plan.set_kernel_variant(1)
        ref = plan.execute(rf).cpu().numpy()
        plan.set_kernel_variant(9)
        w = torch.empty((plan.n_x, plan.n_z), dtype=torch.float32, device=gpu)
        img = plan.execute(rf, weights=w).cpu().numpy()
        assert plan.info()["kernel_variant"] == 9
        assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-5, (ne, na)
        o = sum(O.das_pw_mex(px, pz, rf_np[a].T.astype(np.float64), 20e6, angles[a], arr.width, arr.pitch, 1540.0,
                             (2e6, 7e6), 0.0, win.spec(), FN.spec(), "on")[0] for a in range(na))
        assert np.linalg.norm(img[0].T - o) / np.linalg.norm(o) < 1e-4, (ne, na)
        plan.close()


def test_tensor_core_variant_per_angle_images(gpu):
    """Variant 9 without compounding (one image per angle, launched angle by angle) and
    with a directivity F-number, 192 elements, against variant 1 and the FP64 oracle."""
    import torch
    rng = np.random.default_rng(37)
    ne, na, nt, side = 192, 4, 768, 28
    arr = synth.LinearArray(ne, PITCH, 0.918 * PITCH)
    px = (np.arange(side) - (side - 1) / 2.0) * PITCH
    pz = 8e-3 + np.arange(side) * PITCH / 2
    angles = np.deg2rad(np.linspace(-12.0, 12.0, na))
    fn = f_numbers.directivity.perrot(0.918)
    sc = synth.random_points(rng, 6, (px[0], px[-1]), (pz[0], pz[-1]))
    rf_np = synth.pw_rf(rng, arr, sc, list(angles), nt, 20e6, 1540.0)
    rf = torch.tensor(rf_np, dtype=torch.float32, device=gpu)
    plan = das.PWPlan(px, pz, nt, ne, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0, windows.hann(),
                      fn, compound=False)
    plan.set_kernel_variant(1)
    ref = plan.execute(rf).cpu().numpy()
    plan.set_kernel_variant(9)
    img = plan.execute(rf).cpu().numpy()
    assert img.shape == (na, side, side)
    assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-5
    for a in range(na):
        o = O.das_pw_mex(px, pz, rf_np[a].T.astype(np.float64), 20e6, angles[a], arr.width, arr.pitch, 1540.0,
                         (2e6, 7e6), 0.0, windows.hann().spec(), fn.spec(), "on")[0]
        assert np.linalg.norm(img[a].T - o) / np.linalg.norm(o) < 1e-4, a
    plan.close()


@pytest.mark.parametrize("na", [1, 11])
def test_launch_shapes_keep_results(gpu, na):
    """The launch shapes the autotuner searches (fewer resident blocks, shorter bin
    chunk between exact re-anchorings) change only scheduling and how often the
    phase recurrences are re-anchored: images stay within 1e-5 of the default
    shape's and within the parity bar of the FP64 oracle."""
    rng = np.random.default_rng(31 + na)
    plan, rf, (arr, px, pz, angles) = _frame(rng, 48, na, 1024, 32, True, gpu)
    ref = plan.execute(rf).cpu().numpy()
    inf = plan.info()
    tc = inf["kernel_variant"] == 9
    assert inf["bin_chunk"] == (32 if tc else 256)
    rf_np = rf.cpu().numpy().astype(np.float64)
    o = sum(O.das_pw_mex(px, pz, rf_np[a].T, 20e6, angles[a], arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0,
                         ("hann", 0.0), FN.spec(), "on")[0] for a in range(na))
    for bps, chunk in [(0, 16 if tc else 128), (max(1, inf["blocks_per_sm"] - 1), 0)]:
        plan.set_shape(bps, chunk)
        if chunk:
            assert plan.info()["bin_chunk"] == chunk
        img = plan.execute(rf).cpu().numpy()
        assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-5, (bps, chunk)
        assert np.linalg.norm(img[0].T - o) / np.linalg.norm(o) < 1e-4
    with pytest.raises(_lib.FNumError):
        plan.set_shape(0, 24)
    plan.close()
