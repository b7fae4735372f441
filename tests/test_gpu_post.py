"""Device post-processing: coherent compounding and B-mode log compression
(fnum_bmode), checked against the host computation of the reference's
example script (examples.m:78 sums the per-angle images, examples.m:88,96
take 20 log10(abs(image) / max(abs(image(:))))) done in float64 with numpy."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, synth, windows

pytestmark = pytest.mark.gpu

TOL_DB = 1e-4       # dB against the host computation on the same image, voxels above -100 dB
TOL_DB_PATH = 1e-3  # dB between compounding paths, voxels above -40 dB (the parity bar's range)


def _host_bmode(stack):
    s = stack.astype(np.complex128).sum(axis=0)
    a = np.abs(s)
    return 20 * np.log10(a / a.max()), a.max()


def test_bmode_matches_host_on_beamformed_angles(gpu):
    import torch
    arr = synth.LinearArray(48, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = np.array([-0.1, 0.0, 0.1])
    px = np.linspace(-5e-3, 5e-3, 48)
    pz = np.linspace(6e-3, 18e-3, 64)
    rng = np.random.default_rng(7)
    sc = synth.random_points(rng, 5, (-5e-3, 5e-3), (6e-3, 18e-3))
    rf = torch.tensor(synth.pw_rf(rng, arr, sc, list(angles), 1024, 20e6, 1540.0), dtype=torch.float32, device=gpu)
    plan = das.PWPlan(px, pz, 1024, arr.n_elements, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0,
                      windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5), compound=False)
    stack = plan.execute(rf)                                             # [3, N_x, N_z]
    db, mx = das.bmode(stack)
    ref_db, ref_mx = _host_bmode(stack.cpu().numpy())
    got = db.cpu().numpy()
    sel = ref_db > -100
    assert np.max(np.abs(got[sel] - ref_db[sel])) < TOL_DB
    assert abs(float(mx) - ref_mx) <= 1e-5 * ref_mx
    assert np.isclose(got.max(), 0.0, atol=1e-6)
    # compounding inside the beamformer gives the same B-mode image
    plan_c = das.PWPlan(px, pz, 1024, arr.n_elements, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0,
                        windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5), compound=True)
    db_c, _ = das.bmode(plan_c.execute(rf))
    sel40 = ref_db > -40
    assert np.max(np.abs(db_c.cpu().numpy()[sel40] - got[sel40])) < TOL_DB_PATH
    plan.close()
    plan_c.close()


def test_bmode_floor_and_zero_image(gpu):
    import torch
    img = torch.zeros((2, 8, 9), dtype=torch.complex64, device=gpu)
    db, mx = das.bmode(img, floor_db=-60.0)
    assert float(mx) == 0.0
    assert torch.all(db == -60.0)
    img[0, 3, 4] = 2.0 + 0.0j
    img[1, 3, 4] = 0.0 + 0.0j
    img[0, 1, 1] = 0.002 + 0.0j
    db, mx = das.bmode(img, floor_db=-40.0)
    h = db.cpu().numpy()
    assert float(mx) == pytest.approx(2.0)
    assert h[3, 4] == pytest.approx(0.0, abs=1e-6)
    assert h[1, 1] == -40.0                      # -60 dB clamped to the floor
    assert h[0, 0] == -40.0                      # zero voxel
