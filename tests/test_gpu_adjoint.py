"""Gradients of the image-sharpness loss L = -sum|I|^4 / (sum|I|^2)^2 of a
compounded plane-wave image (fnum_pw_sharpness_grad), against the FP64 oracle
(oracle.pw_sharpness_grad, itself pinned to finite differences in
test_oracle_kat.py) and against finite differences of the library's own loss.
Band, F table and apertures are frozen at the creation speed; only the phases
move with c (fnum_pw_plan_set_sound_speed)."""
import numpy as np
import pytest

from f_number_gb300 import das, f_numbers, synth, windows
from oracle import fnum_oracle as O

pytestmark = pytest.mark.gpu

TOL_LOSS = 1e-5     # relative, loss
TOL_DC = 1e-3       # relative, dL/dc against the FP64 gradient
TOL_GX = 1e-4       # relative L2, dL/dX* against the FP64 gradient
TOL_FD = 1e-3       # relative, analytic vs central differences of the library's loss

F_SPEC = {"kind": "grating.angle_lb", "angle_lb_deg": 60.0, "F_number_ub": 1.5, "distance_deg": 10.0}


def _case(gpu, seed=5):
    import torch
    rng = np.random.default_rng(seed)
    arr = synth.LinearArray(32, 0.3048e-3, 0.918 * 0.3048e-3)
    angles = np.deg2rad([-6.0, 0.0, 6.0])
    px = np.linspace(-3e-3, 3e-3, 20)
    pz = np.linspace(6e-3, 14e-3, 24)
    sc = synth.random_points(rng, 5, (-3e-3, 3e-3), (6e-3, 14e-3))
    rf = synth.pw_rf(rng, arr, sc, list(angles), 768, 20e6, 1500.0)       # echoes at c = 1500
    plan = das.PWPlan(px, pz, 768, arr.n_elements, 20e6, angles, arr.width, arr.pitch, 1540.0, [2e6, 7e6], 0.0,
                      windows.hann(), f_numbers.grating.angle_lb(60.0, 1.5), compound=True)
    return plan, rf, torch.tensor(rf, dtype=torch.float32, device=gpu), (arr, px, pz, angles, rng)


def test_sharpness_gradients_match_fp64(gpu):
    plan, rf, rf_d, (arr, px, pz, angles, _) = _case(gpu)
    kw = dict(f_bounds=(2e6, 7e6), index_t0=0.0, window=("hann", 0.0), F_number=F_SPEC, normalization="on",
              c_freeze=1540.0)
    rf32 = rf.astype(np.float32).astype(np.float64)       # the GPU sees float32 RF
    for c in (1540.0, 1480.0):                           # at the creation speed and re-timed
        plan.set_sound_speed(c)
        L, dc, g = plan.sharpness_grad(rf_d)
        Lr, dcr, gr, _ = O.pw_sharpness_grad(px, pz, rf32, 20e6, angles, arr.width, arr.pitch, c, **kw)
        assert abs(L - Lr) <= TOL_LOSS * abs(Lr), (c, L, Lr)
        assert abs(dc - dcr) <= TOL_DC * abs(dcr), (c, dc, dcr)
        gh = g.cpu().numpy()
        assert np.linalg.norm(gh - gr) / np.linalg.norm(gr) < TOL_GX, c
    plan.close()


def test_sharpness_gradients_match_finite_differences(gpu):
    import torch
    plan, rf, rf_d, (arr, px, pz, angles, rng) = _case(gpu, seed=6)
    plan.set_sound_speed(1520.0)
    L, dc, g = plan.sharpness_grad(rf_d)
    # c: central differences of the library's loss.  The FP32 image puts ~1e-3 of noise
    # on the difference at h = 0.05 m/s; at h = 0.2 m/s the noise is 4x smaller and the
    # truncation error of central differences is 5e-5 (measured with the FP64 oracle)
    h = 0.2
    plan.set_sound_speed(1520.0 + h)
    Lp = plan.sharpness_grad(rf_d, grad_spectra=False)[0]
    plan.set_sound_speed(1520.0 - h)
    Lm = plan.sharpness_grad(rf_d, grad_spectra=False)[0]
    assert abs((Lp - Lm) / (2 * h) - dc) <= TOL_FD * abs(dc)
    # spectra: a random RF direction, dL = 2 Re sum conj(dL/dX*) dX with dX its band DFT
    plan.set_sound_speed(1520.0)
    d_rf = rng.standard_normal(rf.shape) * np.sqrt(np.mean(rf ** 2))
    band = O.band_mex(pz, 768, arr.n_elements, 20e6, arr.width, arr.pitch, 1540.0, (2e6, 7e6), 0.0)
    dX = np.stack([O.rf_band_spectra(d_rf[a].T, band) for a in range(len(angles))], axis=2).transpose(1, 0, 2)
    an = 2 * np.real(np.sum(np.conj(g.cpu().numpy().astype(np.complex128)) * dX))
    # a 1e-3 step (relative to the RF) moves L by ~5e-6 of itself, below the FP32 noise of the
    # loss; at 1e-2 the change is 10x larger and the truncation error of central differences
    # stays near 5e-4 (the FP64 check in test_oracle_kat.py shows its eps^2 behaviour)
    eps = 1e-2
    Lp = plan.sharpness_grad(torch.tensor(rf + eps * d_rf, dtype=torch.float32, device=gpu), grad_spectra=False)[0]
    Lm = plan.sharpness_grad(torch.tensor(rf - eps * d_rf, dtype=torch.float32, device=gpu), grad_spectra=False)[0]
    assert abs((Lp - Lm) / (2 * eps) - an) <= 2 * TOL_FD * abs(an)
    plan.close()


def test_adjoint_inner_product_identity(gpu):
    """fnum_pw_adjoint is the adjoint of the beamformer: for random spectra dX and a
    random image cotangent G, Re <G, A dX> = Re <A^H G, dX> (A linear in X)."""
    import torch
    plan, rf, rf_d, (arr, px, pz, angles, rng) = _case(gpu, seed=7)
    plan.execute(rf_d)
    shape = (plan.n_elements, plan.n_bins, plan.n_angles)
    dX = torch.tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape), dtype=torch.complex64,
                      device=gpu)
    G = torch.tensor(rng.standard_normal((plan.n_x, plan.n_z)) + 1j * rng.standard_normal((plan.n_x, plan.n_z)),
                     dtype=torch.complex64, device=gpu)
    plan.set_spectra(dX)
    img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=gpu)
    plan.execute_beamform(img)
    gX, _ = plan.adjoint(G, dc=False)
    lhs = torch.sum(torch.conj(G.to(torch.complex128)) * img[0].to(torch.complex128)).real.item()
    rhs = torch.sum(torch.conj(gX.to(torch.complex128)) * dX.to(torch.complex128)).real.item()
    scale = torch.linalg.vector_norm(G.abs().double()).item() * torch.linalg.vector_norm(img.abs().double()).item()
    assert abs(lhs - rhs) <= 1e-5 * scale, (lhs, rhs, scale)
    plan.close()


def test_autograd_function_matches_abi_and_finite_differences(gpu):
    """f_number_gb300.autograd.pw_beamform: torch autograd through the C ABI.  The
    sharpness loss written in torch gives the gradients of fnum_pw_sharpness_grad
    (torch's complex grad is 2 dL/dX*), and a second, non-sharpness loss (a
    weighted image energy) matches central differences in c and along a random
    spectra direction."""
    import torch
    from f_number_gb300 import autograd as AG
    plan, rf, rf_d, (arr, px, pz, angles, rng) = _case(gpu, seed=8)
    plan.set_sound_speed(1510.0)
    L_abi, dc_abi, g_abi = plan.sharpness_grad(rf_d)
    X = plan.spectra().clone().requires_grad_(True)
    c = torch.tensor(1510.0, dtype=torch.float64, requires_grad=True)
    L = AG.sharpness(AG.pw_beamform(plan, X, c))
    L.backward()
    assert abs(L.item() - L_abi) <= TOL_LOSS * abs(L_abi)
    assert abs(c.grad.item() - dc_abi) <= TOL_DC * abs(dc_abi), (c.grad.item(), dc_abi)
    assert (torch.linalg.vector_norm(X.grad - 2 * g_abi) / torch.linalg.vector_norm(2 * g_abi)).item() < TOL_GX

    wv = torch.tensor(rng.uniform(0.5, 1.5, (plan.n_x, plan.n_z)), device=gpu)

    def energy(Xv, cv):
        img = AG.pw_beamform(plan, Xv, cv)
        return (wv * (img.real.double() ** 2 + img.imag.double() ** 2)).sum()

    X0 = X.detach().clone()
    Xr = X0.clone().requires_grad_(True)
    cr = torch.tensor(1510.0, dtype=torch.float64, requires_grad=True)
    E = energy(Xr, cr)
    E.backward()
    h = 0.2
    fd_c = (energy(X0, 1510.0 + h).item() - energy(X0, 1510.0 - h).item()) / (2 * h)
    assert abs(fd_c - cr.grad.item()) <= TOL_FD * abs(cr.grad.item()), (fd_c, cr.grad.item())
    d = torch.tensor(rng.standard_normal(X0.shape) + 1j * rng.standard_normal(X0.shape), dtype=torch.complex64,
                     device=gpu) * X0.abs().mean()
    eps = 1e-2
    fd_x = (energy(X0 + eps * d, 1510.0).item() - energy(X0 - eps * d, 1510.0).item()) / (2 * eps)
    an = torch.sum(torch.conj(Xr.grad.to(torch.complex128)) * d.to(torch.complex128)).real.item()
    assert abs(fd_x - an) <= TOL_FD * abs(an), (fd_x, an)
    plan.close()
