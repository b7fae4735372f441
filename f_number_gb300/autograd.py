"""torch.autograd binding of the plane-wave beamformer's C ABI: the compounded
image of a plan as a differentiable function of the band spectra X and the
speed of sound c.

    image = pw_beamform(plan, X, c)       # complex64 [N_x, N_z] on the plan's GPU

The forward is fnum_plan_set_spectra + fnum_pw_plan_set_sound_speed +
fnum_plan_execute_beamform (the fused kernels); the backward is fnum_pw_adjoint
(the hand-written adjoint kernel).  As in fnum_pw_sharpness_grad, the DFT order,
band, F table and apertures are those of the speed the plan was created with;
only the phases follow c.  The reference (das_pw.m, +cuda/gpu_bf_das_pw_rf.cu)
has no derivatives; this binding exists for finite-difference and
reference-gradient checks and for losses written in torch.

PyTorch's convention for a real loss L of complex z is grad = dL/dRe z + i dL/dIm z
= 2 dL/dz*.  The beamformer is C-linear in X, so grad_X = A^H grad_I, which is
what fnum_pw_adjoint returns when handed grad_I; dL/dc from the ABI is
2 Re sum conj(G) dI/dc for its G, hence the factor 1/2 with G = grad_I.
"""
from __future__ import annotations

import torch

from . import das


class PWBeamform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, spectra, c, plan):
        if not isinstance(plan, das.PWPlan) or plan.n_out != 1:
            raise ValueError("pw_beamform needs a compounded PWPlan (compound=True)")
        c_val = float(c)
        spectra = spectra.detach().to(torch.complex64).contiguous()
        plan.set_sound_speed(c_val)
        plan.set_spectra(spectra)
        img = torch.empty((1, plan.n_x, plan.n_z), dtype=torch.complex64, device=spectra.device)
        plan.execute_beamform(img)
        ctx.plan = plan
        ctx.c = c_val
        ctx.c_is_tensor = torch.is_tensor(c)
        ctx.c_like = (c.dtype, c.device) if torch.is_tensor(c) else None
        ctx.save_for_backward(spectra)
        return img[0]

    @staticmethod
    def backward(ctx, grad_img):
        (spectra,) = ctx.saved_tensors
        plan = ctx.plan
        # the plan is stateful: restore the forward's spectra and speed first
        plan.set_sound_speed(ctx.c)
        plan.set_spectra(spectra)
        need_c = ctx.c_is_tensor and ctx.needs_input_grad[1]
        g, dc = plan.adjoint(grad_img.contiguous(), dc=need_c)
        grad_c = None
        if need_c:
            grad_c = torch.tensor(0.5 * dc, dtype=ctx.c_like[0], device=ctx.c_like[1])
        return (g if ctx.needs_input_grad[0] else None), grad_c, None


def pw_beamform(plan, spectra, c):
    """Compounded image of `plan` for band spectra `spectra` (complex64 CUDA tensor
    [n_elements, n_bins, n_angles]) at sound speed `c` (float or 0-d float64
    tensor), differentiable in both."""
    return PWBeamform.apply(spectra, c, plan)


def sharpness(image):
    """The image-sharpness loss L = -sum|I|^4 / (sum|I|^2)^2 (as fnum_pw_sharpness_grad)."""
    p = image.real.double() ** 2 + image.imag.double() ** 2
    return -(p * p).sum() / p.sum() ** 2
