"""PyTorch autograd wrapper of the local-energy gradient (PsiDeep: the adjoint kernels;
Psi: the derivative formed from the estimator sums).

``energy(params, psi, operator_, ensemble)`` returns the real scalar <E_loc> of the
network whose parameters are the complex tensor ``params`` (the reference's layout,
``psi.params``), evaluated on ``ensemble``; its backward pass is the library's adjoint
kernel (``rbmg_ev_eloc_gradient``), which recomputes every forward pass on the device.
PyTorch is used only for this wrapper: the forward value and the gradient both come
from the CUDA library.

    params = torch.tensor(psi.params, requires_grad=True)
    E = energy(params, psi, H, MonteCarloLoop(...))
    E.backward()        # params.grad = dE/dRe + i dE/dIm

With ``score=True`` (default) the gradient is that of <H>, the sampling term included;
``score=False`` differentiates <E_loc> with the samples held fixed.
"""
import numpy as np
import torch

from .api import ExpectationValue


class LocalEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, psi, operator_, ensemble, score):
        psi.params = params.detach().to("cpu", torch.complex128).numpy()
        grad, E = ExpectationValue().eloc_gradient(psi, operator_, ensemble, score)
        ctx.save_for_backward(torch.from_numpy(grad).to(params.device, params.dtype))
        return torch.tensor(E.real, dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return grad_out.to(grad.dtype) * grad, None, None, None, None


def energy(params, psi, operator_, ensemble, score=True):
    """Re <E_loc> of psi with parameters `params` (complex tensor) on `ensemble`."""
    if not torch.is_complex(params):
        raise TypeError("params must be a complex tensor in the reference's parameter layout")
    return LocalEnergy.apply(params, psi, operator_, ensemble, bool(score))
