"""PyTorch autograd wrapper of the local-energy gradient (PsiDeep: the adjoint kernels;
Psi: the derivative formed from the estimator sums).

``energy(params, psi, operator_, ensemble)`` returns the real scalar <E_loc> of the
network whose parameters are the complex tensor ``params`` (the reference's layout,
``psi.params``), evaluated on ``ensemble``.  The gradient comes from the library's
adjoint kernel (``rbmg_ev_eloc_gradient``), which recomputes every forward pass on the
device.  When autograd records the call (grad mode on and ``params.requires_grad``), the
forward pass runs that kernel once, which yields <E_loc> and the gradient together on one
set of configurations, and the backward pass returns the stored gradient.  Otherwise the
forward pass samples (or enumerates) and evaluates the local energies only, with no
gradient work.  (Evaluating the energy in the forward pass and the gradient in the backward
pass on the kept samples gives the same numbers, but for a PsiDeep on Monte Carlo samples
costs the estimator's FP64 local-energy pass on top of the adjoint: 716 ms against 161 ms
per step of the 100-200-100-50 net over 8192 walkers.)  PyTorch is used only for this
wrapper: the value and the gradient both come from the CUDA library.

    params = torch.tensor(psi.params, requires_grad=True)
    E = energy(params, psi, H, MonteCarloLoop(...))
    E.backward()        # params.grad = dE/dRe + i dE/dIm

With ``score=True`` (default) the gradient is that of <H>, the sampling term included;
``score=False`` differentiates <E_loc> with the samples held fixed.
"""
import numpy as np
import torch

from .api import ExpectationValue, FixedSamples, MonteCarloLoop


class LocalEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, psi, operator_, ensemble, score, with_gradient):
        host = params.detach().to("cpu", torch.complex128).numpy().copy()
        psi.params = host
        ctx.grad = None
        if with_gradient:
            # one adjoint pass: <E_loc> and its gradient on the same configurations
            ctx.grad, E = ExpectationValue().eloc_gradient(psi, operator_, ensemble, score)
            return torch.tensor(complex(E).real, dtype=torch.float64, device=params.device)
        if isinstance(ensemble, MonteCarloLoop):
            # one sampling pass; its configurations are kept for the backward pass
            spins, _, eloc = ensemble.samples(psi, operator_, log_psi=False)
            E = complex(np.mean(eloc))
            ctx.ensemble = FixedSamples(psi.N, spins)
        else:
            E = ExpectationValue()(psi, operator_, ensemble)
            ctx.ensemble = ensemble
        ctx.psi, ctx.operator_, ctx.score, ctx.host = psi, operator_, score, host
        return torch.tensor(E.real, dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        grad = ctx.grad
        if grad is None:
            psi = ctx.psi
            psi.params = ctx.host          # the parameters the forward pass evaluated
            grad, _ = ExpectationValue().eloc_gradient(psi, ctx.operator_, ctx.ensemble, ctx.score)
        g = torch.from_numpy(grad).to(grad_out.device)
        return grad_out.to(g.dtype) * g, None, None, None, None, None


def energy(params, psi, operator_, ensemble, score=True):
    """Re <E_loc> of psi with parameters `params` (complex tensor) on `ensemble`."""
    if not torch.is_complex(params):
        raise TypeError("params must be a complex tensor in the reference's parameter layout")
    with_gradient = torch.is_grad_enabled() and params.requires_grad
    return LocalEnergy.apply(params, psi, operator_, ensemble, bool(score), with_gradient)
