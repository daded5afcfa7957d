"""PyTorch autograd wrapper of the local-energy gradient (PsiDeep: the adjoint kernels;
Psi: the derivative formed from the estimator sums).

``energy(params, psi, operator_, ensemble)`` returns the real scalar <E_loc> of the
network whose parameters are the complex tensor ``params`` (the reference's layout,
``psi.params``), evaluated on ``ensemble``.  The forward pass samples (or enumerates)
and evaluates the local energies only; the backward pass runs the library's adjoint
kernel (``rbmg_ev_eloc_gradient``), which recomputes every forward pass on the device,
on the very configurations the forward pass used (a MonteCarloLoop's samples are kept
as a ``FixedSamples`` set), so a forward evaluation without a backward pass costs no
gradient work.  PyTorch is used only for this wrapper: the value and the gradient both
come from the CUDA library.

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
    def forward(ctx, params, psi, operator_, ensemble, score):
        host = params.detach().to("cpu", torch.complex128).numpy().copy()
        psi.params = host
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
        psi = ctx.psi
        psi.params = ctx.host          # the parameters the forward pass evaluated
        grad, _ = ExpectationValue().eloc_gradient(psi, ctx.operator_, ctx.ensemble, ctx.score)
        g = torch.from_numpy(grad).to(grad_out.device)
        return grad_out.to(g.dtype) * g, None, None, None, None


def energy(params, psi, operator_, ensemble, score=True):
    """Re <E_loc> of psi with parameters `params` (complex tensor) on `ensemble`."""
    if not torch.is_complex(params):
        raise TypeError("params must be a complex tensor in the reference's parameter layout")
    return LocalEnergy.apply(params, psi, operator_, ensemble, bool(score))
