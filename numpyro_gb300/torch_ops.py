"""torch.autograd exposure of the hand-written potentials.

``potential(kernel, z)`` returns U(z) for a [K, D] CUDA tensor of latent points;
its backward is the hand-written adjoint of the same potential (gbn_potential_vjp
semantics: the incoming cotangent scales dU/dz), not autodiff.  This is the torch
counterpart of differentiating numpyro's ``potential_fn`` with ``value_and_grad``
(numpyro/infer/hmc_util.py:242-252).
"""
import torch


class _Potential(torch.autograd.Function):
    @staticmethod
    def forward(ctx, z, kernel):
        pe, grad = kernel.potential_and_grad(z.detach())
        ctx.save_for_backward(grad)
        return pe

    @staticmethod
    def backward(ctx, cot):
        (grad,) = ctx.saved_tensors
        return (cot.to(grad.dtype)[:, None] * grad).to(torch.float32), None


def potential(kernel, z):
    """Differentiable U(z) (float64 [K]) for a numpyro_gb300 NUTS/HMC kernel."""
    return _Potential.apply(z.to(device="cuda", dtype=torch.float32).contiguous(), kernel)
