"""torch.autograd binding of the equiprop path.

``propagate(ctx, dt, carr)`` returns the propagator ``U`` as a complex CUDA
tensor and differentiates with respect to the real control samples ``carr``
(shape (amps, pts)) through the library's adjoint kernels: the backward pass
is one call of ``Parament_equipropVJPDevice`` with the incoming gradient as
seed (PyTorch's complex gradient ``G`` satisfies ``dL = Re Tr(G^H dU)``).
"""
import torch


class EquipropFunction(torch.autograd.Function):
    @staticmethod
    def forward(fctx, pctx, dt, carr):
        fctx.pctx = pctx
        fctx.dt = dt
        fctx.save_for_backward(carr)
        return pctx.equiprop_device(dt, carr.detach())

    @staticmethod
    def backward(fctx, grad_U):
        (carr,) = fctx.saved_tensors
        grad = fctx.pctx.vjp_device(fctx.dt, carr.detach(), grad_U.contiguous())
        return None, None, grad.to(carr.real.dtype if carr.is_complex() else carr.dtype)


def propagate(pctx, dt, carr):
    """Differentiable equiprop on a loaded context (see module docstring)."""
    if carr.dim() == 1:
        carr = carr.unsqueeze(0)
    return EquipropFunction.apply(pctx, dt, carr)


def fidelity_loss(U, U_target):
    """1 - |Tr(V^H U)|^2 / d^2 as a differentiable torch expression."""
    d = U.shape[-1]
    g = torch.trace(U_target.conj().transpose(-2, -1).to(U.dtype) @ U)
    return 1.0 - (g.abs() ** 2) / d ** 2
