"""torch.autograd shim over the adjoint C-ABI, for the gradient tests only.

``LBMObjective.apply(F, make_lbm, adjoint_kwargs)`` runs a fresh domain built by ``make_lbm()`` with
the force field F (3N SoA) through ``LBM.run_adjoint`` and returns J; its backward returns dJ/dF from
the same adjoint run.
"""
import torch


class LBMObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, F, make_lbm, adjoint_kwargs):
        lbm = make_lbm()
        try:
            lbm.F.data[:] = F.detach().cpu().numpy()
            J, grad, _ = lbm.run_adjoint(**adjoint_kwargs)
        finally:
            lbm.close()
        ctx.save_for_backward(torch.from_numpy(grad).to(F.device, F.dtype))
        return torch.tensor(J, dtype=torch.float64, device=F.device)

    @staticmethod
    def backward(ctx, grad_output):
        (grad,) = ctx.saved_tensors
        return grad_output.to(grad.dtype) * grad, None, None
