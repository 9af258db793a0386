"""torch.autograd binding of the transient forward/adjoint pair (test harness only).

TransientObjective.apply(xPhys, physics, material) runs CompleteInitialState,
GenerateCheckPoints and ComputeObjectiveSensitivities of a LinearElasticity
object (LinearElasticity.cc:956-1206, :1208-1280, :1625-1908) in `forward`
and returns the objective as a 0-d tensor; `backward` hands back the adjoint
sensitivities that call already computed, scaled by the incoming gradient.
The library itself never imports torch.autograd: this wrapper exists so that
tests can drive the C ABI through torch's gradient machinery.
"""
import torch


class TransientObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xPhys, physics, material):
        physics.CompleteInitialState(xPhys.detach(), *material)
        physics.GenerateCheckPoints()
        dfdx = torch.zeros_like(xPhys)
        fx = physics.ComputeObjectiveSensitivities(dfdx)
        ctx.save_for_backward(dfdx)
        return xPhys.new_tensor(fx)

    @staticmethod
    def backward(ctx, grad):
        (dfdx,) = ctx.saved_tensors
        return grad * dfdx, None, None


def objective(xPhys, physics, material):
    return TransientObjective.apply(xPhys, physics, material)
