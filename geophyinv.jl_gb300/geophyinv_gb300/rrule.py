"""The FWI misfit as a differentiable function.

`rrule(lossvalue, m, loss, dobs, pa, mparams)` follows ChainRulesCore's
convention: it returns the primal J and a pullback dJ -> (tangent of
lossvalue, dm, tangents of loss, dobs, pa, mparams).  The primal pass is the
forward_save run (its boundary store, or the state slots of a checkpointed
plan, stay on the device); the pullback runs the hand-written adjoint and
the imaging condition, once, when it is called.  A checkpointed plan
(`SeisForwExpt(..., checkpoints=n)`) recomputes the forward states from its
slots instead of keeping a per-step store, which is what lets 3-D gradients
fit on the device.

`misfit(m, loss, dobs, pa)` wraps the same pair as a torch.autograd
function of a torch tensor m, for optimisers written against torch.

The reference has no rrule: its FWI hands lossvalue and gradient! to Optim
(src/fwi/fwi.jl:66-76, src/fdtd/func_grad.jl:1-49); the numbers here are
those of gradient!.
"""
import numpy as np

from .fdtd import _adjoint, _forward_save, _loss, lossvalue


class _NoTangent:
    """ChainRulesCore.NoTangent(): the argument is not differentiable."""

    def __repr__(self):
        return "NoTangent()"


NoTangent = _NoTangent()


def rrule(f, m, loss, dobs, pa, mparams=("invK", "rho")):
    """(J, pullback) of f = lossvalue at m (see the module docstring)."""
    if f is not lossvalue:
        raise TypeError("rrule is defined for lossvalue only")
    mparams = tuple(mparams)
    m = np.asarray(m, np.float32)
    _forward_save(pa, m, mparams)
    J = _loss(loss, dobs, pa)
    done = []

    def pullback(dJ):
        if done:
            raise RuntimeError("the pullback of a misfit runs once (the adjoint consumes the forward run)")
        done.append(True)
        dm = _adjoint(pa, m, loss, dobs, mparams, scale=float(dJ))
        return NoTangent, dm, NoTangent, NoTangent, NoTangent, NoTangent

    return J, pullback


def misfit(m, loss, dobs, pa, mparams=("invK", "rho")):
    """J(m) as a torch scalar (float64) whose backward is the adjoint."""
    import torch

    class _Misfit(torch.autograd.Function):
        @staticmethod
        def forward(ctx, mt):
            J, pb = rrule(lossvalue, mt.detach().cpu().numpy(), loss, dobs, pa, mparams)
            ctx.pb = pb
            ctx.like = mt
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, dJ):
            dm = ctx.pb(float(dJ))[1]
            return torch.from_numpy(dm).to(device=ctx.like.device, dtype=ctx.like.dtype)

    return _Misfit.apply(m)
