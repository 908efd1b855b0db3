"""torch.autograd bindings of the QG 1.5-layer step and of the 4D-Var cost.

The reference differentiates its model with jax.vjp (Qgm.step_adj,
mapping/models/model_qg1l/jqgm.py:565-569) and hands the cost and its
gradient to scipy (mapping/src/inv.py:309-414). These Functions give the
same pairs to PyTorch: ``backward()`` runs the library's adjoint kernels, so
torch code (torch.optim, a loss built on the model output) can drive the
windows on the device.

- ``QGStep.apply(h0, hb, plan, nstep)``: the forward step of a
  :class:`vardyn_gb300.qg1l.QG1LPlan`; its backward is ``plan.step_adj``
  (the trajectory is recomputed from h0, as the reference's vjp does). The
  gradient flows to h0 only: the reference's adjoint has no hb derivative.
- ``FourDVarCost.apply(x, engine)``: J per window (float64) of a window
  engine of :mod:`vardyn_gb300.fourdvar` (``QGWindows4DVar``,
  ``QGBasis4DVar``); the forward evaluation already computes the gradient,
  which backward scales by the incoming cotangent.
"""
import torch


class QGStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h0, hb, plan, nstep):
        ctx.plan, ctx.nstep = plan, int(nstep)
        ctx.save_for_backward(h0, hb)
        return plan.step(h0, hb, int(nstep)).reshape(h0.shape)

    @staticmethod
    def backward(ctx, g):
        h0, hb = ctx.saved_tensors
        ad = ctx.plan.step_adj(g.contiguous().to(h0.dtype), h0, hb, ctx.nstep)
        return ad.reshape(h0.shape), None, None, None


class FourDVarCost(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, engine):
        J, G = engine.cost_and_grad(x)
        # the engine owns J and G and overwrites them on its next call
        ctx.save_for_backward(G.detach().clone())
        return J.detach().clone()

    @staticmethod
    def backward(ctx, gJ):
        (G,) = ctx.saved_tensors
        scale = gJ.to(G.dtype).reshape((-1,) + (1,) * (G.dim() - 1))
        return scale * G, None
