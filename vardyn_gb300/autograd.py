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
- ``SWStep.apply(u0, v0, h0, plan, nstep, inputs)``: the multilayer
  shallow-water step of a :class:`vardyn_gb300.sw.SWPlan` (sw.py:752-937);
  ``inputs`` holds the fixed boundary fields, forcing and wind stress
  (keywords of ``plan.step``); backward is ``plan.step_adj`` with respect to
  the initial state.
- ``BasisProjection.apply(X, plan, k)``: phi = G(t_k) X of a reduced-basis
  plan (``BasisPlan``, ``BMPlan``, ``WaveletPlan``; basis.py operg); backward
  is the transpose kernel (operg_transpose).
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


class SWStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, v0, h0, plan, nstep, inputs=None):
        ctx.plan, ctx.nstep, ctx.inputs = plan, int(nstep), dict(inputs or {})
        ctx.save_for_backward(u0, v0, h0)
        u1, v1, h1 = plan.step(u0, v0, h0, nstep=int(nstep), **ctx.inputs)
        return u1.reshape(u0.shape), v1.reshape(v0.shape), h1.reshape(h0.shape)

    @staticmethod
    def backward(ctx, gu, gv, gh):
        u0, v0, h0 = ctx.saved_tensors
        g = [torch.zeros_like(x) if c is None else c.contiguous().to(x.dtype)
             for c, x in zip((gu, gv, gh), (u0, v0, h0))]
        a = ctx.plan.step_adj(u0, v0, h0, *g, nstep=ctx.nstep, **ctx.inputs)
        return a["u0"].reshape(u0.shape), a["v0"].reshape(v0.shape), a["h0"].reshape(h0.shape), None, None, None


class BasisProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, plan, k):
        if X.dtype != plan.dtype:
            raise TypeError(f"control dtype {X.dtype} differs from the basis plan's {plan.dtype}")
        ctx.plan, ctx.k, ctx.shape = plan, int(k), X.shape
        phi = plan.project(int(k), X.reshape(-1, plan.nbasis).contiguous())
        return phi[0] if X.dim() == 1 else phi

    @staticmethod
    def backward(ctx, g):
        g = g.reshape(-1, ctx.plan.ny, ctx.plan.nx).contiguous()
        adX = torch.zeros((g.shape[0], ctx.plan.nbasis), dtype=ctx.plan.dtype, device=g.device)
        ctx.plan.project_T(ctx.k, g.to(ctx.plan.dtype), adX)
        return adX.reshape(ctx.shape), None, None


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
