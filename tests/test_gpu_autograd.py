"""torch.autograd bindings (vardyn_gb300/autograd.py): the QG step's
backward is its adjoint (dot-product identity with the tangent linear), and
the 4D-Var cost's backward returns the engine's gradient, so torch.optim can
minimise it."""
import numpy as np
import pytest
import torch

from test_gpu_basis import make as basis_case
from test_gpu_fourdvar import engine_case
from test_gpu_sw import GOLD as SW_GOLD, plan_a as sw_plan_a

pytestmark = pytest.mark.gpu


def close(a, b, tol):
    return float((a - b).abs().max()) <= tol * float(b.abs().max())


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def test_qg_step_backward_is_the_adjoint():
    from vardyn_gb300.autograd import QGStep
    from vardyn_gb300.qg1l import QG1LPlan
    from vardyn_gb300.synthetic import kminus3_ssh
    ny, nx, dx, nstep = 40, 48, 5e3, 12
    rng = np.random.default_rng(8)
    plan = QG1LPlan(ny, nx, dx, dx, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=torch.float64)
    dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda")
    h0 = dev(kminus3_ssh(ny, nx, dx, dx, rng, rms=0.1, cutoff_km=20.0)).requires_grad_()
    hb = dev(np.zeros((ny, nx)))
    w = dev(rng.standard_normal((ny, nx)))
    dh = dev(rng.standard_normal((ny, nx)))
    out = QGStep.apply(h0, hb, plan, nstep)
    assert out.shape == h0.shape
    (out * w).sum().backward()
    lhs = float((w * plan.step_tgl(dh, h0.detach(), hb, nstep)[0]).sum())
    rhs = float((h0.grad * dh).sum())
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_fourdvar_cost_backward_and_torch_optimiser():
    from vardyn_gb300.autograd import FourDVarCost
    eng, _, _, h0, _ = engine_case(torch.float64)
    x = torch.as_tensor(h0, device="cuda").requires_grad_()
    J = FourDVarCost.apply(x, eng)
    (2.0 * J).sum().backward()
    _, G = eng.cost_and_grad(x.detach())
    assert close(x.grad, 2.0 * G, 1e-12)
    J0 = float(J.detach().sum())
    x2 = torch.as_tensor(h0, device="cuda").requires_grad_()
    opt = torch.optim.LBFGS([x2], max_iter=8, line_search_fn="strong_wolfe")

    def closure():
        opt.zero_grad()
        loss = FourDVarCost.apply(x2, eng).sum()
        loss.backward()
        return loss
    opt.step(closure)
    J1 = float(FourDVarCost.apply(x2.detach(), eng).sum())
    assert J1 < 0.8 * J0


def test_sw_step_backward_is_the_adjoint():
    """Two-layer case with land, boundary fields, forcing and wind: the
    gradient of <w, M(x)> through SWStep equals M'^T w (dot product with
    the tangent linear)."""
    from vardyn_gb300.autograd import SWStep
    g = dict(np.load(SW_GOLD))
    pl = sw_plan_a(g)
    T = lambda k: torch.as_tensor(g["swa_" + k], dtype=torch.float64, device="cuda")
    inputs = dict(taux=T("taux"), tauy=T("tauy"), ub=T("ub"), vb=T("vb"), hb=T("hb"), Fu=T("Fu"), Fv=T("Fv"),
                  Fh=T("Fh"))
    rng = np.random.default_rng(12)
    m = pl.masks
    x = [T("u0").requires_grad_(), T("v0").requires_grad_(), T("h0").requires_grad_()]
    rnd = lambda a, mk: torch.as_tensor(rng.standard_normal(tuple(a.shape)) * mk, device="cuda")
    w = [rnd(a, mk) for a, mk in zip(x, (m.u, m.v, m.h))]
    d = [rnd(a, mk) for a, mk in zip(x, (m.u, m.v, m.h))]
    out = SWStep.apply(*x, pl, 3, inputs)
    assert all(o.shape == a.shape for o, a in zip(out, x))
    sum((o * c).sum() for o, c in zip(out, w)).backward()
    dy = pl.step_tgl(*[a.detach() for a in x], *d, nstep=3, **inputs)
    lhs = sum(float((a.reshape(c.shape) * c).sum()) for a, c in zip(dy, w))
    rhs = sum(float((a.grad * c).sum()) for a, c in zip(x, d))
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def test_basis_projection_backward_is_the_transpose():
    from vardyn_gb300.autograd import BasisProjection
    plan, _, _, _ = basis_case(False, torch.float64)
    rng = np.random.default_rng(9)
    X = torch.as_tensor(rng.standard_normal((2, plan.nbasis)), device="cuda").requires_grad_()
    A = torch.as_tensor(rng.standard_normal((2, plan.ny, plan.nx)), device="cuda")
    k = 30
    phi = BasisProjection.apply(X, plan, k)
    assert close(phi, plan.project(k, X.detach()), 1e-13)
    (phi * A).sum().backward()
    adX = torch.zeros(2, plan.nbasis, dtype=torch.float64, device="cuda")
    plan.project_T(k, A, adX)
    assert close(X.grad, adX, 1e-13)
    x1 = X.detach()[0].clone().requires_grad_()                  # a single control vector
    (BasisProjection.apply(x1, plan, k) * A[0]).sum().backward()
    assert x1.grad.shape == x1.shape and close(x1.grad, adX[0], 1e-13)
