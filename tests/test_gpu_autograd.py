"""torch.autograd bindings (vardyn_gb300/autograd.py): the QG step's
backward is its adjoint (dot-product identity with the tangent linear), and
the 4D-Var cost's backward returns the engine's gradient, so torch.optim can
minimise it."""
import numpy as np
import pytest
import torch

from test_gpu_fourdvar import engine_case

pytestmark = [pytest.mark.gpu, pytest.mark.last]


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
    assert torch.allclose(x.grad, 2.0 * G, rtol=1e-12, atol=0.0)
    J0 = float(J.sum())
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
