"""The single-stage entry points (vd_qg1l_rk_stage / vd_qg1l_rk_stage_adj,
the kernels of the library's steps launched alone) against the reference's
pieces: the stage tendency equals rhs(h2uv(h), q) (jqgm.py:238-262, 321-396,
through vd_qg1l_h2uv / vd_qg1l_rhs, themselves pinned to the reference's own
outputs), and the stage adjoint is the transpose of its linearisation
(central differences, float64)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def _case(seed=3):
    from vardyn_gb300.qg1l import QG1LPlan
    from vardyn_gb300.synthetic import kminus3_ssh
    ny, nx, dx = 40, 52, 5e3
    beta = np.zeros((ny, nx))
    beta[1:-1, :] = 1.6e-11
    plan = QG1LPlan(ny, nx, dx, dx, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=torch.float64, Kdiffus=30.0,
                    beta=beta)
    rng = np.random.default_rng(seed)
    h = torch.as_tensor(np.stack([kminus3_ssh(ny, nx, dx, dx, rng, cutoff_km=20.0) for _ in range(2)]),
                        device="cuda")
    q = plan.h2pv(h, torch.zeros_like(h))
    return plan, h, q, rng


def test_stage_tendency_equals_rhs_of_h2uv():
    plan, h, q, rng = _case()
    base = torch.as_tensor(rng.standard_normal(q.shape), device="cuda")
    k1 = torch.as_tensor(rng.standard_normal(q.shape), device="cuda")
    k = torch.empty_like(q)
    out = plan.rk_stage(h, q, base, k=[k1], c=[0.25], cself=450.0, k_out=k)
    u, v = plan.h2uv(h)
    r = plan.rhs(u, v, q)
    assert float((k - r).abs().max()) <= 1e-14 * float(r.abs().max())
    want = base + 0.25 * k1 + 450.0 * r
    assert float((out - want).abs().max()) <= 1e-13 * float(want.abs().max())


def test_stage_adjoint_is_the_transpose_of_the_tendency():
    plan, h, q, rng = _case(4)
    m3 = torch.as_tensor(plan.mask == 3, device="cuda")
    dh = torch.as_tensor(rng.standard_normal(h.shape), device="cuda") * 1e-3
    dq = torch.as_tensor(rng.standard_normal(q.shape), device="cuda") * 1e-9 * m3
    g = torch.as_tensor(rng.standard_normal(q.shape), device="cuda")
    zero = torch.zeros_like(q)

    def k_of(hh, qq):
        return plan.rk_stage(hh, qq, zero, cself=1.0)

    adq, adh = plan.rk_stage_adj(h, q, g=[g], c=[1.0])
    eps = 1e-3
    dk = (k_of(h + eps * dh, q + eps * dq) - k_of(h - eps * dh, q - eps * dq)) / (2 * eps)
    lhs = float((dk * g).sum())
    rhs = float((dh * adh).sum() + (dq * adq).sum())
    print(f"\nstage tendency transpose: <dk, g> = {lhs:.15e}, <dh, adh> + <dq, adq> = {rhs:.15e}")
    assert abs(lhs - rhs) <= 1e-7 * abs(lhs)
    # the accumulated addends land on the tendency points only
    acc = torch.as_tensor(rng.standard_normal(q.shape), device="cuda")
    adq2, adh2 = plan.rk_stage_adj(h, q, g=[g], c=[1.0], acc=[acc])
    assert torch.allclose(adq2, adq + acc * m3, rtol=1e-14, atol=0)
    assert torch.equal(adh2, adh)
