"""The shallow-water model with open boundaries (flag_obc, sw.py:353-371) on
the GPU against the reference's own outputs (tests/golden/swobc_golden.npz:
the face masks, the right-hand side and a 4-step run with land, sponge,
boundary fields and forcing), with the tangent against central differences
and the adjoint by dot products."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "swobc_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return float(np.abs(a - b).max() / np.abs(b).max())


def model(g):
    from vardyn_gb300.model_qgsw.sw import SW
    p = "ob_"
    sw = SW(dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"],
                 f=g[p + "f"], taux=0.04, tauy=-0.02, bottom_drag_coef=1e-6, dt=20.0, mask=g[p + "mask"],
                 slip_coef=0.6, visc_coef=20.0, diff_coef=10.0, sponge_coef=0.2, flag_obc=True))
    sw.sponge_u, sw.sponge_v, sw.sponge_h = g[p + "sponge_u"], g[p + "sponge_v"], g[p + "sponge_h"]
    return sw


def test_open_boundaries_match_reference(g):
    sw = model(g)
    assert np.array_equal(sw.masks.u[0, 0], g["ob_mask_u"]) and np.array_equal(sw.masks.v[0, 0], g["ob_mask_v"])
    r = sw.step(g["ob_u0"], g["ob_v0"], g["ob_h0"], nstep=4, u_b=g["ob_ub"], v_b=g["ob_vb"], h_b=g["ob_hb"],
                Fu=g["ob_Fu"], Fv=g["ob_Fv"], Fh=g["ob_Fh"])
    for a, k in zip(r, ("u4", "v4", "h4")):
        assert rel(a, g["ob_" + k]) < 1e-12, k


def test_open_boundaries_tangent_adjoint(g):
    sw = model(g)
    pl = sw._plan()
    rng = np.random.default_rng(3)
    T = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda")
    x = [T(g["ob_" + k]) for k in ("u0", "v0", "h0")]
    dx = [T(0.01 * rng.standard_normal(tuple(a.shape))) for a in x]
    tl = pl.step_tgl(*x, *dx, nstep=2)
    eps = 1e-6
    p = pl.step(*[a + eps * b for a, b in zip(x, dx)], nstep=2)
    q = pl.step(*[a - eps * b for a, b in zip(x, dx)], nstep=2)
    for t, a, b in zip(tl, p, q):
        assert rel(t, ((a - b) / (2 * eps)).cpu().numpy()) < 1e-6
    a1 = [T(rng.standard_normal(tuple(t.shape))) for t in tl]
    ad = pl.step_adj(*x, *a1, nstep=2)
    lhs = sum(float((t * a).sum()) for t, a in zip(tl, a1))
    rhs = sum(float((d * ad[k]).sum()) for d, k in zip(dx, ("u0", "v0", "h0")))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
