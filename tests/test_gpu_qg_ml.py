"""Multilayer QG model on the GPU (SW tendencies projected by the vd_qgp
kernels around the spectral Helmholtz solves) against the reference's own
projector outputs, the float64 oracle, finite differences and dot-product
tests."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sw_golden.npz")
NX, NY, NL = 32, 24, 3


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def params(g, island, **kw):
    yw = np.arange(NY + 1)[None, :] * 5.0e3 + np.zeros((NX + 1, 1))
    f = 1.0e-4 + 1.6e-11 * (yw - yw.mean())
    p = dict(nx=NX, ny=NY, nl=NL, dx=5.0e3, dy=5.0e3, f=f, H=np.array([350.0, 750.0, 2900.0]),
             g_prime=np.array([9.81, 0.025, 0.0125]), dt=600.0)
    if island:
        p["mask"] = g["qgi_mask"]
    p.update(kw)
    return p


def plan(g, island, dtype=torch.float64, **kw):
    from vardyn_gb300.qg_ml import QGPlan
    return QGPlan(dtype=dtype, **params(g, island, **kw))


def T(a, dtype=torch.float64):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else a
    return float(np.abs(a - b).max() / np.abs(b).max())


def _dot(a, b):
    return sum(float((x.double() * y.double()).sum()) for x, y in zip(a, b))


@pytest.mark.parametrize("island", [False, True])
def test_projector_matches_reference(g, island):
    pre = "qgi_" if island else "qg_"
    q = plan(g, island)
    assert q.cmm == island
    assert rel(q.homsol, g[pre + "homsol"][0]) < 1e-12
    P = q.project(T(g[pre + "u"]), T(g[pre + "v"]), T(g[pre + "h"]))
    for a, k in zip(P, ["Pu", "Pv", "Ph"]):
        assert rel(a, g[pre + k]) < 1e-11, k


@pytest.mark.parametrize("island", [False, True])
def test_projector_transpose(g, island):
    q = plan(g, island)
    rng = np.random.default_rng(3)
    m = q.masks
    shapes = [(2, NL, NX + 1, NY), (2, NL, NX, NY + 1), (2, NL, NX, NY)]
    x = [T(rng.standard_normal(s) * mk) for s, mk in zip(shapes, (m.u, m.v, m.h))]
    y = [T(rng.standard_normal(s)) for s in shapes]
    Px = q.project(*x)
    Pty = q.project_adj(*y)
    lhs, rhs = _dot(Px, y), _dot(x, Pty)
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def _state(rng, q, B=1):
    m = q.masks
    return (T(0.05 * rng.standard_normal((B, NL, NX + 1, NY)) * m.u),
            T(0.05 * rng.standard_normal((B, NL, NX, NY + 1)) * m.v),
            T(0.2 * rng.standard_normal((B, NL, NX, NY)) * m.h))


@pytest.mark.parametrize("island", [False, True])
def test_step_matches_oracle(g, island):
    from oracle.qg_ml import QGOracle
    kw = dict(bottom_drag_coef=1e-7, visc_coef=20.0, diff_coef=10.0, slip_coef=0.7, taux=0.02, tauy=-0.01)
    q = plan(g, island, **kw)
    p = params(g, island, **kw)
    p["dx"] = np.full((NX, NY), 5.0e3)
    p["dy"] = np.full((NX, NY), 5.0e3)
    p["H"] = p["H"].reshape(NL, 1, 1)
    o = QGOracle(p)
    rng = np.random.default_rng(21)
    u, v, h = _state(rng, q)
    r = q.step(u, v, h, nstep=2)
    ro = o.step(u.cpu().numpy(), v.cpu().numpy(), h.cpu().numpy(), nstep=2)
    for a, b in zip(r, ro):
        assert rel(a, b) < 1e-10


@pytest.mark.parametrize("island", [False, True])
def test_tangent_and_adjoint(g, island):
    q = plan(g, island, bottom_drag_coef=1e-7, visc_coef=20.0, diff_coef=10.0)
    rng = np.random.default_rng(31)
    x = _state(rng, q)
    d = _state(rng, q)
    w = _state(rng, q)
    eps = 1e-5
    dy = q.step_tgl(*x, *d, nstep=2)
    yp = q.step(*[a + eps * b for a, b in zip(x, d)], nstep=2)
    ym = q.step(*[a - eps * b for a, b in zip(x, d)], nstep=2)
    for a, b, c in zip(dy, yp, ym):
        assert rel(a, ((b - c) / (2 * eps)).cpu().numpy()) < 1e-6
    ad = q.step_adj(*x, *w, nstep=2)
    lhs, rhs = _dot(dy, w), _dot(d, [ad["u0"], ad["v0"], ad["h0"]])
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
