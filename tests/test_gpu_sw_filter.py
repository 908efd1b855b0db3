"""The shallow-water model's spectral barotropic filter on the GPU
(sw.py:305-320, 720-750; the Neumann solve of helmholtz.py:187-303):
the solve and the model against the reference's own outputs
(tests/golden/swfilter_golden.npz), the oracle on a non-uniform grid with 3
layers and 2 batch members, central differences of the tangent-linear and
dot products of the adjoint, including the cotangent of H. The same kernel
sources pass the same checks under the host emulation
(tests/test_sw_emulated.py)."""
import os

import numpy as np
import pytest
import torch

from oracle.sw import SWOracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "swfilter_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def T(a, dtype=torch.float64):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else a
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else b
    return float(np.abs(a - b).max() / np.abs(b).max())


def ref_solve(rhs, helm):
    import scipy.fft as sf
    r = sf.dct(sf.dct(rhs, type=2, axis=-1), type=2, axis=-2)
    return sf.idct(sf.idct(r / helm, type=2, axis=-1), type=2, axis=-2)


@pytest.mark.parametrize("nx,ny,nf", [(24, 20, 1), (14, 22, 3), (9, 15, 2), (64, 48, 5), (1024, 768, 2),
                                      (11, 13, 1)])
def test_neumann_solve(nx, ny, nf):
    from vardyn_gb300.helmholtz_neumann import HelmholtzNeumannSolver
    rng = np.random.default_rng(nx + 7 * ny)
    dx = 1e4 * (1 + 0.2 * rng.random((nx, ny)))
    dy = 1.3e4 * (1 + 0.2 * rng.random((nx, ny)))
    lam = 1e-9 * (1 + rng.random((nx, ny)))
    rhs = rng.standard_normal((nf, nx, ny))
    for dtype, tol in ((torch.float64, 1e-12), (torch.float32, 3e-5)):
        s = HelmholtzNeumannSolver(nx, ny, dx, dy, lam, dtype=dtype)
        want = ref_solve(rhs, s.helmholtz_dctII.double().cpu().numpy())
        out = s.solve(T(rhs, dtype))
        assert rel(out.double(), want) < tol, (dtype, rel(out.double(), want))


def test_neumann_golden(g):
    from vardyn_gb300.helmholtz_neumann import HelmholtzNeumannSolver
    lam = 1.0 / (g["fa_gp"][0] * 30.0 * 60.0 * g["fa_H"].sum(axis=-3, keepdims=True))
    s = HelmholtzNeumannSolver(24, 20, g["fa_dx"], g["fa_dy"], lam)
    assert rel(s.helmholtz_dctII, g["fa_helm_dct"][0]) < 1e-14
    assert rel(s.solve(g["fa_rhs"]), g["fa_sol"]) < 1e-12


def _gparam(g, **over):
    p = "fa_"
    d = dict(nx=24, ny=20, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
             taux=0.05, tauy=-0.03, bottom_drag_coef=1e-6, dt=30.0, slip_coef=0.5, visc_coef=10.0, diff_coef=5.0,
             barotropic_filter=True, barotropic_filter_spectral=True)
    d.update(over)
    return d


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 3e-5)])
def test_model_golden(g, dtype, tol):
    from vardyn_gb300.model_qgsw.sw import SW
    sw = SW(_gparam(g, dtype=dtype))
    r = sw.step(g["fa_u0"], g["fa_v0"], g["fa_h0"], nstep=3)
    for a, k in zip(r, ["u3", "v3", "h3"]):
        assert rel(np.asarray(a, dtype=np.float64), g["fa_" + k]) < tol, k
    if dtype == torch.float64:
        pl = sw._plan()
        o = SWOracle(_gparam(g))
        u, v, h = o.to_model(g["fa_u0"], g["fa_v0"], g["fa_h0"])
        du, dv, dh = pl.rhs(T(u), T(v), T(h))
        assert rel(du, g["fa_dtu"]) < 1e-12 and rel(dv, g["fa_dtv"]) < 1e-12 and rel(dh, g["fa_dth"]) < 1e-12


def test_refusals(g):
    from vardyn_gb300.model_qgsw.sw import SW
    with pytest.raises(NotImplementedError):
        SW(_gparam(g, barotropic_filter_spectral=False))
    mask = np.ones((24, 20))
    mask[8:12, 7:11] = 0
    with pytest.raises(NotImplementedError):
        SW(_gparam(g, mask=mask))


def _case(B=2, seed=5):
    nx, ny, nl = 14, 10, 3
    rng = np.random.default_rng(seed)
    dx = 2e3 * (1 + 0.15 * rng.random((nx, ny)))
    dy = 2.5e3 * (1 + 0.15 * rng.random((nx, ny)))
    f = 1e-4 + 2e-11 * np.arange(ny + 1)[None, :] * 2.5e3 + np.zeros((nx + 1, 1))
    H = np.array([150.0, 350.0, 800.0]).reshape(nl, 1, 1)
    prm = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=np.array([9.81, 0.02, 0.01]), f=f, taux=0.04,
               tauy=-0.02, bottom_drag_coef=2e-6, dt=20.0, slip_coef=0.7, visc_coef=5.0, diff_coef=2.0,
               barotropic_filter=True, barotropic_filter_spectral=True)
    o = SWOracle(prm)
    m = o.masks
    x = (0.05 * rng.standard_normal((B, nl, nx + 1, ny)) * m.u, 0.05 * rng.standard_normal((B, nl, nx, ny + 1)) * m.v,
         0.4 * rng.standard_normal((B, nl, nx, ny)))
    return prm, o, x, rng


def test_steps_vs_oracle():
    from vardyn_gb300.model_qgsw.sw import SW
    prm, o, x, _ = _case()
    r = SW(prm).step(*x, nstep=4)
    want = o.step(*x, nstep=4)
    for a, b, k in zip(r, want, "uvh"):
        assert rel(np.asarray(a), b) < 1e-11, k


def test_tangent_adjoint_and_H():
    from vardyn_gb300.model_qgsw.sw import SW
    prm, o, x, rng = _case()
    sw = SW(prm)
    pl = sw._plan()
    m = o.masks
    tx = [T(a) for a in x]
    dx = [T(0.01 * rng.standard_normal(x[0].shape) * m.u), T(0.01 * rng.standard_normal(x[1].shape) * m.v),
          T(0.1 * rng.standard_normal(x[2].shape))]
    n = 3
    tl = pl.step_tgl(*tx, *dx, nstep=n)
    eps = 1e-5
    p = pl.step(*[a + eps * b for a, b in zip(tx, dx)], nstep=n)
    q = pl.step(*[a - eps * b for a, b in zip(tx, dx)], nstep=n)
    for t, a, b, k in zip(tl, p, q, "uvh"):
        assert rel(t, (a - b) / (2 * eps)) < 1e-6, k
    a1 = [T(rng.standard_normal(tuple(t.shape))) for t in tl]
    ad = pl.step_adj(*tx, *a1, nstep=n, want_ref=True)
    lhs = sum(float((t * a).sum()) for t, a in zip(tl, a1))
    rhs = sum(float((d * ad[k]).sum()) for d, k in zip(dx, ("u0", "v0", "h0")))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
    # H: the adjoint's cotangent against the tangent with respect to H. The
    # model's H has unit spatial axes, so its cotangent is that of per-layer
    # thicknesses (the reference pressure gradients are then the constant 0,
    # sw.py:403-404): the direction is constant in space.
    dH = np.broadcast_to(rng.standard_normal((prm["nl"], 1, 1)), (prm["nl"], prm["nx"], prm["ny"])).copy()
    zero = [torch.zeros_like(a) for a in tx]
    tlH = pl.step_tgl(*tx, *zero, nstep=n, dH=dH)
    lhs = sum(float((t * a).sum()) for t, a in zip(tlH, a1))
    rhs = float((ad["H"].double().cpu() * torch.as_tensor(dH)).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-10
