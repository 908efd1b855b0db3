"""Cotangents of the shallow-water step with respect to its H and h_wind
arguments (the H / h_wind entries of jax.vjp in sw.py:924-938, used by
Model_qgsw for the 'H' and 'h_wind' controls, mod.py:3255-3290), checked
against central finite differences of the GPU forward; and the forward with a
perturbed H against the float64 oracle, whose wind depth stays the model's
own H (sw.py:622-630)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NX, NY, NL = 26, 22, 2
DX = 1.0e4
H0 = np.array([150.0, 600.0])
GP = np.array([9.81, 0.03])


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def _f():
    yw = np.arange(NY + 1)[None, :] * DX + np.zeros((NX + 1, 1))
    return 1.0e-4 + 1.0e-11 * (yw - yw.mean())


def _mask():
    m = np.ones((NX, NY))
    m[8:12, 6:10] = 0
    return m


def _kw(**over):
    kw = dict(mask=_mask(), slip_coef=0.5, bottom_drag_coef=1e-6, visc_coef=20.0, diff_coef=10.0, taux=0.05,
              tauy=-0.02, dtype=torch.float64)
    kw.update(over)
    return kw


def _plan(H, **over):
    from vardyn_gb300.sw import SWPlan
    return SWPlan(NX, NY, NL, DX, DX, _f(), H, GP, 30.0, **_kw(**over))


def T(a):
    return torch.as_tensor(np.asarray(a), dtype=torch.float64, device="cuda")


def _state(seed):
    rng = np.random.default_rng(seed)
    m = _mask()
    mu = np.pad(m, ((1, 1), (0, 0)))
    mu = (mu[1:] * mu[:-1])
    mv = np.pad(m, ((0, 0), (1, 1)))
    mv = (mv[:, 1:] * mv[:, :-1])
    return (0.05 * rng.standard_normal((1, NL, NX + 1, NY)) * mu, 0.05 * rng.standard_normal((1, NL, NX, NY + 1)) * mv,
            0.3 * rng.standard_normal((1, NL, NX, NY)) * m)


def _J(pl, x, w, forcing, nstep=3):
    out = pl.step(*map(T, x), nstep=nstep, **forcing)
    return sum(float((a * T(b)).sum()) for a, b in zip(out, w))


def _forcing(seed):
    rng = np.random.default_rng(seed)
    return dict(Fu=T(1e-7 * rng.standard_normal((1, NL, NX + 1, NY))),
                Fv=T(1e-7 * rng.standard_normal((1, NL, NX, NY + 1))),
                Fh=T(1e-6 * rng.standard_normal((1, NL, NX, NY))))


@pytest.mark.parametrize("forcing_momentum", ["direct", "mass_consistent"])
def test_adjoint_wrt_H_matches_finite_differences(forcing_momentum):
    """Per-layer H cotangent through the total thickness, the reference
    pressure gradients (H varies in space) and, with mass-consistent forcing,
    the face thickness of the forcing term; wind depth from the model's H."""
    rng = np.random.default_rng(11)
    Hb = H0.reshape(NL, 1, 1)
    Ht = Hb + 5.0 * rng.standard_normal((NL, NX, NY))
    x, w = _state(1), _state(2)
    F = _forcing(3)
    mk = lambda H: _plan(H, H_wind=Hb, forcing_momentum=forcing_momentum)
    pl = mk(Ht)
    a = pl.step_adj(*map(T, x), *map(T, w), nstep=3, want_ref=True, **F)
    dH = rng.standard_normal((NL, NX, NY))
    # the response to a spatial H is strongly nonlinear (the top layer's
    # pressure gradient scales with g' = 9.81): central differences reach
    # 3e-7 at eps = 1e-3 and 3e-9 at 1e-4
    eps = 1e-4
    fd = (_J(mk(Ht + eps * dH), x, w, F) - _J(mk(Ht - eps * dH), x, w, F)) / (2 * eps)
    ad = float((a["H"] * T(dH)).sum())
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
    assert float(a["h_wind"].abs().max()) == 0.0


def test_adjoint_wrt_h_wind_matches_finite_differences():
    rng = np.random.default_rng(12)
    hw = 60.0 + 10.0 * rng.standard_normal((NX, NY))
    x, w = _state(4), _state(5)
    mk = lambda h: _plan(H0.reshape(NL, 1, 1), h_wind=h)
    a = mk(hw).step_adj(*map(T, x), *map(T, w), nstep=3, want_ref=True)
    d = rng.standard_normal((NX, NY))
    # the wind factor is a smooth 1/H (truncation ~ (eps/60)^2), while the
    # sensitivity is small (tau / (rho H) over three steps): a larger step
    # keeps the differences of J above its round-off
    eps = 1e-2
    fd = (_J(mk(hw + eps * d), x, w, {}) - _J(mk(hw - eps * d), x, w, {})) / (2 * eps)
    ad = float((a["h_wind"] * T(d)).sum())
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def _sw(h_wind=None):
    from vardyn_gb300.model_qgsw.sw import SW
    p = dict(nx=NX, ny=NY, nl=NL, dx=np.full((NX, NY), DX), dy=np.full((NX, NY), DX), f=_f(),
             H=H0.reshape(NL, 1, 1), g_prime=GP, dt=30.0, h_wind=h_wind, **_kw())
    p["dtype"] = "float64"
    return SW(p)


def test_dropin_step_adj_returns_H_and_h_wind_cotangents():
    """SW.step_adj with H (1, nx, ny) and h_wind (nx, ny), as Model_qgsw
    passes them: cotangents summed to those shapes, equal to the plan's."""
    rng = np.random.default_rng(13)
    m = _sw(h_wind=40.0)
    dH = 3.0 * rng.standard_normal((1, NX, NY))
    dhw = 5.0 * rng.standard_normal((NX, NY))
    x, w = _state(6), _state(7)
    r = m.step_adj(*x, *w, H=dH, nstep=2, h_wind=dhw)[0]
    assert r[3].shape == (1, NX, NY) and r[4].shape == (NX, NY)
    pl = _plan(H0.reshape(NL, 1, 1) + dH, h_wind=40.0 + dhw, H_wind=H0.reshape(NL, 1, 1))
    a = pl.step_adj(*map(T, x), *map(T, w), nstep=2, want_ref=True)
    ref_H = a["H"].sum(0, keepdim=True).cpu().numpy()
    assert np.abs(r[3] - ref_H).max() <= 1e-13 * np.abs(ref_H).max()
    assert np.abs(r[4] - a["h_wind"].cpu().numpy()).max() <= 1e-13 * float(a["h_wind"].abs().max())
    # without H / h_wind there is no cotangent, as for jax.vjp of an absent input
    r0 = m.step_adj(*x, *w, nstep=2)[0]
    assert r0[3] is None and r0[4] is None


def test_forward_with_perturbed_H_matches_oracle():
    """The wind depth stays the model's own H when step gets an H
    perturbation (sw.py:622-630); the rest sees H + dH."""
    from oracle.sw import SWOracle
    rng = np.random.default_rng(14)
    dH = 4.0 * rng.standard_normal((1, NX, NY))
    x = _state(8)
    m = _sw()
    got = m.step(*x, H=dH, nstep=3)
    p = dict(nx=NX, ny=NY, nl=NL, dx=np.full((NX, NY), DX), dy=np.full((NX, NY), DX), f=_f(),
             H=H0.reshape(NL, 1, 1), g_prime=GP, dt=30.0, mask=_mask(), slip_coef=0.5, bottom_drag_coef=1e-6,
             visc_coef=20.0, diff_coef=10.0, taux=0.05, tauy=-0.02)
    o = SWOracle(p)
    exp = o.step(*x, H=dH, nstep=3)
    for a, b in zip(got, exp):
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()


def test_dropin_H_and_h_wind_steps_match_reference():
    """The drop-in SW.step with the per-call H and h_wind arguments against
    the reference's own sw.py outputs (non-uniform metrics, land)."""
    import os
    from vardyn_gb300.model_qgsw.sw import SW
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "sw_golden.npz")))
    p = "swh_"
    base = dict(nx=26, ny=20, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
                taux=0.08, tauy=-0.05, bottom_drag_coef=1e-6, dt=20.0, mask=g[p + "mask"], slip_coef=0.5,
                visc_coef=20.0, diff_coef=10.0, dtype="float64")
    r = SW(dict(base)).step(g[p + "u0"], g[p + "v0"], g[p + "h0"], H=g[p + "dH"], nstep=3)
    for a, k in zip(r, ("uH", "vH", "hH")):
        assert np.abs(a - g[p + k]).max() <= 1e-11 * np.abs(g[p + k]).max(), k
    r = SW(dict(base, h_wind=50.0)).step(g[p + "u0"], g[p + "v0"], g[p + "h0"], nstep=3, h_wind=g[p + "hw"])
    for a, k in zip(r, ("uW", "vW", "hW")):
        assert np.abs(a - g[p + k]).max() <= 1e-11 * np.abs(g[p + k]).max(), k


def _tl_J(pl, x, dx, w, forcing, nstep=3, **d):
    out = pl.step_tgl(*map(T, x), *map(T, dx), nstep=nstep, **forcing, **d)
    return sum(float((a * T(b)).sum()) for a, b in zip(out, w))


@pytest.mark.parametrize("forcing_momentum", ["direct", "mass_consistent"])
def test_tangent_wrt_H_matches_finite_differences(forcing_momentum):
    """The tangent of the step in a spatial, per-layer H (the H entry of
    jax.jvp, sw.py:906-922) against central differences of the forward, with
    the state tangent zero; wind depth from the model's H."""
    rng = np.random.default_rng(31)
    Hb = H0.reshape(NL, 1, 1)
    Ht = Hb + 5.0 * rng.standard_normal((NL, NX, NY))
    x, w = _state(8), _state(9)
    F = _forcing(10)
    mk = lambda H: _plan(H, H_wind=Hb, forcing_momentum=forcing_momentum)
    dH = rng.standard_normal((NL, NX, NY))
    zero = tuple(np.zeros_like(a) for a in x)
    tl = _tl_J(mk(Ht), x, zero, w, F, dH=dH)
    # strongly nonlinear in H: central differences reach ~3e-9 at eps = 1e-4
    eps = 1e-4
    fd = (_J(mk(Ht + eps * dH), x, w, F) - _J(mk(Ht - eps * dH), x, w, F)) / (2 * eps)
    assert abs(tl - fd) <= 1e-6 * abs(fd), (tl, fd)


@pytest.mark.parametrize("h_wind", ["field", "scalar"])
def test_tangent_wrt_h_wind_matches_finite_differences(h_wind):
    rng = np.random.default_rng(32)
    hw = 60.0 + 10.0 * rng.standard_normal((NX, NY)) if h_wind == "field" else 55.0
    d = rng.standard_normal((NX, NY)) if h_wind == "field" else 1.0
    x, w = _state(11), _state(12)
    mk = lambda h: _plan(H0.reshape(NL, 1, 1), h_wind=h)
    zero = tuple(np.zeros_like(a) for a in x)
    tl = _tl_J(mk(hw), x, zero, w, {}, dh_wind=d)
    eps = 1e-2
    fd = (_J(mk(hw + eps * d), x, w, {}) - _J(mk(hw - eps * d), x, w, {})) / (2 * eps)
    assert abs(tl - fd) <= 1e-6 * abs(fd), (tl, fd)


def test_tangent_and_adjoint_wrt_H_and_h_wind_are_transposes():
    """<TL(dx, dH, dh_wind), w> = <dx, adj_x(w)> + <dH, adj_H(w)> +
    <dh_wind, adj_h_wind(w)> to rounding, with forcing and mass-consistent
    momentum forcing on."""
    rng = np.random.default_rng(33)
    Hb = H0.reshape(NL, 1, 1)
    Ht = Hb + 5.0 * rng.standard_normal((NL, NX, NY))
    hw = 60.0 + 10.0 * rng.standard_normal((NX, NY))
    pl = _plan(Ht, H_wind=Hb, h_wind=hw, forcing_momentum="mass_consistent")
    x, dx, w = _state(13), _state(14), _state(15)
    F = _forcing(16)
    dH = rng.standard_normal((NL, NX, NY))
    dhw = rng.standard_normal((NX, NY))
    lhs = _tl_J(pl, x, dx, w, F, dH=dH, dh_wind=dhw)
    a = pl.step_adj(*map(T, x), *map(T, w), nstep=3, want_ref=True, **F)
    rhs = sum(float((a[k] * T(b)).sum()) for k, b in zip(("u0", "v0", "h0"), dx))
    rhs += float((a["H"] * T(dH)).sum()) + float((a["h_wind"] * T(dhw)).sum())
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs), (lhs, rhs)
    # the tangent tables are unregistered after the call: a plain tangent
    # again ignores H / h_wind
    plain = _tl_J(pl, x, dx, w, F)
    rhs0 = sum(float((a[k] * T(b)).sum()) for k, b in zip(("u0", "v0", "h0"), dx))
    assert abs(plain - rhs0) <= 1e-11 * abs(plain), (plain, rhs0)


def test_dropin_step_tgl_with_H_and_h_wind_tangents():
    """SW.step_tgl with H / dH (1, nx, ny) and h_wind / dh_wind (nx, ny), as
    Model_qgsw passes them, equals the plan's tangent at H + dH-base."""
    rng = np.random.default_rng(34)
    m = _sw(h_wind=40.0)
    Hp = 3.0 * rng.standard_normal((1, NX, NY))
    hwp = 5.0 * rng.standard_normal((NX, NY))
    dH = rng.standard_normal((1, NX, NY))
    dhw = rng.standard_normal((NX, NY))
    x, dx = _state(17), _state(18)
    r = m.step_tgl(*x, *dx, H=Hp, dH=dH, nstep=2, h_wind=hwp, dh_wind=dhw)
    pl = _plan(H0.reshape(NL, 1, 1) + Hp, h_wind=40.0 + hwp, H_wind=H0.reshape(NL, 1, 1))
    ref = pl.step_tgl(*map(T, x), *map(T, dx), nstep=2, dH=np.broadcast_to(dH, (NL, NX, NY)), dh_wind=dhw)
    for a, b in zip(r, ref):
        b = b.cpu().numpy()
        assert np.abs(np.asarray(a) - b).max() <= 1e-13 * np.abs(b).max()
    r0 = m.step_tgl(*x, *dx, H=Hp, nstep=2, h_wind=hwp)
    assert max(float(np.abs(np.asarray(a) - b.cpu().numpy()).max()) for a, b in zip(r0, ref)) > 0.0
