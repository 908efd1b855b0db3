"""Shallow-water model on the GPU (vd_sw_*) against the reference's own
outputs, finite differences and dot-product tests (the form of the
reference's adjoint_test_sw, sw.py:940-1035)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sw_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def plan_a(g, dtype=torch.float64):
    from vardyn_gb300.sw import SWPlan
    p = "swa_"
    return SWPlan(28, 22, 2, g[p + "dx"], g[p + "dy"], g[p + "f"], g[p + "H"], g[p + "gp"], 15.0, mask=g[p + "mask"],
                  slip_coef=0.5, bottom_drag_coef=2e-7, visc_coef=30.0, diff_coef=20.0, sponge_coef=0.3,
                  taux=g[p + "taux0"], tauy=g[p + "tauy0"], sponge_u=g[p + "sponge_u"], sponge_v=g[p + "sponge_v"],
                  sponge_h=g[p + "sponge_h"], dtype=dtype)


def plan_b(g, dtype=torch.float64):
    from vardyn_gb300.sw import SWPlan
    p = "swb_"
    return SWPlan(24, 26, 1, g[p + "dx"], g[p + "dy"], g[p + "f"], g[p + "H"], g[p + "gp"], 60.0, slip_coef=1.0,
                  bottom_drag_coef=1e-6, h_wind=80.0, forcing_momentum="mass_consistent", h_min=0.05, dtype=dtype)


def T(a, dtype=torch.float64):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else a
    return float(np.abs(a - b).max() / np.abs(b).max())


def to_model(pl, g, p):
    o_m = pl.masks
    dxu = np.pad(g[p + "dx"], ((1, 1), (0, 0)), mode="edge")
    dxu = 0.5 * (dxu[1:] + dxu[:-1])
    dyv = np.pad(g[p + "dy"], ((0, 0), (1, 1)), mode="edge")
    dyv = 0.5 * (dyv[:, 1:] + dyv[:, :-1])
    return (g[p + "u0"] * o_m.u * dxu, g[p + "v0"] * o_m.v * dyv, g[p + "h0"] * o_m.h * g[p + "dx"] * g[p + "dy"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_rhs_matches_reference(g, case):
    pl = plan_a(g) if case == "a" else plan_b(g)
    p = "sw" + case + "_"
    u, v, h = to_model(pl, g, p)
    du, dv, dh = pl.rhs(T(u), T(v), T(h), taux=T(g[p + "taux"]), tauy=T(g[p + "tauy"]))
    assert rel(du, g[p + "dtu"]) < 1e-12
    assert rel(dv, g[p + "dtv"]) < 1e-12
    assert rel(dh, g[p + "dth"]) < 1e-12


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-4)])
def test_step_matches_reference(g, dtype, tol):
    p = "swa_"
    pl = plan_a(g, dtype)
    t = lambda k: T(g[p + k], dtype)
    r = pl.step(t("u0"), t("v0"), t("h0"), nstep=4, ub=t("ub"), vb=t("vb"), hb=t("hb"), Fu=t("Fu"), Fv=t("Fv"),
                Fh=t("Fh"), taux=t("taux"), tauy=t("tauy"))
    for a, k in zip(r, ["u4", "v4", "h4"]):
        assert rel(a, g[p + k]) < tol, k
    r = pl.step(t("u0"), t("v0"), t("h0"), nstep=2)
    for a, k in zip(r, ["u2d", "v2d", "h2d"]):
        assert rel(a, g[p + k]) < tol, k


def test_step_mass_consistent_matches_reference(g):
    p = "swb_"
    pl = plan_b(g)
    t = lambda k: T(g[p + k])
    r = pl.step(t("u0"), t("v0"), t("h0"), nstep=5, Fh=t("Fh"), taux=t("taux"), tauy=t("tauy"))
    for a, k in zip(r, ["u5", "v5", "h5"]):
        assert rel(a, g[p + k]) < 1e-12, k


def test_batch_members_independent(g):
    p = "swa_"
    pl = plan_a(g)
    t = lambda k: T(g[p + k])
    rng = np.random.default_rng(1)
    u2 = torch.cat([t("u0"), t("u0") * 0.5])
    v2 = torch.cat([t("v0"), t("v0") * 0.5])
    h2 = torch.cat([t("h0"), T(rng.standard_normal(g[p + "h0"].shape) * 0.1)])
    r2 = pl.step(u2, v2, h2, nstep=3)
    for b in range(2):
        r1 = pl.step(u2[b:b + 1], v2[b:b + 1], h2[b:b + 1], nstep=3)
        for a, c in zip(r1, r2):
            assert torch.equal(a, c[b:b + 1])


def _rand_like(shape, rng, mask=None):
    a = rng.standard_normal(shape)
    return a if mask is None else a * mask


def _dot(a, b):
    return sum(float((x.double() * y.double()).sum()) for x, y in zip(a, b))


@pytest.mark.parametrize("case", ["a", "b"])
def test_tangent_matches_finite_differences(g, case):
    pl = plan_a(g) if case == "a" else plan_b(g)
    p = "sw" + case + "_"
    t = lambda k: T(g[p + k])
    kw = dict(taux=t("taux"), tauy=t("tauy"))
    if case == "a":
        kw.update(ub=t("ub"), vb=t("vb"), hb=t("hb"), Fu=t("Fu"), Fv=t("Fv"), Fh=t("Fh"))
    else:
        kw.update(Fh=t("Fh"))
    rng = np.random.default_rng(7)
    x = [t("u0"), t("v0"), t("h0")]
    m = pl.masks
    d = [T(_rand_like(a.shape, rng, mk)) * s for a, mk, s in zip(x, (m.u, m.v, m.h), (0.05, 0.05, 0.1))]
    dy = pl.step_tgl(*x, *d, nstep=3, **kw)
    eps = 1e-5
    yp = pl.step(*[a + eps * b for a, b in zip(x, d)], nstep=3, **kw)
    ym = pl.step(*[a - eps * b for a, b in zip(x, d)], nstep=3, **kw)
    for a, b, c in zip(dy, yp, ym):
        fd = ((b - c) / (2 * eps)).cpu().numpy()
        assert rel(a, fd) < 1e-6


@pytest.mark.parametrize("case", ["a", "b"])
def test_adjoint_dot_product(g, case):
    pl = plan_a(g) if case == "a" else plan_b(g)
    p = "sw" + case + "_"
    t = lambda k: T(g[p + k])
    kw = dict(taux=t("taux"), tauy=t("tauy"))
    if case == "a":
        kw.update(ub=t("ub"), vb=t("vb"), hb=t("hb"), Fu=t("Fu"), Fv=t("Fv"), Fh=t("Fh"))
    else:
        kw.update(Fh=t("Fh"))
    rng = np.random.default_rng(11)
    x = [t("u0"), t("v0"), t("h0")]
    m = pl.masks
    d = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, (m.u, m.v, m.h))]
    w = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, (m.u, m.v, m.h))]
    dy = pl.step_tgl(*x, *d, nstep=3, **kw)
    ad = pl.step_adj(*x, *w, nstep=3, **kw)
    lhs = _dot(dy, w)
    rhs = _dot(d, [ad["u0"], ad["v0"], ad["h0"]])
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def test_adjoint_of_forcing_and_sponge_targets(g):
    pl = plan_a(g)
    p = "swa_"
    t = lambda k: T(g[p + k])
    rng = np.random.default_rng(12)
    x = [t("u0"), t("v0"), t("h0")]
    b = [t("ub"), t("vb"), t("hb")]
    F = [t("Fu"), t("Fv"), t("Fh")]
    m = pl.masks
    masks = (m.u, m.v, m.h)
    dx = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, masks)]
    db = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, masks)]
    dF = [T(_rand_like(a.shape, rng, mk)) * 1e-4 for a, mk in zip(x, masks)]
    w = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, masks)]
    kw = dict(taux=t("taux"), tauy=t("tauy"))
    dy = pl.step_tgl(*x, *dx, nstep=2, ub=b[0], vb=b[1], hb=b[2], dub=db[0], dvb=db[1], dhb=db[2], Fu=F[0], Fv=F[1],
                     Fh=F[2], dFu=dF[0], dFv=dF[1], dFh=dF[2], **kw)
    ad = pl.step_adj(*x, *w, nstep=2, ub=b[0], vb=b[1], hb=b[2], Fu=F[0], Fv=F[1], Fh=F[2], want_bc=True,
                     want_forcing=True, **kw)
    lhs = _dot(dy, w)
    rhs = (_dot(dx, [ad["u0"], ad["v0"], ad["h0"]]) + _dot(db, [ad["ub"], ad["vb"], ad["hb"]])
           + _dot(dF, [ad["Fu"], ad["Fv"], ad["Fh"]]))
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def test_float32_adjoint_dot_product(g):
    pl = plan_a(g, torch.float32)
    p = "swa_"
    t = lambda k: T(g[p + k], torch.float32)
    rng = np.random.default_rng(13)
    x = [t("u0"), t("v0"), t("h0")]
    m = pl.masks
    d = [T(_rand_like(a.shape, rng, mk), torch.float32) for a, mk in zip(x, (m.u, m.v, m.h))]
    w = [T(_rand_like(a.shape, rng, mk), torch.float32) for a, mk in zip(x, (m.u, m.v, m.h))]
    dy = pl.step_tgl(*x, *d, nstep=2)
    ad = pl.step_adj(*x, *w, nstep=2)
    lhs, rhs = _dot(dy, w), _dot(d, [ad["u0"], ad["v0"], ad["h0"]])
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_adjoint_is_bit_reproducible(g, dtype):
    """The tendency adjoint runs in two passes without atomics (per-source
    terms, then a fixed-order gather per target), so repeated adjoints agree
    bit for bit (two layers, land, viscosity, diffusion, drag, sponge, wind,
    boundary fields and forcing)."""
    pl = plan_a(g, dtype)
    p = "swa_"
    t = lambda k: T(g[p + k], dtype)
    rng = np.random.default_rng(14)
    x = [t("u0"), t("v0"), t("h0")]
    m = pl.masks
    w = [T(_rand_like(a.shape, rng, mk), dtype) for a, mk in zip(x, (m.u, m.v, m.h))]
    kw = dict(taux=t("taux"), tauy=t("tauy"), ub=t("ub"), vb=t("vb"), hb=t("hb"), Fu=t("Fu"), Fv=t("Fv"),
              Fh=t("Fh"), want_bc=True, want_forcing=True)
    a1 = pl.step_adj(*x, *w, nstep=3, **kw)
    a2 = pl.step_adj(*x, *w, nstep=3, **kw)
    for k in ("u0", "v0", "h0", "ub", "vb", "hb", "Fu", "Fv", "Fh"):
        assert torch.equal(a1[k], a2[k]), k


def test_mass_consistent_adjoint_is_bit_reproducible(g):
    """The mass-consistent forcing adjoint gathers over the replicate-padded
    cells in a fixed order (no atomics): with land next to the forced faces,
    repeated adjoints agree bit for bit."""
    from vardyn_gb300.sw import SWPlan
    p = "swa_"
    pl = SWPlan(28, 22, 2, g[p + "dx"], g[p + "dy"], g[p + "f"], g[p + "H"], g[p + "gp"], 15.0, mask=g[p + "mask"],
                slip_coef=0.5, bottom_drag_coef=2e-7, visc_coef=30.0, diff_coef=20.0,
                forcing_momentum="mass_consistent", dtype=torch.float64)
    t = lambda k: T(g[p + k])
    rng = np.random.default_rng(15)
    x = [t("u0"), t("v0"), t("h0")]
    m = pl.masks
    w = [T(_rand_like(a.shape, rng, mk)) for a, mk in zip(x, (m.u, m.v, m.h))]
    kw = dict(Fh=T(1e-4 * rng.standard_normal(g[p + "h0"].shape)), want_forcing=True)
    a1 = pl.step_adj(*x, *w, nstep=3, **kw)
    a2 = pl.step_adj(*x, *w, nstep=3, **kw)
    for k in ("u0", "v0", "h0", "Fh"):
        assert torch.equal(a1[k], a2[k]), k
