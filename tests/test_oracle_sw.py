"""Shallow-water oracle (restatement of sw.py and helpers) and the library's
host mask builder against outputs of the reference's own sw.py."""
import os

import numpy as np
import pytest

from oracle.sw import SWOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sw_golden.npz")
MASKS = ["u", "v", "w", "psi", "w_valid", "w_cornerout_bound", "w_vertical_bound", "w_horizontal_bound",
         "u_sten_hx_eq2", "u_sten_hx_eq4", "u_sten_hx_gt6", "u_sten_wy_eq2", "u_sten_wy_eq4", "u_sten_wy_gt4",
         "v_sten_hy_eq2", "v_sten_hy_eq4", "v_sten_hy_gt6", "v_sten_wx_eq2", "v_sten_wx_eq4", "v_sten_wx_gt6"]


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def param_a(g):
    p = "swa_"
    return dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
                taux=g[p + "taux0"], tauy=g[p + "tauy0"], bottom_drag_coef=2e-7, dt=15.0, mask=g[p + "mask"],
                slip_coef=0.5, visc_coef=30.0, diff_coef=20.0, sponge_coef=0.3)


def param_b(g):
    p = "swb_"
    return dict(nx=24, ny=26, nl=1, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
                taux=0.0, tauy=0.0, bottom_drag_coef=1e-6, dt=60.0, slip_coef=1.0, visc_coef=0.0, diff_coef=0.0,
                h_wind=80.0, forcing_momentum="mass_consistent", h_min=0.05)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_oracle_masks(g):
    o = SWOracle(param_a(g))
    m = o.masks
    ours = dict(u=m.u, v=m.v, w=m.w, psi=m.psi, w_valid=m.w_valid, w_cornerout_bound=m.w_cornerout_bound,
                w_vertical_bound=m.w_vertical_bound, w_horizontal_bound=m.w_horizontal_bound)
    for k, a in zip(["hx_eq2", "hx_eq4", "hx_gt6"], m.u_hx):
        ours["u_sten_" + k] = a
    for k, a in zip(["wy_eq2", "wy_eq4", "wy_gt4"], m.u_wy):
        ours["u_sten_" + k] = a
    for k, a in zip(["hy_eq2", "hy_eq4", "hy_gt6"], m.v_hy):
        ours["v_sten_" + k] = a
    for k, a in zip(["wx_eq2", "wx_eq4", "wx_gt6"], m.v_wx):
        ours["v_sten_" + k] = a
    for name in MASKS:
        assert np.array_equal(np.asarray(ours[name], float), g["swa_mask_" + name]), name
    assert np.array_equal(m.irr_x, g["swa_irr_x"]) and np.array_equal(m.irr_y, g["swa_irr_y"])


def test_library_host_masks(g):
    from vardyn_gb300.sw import SWMasks
    m = SWMasks(28, 22, g["swa_mask"])
    for name in MASKS:
        assert np.array_equal(getattr(m, name), g["swa_mask_" + name]), name
    assert np.array_equal(m.psi_irrbound_xids, g["swa_irr_x"])
    assert np.array_equal(m.psi_irrbound_yids, g["swa_irr_y"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_oracle_rhs(g, case):
    p = "sw" + case + "_"
    o = SWOracle(param_a(g) if case == "a" else param_b(g))
    u, v, h = o.to_model(g[p + "u0"], g[p + "v0"], g[p + "h0"])
    du, dv, dh = o.rhs(u, v, h, o.ref_values(o.H), g[p + "taux"], g[p + "tauy"])
    assert rel(du, g[p + "dtu"]) < 1e-13 and rel(dv, g[p + "dtv"]) < 1e-13 and rel(dh, g[p + "dth"]) < 1e-13


def test_oracle_steps(g):
    p = "swa_"
    o = SWOracle(param_a(g))
    o.sponge_u, o.sponge_v, o.sponge_h = g[p + "sponge_u"][0, 0], g[p + "sponge_v"][0, 0], g[p + "sponge_h"][0, 0]
    r = o.step(g[p + "u0"], g[p + "v0"], g[p + "h0"], nstep=4, u_b=g[p + "ub"], v_b=g[p + "vb"], h_b=g[p + "hb"],
               Fu=g[p + "Fu"], Fv=g[p + "Fv"], Fh=g[p + "Fh"], taux=g[p + "taux"], tauy=g[p + "tauy"])
    for a, k in zip(r, ["u4", "v4", "h4"]):
        assert rel(a, g[p + k]) < 1e-13
    r = o.step(g[p + "u0"], g[p + "v0"], g[p + "h0"], nstep=2)
    for a, k in zip(r, ["u2d", "v2d", "h2d"]):
        assert rel(a, g[p + k]) < 1e-13
    p = "swb_"
    o = SWOracle(param_b(g))
    r = o.step(g[p + "u0"], g[p + "v0"], g[p + "h0"], nstep=5, Fh=g[p + "Fh"], taux=g[p + "taux"], tauy=g[p + "tauy"])
    for a, k in zip(r, ["u5", "v5", "h5"]):
        assert rel(a, g[p + k]) < 1e-13


def param_h(g, **over):
    p = "swh_"
    d = dict(nx=26, ny=20, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
             taux=0.08, tauy=-0.05, bottom_drag_coef=1e-6, dt=20.0, mask=g[p + "mask"], slip_coef=0.5,
             visc_coef=20.0, diff_coef=10.0)
    d.update(over)
    return d


def test_oracle_step_with_H_and_h_wind_arguments(g):
    """SW.step(H=dH) (the wind depth stays the model's own H, sw.py:622-630)
    and SW.step(h_wind=field) on a model whose h_wind is a scalar (the two
    add, sw.py:810-817), on non-uniform metrics."""
    p = "swh_"
    o = SWOracle(param_h(g))
    r = o.step(g[p + "u0"], g[p + "v0"], g[p + "h0"], H=g[p + "dH"], nstep=3)
    for a, k in zip(r, ("uH", "vH", "hH")):
        assert rel(a, g[p + k]) < 1e-12, k
    o = SWOracle(param_h(g, h_wind=50.0 + g[p + "hw"]))
    r = o.step(g[p + "u0"], g[p + "v0"], g[p + "h0"], nstep=3)
    for a, k in zip(r, ("uW", "vW", "hW")):
        assert rel(a, g[p + k]) < 1e-12, k
