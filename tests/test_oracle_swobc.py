"""The oracle's shallow-water model with open boundaries (flag_obc,
sw.py:353-371) against outputs of the reference's own sw.py
(tests/golden/gen_golden_swobc.py): the face masks, the right-hand side and a
4-step run with land, sponge, boundary fields and forcing."""
import os

import numpy as np
import pytest

from oracle.sw import SWOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "swobc_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def param(g, **over):
    p = "ob_"
    d = dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
             taux=0.04, tauy=-0.02, bottom_drag_coef=1e-6, dt=20.0, mask=g[p + "mask"], slip_coef=0.6,
             visc_coef=20.0, diff_coef=10.0, sponge_coef=0.2, flag_obc=True)
    d.update(over)
    return d


def oracle(g, **over):
    o = SWOracle(param(g, **over))
    o.sponge_u = g["ob_sponge_u"].reshape(29, 22)
    o.sponge_v = g["ob_sponge_v"].reshape(28, 23)
    o.sponge_h = g["ob_sponge_h"].reshape(28, 22)
    return o


def rel(a, b):
    return np.abs(np.asarray(a) - b).max() / np.abs(b).max()


def test_masks(g):
    o = oracle(g)
    assert np.array_equal(o.masks.u, g["ob_mask_u"]) and np.array_equal(o.masks.v, g["ob_mask_v"])
    # the walls are open, land included
    assert o.masks.u[0].min() == 1 and o.masks.v[:, -1].min() == 1


def test_rhs_and_steps(g):
    o = oracle(g)
    u, v, h = o.to_model(g["ob_u0"], g["ob_v0"], g["ob_h0"])
    du, dv, dh = o.rhs(u, v, h, o.ref_values(o.H), o.taux, o.tauy)
    assert rel(du, g["ob_dtu"]) < 1e-12 and rel(dv, g["ob_dtv"]) < 1e-12 and rel(dh, g["ob_dth"]) < 1e-12
    r = o.step(g["ob_u0"], g["ob_v0"], g["ob_h0"], nstep=4, u_b=g["ob_ub"], v_b=g["ob_vb"], h_b=g["ob_hb"],
               Fu=g["ob_Fu"], Fv=g["ob_Fv"], Fh=g["ob_Fh"])
    for a, k in zip(r, ("u4", "v4", "h4")):
        assert rel(a, g["ob_" + k]) < 1e-12, k
    # open walls change the run (the boundary velocities enter the diagnostics)
    c = oracle(g, flag_obc=False).step(g["ob_u0"], g["ob_v0"], g["ob_h0"], nstep=4, u_b=g["ob_ub"],
                                       v_b=g["ob_vb"], h_b=g["ob_hb"], Fu=g["ob_Fu"], Fv=g["ob_Fv"], Fh=g["ob_Fh"])
    assert rel(c[0], g["ob_u4"]) > 1e-3


def test_library_host_masks(g):
    """The library's host mask builder with open boundaries (no GPU): the
    face masks equal the reference's."""
    from vardyn_gb300.sw import SWMasks
    m = SWMasks(28, 22, g["ob_mask"], obc=True)
    assert np.array_equal(m.u, g["ob_mask_u"]) and np.array_equal(m.v, g["ob_mask_v"])
    c = SWMasks(28, 22, g["ob_mask"])
    assert not np.array_equal(c.u, g["ob_mask_u"])
