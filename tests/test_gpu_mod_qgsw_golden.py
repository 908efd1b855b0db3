"""The multilayer model wrapper Model_qgsw (mapping/src/mod.py:2412-3617) on
the GPU against golden vectors from the reference's own class
(tests/golden/gen_golden_qgsw.py): constructor, boundary fields by nearest
time, and the chunked step with forcing and boundary perturbation
parameters, for 1 layer with an island and for 2 layers."""
import datetime
import os
from types import SimpleNamespace as NS

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgsw_golden.npz")
NAMES = {"U": "u", "V": "v", "SSH": "ssh"}
CASES = {
    "a": dict(nl=1, island=True, ny=20, nx=26, dx=4.5e3, dy=4.0e3, dt=15.0, nstep=5, max_nstep=2,
              name_params=["bc"], bc=True),
    "b": dict(nl=2, island=False, ny=18, nx=22, dx=4.5e3, dy=4.0e3, dt=10.0, nstep=4, max_nstep=3,
              name_params=[], bc=False),
}


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


class State:
    def __init__(self, ny, nx, dx, dy, f, mask):
        self.ny, self.nx = ny, nx
        self.DX, self.DY = np.full((ny, nx), dx), np.full((ny, nx), dy)
        self.f, self.mask = f, mask
        self.var, self.params = {}, {}

    def getvar(self, name_var=None):
        return self.var[name_var]

    def setvar(self, var, name_var=None):
        self.var[name_var] = np.asarray(var)


@pytest.mark.parametrize("tag", ["a", "b"])
def test_chunked_step_matches_reference(tag):
    from vardyn_gb300.mod_qgsw import Model_qgsw
    g = dict(np.load(GOLD))
    p = CASES[tag]
    ny, nx, nl = p["ny"], p["nx"], p["nl"]
    yy = np.arange(ny)[:, None] * 4.0e3 + np.zeros((1, nx))
    f = 1.0e-4 + 1.6e-11 * (yy - yy.mean())
    mask = np.zeros((ny, nx), dtype=bool)
    if p["island"]:
        mask[8:12, 10:14] = True
    st = State(ny, nx, p["dx"], p["dy"], f, mask)
    H = [350.0, 750.0, 2900.0][:nl]
    gp = [9.81, 0.025, 0.0125][:nl]
    MOD = NS(name_var=NAMES, nl=nl, name_class="SW", f0=None, constant_f=False, c0=2.7,
             g_prime=np.array(gp) if nl > 1 else gp[0], H=np.array(H) if nl > 1 else H[0], dtmodel=p["dt"],
             cfl=None, bottom_drag_coef=2e-7, slip_coef=0.5, visc_coef=30.0, diff_coef=20.0, sponge_coef=0.0,
             max_nstep=p["max_nstep"], name_params=p["name_params"], init_from_bc=None, rho_water=1025.0,
             h_wind=None, forcing_momentum="direct")
    EXP = NS(init_date=datetime.datetime(2020, 1, 1), final_date=datetime.datetime(2020, 1, 2))
    M = Model_qgsw(NS(MOD=MOD, EXP=EXP, GRID=None), st, dtype=torch.float64)
    assert M.dt == float(g[f"{tag}_dt"])
    for k in [k for k in g if k.startswith(f"{tag}_in_var_")]:
        st.var[k[len(f"{tag}_in_var_"):]] = g[k].copy()
    for k in [k for k in g if k.startswith(f"{tag}_in_par_")]:
        st.params[k[len(f"{tag}_in_par_"):]] = g[k].copy()
    if p["bc"]:
        M.set_bc([0.0, 30.0], {v: list(g[f"{tag}_bc_{v}"]) for v in ("SSH", "U", "V")})
    M.step(st, nstep=p["nstep"], t=0)
    keys = [k for k in g if k.startswith(f"{tag}_out_var_")]
    assert keys
    for k in keys:
        name = k[len(f"{tag}_out_var_"):]
        got, want = np.asarray(st.var[name], dtype=np.float64), g[k]
        err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-300)
        print(f"\nModel_qgsw {tag} {name}: {err:.1e}")
        assert err <= 1e-11, (name, err)
