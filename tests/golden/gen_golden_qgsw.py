"""Generate golden vectors for the multilayer model wrapper ``Model_qgsw``
(mapping/src/mod.py:2412-3617) from the reference's own source: its
constructor (reduced gravities, layer thicknesses, time step, State
variables and parameters, the SW model built from ``model_qgsw/sw.py``),
``set_bc`` / ``_apply_bc`` (boundary fields by nearest time), and the chunked
``step`` (mod.py:3292-3358: State <-> model layout, forcing per day, boundary
perturbation parameters, chunks of ``max_nstep`` steps, the surface fields
diagnosed from the layers).

Everything runs unmodified from the reference checkout under the NumPy
stand-in for jax (float64); the model files are loaded by the wrapper's own
``SourceFileLoader`` calls from ``config.MOD.dir_model``. The tangent and
adjoint of the wrapper wrap ``jax.jvp`` / ``jax.vjp`` (mod.py:3360-3617),
which the stand-in does not provide, so only the forward is recorded. QG
cannot step in the reference as shipped (``SW.step`` passes arguments
``QG.compute_time_derivatives`` does not take), so the cases are SW.

Cases:
- ``a``: 1 layer, an island, 'bc' perturbation parameters, 5 steps in
  chunks of 2, boundary fields at two times, forcing on u, v and SSH;
- ``b``: 2 layers, no land, 4 steps in chunks of 3, no boundary fields.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_qgsw.py <VarDyn checkout>
Writes ``tests/golden/qgsw_golden.npz``.
"""
import datetime
import os
import sys
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden_fourdvar import load_all  # noqa: E402

NAMES = {"U": "u", "V": "v", "SSH": "ssh"}


class State:
    """The State methods Model_qgsw uses (getvar / setvar on var dicts)."""

    def __init__(self, ny, nx, dx, dy, f, mask):
        self.ny, self.nx = ny, nx
        self.DX, self.DY = np.full((ny, nx), dx), np.full((ny, nx), dy)
        self.X = self.Y = None
        self.f, self.mask = f, mask
        self.lon_unit = "-180_180"
        self.var, self.params = {}, {}

    def getvar(self, name_var=None):
        return self.var[name_var]

    def setvar(self, var, name_var=None):
        self.var[name_var] = np.asarray(var)


CASES = {
    "a": dict(nl=1, island=True, ny=20, nx=26, dx=4.5e3, dy=4.0e3, dt=15.0, nstep=5, max_nstep=2,
              name_params=["bc"], bc=True, seed=5),
    "b": dict(nl=2, island=False, ny=18, nx=22, dx=4.5e3, dy=4.0e3, dt=10.0, nstep=4, max_nstep=3,
              name_params=[], bc=False, seed=6),
}


def run_case(tag, p, mod, ref_root, out):
    ny, nx, nl = p["ny"], p["nx"], p["nl"]
    yy = np.arange(ny)[:, None] * 4.0e3 + np.zeros((1, nx))
    f = 1.0e-4 + 1.6e-11 * (yy - yy.mean())
    mask = np.zeros((ny, nx), dtype=bool)   # True = land
    if p["island"]:
        mask[8:12, 10:14] = True
    st = State(ny, nx, p["dx"], p["dy"], f.copy(), mask)
    H = [350.0, 750.0, 2900.0][:nl]
    gp = [9.81, 0.025, 0.0125][:nl]
    MOD = NS(dir_model=os.path.join(ref_root, "mapping", "models", "model_qgsw"), name_var=NAMES, var_to_save=None,
             nl=nl, name_class="SW", f0=None, constant_f=False, c0=2.7, path_mdt=None, filec_aux=None,
             g_prime=np.array(gp) if nl > 1 else gp[0], H=np.array(H) if nl > 1 else H[0], dtmodel=p["dt"],
             cfl=None, bottom_drag_coef=2e-7, slip_coef=0.5, visc_coef=30.0, diff_coef=20.0, sponge_coef=0.0,
             dist_sponge_bc=None, use_sponge_on_coast=False, tangential_sponge_factor=1.0, rho_water=1025.0,
             h_wind=None, forcing_momentum="direct", max_nstep=p["max_nstep"], name_params=p["name_params"],
             init_from_bc=None, name_init_var=None, path_wind=None, name_var_wind=None)
    EXP = NS(init_date=datetime.datetime(2020, 1, 1), final_date=datetime.datetime(2020, 1, 2), flag_plot=0)
    config = NS(MOD=MOD, EXP=EXP, GRID=NS(super="GRID_CAR"), INV=None)
    M = mod.Model_qgsw(config, st)
    rng = np.random.default_rng(p["seed"])
    ocean = ~mask
    if nl > 1:
        st.var["u_layers"] = 0.05 * rng.standard_normal((nl, ny, nx + 1))
        st.var["v_layers"] = 0.05 * rng.standard_normal((nl, ny + 1, nx))
        st.var["h_layers"] = 0.2 * rng.standard_normal((nl, ny, nx)) * ocean
    else:
        st.var["u"] = 0.05 * rng.standard_normal((ny, nx + 1))
        st.var["v"] = 0.05 * rng.standard_normal((ny + 1, nx))
        st.var["ssh"] = 0.2 * rng.standard_normal((ny, nx)) * ocean
    st.params["u"] = 0.1 * rng.standard_normal((ny, nx + 1))
    st.params["v"] = 0.1 * rng.standard_normal((ny + 1, nx))
    st.params["ssh"] = 0.3 * rng.standard_normal((ny, nx))
    if "bc" in p["name_params"]:
        st.params["u_b"] = 0.01 * rng.standard_normal((ny, nx + 1))
        st.params["v_b"] = 0.01 * rng.standard_normal((ny + 1, nx))
        st.params["h_b"] = 0.02 * rng.standard_normal((ny, nx))
    tb = [0.0, 30.0]
    var_bc = None
    if p["bc"]:
        var_bc = {"SSH": [0.05 * rng.standard_normal((ny, nx)) for _ in tb],
                  "U": [0.02 * rng.standard_normal((ny, nx + 1)) for _ in tb],
                  "V": [0.02 * rng.standard_normal((ny + 1, nx)) for _ in tb]}
        M.set_bc(tb, var_bc)
    out[f"{tag}_dt"] = np.float64(M.dt)
    for k, v in st.var.items():
        out[f"{tag}_in_var_{k}"] = np.asarray(v, dtype=np.float64)
    for k, v in st.params.items():
        out[f"{tag}_in_par_{k}"] = np.asarray(v, dtype=np.float64)
    if var_bc is not None:
        for k, arrs in var_bc.items():
            out[f"{tag}_bc_{k}"] = np.stack(arrs)
    M.step(st, nstep=p["nstep"], t=0)
    for k, v in st.var.items():
        out[f"{tag}_out_var_{k}"] = np.asarray(v, dtype=np.float64)


def main():
    ref_root = _jax_standin.reference_root()
    mods = load_all(ref_root)
    mod = mods[4]
    out = {}
    for tag, p in CASES.items():
        run_case(tag, p, mod, ref_root, out)
    np.savez_compressed(os.path.join(HERE, "qgsw_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
