"""Generate golden cost and gradient values of the reference's own 4D-Var
assembly: ``Variational.cost_and_grad`` (mapping/src/tools_4Dvar.py:252-400)
driving ``Model_qg1l_jax.step`` / ``step_adj`` (mapping/src/mod.py:867-913,
1018-1076), the jax along-track operator ``Obsop_interp_l3_jax``
(mapping/src/obsop.py:375-678, observations read through its own
``process_obs``) and a ``Basis_gauss3d`` reduced basis (basis.py:1170-1555),
with the checkpoint rule of mapping/src/inv.py:144-163.

Everything runs unmodified from the reference checkout under the NumPy
stand-in for jax (``_jax_standin.py``, float64), on a lon/lat grid with the
model class ``Qgm`` of mapping/models/model_qg1l/jqgm.py. Two reverse-mode
pieces need ``jax.vjp``, which the stand-in does not provide; they take the
oracle's restatements, each pinned on its own:

- ``Model_qg1l_jax.qgm_step_adj`` (the vjp of ``Qgm.step``) is
  ``oracle.qg1l.QgmOracle.step_adj``, which matches central differences of
  the pinned forward and passes the dot-product test;
- ``Obsop_interp_l3_jax._misfit_reduced`` (the vjp of the linear misfit) is
  H^T (inverr * cotangent) written out below from the operator's own arrays.

So these vectors pin the assembly itself: the checkpoint walk and its order of
misfits, basis projections and model calls, the State copies, the SSH forcing
n dt/86400 F and its adjoint accumulation into the parameters, the
preconditioned / plain background term, J = (Jo + Jb)/2 and G. Cases:

- ``p``: prec = True, observations at steps 0, 2, 5, 9 and 12 of a 12-step
  window, basis checkpoints every 3 steps;
- ``n``: prec = False, a different basis and observation steps 4, 7 and 11,
  a non-zero background Xb.

Files read by ``process_obs`` (``xr.open_dataset``) are dicts held in memory.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_fourdvar.py <VarDyn checkout>
Writes ``tests/golden/fourdvar_golden.npz``.
"""
import datetime
import importlib.util
import os
import sys
import tempfile
from types import SimpleNamespace as NS

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _jax_standin  # noqa: E402

from gen_golden import load_reference  # noqa: E402
from gen_golden_basis import load_basis  # noqa: E402
from gen_golden_obs import _empty  # noqa: E402

LON0, LAT0, DDEG, NX, NY = -60.0, 35.0, 0.05, 32, 26
DT, NSTEP, CHECK = 1200.0, 12, 3
CASES = {
    "p": dict(prec=True, obs_steps=(0, 2, 5, 9, 12), basis=dict(sigma_D=50.0, sigma_T=0.1, facns=1.5, facnlt=2.0,
                                                                   sigma_Q=0.05), xb=0.0, seed=11),
    "n": dict(prec=False, obs_steps=(4, 7, 11), basis=dict(sigma_D=70.0, sigma_T=0.15, facns=1.0, facnlt=1.5,
                                                           sigma_Q=0.08), xb=0.01, seed=12),
}


class _Dataset(dict):
    """What process_obs reads from a file: ``ds[name].values`` and ``in``."""

    def __getitem__(self, k):
        return NS(values=dict.__getitem__(self, k))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


FILES = {}


def _open_dataset(path):
    return FILES[path]


def _load(name, ref_root):
    spec = importlib.util.spec_from_file_location(f"src.{name}", os.path.join(ref_root, "mapping", "src",
                                                                              f"{name}.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[f"src.{name}"] = mod
    setattr(sys.modules["src"], name, mod)
    spec.loader.exec_module(mod)
    return mod


def load_all(ref_root):
    jqgm = load_reference(ref_root)                   # Qgm under the stand-in
    basis = load_basis(ref_root)                      # installs again; src.grid, src.obsop, src.basis
    obsop = sys.modules["src.obsop"]
    sys.modules["xarray"].open_dataset = _open_dataset
    obsop.xr = sys.modules["xarray"]
    _empty("jaxparrow")
    for name in ("exp", "state", "mod", "tools_4Dvar"):
        _load(name, ref_root)
    return jqgm, basis, obsop, sys.modules["src.state"], sys.modules["src.mod"], sys.modules["src.tools_4Dvar"]


def grid():
    lon1d = LON0 + DDEG * np.arange(NX)
    lat1d = LAT0 + DDEG * np.arange(NY)
    lon, lat = np.meshgrid(lon1d, lat1d)
    DX = np.radians(DDEG) * 6371e3 * np.cos(np.radians(lat))
    DY = np.full((NY, NX), np.radians(DDEG) * 6371e3)
    return lon1d, lat1d, lon, lat, DX, DY


def smooth_field(rng, amp):
    k = np.fft.fftfreq(NX)[None, :] ** 2 + np.fft.fftfreq(NY)[:, None] ** 2
    spec = np.exp(-k / 0.004) * (rng.standard_normal((NY, NX)) + 1j * rng.standard_normal((NY, NX)))
    f = np.real(np.fft.ifft2(spec))
    return amp * f / f.std()


def run_case(tag, p, mods, out):
    jqgm, basis_mod, obsop, state_mod, mod, t4d = mods
    rng = np.random.default_rng(p["seed"])
    lon1d, lat1d, lon, lat, DX, DY = grid()
    t0 = datetime.datetime(2020, 1, 1)
    T = np.arange(NSTEP + 1) * DT
    timestamps = [t0 + datetime.timedelta(seconds=float(t)) for t in T]
    tmp = tempfile.mkdtemp()
    config = NS(EXP=NS(name_time="time", name_lon="lon", name_lat="lat", name_exp_save="g", path_save=tmp,
                       tmp_DA_path=tmp, flag_plot=0, lon_obs_max=None, lon_obs_min=None, lat_obs_max=None,
                       lat_obs_min=None, assimilation_time_step=datetime.timedelta(seconds=DT)),
                OBSOP=NS(compute_op=True, write_op=False, path_save=None, mask_borders=False, Npix=4,
                         name_obs=None, name_var="SSH"),
                INV=NS(prec=p["prec"], timestep_checkpoint=datetime.timedelta(seconds=CHECK * DT),
                       save_minimization=False, compute_test=False))
    # State: the reference class, grid attributes set as its grid set-up would
    State = state_mod.State(config, first=False)
    State.ny, State.nx, State.lon, State.lat = NY, NX, lon, lat
    State.DX, State.DY, State.X, State.Y = DX, DY, None, None
    State.dx, State.dy = float(DX.mean()), float(DY.mean())
    State.f = np.full((NY, NX), 1e-4)
    State.mask = np.zeros((NY, NX), dtype=bool)
    State.lon_u = State.lat_u = State.lon_v = State.lat_v = None
    State.geo_grid = True
    State.lon_min, State.lon_max, State.lat_min, State.lat_max = lon.min(), lon.max(), lat.min(), lat.max()
    State.lon_unit = "-180_180"
    h_init = smooth_field(rng, 0.1)
    State.var = {"ssh": h_init.copy()}
    State.params = {"ssh": np.zeros((NY, NX))}

    # Model: Model_qg1l_jax's own step / step_adj around the reference's Qgm
    # (forward) and the oracle's adjoint in place of jax.vjp
    from oracle.qg1l import QgmOracle
    qgm = jqgm.Qgm(dx=DX, dy=DY, dt=DT, SSH=h_init, c=np.float64(2.7), g=9.81, f=np.float64(1e-4),
                   time_scheme="rk2")
    qo = QgmOracle(dx=DX, dy=DY, dt=DT, c=2.7, g=9.81, f=1e-4, time_scheme="rk2")
    M = mod.Model_qg1l_jax.__new__(mod.Model_qg1l_jax)
    M.name_var = {"SSH": "ssh"}
    M.bc = {}
    M.ny, M.nx = NY, NX
    M.dt, M.T, M.timestamps = DT, T, timestamps
    M.advect_tracer = False
    M.ageo_velocities = False
    M.forcing_tracer_from_bc = False
    M.Wbc = np.zeros((NY, NX))
    M.qgm_step = qgm.step_jit
    M.qgm_step_adj = lambda adX1, X1, Xb, nstep: qo.step_adj(np.asarray(adX1), np.asarray(X1), np.asarray(Xb),
                                                             nstep)

    # Observations through the reference's own process_obs
    dict_obs = {}
    sat = {"name_var": ["SSH"], "name_lon": "lon", "name_lat": "lat", "sigma_noise": None}
    for s in p["obs_steps"]:
        n = int(rng.integers(50, 90))
        path = f"{tag}_obs_{s}"
        FILES[path] = _Dataset(lon=rng.uniform(lon1d[1], lon1d[-2], n), lat=rng.uniform(lat1d[1], lat1d[-2], n),
                               SSH=0.1 * rng.standard_normal(n), SSH_err=rng.uniform(0.02, 0.05, n))
        dict_obs[timestamps[s]] = {"attributes": [sat], "obs_path": [path], "obs_name": ["alg"]}
        for k in ("lon", "lat", "SSH", "SSH_err"):
            out[f"{tag}_obs{s}_{k}"] = dict.__getitem__(FILES[path], k)
    H = obsop.Obsop_interp_l3_jax(config, State, dict_obs, M)
    H.process_obs()

    def misfit_reduced(t, grad_obs, X):
        # vjp of the linear misfit inverr * (H X - y) (NaN entries carry no
        # cotangent; none occur here)
        idt = int(np.nonzero(np.asarray(H.t_obs) == t)[0][0])
        data = np.asarray(H.data_arr[idt])
        row = np.asarray(H.indices_arr[idt][0]).astype(int)
        col = np.asarray(H.indices_arr[idt][1]).astype(int)
        inverr = 1.0 / np.asarray(H.errobs_arr[idt])
        g = np.zeros(np.asarray(X).size)
        np.add.at(g, col, data * (inverr * np.asarray(grad_obs))[row])
        return g

    H._misfit_reduced_jit = misfit_reduced

    # Basis and the checkpoint rule of inv.py:144-163 (H.is_obs on timestamps)
    nstep_check = int(config.INV.timestep_checkpoint.total_seconds() // M.dt)
    checkpoints, check = [0], 0
    for i, t in enumerate(timestamps[:-1]):
        if i > 0 and (H.is_obs(t) or check == nstep_check):
            checkpoints.append(i)
            if check == nstep_check:
                check = 0
        check += 1
    checkpoints.append(len(timestamps) - 1)
    checkpoints = np.asarray(checkpoints)
    bp = p["basis"]
    cfg_b = NS(BASIS=NS(name_mod_var="ssh", fcor=None, flag_variable_Q=False, path_sad=None, name_var_sad=None,
                        path_background=None, var_background=None, c_grid_var=None, compute_velocities=False,
                        name_mod_u=None, name_mod_v=None, normalize_fact=True, flux=False, time_spinup=None, **bp))
    B = basis_mod.Basis_gauss3d(cfg_b, State)
    time_basis = np.array([T[c] / 3600 / 24 for c in range(0, NSTEP + 1, nstep_check)])
    _, Q = B.set_basis(time_basis, return_q=True)
    Q = np.asarray(Q, dtype=np.float64)
    Xb = np.full(B.nbasis, p["xb"])
    X0 = rng.standard_normal(B.nbasis) * (1.0 if p["prec"] else Q)

    var = t4d.Variational(config=config, M=M, H=H, State=State, R=t4d.Cov(None), B=t4d.Cov(Q), Basis=B, Xb=Xb,
                          checkpoints=checkpoints)
    J, G = var.cost_and_grad(X0)
    out.update({f"{tag}_h_init": h_init, f"{tag}_X0": X0, f"{tag}_Xb": Xb, f"{tag}_Q": Q, f"{tag}_J": np.float64(J),
                f"{tag}_G": np.asarray(G, dtype=np.float64), f"{tag}_checkpoints": checkpoints,
                f"{tag}_time_basis": time_basis, f"{tag}_obs_steps": np.array(p["obs_steps"]),
                f"{tag}_prec": np.array(p["prec"])})
    for k, v in bp.items():
        out[f"{tag}_basis_{k}"] = np.float64(v)
    print(f"case {tag}: nbasis {B.nbasis}, checkpoints {list(checkpoints)}, J {J:.12e}")


def main():
    ref_root = _jax_standin.reference_root()
    mods = load_all(ref_root)
    lon1d, lat1d, *_ = grid()
    out = {"lon": lon1d, "lat": lat1d, "dt": np.float64(DT), "nstep": np.int64(NSTEP),
           "nstep_check": np.int64(CHECK)}
    for tag, p in CASES.items():
        run_case(tag, p, mods, out)
    np.savez_compressed(os.path.join(HERE, "fourdvar_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
