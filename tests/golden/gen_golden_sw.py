"""Generate golden vectors for the multilayer shallow-water model and the QG
projector from the reference's own source code.

Loads ``mapping/models/model_qgsw/sw.py`` and ``qg.py`` (with their helper
modules) unmodified, with the NumPy stand-in for jax of ``_jax_standin.py``,
and records in float64:

- the SW masks (masks.py) of a domain with land;
- ``SW.compute_time_derivatives`` and ``SW.step`` for two configurations that
  between them exercise every term (2 layers with land, partial slip, wind
  arrays, drag, viscosity, thickness diffusion, sponge, direct forcing; 1
  layer with varying H, scalar h_wind, free slip, mass-consistent forcing);
- the QG operators (layer/mode matrices, ``project_qg``) with and without an
  island (capacitance-matrix branch).

``QG.step`` itself cannot run in the reference as shipped: ``SW.step`` passes
``ref_vals`` and wind arguments that ``QG.compute_time_derivatives`` and
``QG.add_wind_forcing`` do not accept, so only its operators are recorded.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_sw.py <VarDyn checkout>
Writes ``tests/golden/sw_golden.npz``.
"""
import os
import sys
from importlib.machinery import SourceFileLoader

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402


def J(a):
    return np.asarray(a, dtype="float64").view(_jax_standin.JArray)


def load(ref_root):
    _jax_standin.install(enable_x64=True)
    d = os.path.join(ref_root, "mapping", "models", "model_qgsw")
    sys.path.insert(0, d)
    mods = {}
    for name in ("tools", "finite_diff", "reconstruction", "flux", "masks", "helmholtz",
                 "helmholtz_multigrid", "sw", "qg"):
        mods[name] = SourceFileLoader(name, os.path.join(d, name + ".py")).load_module()
        sys.modules[name] = mods[name]
    return mods


def grid(nx, ny, rng, vary=True):
    xx = np.arange(nx)[:, None] + np.zeros((1, ny))
    yy = np.zeros((nx, 1)) + np.arange(ny)[None, :]
    dx = 5.0e3 * (1 + (0.02 * np.sin(0.3 * xx + 0.2 * yy) if vary else 0 * xx))
    dy = 4.0e3 * (1 + (0.015 * np.cos(0.25 * yy - 0.1 * xx) if vary else 0 * xx))
    yw = np.arange(ny + 1)[None, :] * 4.0e3 + np.zeros((nx + 1, 1))
    f = 1.0e-4 + 1.6e-11 * (yw - yw.mean())
    return dx, dy, f


def land_mask(nx, ny):
    m = np.ones((nx, ny))
    m[9:14, 6:10] = 0          # island
    m[0:4, 0:3] = 0            # corner
    m[nx - 2:, 12:15] = 0      # coast notch
    m[17, 3] = 0               # single cell
    return m


def sw_case_a(M, out, rng):
    nx, ny, nl = 28, 22, 2
    dx, dy, f = grid(nx, ny, rng)
    mask = land_mask(nx, ny)
    H = np.array([350.0, 750.0]).reshape(2, 1, 1)
    gp = np.array([9.81, 0.025])
    param = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f,
                 taux=0.05 * rng.standard_normal((nx - 1, ny)), tauy=0.05 * rng.standard_normal((nx, ny - 1)),
                 bottom_drag_coef=2e-7, dt=15.0, mask=mask, slip_coef=0.5, visc_coef=30.0, diff_coef=20.0,
                 compile=False, sponge_coef=0.3, dtype=np.float64)
    sw = M["sw"].SW(param)
    sw.sponge_u = J(rng.random((1, 1, nx + 1, ny)))
    sw.sponge_v = J(rng.random((1, 1, nx, ny + 1)))
    sw.sponge_h = J(rng.random((1, 1, nx, ny)))
    u0 = 0.1 * rng.standard_normal((1, nl, nx + 1, ny))
    v0 = 0.1 * rng.standard_normal((1, nl, nx, ny + 1))
    h0 = 0.3 * rng.standard_normal((1, nl, nx, ny))
    ub = 0.05 * rng.standard_normal(u0.shape)
    vb = 0.05 * rng.standard_normal(v0.shape)
    hb = 0.1 * rng.standard_normal(h0.shape)
    Fu = 1e-5 * rng.standard_normal(u0.shape)
    Fv = 1e-5 * rng.standard_normal(v0.shape)
    Fh = 1e-5 * rng.standard_normal(h0.shape)
    taux = 0.05 * rng.standard_normal((nx - 1, ny))
    tauy = 0.05 * rng.standard_normal((nx, ny - 1))
    p = "swa_"
    for k, val in dict(dx=dx, dy=dy, f=f, mask=mask, H=H, gp=gp, taux0=param["taux"], tauy0=param["tauy"],
                       sponge_u=sw.sponge_u, sponge_v=sw.sponge_v, sponge_h=sw.sponge_h, u0=u0, v0=v0, h0=h0,
                       ub=ub, vb=vb, hb=hb, Fu=Fu, Fv=Fv, Fh=Fh, taux=taux, tauy=tauy).items():
        out[p + k] = np.asarray(val)
    ms = sw.masks
    for name in ("u", "v", "w", "psi", "w_valid", "w_cornerout_bound", "w_vertical_bound", "w_horizontal_bound",
                 "u_sten_hx_eq2", "u_sten_hx_eq4", "u_sten_hx_gt6", "u_sten_wy_eq2", "u_sten_wy_eq4",
                 "u_sten_wy_gt4", "v_sten_hy_eq2", "v_sten_hy_eq4", "v_sten_hy_gt6", "v_sten_wx_eq2",
                 "v_sten_wx_eq4", "v_sten_wx_gt6"):
        out[p + "mask_" + name] = np.asarray(getattr(ms, name), dtype=np.float64)[0, 0]
    out[p + "irr_x"] = np.asarray(ms.psi_irrbound_xids)
    out[p + "irr_y"] = np.asarray(ms.psi_irrbound_yids)
    u, v, h = sw.set_input_uvh(J(u0), J(v0), J(h0))
    ref_vals = sw._compute_ref_values(sw.H)
    du, dv, dh = sw.compute_time_derivatives(u, v, h, ref_vals, taux=J(taux), tauy=J(tauy))
    out[p + "dtu"], out[p + "dtv"], out[p + "dth"] = np.asarray(du), np.asarray(dv), np.asarray(dh)
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=4, u_b=J(ub), v_b=J(vb), h_b=J(hb), Fu=J(Fu), Fv=J(Fv),
                         Fh=J(Fh), taux=J(taux), tauy=J(tauy))
    out[p + "u4"], out[p + "v4"], out[p + "h4"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)
    # default forcing / boundary arguments, wind from the constructor
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=2)
    out[p + "u2d"], out[p + "v2d"], out[p + "h2d"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)


def sw_case_b(M, out, rng):
    nx, ny, nl = 24, 26, 1
    dx, dy, f = grid(nx, ny, rng, vary=False)
    xx = np.arange(nx)[:, None] + np.zeros((1, ny))
    H = (0.8 + 0.1 * np.sin(0.2 * xx + 0.1 * np.arange(ny)[None, :]))[None]
    gp = np.array([9.81])
    param = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f, taux=0.0, tauy=0.0,
                 bottom_drag_coef=1e-6, dt=60.0, slip_coef=1.0, visc_coef=0.0, diff_coef=0.0, compile=False,
                 h_wind=80.0, forcing_momentum="mass_consistent", h_min=0.05, dtype=np.float64)
    sw = M["sw"].SW(param)
    u0 = 0.05 * rng.standard_normal((1, nl, nx + 1, ny))
    v0 = 0.05 * rng.standard_normal((1, nl, nx, ny + 1))
    h0 = 0.05 * rng.standard_normal((1, nl, nx, ny))
    Fh = 1e-5 * rng.standard_normal(h0.shape)
    taux = 0.1 * rng.standard_normal((nx - 1, ny))
    tauy = 0.1 * rng.standard_normal((nx, ny - 1))
    p = "swb_"
    for k, val in dict(dx=dx, dy=dy, f=f, H=H, gp=gp, u0=u0, v0=v0, h0=h0, Fh=Fh, taux=taux, tauy=tauy).items():
        out[p + k] = np.asarray(val)
    u, v, h = sw.set_input_uvh(J(u0), J(v0), J(h0))
    ref_vals = sw._compute_ref_values(sw.H)
    du, dv, dh = sw.compute_time_derivatives(u, v, h, ref_vals, taux=J(taux), tauy=J(tauy))
    out[p + "dtu"], out[p + "dtv"], out[p + "dth"] = np.asarray(du), np.asarray(dv), np.asarray(dh)
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=5, Fh=J(Fh), taux=J(taux), tauy=J(tauy))
    out[p + "u5"], out[p + "v5"], out[p + "h5"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)


def qg_case(M, out, rng, island):
    nx, ny, nl = 32, 24, 3
    dx, dy, f = 5.0e3, 5.0e3, None
    yw = np.arange(ny + 1)[None, :] * 5.0e3 + np.zeros((nx + 1, 1))
    f = 1.0e-4 + 1.6e-11 * (yw - yw.mean())
    H = np.array([350.0, 750.0, 2900.0]).reshape(3, 1, 1)
    gp = np.array([9.81, 0.025, 0.0125])
    param = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f, taux=0.0, tauy=0.0,
                 bottom_drag_coef=0.0, dt=600.0, compile=False, dtype=np.float64)
    p = "qgi_" if island else "qg_"
    if island:
        mask = np.ones((nx, ny))
        mask[10:15, 8:13] = 0
        mask[25:27, 3:5] = 0
        param["mask"] = mask
        out[p + "mask"] = mask
    qg = M["qg"].QG(param)
    u0 = 0.1 * rng.standard_normal((1, nl, nx + 1, ny))
    v0 = 0.1 * rng.standard_normal((1, nl, nx, ny + 1))
    h0 = 0.3 * rng.standard_normal((1, nl, nx, ny))
    u, v, h = qg.set_input_uvh(J(u0), J(v0), J(h0))
    out[p + "u"], out[p + "v"], out[p + "h"] = np.asarray(u), np.asarray(v), np.asarray(h)
    out[p + "A"] = np.asarray(qg.A)
    out[p + "lambd"] = np.asarray(qg.lambd)
    out[p + "Cl2m"] = np.asarray(qg.Cl2m)
    out[p + "Cm2l"] = np.asarray(qg.Cm2l)
    out[p + "homsol"] = np.asarray(qg.homsol_wgrid)
    pu, pv, ph = qg.project_qg(u, v, h)
    out[p + "Pu"], out[p + "Pv"], out[p + "Ph"] = np.asarray(pu), np.asarray(pv), np.asarray(ph)
    q = qg.Q(u, v, h)
    out[p + "Q"] = np.asarray(q)
    pq, pqi = qg.QoG_inv(q)
    out[p + "pqg"], out[p + "pqgi"] = np.asarray(pq), np.asarray(pqi)


def sw_case_h(M, out, rng):
    """Steps with the per-call H and h_wind arguments (sw.py:752-817): H
    enters the reference values, the wind depth stays the model's own H
    (sw.py:622-630); h_wind adds to the model's mixed-layer depth."""
    nx, ny, nl = 26, 20, 2
    dx, dy, f = grid(nx, ny, rng)
    mask = land_mask(nx, ny)[:nx, :ny]
    H = np.array([150.0, 600.0]).reshape(2, 1, 1)
    gp = np.array([9.81, 0.03])
    base = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f, taux=0.08, tauy=-0.05,
                bottom_drag_coef=1e-6, dt=20.0, mask=mask, slip_coef=0.5, visc_coef=20.0, diff_coef=10.0,
                compile=False, dtype=np.float64)
    u0 = 0.05 * rng.standard_normal((1, nl, nx + 1, ny))
    v0 = 0.05 * rng.standard_normal((1, nl, nx, ny + 1))
    h0 = 0.3 * rng.standard_normal((1, nl, nx, ny))
    dH = 4.0 * rng.standard_normal((1, nx, ny))
    hw = 8.0 * rng.standard_normal((nx, ny))
    p = "swh_"
    for k, val in dict(dx=dx, dy=dy, f=f, mask=mask, H=H, gp=gp, u0=u0, v0=v0, h0=h0, dH=dH, hw=hw).items():
        out[p + k] = np.asarray(val)
    sw = M["sw"].SW(dict(base))
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), H=J(dH), nstep=3)
    out[p + "uH"], out[p + "vH"], out[p + "hH"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)
    sw = M["sw"].SW(dict(base, h_wind=50.0))
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=3, h_wind=J(hw))
    out[p + "uW"], out[p + "vW"], out[p + "hW"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)


def main():
    ref_root = _jax_standin.reference_root()
    M = load(ref_root)
    out = {}
    rng = np.random.default_rng(4242)
    sw_case_a(M, out, rng)
    sw_case_b(M, out, rng)
    qg_case(M, out, rng, island=False)
    qg_case(M, out, rng, island=True)
    sw_case_h(M, out, rng)
    np.savez_compressed(os.path.join(HERE, "sw_golden.npz"), **out)
    print("wrote", len(out), "arrays,", os.path.getsize(os.path.join(HERE, "sw_golden.npz")), "bytes")


if __name__ == "__main__":
    main()
