"""Generate golden vectors for the shallow-water model with open boundaries
(``flag_obc``, mapping/models/model_qgsw/sw.py:353-371) from the reference's
own source code loaded unmodified behind the NumPy stand-in for jax
(float64).

With ``flag_obc`` the reference sets the u masks of the west / east faces and
the v masks of the south / north faces to 1 after the other masks are built,
and allocates boundary arrays that nothing reads. Inflow velocities on those
faces are then kept by ``set_input_uvh`` (440-441) and enter the diagnostics
(vorticity, kinetic energy, the 4-point averages of the Coriolis and vortex
terms); the faces' own tendencies stay zero, and the sponge relaxes them to
the boundary fields. Case ``ob``: 2 layers with land (including land on the
outer walls), partial slip, viscosity, diffusion, a sponge on every grid,
boundary fields and forcing: the masks, ``compute_time_derivatives`` and a
4-step ``step``.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_swobc.py <VarDyn checkout>
Writes ``tests/golden/swobc_golden.npz``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402
from gen_golden_sw import J, grid, land_mask, load  # noqa: E402


def main():
    ref_root = _jax_standin.reference_root()
    M = load(ref_root)
    rng = np.random.default_rng(777)
    out = {}
    nx, ny, nl = 28, 22, 2
    dx, dy, f = grid(nx, ny, rng)
    mask = land_mask(nx, ny)
    H = np.array([300.0, 800.0]).reshape(2, 1, 1)
    gp = np.array([9.81, 0.02])
    param = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f, taux=0.04, tauy=-0.02,
                 bottom_drag_coef=1e-6, dt=20.0, mask=mask, slip_coef=0.6, visc_coef=20.0, diff_coef=10.0,
                 compile=False, sponge_coef=0.2, flag_obc=True, dtype=np.float64)
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
    p = "ob_"
    for k, val in dict(dx=dx, dy=dy, f=f, mask=mask, H=H, gp=gp, sponge_u=sw.sponge_u, sponge_v=sw.sponge_v,
                       sponge_h=sw.sponge_h, u0=u0, v0=v0, h0=h0, ub=ub, vb=vb, hb=hb, Fu=Fu, Fv=Fv,
                       Fh=Fh).items():
        out[p + k] = np.asarray(val)
    out[p + "mask_u"] = np.asarray(sw.masks.u, dtype=np.float64)[0, 0]
    out[p + "mask_v"] = np.asarray(sw.masks.v, dtype=np.float64)[0, 0]
    u, v, h = sw.set_input_uvh(J(u0), J(v0), J(h0))
    ref_vals = sw._compute_ref_values(sw.H)
    du, dv, dh = sw.compute_time_derivatives(u, v, h, ref_vals)
    out[p + "dtu"], out[p + "dtv"], out[p + "dth"] = np.asarray(du), np.asarray(dv), np.asarray(dh)
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=4, u_b=J(ub), v_b=J(vb), h_b=J(hb), Fu=J(Fu), Fv=J(Fv),
                         Fh=J(Fh))
    out[p + "u4"], out[p + "v4"], out[p + "h4"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)
    np.savez_compressed(os.path.join(HERE, "swobc_golden.npz"), **out)
    print("wrote", len(out), "arrays,", os.path.getsize(os.path.join(HERE, "swobc_golden.npz")), "bytes")


if __name__ == "__main__":
    main()
