"""Generate golden vectors for the shallow-water model's barotropic filter in
its spectral form (mapping/models/model_qgsw/sw.py:305-320, 695-725) and its
DCT-II Neumann Helmholtz solver with the capacitance correction for land
(helmholtz.py:20-87, 187-305), from the reference's own source code loaded
unmodified behind the NumPy stand-in for jax (float64).

Case ``fa`` (uniform spacings: the solver diagonalises the Laplacian with one
DCT-II per direction): 2 layers, no land: the solver's spectral eigenvalues,
a solve of a random right-hand side, ``compute_time_derivatives`` and a 3-step
``step``. With any land the reference's solver does not construct: SW passes
its [nx, ny] spacing arrays, and the masked operator that the capacitance
matrix is built from divides a face-grid difference by them
(helmholtz.py:254, shapes (nx+1, ny) and (nx, ny) do not broadcast), so no
land case exists to record.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_swfilter.py <VarDyn checkout>
Writes ``tests/golden/swfilter_golden.npz``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402
from gen_golden_sw import J, grid, load  # noqa: E402


def case(M, out, rng, tag, land):
    nx, ny, nl = 24, 20, 2
    dx, dy, f = grid(nx, ny, rng, vary=False)
    H = np.array([300.0, 700.0]).reshape(2, 1, 1)
    gp = np.array([9.81, 0.03])
    param = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=gp, f=f, taux=0.05, tauy=-0.03,
                 bottom_drag_coef=1e-6, dt=30.0, slip_coef=0.5, visc_coef=10.0, diff_coef=5.0, compile=False,
                 barotropic_filter=True, barotropic_filter_spectral=True, dtype=np.float64)
    if land:
        mask = np.ones((nx, ny))
        mask[8:12, 7:11] = 0
        mask[nx - 3:, 14:17] = 0
        param["mask"] = mask
        out[tag + "mask"] = mask
    sw = M["sw"].SW(param)
    hs = sw.helm_solver
    out[tag + "dx"], out[tag + "dy"], out[tag + "f"] = dx, dy, f
    out[tag + "H"], out[tag + "gp"] = H, gp
    out[tag + "helm_dct"] = np.asarray(hs.helmholtz_dctII, dtype=np.float64)
    out[tag + "irr_x"] = np.asarray(hs.irrbound_xids)
    out[tag + "irr_y"] = np.asarray(hs.irrbound_yids)
    if hs.cap_matrix is not None:
        out[tag + "cap"] = np.asarray(hs.cap_matrix, dtype=np.float64)
    rhs = rng.standard_normal((1, 1, nx, ny)) * 1e-6
    out[tag + "rhs"] = rhs
    out[tag + "sol"] = np.asarray(hs.solve(J(rhs)), dtype=np.float64)
    u0 = 0.05 * rng.standard_normal((1, nl, nx + 1, ny))
    v0 = 0.05 * rng.standard_normal((1, nl, nx, ny + 1))
    h0 = 0.3 * rng.standard_normal((1, nl, nx, ny))
    out[tag + "u0"], out[tag + "v0"], out[tag + "h0"] = u0, v0, h0
    u, v, h = sw.set_input_uvh(J(u0), J(v0), J(h0))
    ref_vals = sw._compute_ref_values(sw.H)
    du, dv, dh = sw.compute_time_derivatives(u, v, h, ref_vals)
    out[tag + "dtu"], out[tag + "dtv"], out[tag + "dth"] = np.asarray(du), np.asarray(dv), np.asarray(dh)
    u1, v1, h1 = sw.step(J(u0), J(v0), J(h0), nstep=3)
    out[tag + "u3"], out[tag + "v3"], out[tag + "h3"] = np.asarray(u1), np.asarray(v1), np.asarray(h1)


def main():
    ref_root = _jax_standin.reference_root()
    M = load(ref_root)
    rng = np.random.default_rng(31)
    out = {}
    case(M, out, rng, "fa_", land=False)
    np.savez_compressed(os.path.join(HERE, "swfilter_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
