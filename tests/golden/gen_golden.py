"""Generate golden vectors for the QG 1.5-layer forward path from the
reference's own source code.

The reference (datlas-ocean/VarDyn) is JAX code and jax is not installable in
this container. This script installs a NumPy stand-in for the few jax entry
points that ``mapping/models/model_qg1l/jqgm.py`` touches (see
``_jax_standin.py``), loads that file unmodified from the reference checkout,
and records the outputs of ``Qgm``'s forward functions on seeded inputs in
float64 (``USE_FLOAT64 = True``).

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden.py <VarDyn checkout>
Writes ``tests/golden/qg1l_golden.npz``.
"""
import os
import sys
from importlib.machinery import SourceFileLoader

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _jax_standin  # noqa: E402


def load_reference(ref_root):
    _jax_standin.install(enable_x64=True)
    path = os.path.join(ref_root, "mapping", "models", "model_qg1l", "jqgm.py")
    return SourceFileLoader("jqgm_reference", path).load_module()


def J(a):
    return np.asarray(a, dtype="float64").view(_jax_standin.JArray)


def small_case(ref, out):
    """24x30 grid: land blob, beta plane, diffusion, bathymetry term, hb != 0."""
    rng = np.random.default_rng(1234)
    ny, nx = 24, 30
    dx = np.full((ny, nx), 1.0e4)
    dy = np.full((ny, nx), 1.2e4)
    yy = np.arange(ny)[:, None] * 1.2e4 + np.zeros((1, nx))
    f = 1.0e-4 + 1.6e-11 * (yy - yy.mean())
    ssh = 0.1 * rng.standard_normal((ny, nx))
    ssh[9:12, 14:17] = np.nan          # land blob
    bathy = 0.05 * rng.standard_normal((ny, nx))
    hb = 0.02 * rng.standard_normal((ny, nx))
    hb[np.isnan(ssh)] = 0.0
    out["small_ssh"] = ssh
    out["small_dx"] = dx
    out["small_dy"] = dy
    out["small_f"] = f
    out["small_bathy"] = bathy
    out["small_hb"] = hb
    for scheme in ("Euler", "rk2", "rk3"):
        m = ref.Qgm(dx=dx, dy=dy, dt=1200.0, SSH=ssh, c=np.float64(2.7), g=9.81,
                    f=f, time_scheme=scheme, Kdiffus=50.0,
                    bathymetry_PV_term=bathy)
        if scheme == "Euler":
            out["small_mask"] = np.asarray(m.mask)
            h0 = J(np.nan_to_num(ssh))
            u, v = m.h2uv(J(ssh))
            out["small_h2uv_u"] = np.asarray(u)
            out["small_h2uv_v"] = np.asarray(v)
            q = m.h2pv(J(ssh), J(hb))
            out["small_h2pv"] = np.asarray(q)
            qb = m.h2pv(J(hb), J(hb))
            out["small_qb"] = np.asarray(qb)
            out["small_pv2h"] = np.asarray(m.pv2h(q, J(hb), qb))
            u0, v0 = m.h2uv(h0)
            out["small_rhs"] = np.asarray(m.rhs(u0, v0, q))
        out[f"small_step_{scheme}"] = np.asarray(m.step(J(ssh), J(hb), nstep=3))

    # DST-I of the reference on a ragged 2-D array
    x = rng.standard_normal((10, 14))
    out["dst_in"] = x
    out["dst_out"] = np.asarray(ref.dstI2D(J(x)))


def sf_case(ref, out):
    """Qgm_sf (streamfunction form, jqgm.py:571-1031) on the small case: land,
    f varying in y (phi = g/f h pointwise), diffusion, bathymetry, hb != 0."""
    ssh, dx, dy, f = out["small_ssh"], out["small_dx"], out["small_dy"], out["small_f"]
    bathy, hb = out["small_bathy"], out["small_hb"]
    for scheme in ("Euler", "rk2", "rk3"):
        m = ref.Qgm_sf(dx=dx, dy=dy, dt=1200.0, SSH=ssh, c=np.float64(2.7), g=9.81,
                       f=f, time_scheme=scheme, Kdiffus=50.0, bathymetry_PV_term=bathy)
        if scheme == "Euler":
            out["sf_mask"] = np.asarray(m.mask)
            phi = J(9.81 / f * np.nan_to_num(ssh))
            phib = J(9.81 / f * hb)
            q = m.phi2pv(phi, phib)
            out["sf_phi2pv"] = np.asarray(q)
            qb = m.phi2pv(phib, phib)
            out["sf_pv2phi"] = np.asarray(m.pv2phi(q, phib, qb))
        out[f"sf_step_{scheme}"] = np.asarray(m.step(J(ssh), J(hb), nstep=3))


def helm_case(ref_root, out):
    """Spectral Helmholtz solvers of mapping/models/model_qgsw/helmholtz.py:
    DST-I solve with edge padding (138-143) for two modes, capacitance
    matrices (146-169) and the capacitance-matrix solve (172-184) on a
    domain with an island."""
    sys.path.insert(0, os.path.join(ref_root, "mapping", "models", "model_qgsw"))
    path = os.path.join(ref_root, "mapping", "models", "model_qgsw", "helmholtz.py")
    hm = SourceFileLoader("helmholtz_reference", path).load_module()
    rng = np.random.default_rng(77)
    nx, ny, dx, dy = 40, 30, 2.0e3, 2.5e3
    f0, lam = 1.0e-4, np.array([0.0, 3.0e-1 * 1e-6 / 1e-8])
    lap = np.asarray(hm.compute_laplace_dstI(nx, ny, dx, dy, {"dtype": np.float64}))
    helm = J(lap[None, None] - f0 ** 2 * lam.reshape(1, 2, 1, 1))
    rhs = J(rng.standard_normal((1, 2, nx - 1, ny - 1)))
    out["helm_lam"] = lam
    out["helm_rhs"] = np.asarray(rhs)
    out["helm_dst_sol"] = np.asarray(hm.solve_helmholtz_dstI(rhs, helm))
    mask = np.ones((nx + 1, ny + 1))
    mask[0, :] = mask[-1, :] = 0
    mask[:, 0] = mask[:, -1] = 0
    mask[14:20, 10:16] = 0                       # island on the W grid
    isl = np.argwhere(mask[1:-1, 1:-1] == 0)     # its cells in interior indices
    bx, by = isl[:, 0], isl[:, 1]
    cap = hm.compute_capacitance_matrices(helm, bx, by)
    out["helm_mask"] = mask
    out["helm_bx"], out["helm_by"] = bx, by
    out["helm_cap"] = np.asarray(cap)
    out["helm_cmm_sol"] = np.asarray(hm.solve_helmholtz_dstI_cmm(rhs, helm, cap, bx, by, J(mask)))


def c1_case(ref, out):
    """128x128, dx=dy=10 km, f0=1e-4, c=2.7, dt=1200 s, 72 steps, hb=0."""
    from vardyn_gb300.synthetic import kminus3_ssh
    ny = nx = 128
    dx = np.full((ny, nx), 1.0e4)
    rng = np.random.default_rng(20240101)
    h0 = kminus3_ssh(ny, nx, 1.0e4, 1.0e4, rng, rms=0.1, cutoff_km=50.0)
    hb = np.zeros((ny, nx))
    out["c1_h0"] = h0
    for scheme in ("rk2", "rk3"):
        m = ref.Qgm(dx=dx, dy=dx, dt=1200.0, SSH=None, c=np.float64(2.7), g=9.81,
                    f=np.float64(1.0e-4), time_scheme=scheme)
        out[f"c1_step72_{scheme}"] = np.asarray(m.step(J(h0), J(hb), nstep=72))


def main():
    ref_root = _jax_standin.reference_root()
    ref = load_reference(ref_root)
    out = {}
    small_case(ref, out)
    sf_case(ref, out)
    helm_case(ref_root, out)
    c1_case(ref, out)
    np.savez_compressed(os.path.join(HERE, "qg1l_golden.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
