"""Generate golden vectors for the QG 1.5-layer model with tracers
(``Qgm_trac``, mapping/models/model_qg1l/jqgm.py:1551-2151) from the
reference's own source code, through the NumPy stand-in for jax
(``_jax_standin.py``), in float64.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_trac.py <VarDyn checkout>
Writes ``tests/golden/qgtrac_golden.npz``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden import J, load_reference  # noqa: E402


def _fields(rng, ny, nx, ntrac, land):
    ssh = 0.1 * rng.standard_normal((ny, nx))
    if land:
        ssh[10:13, 14:18] = np.nan
    c = 1.0 + 0.2 * rng.standard_normal((ntrac, ny, nx))
    hb = 0.02 * rng.standard_normal((ny, nx))
    cb = 1.0 + 0.1 * rng.standard_normal((ntrac, ny, nx))
    return ssh, c, hb, cb


def case_a(ref, out):
    """Euler, 2 tracers, open boundaries, land, beta plane, MDT, PV and tracer
    diffusion, default relaxation weights."""
    rng = np.random.default_rng(2468)
    ny, nx = 26, 32
    dx = np.full((ny, nx), 1.0e4)
    dy = np.full((ny, nx), 1.1e4)
    yy = np.arange(ny)[:, None] * 1.1e4 + np.zeros((1, nx))
    f = 1.0e-4 + 1.6e-11 * (yy - yy.mean())
    ssh, c, hb, cb = _fields(rng, ny, nx, 2, True)
    mdt = 0.03 * rng.standard_normal((ny, nx))
    m = ref.Qgm_trac(dx=dx, dy=dy, dt=900.0, SSH=ssh, c=np.float64(2.7), g=9.81, f=f, time_scheme="Euler",
                     Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC", mdt=J(mdt))
    X0 = np.concatenate([np.nan_to_num(ssh)[None], c])
    Xb = np.concatenate([hb[None], cb])
    X1 = np.asarray(m.step(J(X0.copy()), J(Xb.copy()), nstep=4))
    out.update(a_ssh=ssh, a_dx=dx, a_dy=dy, a_f=f, a_mdt=mdt, a_X0=X0, a_Xb=Xb, a_X1=X1)


def case_b(ref, out):
    """rk2, 1 tracer, Dirichlet tracer boundaries on the ring classes, a
    custom relaxation map, no PV advection, no land."""
    rng = np.random.default_rng(1357)
    ny, nx = 24, 28
    dx = np.full((ny, nx), 1.2e4)
    ssh, c, hb, cb = _fields(rng, ny, nx, 1, False)
    wbc = np.zeros((ny, nx))
    wbc[:3, :] = np.linspace(1.0, 0.2, 3)[:, None]
    m = ref.Qgm_trac(dx=dx, dy=dx, dt=600.0, SSH=ssh, c=np.float64(2.5), g=9.81, f=np.float64(1.0e-4),
                     time_scheme="rk2", Wbc=wbc, Kdiffus=None, Kdiffus_trac=5.0, bc_trac="dirichlet",
                     advect_pv=False)
    X0 = np.concatenate([ssh[None], c])
    Xb = np.concatenate([hb[None], cb])
    X1 = np.asarray(m.step(J(X0.copy()), J(Xb.copy()), nstep=3))
    out.update(b_ssh=ssh, b_dx=dx, b_wbc=wbc, b_X0=X0, b_Xb=Xb, b_X1=X1)


def case_c(ref, out):
    """rk2 without tracers (the state is the SSH alone)."""
    rng = np.random.default_rng(9753)
    ny, nx = 22, 26
    dx = np.full((ny, nx), 1.0e4)
    ssh = 0.1 * rng.standard_normal((ny, nx))
    hb = 0.02 * rng.standard_normal((ny, nx))
    m = ref.Qgm_trac(dx=dx, dy=dx, dt=900.0, SSH=ssh, c=np.float64(2.7), g=9.81, f=np.float64(1.0e-4),
                     time_scheme="rk2", Kdiffus=15.0)
    h1 = np.asarray(m.step(J(ssh.copy()), J(hb.copy()), nstep=3))
    out.update(c_ssh=ssh, c_dx=dx, c_hb=hb, c_h1=h1)


def main():
    ref_root = _jax_standin.reference_root()
    ref = load_reference(ref_root)
    out = {}
    case_a(ref, out)
    case_b(ref, out)
    case_c(ref, out)
    np.savez_compressed(os.path.join(HERE, "qgtrac_golden.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
