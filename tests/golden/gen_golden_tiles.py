"""Generate golden vectors for the overlapping-tile QG 1.5-layer model
(``QgmWithTiles``, mapping/models/model_qg1l/jqgm.py:1033-1376) from the
reference's own source code.

As ``gen_golden.py`` does, this installs the NumPy stand-in for jax
(``_jax_standin.py``: vmap, dynamic_slice and dynamic_update_slice included),
loads ``jqgm.py`` unmodified from the reference checkout and records
``QgmWithTiles.step`` on seeded inputs in float64.

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_tiles.py <VarDyn checkout>
Writes ``tests/golden/qgt_golden.npz``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

from gen_golden import J, load_reference  # noqa: E402


def case_a(ref, out):
    """40 x 52, tiles of 20 with overlap 6, Euler, f-plane, land blob, hb != 0,
    diffusion, MDT."""
    rng = np.random.default_rng(4321)
    ny, nx = 40, 52
    dx = np.full((ny, nx), 1.0e4)
    dy = np.full((ny, nx), 1.1e4)
    ssh = 0.1 * rng.standard_normal((ny, nx))
    ssh[17:21, 25:29] = np.nan
    hb = 0.02 * rng.standard_normal((ny, nx))
    hb[np.isnan(ssh)] = 0.0
    mdt = 0.05 * rng.standard_normal((ny, nx))
    m = ref.QgmWithTiles(dx=dx, dy=dy, dt=900.0, SSH=ssh, c=np.float64(2.7), Kdiffus=30.0, g=9.81,
                         f=np.float64(1.0e-4), time_scheme="Euler", mdt=J(mdt), tile_size=20, tile_overlap=6)
    h0 = np.nan_to_num(ssh)
    # step adds the MDT with "+=" (jqgm.py:1346-1348): in jax that rebinds the
    # name, on the NumPy stand-in it writes through, so pass private copies
    h1 = np.asarray(m.step(J(h0.copy()), J(hb.copy()), nstep=4))
    out.update(a_ssh=ssh, a_dx=dx, a_dy=dy, a_hb=hb, a_mdt=mdt, a_h0=h0, a_h1=h1,
               a_tiles=np.asarray(m.tiles, dtype=np.int64), a_wsum=np.asarray(m.weights_space_sum))


def case_b(ref, out):
    """36 x 44, tiles of 16 with overlap 4, rk2, beta plane and spatial c (tile
    means differ), no land, no MDT."""
    rng = np.random.default_rng(8765)
    ny, nx = 36, 44
    dx = np.full((ny, nx), 1.2e4)
    dy = np.full((ny, nx), 1.2e4)
    yy = np.arange(ny)[:, None] * 1.2e4 + np.zeros((1, nx))
    f = 1.0e-4 + 1.6e-11 * (yy - yy.mean())
    c = 2.5 + 0.3 * rng.random((ny, nx))
    ssh = 0.1 * rng.standard_normal((ny, nx))
    hb = 0.01 * rng.standard_normal((ny, nx))
    m = ref.QgmWithTiles(dx=dx, dy=dy, dt=900.0, SSH=ssh, c=c, Kdiffus=None, g=9.81, f=f,
                         time_scheme="rk2", tile_size=16, tile_overlap=4)
    h1 = np.asarray(m.step(J(ssh.copy()), J(hb.copy()), nstep=3))
    out.update(b_ssh=ssh, b_dx=dx, b_dy=dy, b_f=f, b_c=c, b_hb=hb, b_h1=h1,
               b_tiles=np.asarray(m.tiles, dtype=np.int64))


def main():
    ref_root = _jax_standin.reference_root()
    ref = load_reference(ref_root)
    out = {}
    case_a(ref, out)
    case_b(ref, out)
    np.savez_compressed(os.path.join(HERE, "qgt_golden.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
