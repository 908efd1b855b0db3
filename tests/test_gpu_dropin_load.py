"""The drop-in model module loaded the way the reference's model wrapper
loads a model class: by file path with SourceFileLoader and instantiated
with the keyword arguments of Model_qg1l_jax.__init__
(mapping/src/mod.py:479-486, 697-718), then driven through the step_jit /
step_tgl_jit / step_adj_jit names it binds (mod.py:721-723) with the
call forms of mod.py:892, 991, 1055. Results must equal the package import
of the same class bit for bit and the float64 oracle to rounding."""
import os
import warnings
from importlib.machinery import SourceFileLoader

import numpy as np
import pytest
import torch

from oracle.qg1l import QgmOracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIR_MODEL = os.path.join(ROOT, "vardyn_gb300", "model_qg1l")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def load_by_path():
    # mod.py:485 calls SourceFileLoader(...).load_module(), deprecated in
    # Python 3.12 but still what the reference runs
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)
        return SourceFileLoader("qgm", f"{DIR_MODEL}/jqgm.py").load_module()


def reference_kwargs(n, dx, dt, ssh, time_scheme):
    """The keyword arguments of mod.py:697-718 with the defaults of
    config_default.py's QG1L model section."""
    DX = np.full((n, n), dx)
    return dict(dx=DX, dy=DX, dt=dt, SSH=ssh, c=2.7, upwind=3, time_scheme=time_scheme, g=9.81, f=1e-4,
                Wbc=None, Kdiffus=None, Kdiffus_trac=None, bc_trac="OBC", advect_pv=True,
                ageo_velocities=False, constant_c=True, constant_f=True, solver="spectral", tile_size=32,
                tile_overlap=16, mdt=None, bathymetry_PV_term=None)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name_class", ["Qgm", "Qgm_sf"])
def test_loaded_by_path_steps_like_the_package_class(name_class):
    from vardyn_gb300.model_qg1l import jqgm as pkg
    from vardyn_gb300.synthetic import kminus3_ssh
    n, dx, dt, nstep = 48, 1e4, 1200.0, 6
    rng = np.random.default_rng(11)
    h0 = kminus3_ssh(n, n, dx, dx, rng, cutoff_km=30.0)
    hb = np.zeros((n, n))
    kw = reference_kwargs(n, dx, dt, h0, "rk2")
    qgm = load_by_path()
    model = getattr(qgm, name_class)(dtype="float64", **kw)
    twin = getattr(pkg, name_class)(dtype="float64", **kw)
    step, step_tgl, step_adj = model.step_jit, model.step_tgl_jit, model.step_adj_jit
    h1 = step(h0, hb, nstep=nstep)
    dh = 0.01 * rng.standard_normal((n, n))
    ad = rng.standard_normal((n, n))
    dh1 = step_tgl(dh, h0, hb, nstep=nstep)
    adh0 = step_adj(ad, h0, hb, nstep=nstep)
    assert np.array_equal(h1, twin.step_jit(h0, hb, nstep=nstep), equal_nan=True)
    assert np.array_equal(dh1, twin.step_tgl_jit(dh, h0, hb, nstep=nstep))
    assert np.array_equal(adh0, twin.step_adj_jit(ad, h0, hb, nstep=nstep))
    if name_class == "Qgm":
        ref = QgmOracle(dx=kw["dx"], dy=kw["dy"], dt=dt, c=2.7, f=1e-4, time_scheme="rk2")
        assert rel(h1, ref.step(h0, hb, nstep)) < 1e-11
        assert rel(dh1, ref.step_tgl(dh, h0, hb, nstep)) < 1e-10
        assert rel(adh0, ref.step_adj(ad, h0, hb, nstep)) < 1e-10


def test_loaded_by_path_tiles_forward():
    from vardyn_gb300.model_qg1l import jqgm as pkg
    from vardyn_gb300.synthetic import kminus3_ssh
    n, dx, dt = 64, 1e4, 1200.0
    rng = np.random.default_rng(12)
    h0 = kminus3_ssh(n, n, dx, dx, rng, cutoff_km=30.0)
    hb = np.zeros((n, n))
    kw = reference_kwargs(n, dx, dt, h0, "Euler")
    model = load_by_path().QgmWithTiles(dtype="float64", **kw)
    twin = pkg.QgmWithTiles(dtype="float64", **kw)
    h1 = model.step_jit(h0, hb, nstep=3)
    assert np.array_equal(h1, twin.step_jit(h0, hb, nstep=3), equal_nan=True)
    assert np.isfinite(h1).all()
