"""QG 1.5-layer model with passive tracers on the GPU (vd_qgtrac_step,
drop-in Qgm_trac.step) against the reference's own Qgm_trac outputs
(tests/golden/gen_golden_trac.py) and the float64 oracle."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgtrac_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _rel(a, b):
    m = ~np.isnan(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    return float(np.abs(a[m] - b[m]).max() / np.abs(b[m]).max())


def _case_a(g, cls, **kw):
    return cls(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
               time_scheme=kw.pop("time_scheme", "Euler"), Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC",
               mdt=g["a_mdt"], **kw)


def test_euler_two_tracers_open_boundaries_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, dtype="float64")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=4), g["a_X1"]) < 1e-11


def test_rk2_dirichlet_relaxation_no_pv_advection_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = Qgm_trac(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4,
                 time_scheme="rk2", Wbc=g["b_wbc"], Kdiffus=None, Kdiffus_trac=5.0, bc_trac="dirichlet",
                 advect_pv=False, dtype="float64")
    assert _rel(m.step(g["b_X0"], g["b_Xb"], nstep=3), g["b_X1"]) < 1e-11


def test_rk2_ssh_alone_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = Qgm_trac(dx=g["c_dx"], dy=g["c_dx"], dt=900.0, SSH=g["c_ssh"], c=2.7, g=9.81, f=1.0e-4,
                 time_scheme="rk2", Kdiffus=15.0, dtype="float64")
    assert _rel(m.step(g["c_ssh"], g["c_hb"], nstep=3), g["c_h1"]) < 1e-11


def test_rk4_extension_matches_oracle(g):
    from oracle.qg1l_trac import QgmTracOracle
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, time_scheme="rk4", dtype="float64")
    o = _case_a(g, QgmTracOracle, time_scheme="rk4")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=5), o.step(g["a_X0"], g["a_Xb"], nstep=5)) < 1e-11


def test_float32_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, dtype="float32")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=4), g["a_X1"]) < 1e-4


def test_batched_windows_equal_single_windows(g):
    """Three windows in one call equal three calls (the windows are
    independent); zero steps give the input with NaN on land."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, time_scheme="rk2", dtype="float64")
    rng = np.random.default_rng(4)
    X0 = np.stack([g["a_X0"] + 0.02 * b * rng.standard_normal(g["a_X0"].shape) for b in range(3)])
    Xb = np.stack([g["a_Xb"]] * 3)
    dev = lambda a: torch.as_tensor(a, device="cuda")
    h1, c1 = m.step_windows(dev(X0[:, 0]), dev(X0[:, 1:]), dev(Xb[:, 0]), dev(Xb[:, 1:]), nstep=3)
    for b in range(3):
        one = m.step(X0[b], Xb[b], nstep=3)
        assert _rel(h1[b].cpu().numpy(), one[0]) < 1e-13
        assert _rel(c1[b].cpu().numpy(), one[1:]) < 1e-13
    z = m.step(g["a_X0"], g["a_Xb"], nstep=0)
    land = np.isnan(g["a_X1"][0])
    assert np.all(np.isnan(z[:, land]))
    assert np.allclose(z[:, ~land], g["a_X0"][:, ~land], rtol=0, atol=1e-15)
