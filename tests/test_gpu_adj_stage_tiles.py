"""The QG 1.5-layer adjoint stage in its two staging forms.

Grids whose rows are a multiple of 16 elements stage the stage's tiles (h, q,
q + bathymetry, the stage adjoints G_t, beta and the mask) in shared memory
with bulk tensor copies, which fill out-of-grid cells with zeros; other grids,
or the schedule choice ``stencil_loads=1``, load the same tiles with
bounds-checked loads. The arithmetic after staging is the same, so the two
forms agree bit for bit. The staged form is also checked against the float64
oracle's adjoint (jqgm.py:559-569) and by a dot product with the tangent."""
import numpy as np
import pytest
import torch

from oracle.qg1l import QgmOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def _plan(ny, nx, dtype, scheme, bathy, beta, K, land, seed=0):
    from vardyn_gb300.qg1l import QG1LPlan, build_mask
    rng = np.random.default_rng(seed)
    ssh = np.zeros((ny, nx))
    if land:
        ssh[ny // 3:ny // 3 + 3, nx // 2:nx // 2 + 2] = np.nan
    kw = dict(Kdiffus=30.0 if K else None, mask=build_mask(ny, nx, ssh),
              beta=(1.6e-11 + 1e-13 * (np.arange(ny)[:, None] - ny / 2)) * np.ones((1, nx)) if beta else None,
              fbathy=1e-5 * rng.standard_normal((ny, nx)) if bathy else None)
    return QG1LPlan(ny, nx, 1e4, 1e4, 900.0, 1e-4, 2.7, time_scheme=scheme, dtype=dtype, **kw), rng


def _both(plan, fn):
    out = []
    for mode in (0, 1):
        plan.set_schedule(stencil_loads=mode)
        r = fn()
        out.append([x.clone() for x in (r if isinstance(r, (tuple, list)) else (r,))])
    plan.set_schedule(stencil_loads=0)
    return out


def _device_error():
    import ctypes
    from vardyn_gb300 import _lib
    v = ctypes.c_int(0)
    _lib.call("vd_device_error", ctypes.byref(v), 1)
    return v.value


CASES = [(40, 48, True, True, True, True), (72, 80, False, True, False, True), (64, 128, True, False, True, False),
         (37, 16, False, False, True, False)]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("ny,nx,bathy,beta,K,land", CASES)
def test_stage_building_block_staged_equals_checked(dtype, ny, nx, bathy, beta, K, land):
    """vd_qg1l_rk_stage_adj with 1 to 4 stage adjoints and 0 to 4 addends over
    3 fields (ragged tiles in x and y, land, every optional term)."""
    plan, rng = _plan(ny, nx, dtype, "rk4", bathy, beta, K, land)
    T = lambda a: torch.as_tensor(a, dtype=dtype, device="cuda")
    B = 3
    hs = T(0.1 * rng.standard_normal((B, ny, nx)))
    qs = T(1e-5 * rng.standard_normal((B, ny, nx)))
    for ng, na in ((1, 0), (2, 2), (4, 4), (3, 1)):
        g = [T(rng.standard_normal((B, ny, nx))) for _ in range(ng)]
        c = list(rng.uniform(0.1, 1.0, ng))
        acc = [T(rng.standard_normal((B, ny, nx))) for _ in range(na)]
        a, b = _both(plan, lambda: plan.rk_stage_adj(hs, qs, g, c, acc))
        for x, y in zip(a, b):
            assert torch.equal(x, y), (ng, na, float((x - y).abs().max()))
    torch.cuda.synchronize()
    assert _device_error() == 0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("scheme", ["rk2", "rk3"])
def test_window_adjoint_staged_equals_checked(dtype, scheme):
    plan, rng = _plan(72, 80, dtype, scheme, True, True, True, True, seed=3)
    T = lambda a: torch.as_tensor(a, dtype=dtype, device="cuda")
    h0 = T(0.1 * rng.standard_normal((2, 72, 80)))
    hb = T(0.01 * rng.standard_normal((2, 72, 80)))
    ad = T(rng.standard_normal((2, 72, 80)))
    a, b = _both(plan, lambda: plan.step_adj(ad, h0, hb, 4))
    assert torch.isfinite(a[0]).all()
    assert torch.equal(a[0], b[0])


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk4"])
def test_staged_adjoint_fp64_matches_oracle(scheme):
    """nx = 48: the staged form, with land, beta, bathymetry and diffusion."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm
    ny, nx = 40, 48
    rng = np.random.default_rng(11)
    dx = np.full((ny, nx), 1.0e4)
    f = 1e-4 + 1.6e-11 * (np.arange(ny)[:, None] * 1e4 + np.zeros((1, nx)))
    ssh = 0.1 * rng.standard_normal((ny, nx))
    ssh[20:22, 30:33] = np.nan
    kw = dict(dx=dx, dy=dx, dt=900.0, SSH=ssh, c=2.7, f=f, time_scheme=scheme, Kdiffus=30.0,
              bathymetry_PV_term=0.03 * rng.standard_normal((ny, nx)))
    ref = QgmOracle(**kw)
    m = Qgm(dtype="float64", **kw)
    assert m.plan.schedule()["stencil_loads"] == 0
    h0, hb = np.nan_to_num(ssh), 0.01 * rng.standard_normal((ny, nx))
    ad = rng.standard_normal((ny, nx))
    got, exp = np.asarray(m.step_adj(ad, h0, hb, 4)), ref.step_adj(ad, h0, hb, 4)
    assert np.linalg.norm(got - exp) <= 1e-10 * np.linalg.norm(exp)
