"""The library's reduced-basis 4D-Var engine (QGBasis4DVar, float64) against
golden cost and gradient values produced by the reference's own
Variational.cost_and_grad with Model_qg1l_jax, the jax along-track operator
and Basis_gauss3d on a lon/lat grid (tests/golden/gen_golden_fourdvar.py).

The observation operator's rows are the reference's (3-D Cartesian distances
on the lon/lat grid, pinned in tests/test_oracle_obs_golden.py) handed to the
engine; the basis is the library's own geographic BasisPlan; the model is the
QG1.5L plan with the grid's centre spacing (jqgm.py:126-131)."""
import numpy as np
import pytest
import torch

from test_oracle_fourdvar_golden import GeoObs, basis_params, geometry, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.mark.parametrize("tag", ["p", "n"])
def test_reduced_basis_engine_matches_reference(tag):
    from vardyn_gb300.basis import BasisPlan, Gauss3dParams
    from vardyn_gb300.fourdvar import QGBasis4DVar
    from vardyn_gb300.obsop import AlongTrackObs
    from vardyn_gb300.qg1l import QG1LPlan
    g = golden()
    lon, lat, DX, DY = geometry(g)
    ny, nx = lon.shape
    dt64 = torch.float64
    plan = QG1LPlan(ny, nx, DX[ny // 2, nx // 2], DY[ny // 2, nx // 2], float(g["dt"]), 1e-4, 2.7,
                    time_scheme="rk2", dtype=dt64)
    bp = basis_params(g, tag)
    basis = BasisPlan(g["lon"], g["lat"], g[f"{tag}_time_basis"],
                      [Gauss3dParams(normalize_fact=True, flux=False, **bp)], geographic=True, dtype=dt64)
    assert np.allclose(basis.q(), g[f"{tag}_Q"], rtol=1e-14, atol=0)
    geo = GeoObs(g, tag)
    idx, w, step = geo.operator_rows()
    yobs = np.concatenate([g[f"{tag}_obs{s}_SSH"] for s in geo.steps])
    err = np.concatenate([g[f"{tag}_obs{s}_SSH_err"] for s in geo.steps])
    win = dict(step=step, yobs=yobs, err=err)
    obs = AlongTrackObs([win], ny, nx, DX[0, 0], DY[0, 0], dtype=dt64, operator=[(idx, w)])
    hb = torch.zeros(1, ny, nx, dtype=dt64, device="cuda")
    h_init = torch.as_tensor(g[f"{tag}_h_init"][None], device="cuda")
    eng = QGBasis4DVar(plan, basis, h_init, hb, int(g["nstep"]), int(g["nstep_check"]), obs, Q=g[f"{tag}_Q"],
                       Xb=g[f"{tag}_Xb"], prec=bool(g[f"{tag}_prec"]))
    assert eng.cps == [int(c) for c in g[f"{tag}_checkpoints"]]
    J, G = eng.cost_and_grad(torch.as_tensor(g[f"{tag}_X0"][None], device="cuda"))
    J, G = float(J[0]), G[0].cpu().numpy()
    Jr, Gr = float(g[f"{tag}_J"]), g[f"{tag}_G"]
    e_J, e_G = abs(J - Jr) / abs(Jr), np.linalg.norm(G - Gr) / np.linalg.norm(Gr)
    print(f"\ncase {tag}: J {J:.14e} vs reference {Jr:.14e} (rel {e_J:.1e}), gradient rel-L2 {e_G:.1e}")
    assert e_J < 1e-11
    assert e_G < 1e-10
