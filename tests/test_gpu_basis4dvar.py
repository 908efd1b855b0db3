"""4D-Var with a reduced-basis control forcing the SSH (the reference's
Inv_4Dvar with Basis_multi of Gaussian components) on the GPU, against the
float64 oracle of tools_4Dvar.py:252-400 + mod.py:867-1076."""
import numpy as np
import pytest
import torch

from oracle.basis import Gauss3dOracle, MultiOracle
from oracle.fourdvar import ObsSet, checkpoints, cost_and_grad_basis
from oracle.qg1l import QgmOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


COMPS = [dict(sigma_D=60, sigma_T=0.15, facns=1.0, facnlt=2.0, sigma_Q=0.05),
         dict(sigma_D=110, sigma_T=0.3, facns=1.5, facnlt=2.0, sigma_Q=0.08)]


def case(dtype, B=2, ny=40, nx=48, nstep=30, nstep_check=6, nobs=300, seed=11):
    from vardyn_gb300.basis import BasisPlan, Gauss3dParams
    from vardyn_gb300.fourdvar import QGBasis4DVar
    from vardyn_gb300.obsop import AlongTrackObs
    from vardyn_gb300.qg1l import QG1LPlan
    from vardyn_gb300.synthetic import kminus3_ssh, satellite_tracks
    dx, dt = 5e3, 900.0
    rng = np.random.default_rng(seed)
    xk, yk = np.arange(nx) * dx / 1e3, np.arange(ny) * dx / 1e3
    time_basis = np.arange(0, nstep * dt + nstep_check * dt, nstep_check * dt) / 24 / 3600
    plan_b = BasisPlan(xk, yk, time_basis, [Gauss3dParams(**c) for c in COMPS], dtype=dtype)
    lon, lat = np.meshgrid(xk, yk)
    orc_b = MultiOracle([Gauss3dOracle(lon, lat, **c) for c in COMPS])
    Xb, Q = orc_b.set_basis(time_basis)
    wins, obs_sets, h_init = [], [], []
    for b in range(B):
        x, y, st = satellite_tracks(ny, nx, dx, dx, nstep, nobs, rng, spacing_km=6.5)
        st[:8] = 0
        st[-5:] = nstep
        w = dict(x_km=x, y_km=y, step=st, err=np.full(x.size, 0.03),
                 yobs=0.1 * rng.standard_normal(x.size))
        wins.append(w)
        obs_sets.append(ObsSet(x, y, st, w["yobs"], w["err"], ny, nx, dx, dx))
        h_init.append(kminus3_ssh(ny, nx, dx, dx, rng, rms=0.1, cutoff_km=20.0))
    h_init = np.stack(h_init)
    ref = QgmOracle(dx=np.full((ny, nx), dx), dy=np.full((ny, nx), dx), dt=dt, c=2.7, f=1e-4,
                    time_scheme="rk2")
    plan = QG1LPlan(ny, nx, dx, dx, dt, 1e-4, 2.7, time_scheme="rk2", dtype=dtype)
    obs = AlongTrackObs(wins, ny, nx, dx, dx, dtype=dtype)
    hb = torch.zeros(B, ny, nx, dtype=dtype, device="cuda")
    eng = QGBasis4DVar(plan, plan_b, torch.as_tensor(h_init, device="cuda").to(dtype), hb, nstep, nstep_check,
                       obs)
    X0 = rng.standard_normal((B, plan_b.nbasis))
    return eng, ref, orc_b, time_basis, Xb, Q, obs_sets, h_init, X0


def test_checkpoint_list_matches_oracle():
    from vardyn_gb300.fourdvar import checkpoints as cps_gpu
    rng = np.random.default_rng(0)
    for _ in range(20):
        nstep = int(rng.integers(5, 60))
        nck = int(rng.integers(1, 12))
        obs = rng.integers(0, nstep + 1, size=int(rng.integers(0, 10)))
        assert cps_gpu(nstep, nck, obs) == checkpoints(nstep, nck, obs)


def test_basis_4dvar_fp64_matches_oracle():
    eng, ref, orc_b, tb, Xb, Q, obs_sets, h_init, X0 = case(torch.float64)
    assert len(eng.cps) > eng.nstep // eng.nstep_check + 2      # observation intervals split basis intervals
    J, G = eng.cost_and_grad(torch.as_tensor(X0, device="cuda"))
    J, G = J.cpu().numpy(), G.cpu().numpy()
    hb = np.zeros(h_init.shape[1:])
    for b in range(X0.shape[0]):
        Jr, Gr = cost_and_grad_basis(ref, orc_b, tb, X0[b], Xb, Q, h_init[b], hb, eng.nstep, eng.nstep_check,
                                     obs_sets[b])
        assert abs(J[b] - Jr) / Jr < 1e-11, (J[b], Jr)
        assert rel(G[b], Gr) < 1e-10, rel(G[b], Gr)


def test_basis_4dvar_fp32_error_and_graph():
    eng, ref, orc_b, tb, Xb, Q, obs_sets, h_init, X0 = case(torch.float32)
    x = torch.as_tensor(X0, device="cuda", dtype=torch.float32)
    J, G = [t.clone() for t in eng.cost_and_grad(x)]
    hb = np.zeros(h_init.shape[1:])
    for b in range(X0.shape[0]):
        Jr, Gr = cost_and_grad_basis(ref, orc_b, tb, X0[b], Xb, Q, h_init[b], hb, eng.nstep, eng.nstep_check,
                                     obs_sets[b])
        print(f"window {b}: J rel err {abs(float(J[b]) - Jr) / Jr:.2e}, grad rel-L2 "
              f"{rel(G[b].double().cpu().numpy(), Gr):.2e}")
        assert abs(float(J[b]) - Jr) / Jr < 1e-5
        assert rel(G[b].double().cpu().numpy(), Gr) < 1e-4
    eng.capture()
    J2, G2 = [t.clone() for t in eng.cost_and_grad(x)]
    assert torch.equal(J, J2) and torch.equal(G, G2)


def test_basis_4dvar_central_differences_fp64():
    eng, *_, X0 = case(torch.float64, B=1, nstep=18)
    x = torch.as_tensor(X0, device="cuda")
    J0, G = [t.clone() for t in eng.cost_and_grad(x)]
    d = torch.as_tensor(np.random.default_rng(3).standard_normal(X0.shape), device="cuda")
    d /= d.abs().max()
    gd = float((G * d).sum())
    errs = []
    for eps in (1e-2, 1e-3, 1e-4, 1e-5):
        Jp = float(eng.cost_and_grad(x + eps * d)[0][0])
        Jm = float(eng.cost_and_grad(x - eps * d)[0][0])
        errs.append(abs((Jp - Jm) / (2 * eps) - gd) / abs(gd))
    print("central-difference relative errors:", ["%.1e" % e for e in errs])
    assert min(errs) < 1e-7, errs
