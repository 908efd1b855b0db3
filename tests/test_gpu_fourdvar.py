"""4D-Var cost and gradient on the GPU (observation operator, window engine,
checkpointing, CUDA-graph replay) against the float64 oracle."""
import numpy as np
import pytest
import torch

from oracle import obsop as oob
from oracle.fourdvar import ObsSet, cost_and_grad_h0
from oracle.qg1l import QgmOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make_windows(B, ny, nx, dx, nstep, nobs, seed, with_step0=True):
    from vardyn_gb300.synthetic import kminus3_ssh, satellite_tracks
    rng = np.random.default_rng(seed)
    wins, truths = [], []
    for b in range(B):
        truth = kminus3_ssh(ny, nx, dx, dx, rng, rms=0.1, cutoff_km=4 * dx / 1e3)
        x, y, st = satellite_tracks(ny, nx, dx, dx, nstep, nobs, rng, spacing_km=dx / 1e3 * 1.3)
        if with_step0:
            st[:10] = 0
        st[-7:] = nstep
        wins.append(dict(x_km=x, y_km=y, step=st, err=np.full(x.size, 0.03)))
        truths.append(truth)
    return wins, truths


def test_obs_operator_matches_oracle():
    from vardyn_gb300.obsop import AlongTrackObs
    ny, nx, dx = 40, 52, 5e3
    rng = np.random.default_rng(3)
    wins, _ = make_windows(2, ny, nx, dx, 10, 300, seed=1)
    fields = rng.standard_normal((2, ny, nx))
    fields[1, 5, 5] = np.nan
    for w in wins:
        w["yobs"] = rng.standard_normal(w["x_km"].size)
    obs = AlongTrackObs(wins, ny, nx, dx, dx, dtype=torch.float64)
    F = torch.as_tensor(fields, device="cuda")
    ad = torch.zeros(2, ny, nx, dtype=torch.float64, device="cuda")
    for s in obs.steps:
        obs.apply_misfit(int(s), F)
        obs.apply_adjoint(int(s), ad)
    mis = obs.misfit.cpu().numpy()
    exp_ad = np.zeros((2, ny, nx))
    for b, w in enumerate(wins):
        for s in np.unique(w["step"]):
            sel = w["step"] == s
            data, rows, cols = oob.sparse_op(w["x_km"][sel], w["y_km"][sel], ny, nx, dx, dx)
            m = oob.misfit(fields[b].ravel(), data, rows, cols, w["yobs"][sel], w["err"][sel])
            got = mis[(obs.obs_window == b) & (obs.obs_step == s)]
            # GPU storage is time-major, within a step window-major, within a
            # window in input order
            assert np.allclose(got, m, rtol=1e-13, atol=1e-13)
            exp_ad[b] += oob.misfit_adj(m, data, rows, cols, w["err"][sel], ny * nx).reshape(ny, nx)
    assert rel(ad.cpu().numpy(), exp_ad) < 1e-13


def engine_case(dtype, B=2, ny=48, nx=56, nstep=24, nobs=400, seed=5, checkpoint=None):
    from vardyn_gb300.fourdvar import QGWindows4DVar
    from vardyn_gb300.obsop import AlongTrackObs
    from vardyn_gb300.qg1l import QG1LPlan
    dx = 5e3
    wins, truths = make_windows(B, ny, nx, dx, nstep, nobs, seed)
    ref = QgmOracle(dx=np.full((ny, nx), dx), dy=np.full((ny, nx), dx), dt=900.0, c=2.7, f=1e-4,
                    time_scheme="rk2")
    hb = np.zeros((ny, nx))
    rng = np.random.default_rng(seed + 100)
    obs_sets = []
    for b, w in enumerate(wins):
        # observations of a model run from the truth plus noise
        ytrue = np.zeros(w["x_km"].size)
        h = truths[b]
        prev = 0
        for s in sorted(np.unique(w["step"])):
            if s > prev:
                h = ref.step(h, hb, int(s - prev))
                prev = s
            sel = w["step"] == s
            data, rows, cols = oob.sparse_op(w["x_km"][sel], w["y_km"][sel], ny, nx, dx, dx)
            hx = np.zeros(sel.sum())
            np.add.at(hx, rows, data * h.ravel()[cols])
            ytrue[sel] = hx
        w["yobs"] = ytrue + 0.03 * rng.standard_normal(ytrue.size)
        obs_sets.append(ObsSet(w["x_km"], w["y_km"], w["step"], w["yobs"], w["err"], ny, nx, dx, dx))
    plan = QG1LPlan(ny, nx, dx, dx, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=dtype)
    obs = AlongTrackObs(wins, ny, nx, dx, dx, dtype=dtype)
    hbt = torch.zeros(B, ny, nx, dtype=dtype, device="cuda")
    eng = QGWindows4DVar(plan, hbt, nstep, obs, checkpoint=checkpoint)
    h0 = np.stack([0.5 * t for t in truths])
    return eng, ref, obs_sets, h0, hb


def test_cost_and_grad_fp64_matches_oracle():
    eng, ref, obs_sets, h0, hb = engine_case(torch.float64)
    J, G = eng.cost_and_grad(torch.as_tensor(h0, device="cuda"))
    J, G = J.cpu().numpy(), G.cpu().numpy()
    for b in range(h0.shape[0]):
        Jr, Gr = cost_and_grad_h0(ref, h0[b], hb, eng.nstep, obs_sets[b])
        assert abs(J[b] - Jr) / Jr < 1e-11
        assert rel(G[b], Gr) < 1e-10


def test_cost_and_grad_fp32_error():
    """FP32 bulk with FP64 reductions: gradient relative L2 <= 1e-4 vs FP64."""
    eng, ref, obs_sets, h0, hb = engine_case(torch.float32)
    J, G = eng.cost_and_grad(torch.as_tensor(h0, device="cuda", dtype=torch.float32))
    J, G = J.cpu().numpy(), G.cpu().numpy()
    for b in range(h0.shape[0]):
        Jr, Gr = cost_and_grad_h0(ref, h0[b], hb, eng.nstep, obs_sets[b])
        print(f"window {b}: J rel err {abs(J[b] - Jr) / Jr:.2e}, grad rel-L2 {rel(G[b], Gr):.2e}")
        assert abs(J[b] - Jr) / Jr < 1e-5
        assert rel(G[b], Gr) < 1e-4


def test_checkpointed_equals_full():
    eng, _, _, h0, _ = engine_case(torch.float64, nstep=30)
    eng_c, _, _, _, _ = engine_case(torch.float64, nstep=30, checkpoint=7)
    x = torch.as_tensor(h0, device="cuda")
    J1, G1 = [t.clone() for t in eng.cost_and_grad(x)]
    J2, G2 = [t.clone() for t in eng_c.cost_and_grad(x)]
    assert torch.allclose(J1, J2, rtol=1e-13, atol=0)
    assert rel(G2.cpu().numpy(), G1.cpu().numpy()) < 1e-13
    assert eng_c.memory_bytes() < eng.memory_bytes()


@pytest.mark.parametrize("dtype,slots,unit", [(torch.float64, 2, 3), (torch.float32, 3, 2), (torch.float32, 0, 4),
                                              (torch.float64, 5, 1)])
def test_revolve_equals_full_trajectory(dtype, slots, unit):
    """The binomial schedule recomputes the same trajectory: cost and gradient
    equal the full-trajectory engine's bit for bit, with the memory of
    slots + 1 snapshots and one unit."""
    eng, _, _, h0, _ = engine_case(dtype, nstep=30)
    eng_r, _, _, _, _ = engine_case(dtype, nstep=30, checkpoint=("revolve", slots, unit))
    x = torch.as_tensor(h0, device="cuda", dtype=dtype)
    J1, G1 = [t.clone() for t in eng.cost_and_grad(x)]
    J2, G2 = [t.clone() for t in eng_r.cost_and_grad(x)]
    assert torch.equal(J1, J2) and torch.equal(G1, G2)
    assert eng_r.memory_bytes() < eng.memory_bytes()
    eng_r.capture()
    J3, G3 = [t.clone() for t in eng_r.cost_and_grad(x)]
    assert torch.equal(J3, J1) and torch.equal(G3, G1)


def test_graph_replay_equals_eager():
    eng, _, _, h0, _ = engine_case(torch.float32, nstep=16)
    x = torch.as_tensor(h0, device="cuda", dtype=torch.float32)
    J1, G1 = [t.clone() for t in eng.cost_and_grad(x)]
    eng.capture()
    J2, G2 = [t.clone() for t in eng.cost_and_grad(x)]
    assert torch.equal(J1, J2) and torch.equal(G1, G2)
    J3, G3 = [t.clone() for t in eng.cost_and_grad(1.1 * x)]
    assert not torch.equal(J3, J2)


def test_gradient_central_differences_fp64():
    """dJ/dh0 . d against (J(h0+eps d) - J(h0-eps d)) / 2eps for eps = 1e-3 ..
    1e-6 along a smooth direction of unit maximum (the form of the
    reference's grad_test, tools_4Dvar.py:402-413): the error falls with eps
    until rounding and gets below 1e-7."""
    from vardyn_gb300.synthetic import kminus3_ssh
    eng, _, _, h0, _ = engine_case(torch.float64, B=1, nstep=20)
    x = torch.as_tensor(h0, device="cuda")
    J0, G = [t.clone() for t in eng.cost_and_grad(x)]
    dd = kminus3_ssh(h0.shape[1], h0.shape[2], 5e3, 5e3, np.random.default_rng(9), cutoff_km=30.0)
    d = torch.as_tensor((dd / np.abs(dd).max())[None], device="cuda")
    gd = float((G * d).sum())
    errs = []
    for eps in (1e-3, 1e-4, 1e-5, 1e-6):
        Jp = float(eng.cost_and_grad(x + eps * d)[0][0])
        Jm = float(eng.cost_and_grad(x - eps * d)[0][0])
        errs.append(abs((Jp - Jm) / (2 * eps) - gd) / abs(gd))
    print("central-difference relative errors:", ["%.1e" % e for e in errs])
    assert min(errs) < 1e-7, errs
    assert errs[1] < errs[0] or errs[0] < 1e-7


def test_mixed_sizes_match_single_windows_and_graph():
    """Windows of three grid sizes on concurrent streams (and as one CUDA
    graph) give each window's single-window cost and gradient."""
    from vardyn_gb300.fourdvar import MixedWindows4DVar, QGWindows4DVar
    from vardyn_gb300.obsop import AlongTrackObs
    from vardyn_gb300.qg1l import QG1LPlan
    dx, nstep = 5e3, 12
    engines, xs, singles = [], [], []
    for n, B, seed in ((40, 2, 1), (56, 1, 2), (72, 2, 3)):
        wins, truths = make_windows(B, n, n, dx, nstep, 150, seed)
        rng = np.random.default_rng(seed)
        for w in wins:
            w["yobs"] = 0.05 * rng.standard_normal(w["x_km"].size)
        plan = QG1LPlan(n, n, dx, dx, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=torch.float64)
        obs = AlongTrackObs(wins, n, n, dx, dx, dtype=torch.float64)
        engines.append(QGWindows4DVar(plan, torch.zeros(B, n, n, dtype=torch.float64, device="cuda"), nstep, obs))
        x = torch.as_tensor(0.5 * np.stack(truths), device="cuda")
        xs.append(x)
        for b in range(B):
            o1 = AlongTrackObs(wins[b:b + 1], n, n, dx, dx, dtype=torch.float64)
            e1 = QGWindows4DVar(plan, torch.zeros(1, n, n, dtype=torch.float64, device="cuda"), nstep, o1)
            J1, G1 = e1.cost_and_grad(x[b:b + 1])
            singles.append((float(J1[0]), G1[0].cpu().numpy().copy()))
    mixed = MixedWindows4DVar(engines)
    out = [(J.cpu().numpy().copy(), G.cpu().numpy().copy()) for J, G in mixed.cost_and_grad(xs)]
    k = 0
    for J, G in out:
        for b in range(J.shape[0]):
            Js, Gs = singles[k]
            assert abs(J[b] - Js) <= 1e-12 * abs(Js)
            assert rel(G[b], Gs) < 1e-12
            k += 1
    mixed.capture()
    out2 = [(J.cpu().numpy().copy(), G.cpu().numpy().copy()) for J, G in mixed.cost_and_grad(xs)]
    for (J, G), (J2, G2) in zip(out, out2):
        assert np.array_equal(J, J2) and np.array_equal(G, G2)
