"""Batched L-BFGS (the outer 4D-Var loop on the device) against scipy's
L-BFGS-B, the algorithm the reference's Inv_4Dvar calls (inv.py:369-375):
window by window the same iterates, iteration and evaluation counts."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
opt = pytest.importorskip("scipy.optimize")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def scipy_run(fun_np, x0, **options):
    r = opt.minimize(fun_np, x0, jac=True, method="L-BFGS-B", options=options)
    return r


def quad_problem(B, n, seed):
    rng = np.random.default_rng(seed)
    As, bs = [], []
    for k in range(B):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        ev = np.logspace(0, 1 + k, n)              # condition 10 .. 10^B
        As.append((Q * ev) @ Q.T)
        bs.append(rng.standard_normal(n))
    return np.stack(As), np.stack(bs)


def test_quadratics_match_scipy():
    from vardyn_gb300.minimize import BatchedLBFGS
    B, n = 3, 40
    A, b = quad_problem(B, n, 1)
    At = torch.as_tensor(A, device="cuda")
    bt = torch.as_tensor(b, device="cuda")

    def fun(x):
        Ax = torch.einsum("bij,bj->bi", At, x)
        return (0.5 * (x * Ax).sum(1) - (bt * x).sum(1)).cpu().numpy(), Ax - bt

    x0 = np.random.default_rng(2).standard_normal((B, n))
    # the first 40 iterations: the same iterates (the direction differs from
    # scipy's compact form only by rounding)
    res = BatchedLBFGS(fun, B, n, maxiter=40).minimize(torch.as_tensor(x0, device="cuda"))
    for k in range(B):
        r = scipy_run(lambda x: (0.5 * x @ A[k] @ x - b[k] @ x, A[k] @ x - b[k]), x0[k], maxiter=40)
        xk = res["x"][k].cpu().numpy()
        assert res["nit"][k] == r.nit, (k, res["nit"][k], r.nit)
        assert res["nfev"][k] == r.nfev, (k, res["nfev"][k], r.nfev)
        assert np.abs(xk - r.x).max() <= 1e-8 * max(1.0, np.abs(r.x).max())
        assert abs(res["fun"][k] - r.fun) <= 1e-10 * max(1.0, abs(r.fun))
    # to convergence: the minimiser (iteration counts may differ by rounding
    # once the reduction test is near its threshold)
    res = BatchedLBFGS(fun, B, n, gtol=1e-9, ftol=1e-15).minimize(torch.as_tensor(x0, device="cuda"))
    for k in range(B):
        xs = np.linalg.solve(A[k], b[k])
        assert res["status"][k] == 0
        assert np.abs(res["x"][k].cpu().numpy() - xs).max() <= 1e-5 * np.abs(xs).max()


def rosen(x):
    return (100.0 * (x[..., 1:] - x[..., :-1] ** 2) ** 2 + (1 - x[..., :-1]) ** 2).sum(-1)


def rosen_grad(x):
    g = np.zeros_like(x)
    xm, xp = x[..., :-1], x[..., 1:]
    g[..., :-1] += -400.0 * xm * (xp - xm ** 2) - 2 * (1 - xm)
    g[..., 1:] += 200.0 * (xp - xm ** 2)
    return g


@pytest.mark.parametrize("n", [2, 6])
def test_rosenbrock_matches_scipy(n):
    from vardyn_gb300.minimize import BatchedLBFGS
    B = 4
    x0 = np.random.default_rng(n).uniform(-2, 2, (B, n))

    def fun(x):
        xn = x.cpu().numpy()
        return rosen(xn), torch.as_tensor(rosen_grad(xn), device="cuda")

    res = BatchedLBFGS(fun, B, n, maxiter=200).minimize(torch.as_tensor(x0, device="cuda"))
    for k in range(B):
        r = scipy_run(lambda x: (rosen(x), rosen_grad(x)), x0[k], maxiter=200)
        assert res["nit"][k] == r.nit and res["nfev"][k] == r.nfev, (k, res["nit"][k], r.nit, res["nfev"][k], r.nfev)
        assert np.abs(res["x"][k].cpu().numpy() - r.x).max() <= 1e-7


def test_4dvar_minimisation_matches_scipy():
    """The outer loop on the real cost: a batch of 2 QG windows (float64
    plan), 8 iterations, against scipy driving the same cost window by
    window."""
    from vardyn_gb300.fourdvar import QGWindows4DVar
    from vardyn_gb300.minimize import minimize_4dvar
    from vardyn_gb300.obsop import AlongTrackObs
    from vardyn_gb300.qg1l import QG1LPlan
    from vardyn_gb300.synthetic import kminus3_ssh, satellite_tracks
    n, nstep, dx = 48, 24, 1.0e4
    wins, guess, truth = [], [], []
    for b in range(2):
        rng = np.random.default_rng(70 + b)
        truth.append(kminus3_ssh(n, n, dx, dx, rng, rms=0.1, cutoff_km=60.0))
        guess.append(0.5 * kminus3_ssh(n, n, dx, dx, rng, rms=0.1, cutoff_km=60.0))
        x, y, st = satellite_tracks(n, n, dx, dx, nstep, 600, rng, spacing_km=12.0)
        wins.append(dict(x_km=x, y_km=y, step=st, err=np.full(x.size, 0.03), yobs=np.zeros(x.size)))
    plan = QG1LPlan(n, n, dx, dx, 1200.0, 1e-4, 2.7, time_scheme="rk2", dtype=torch.float64)
    obs = AlongTrackObs(wins, n, n, dx, dx, dtype=torch.float64)
    eng = QGWindows4DVar(plan, torch.zeros(2, n, n, dtype=torch.float64, device="cuda"), nstep, obs)
    eng.cost_and_grad(torch.as_tensor(np.stack(truth), device="cuda"))
    torch.cuda.synchronize()
    obs.d_y.copy_(obs.misfit[:obs.nobs] * 0.03)

    def cg(x):
        J, G = eng.cost_and_grad(x.reshape(2, n, n))
        return J, G

    x0 = np.stack(guess)
    res = minimize_4dvar(cg, torch.as_tensor(x0, device="cuda"), maxiter=8)
    for k in range(2):
        def fk(xk):
            xb = torch.as_tensor(x0, device="cuda").clone()
            xb[k] = torch.as_tensor(xk.reshape(n, n), device="cuda")
            J, G = eng.cost_and_grad(xb)
            return float(J[k]), G[k].double().cpu().numpy().ravel()
        r = scipy_run(fk, x0[k].ravel(), maxiter=8)
        assert res["nit"][k] == r.nit and res["nfev"][k] == r.nfev, (k, res["nit"][k], r.nit, res["nfev"][k], r.nfev)
        xk = res["x"][k].cpu().numpy().ravel()
        assert np.abs(xk - r.x).max() <= 1e-7 * np.abs(r.x).max()
        assert abs(res["fun"][k] - r.fun) <= 1e-9 * abs(r.fun)


def test_crazy_gradient_restarts_from_best():
    """A window whose gradient blows up restarts from its best state (the
    reference's CrazyGradient handling); the other window is unaffected."""
    from vardyn_gb300.minimize import minimize_4dvar
    B, n = 2, 10
    A, b = quad_problem(B, n, 3)
    At, bt = torch.as_tensor(A, device="cuda"), torch.as_tensor(b, device="cuda")
    calls = {"n": 0}

    def cg(x):
        calls["n"] += 1
        Ax = torch.einsum("bij,bj->bi", At, x)
        J = (0.5 * (x * Ax).sum(1) - (bt * x).sum(1)).cpu().numpy()
        G = Ax - bt
        if calls["n"] == 4:       # one non-finite cost for window 1
            J = J.copy()
            J[1] = np.nan
        return J, G

    x0 = torch.as_tensor(np.ones((B, n)), device="cuda")
    res = minimize_4dvar(cg, x0, gtol=1e-8, ftol=1e-15, max_retries=2)
    assert res["retries"][0] == 0 and res["retries"][1] == 1
    for k in range(B):
        xs = np.linalg.solve(A[k], b[k])
        assert np.abs(res["x"][k].cpu().numpy() - xs).max() <= 1e-5 * np.abs(xs).max()
