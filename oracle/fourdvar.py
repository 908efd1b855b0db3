"""Restatement of the 4D-Var cost and gradient of the reference
(mapping/src/tools_4Dvar.py:252-400, Variational.cost_and_grad) for a QG
1.5-layer model whose control is the initial SSH. Test infrastructure only.

Semantics kept from the reference:
- checkpoints at every observation step plus the window ends
  (mapping/src/inv.py:144-163); the model is called once per checkpoint
  interval, each call re-deriving PV from SSH (jqgm.py:536);
- Jo accumulates misfit.R^-1.misfit with misfit = inverr*(Hx - y)
  (tools_4Dvar.py:292, obsop.py:610-628); J = (Jo + Jb)/2 (326);
- the observation adjoint uses the misfit itself as cotangent
  (tools_4Dvar.py:391, obsop.py:668-678), which is the gradient of J when
  sigma_R = 1 (the only case used here);
- the background term (optional) is the preconditioned X0.X0 (265, 395-398)
  with X = sigma_B*X0 + Xb.
"""
import numpy as np

from . import obsop as ob


class ObsSet:
    """Observations of one window: per model step, the H rows and data."""

    def __init__(self, x_km, y_km, step, yobs, err, ny, nx, dx, dy, npix=4):
        self.steps = np.unique(step)
        self.ny, self.nx = ny, nx
        self.per_step = {}
        for s in self.steps:
            sel = step == s
            data, rows, cols = ob.sparse_op(x_km[sel], y_km[sel], ny, nx, dx, dy, npix)
            self.per_step[int(s)] = (data, rows, cols, yobs[sel], err[sel])

    def misfit(self, s, h):
        data, rows, cols, y, e = self.per_step[s]
        return ob.misfit(np.asarray(h).ravel(), data, rows, cols, y, e)

    def adj(self, s, mis, h):
        data, rows, cols, y, e = self.per_step[s]
        return ob.misfit_adj(mis, data, rows, cols, e, self.ny * self.nx,
                             x_flat=np.asarray(h).ravel(), yobs=y).reshape(self.ny, self.nx)


def cost_and_grad_h0(qgm, h0, hb, nstep, obs, sigma_R=1.0, sigma_B=None, hbg=None):
    """J(h0) and dJ/dh0 for one window (float64)."""
    steps = [int(s) for s in obs.steps if 0 <= s <= nstep]
    cps = sorted(set([0, nstep] + [s for s in steps if s < nstep]))
    obs_set = set(steps)
    Jo = 0.0
    states = {}
    mis = {}
    h = np.array(h0, dtype=np.float64)
    for i in range(len(cps) - 1):
        t = cps[i]
        if t in obs_set:
            mis[t] = obs.misfit(t, h)
            Jo += mis[t].dot(mis[t]) / sigma_R ** 2
        states[t] = h
        h = qgm.step(h, hb, cps[i + 1] - cps[i])
    states[nstep] = h
    if nstep in obs_set:
        mis[nstep] = obs.misfit(nstep, h)
        Jo += mis[nstep].dot(mis[nstep]) / sigma_R ** 2
    Jb = 0.0
    if sigma_B is not None:
        x0 = (np.asarray(h0) - hbg) / sigma_B
        Jb = x0.ravel().dot(x0.ravel())
    J = 0.5 * (Jo + Jb)

    ad = np.zeros_like(np.asarray(h0, dtype=np.float64))
    if nstep in obs_set:
        ad = ad + obs.adj(nstep, mis[nstep], states[nstep])
    for i in reversed(range(len(cps) - 1)):
        t = cps[i]
        ad = qgm.step_adj(ad, states[t], hb, cps[i + 1] - cps[i])
        if t in obs_set:
            ad = ad + obs.adj(t, mis[t], states[t])
    if sigma_B is not None:
        ad = ad + (np.asarray(h0) - hbg) / sigma_B ** 2
    return J, ad


def checkpoints(nstep, nstep_check, obs_steps):
    """Model steps at which the cost function is evaluated
    (mapping/src/inv.py:144-163): step 0, every observation step, every
    nstep_check-th step, and the last step."""
    obs_steps = set(int(s) for s in obs_steps)
    cps, check = [0], 0
    for i in range(nstep):
        if i > 0 and (i in obs_steps or check == nstep_check):
            cps.append(i)
            if check == nstep_check:
                check = 0
        check += 1
    cps.append(nstep)
    return cps


def cost_and_grad_basis(qgm, basis, time_basis, X0, Xb, Q, h_init, hb, nstep, nstep_check, obs,
                        sigma_R=1.0, prec=True):
    """J(X0) and dJ/dX0 for a reduced-basis control forcing the SSH
    (tools_4Dvar.py:252-400 with Model_qg1l_jax.step / step_adj,
    mod.py:867-913, 1020-1076): at every checkpoint that is a multiple of
    nstep_check the basis writes the forcing F = G(t) X; every model call of
    n steps ends with h += n*dt/86400*F; the adjoint adds n*dt/86400*adh to
    the forcing adjoint before the model adjoint and maps it back with G^T at
    the basis checkpoints. prec: X = Q*X0 + Xb, Jb = X0.X0, G = Q*adX + X0."""
    dt = qgm.dt
    steps = [int(s) for s in obs.steps if 0 <= s <= nstep]
    obs_set = set(steps)
    cps = checkpoints(nstep, nstep_check, [s for s in steps if 0 < s < nstep])
    X0 = np.asarray(X0, np.float64)
    if prec:
        X = Q * X0 + Xb
        Jb = X0.dot(X0)
    else:
        X = X0 + Xb
        Jb = np.dot(X0, X0 / Q ** 2)
    h = np.array(h_init, dtype=np.float64)
    F = np.zeros_like(h)
    Jo = 0.0
    states, mis = {}, {}
    for i in range(len(cps) - 1):
        c, n = cps[i], cps[i + 1] - cps[i]
        if c in obs_set:
            mis[c] = obs.misfit(c, h)
            Jo += mis[c].dot(mis[c]) / sigma_R ** 2
        if c % nstep_check == 0:
            F = basis.operg(time_basis[c // nstep_check], X)
        states[c] = h
        h = qgm.step(h, hb, n) + n * dt / (3600 * 24) * F
    states[nstep] = h
    if nstep in obs_set:
        mis[nstep] = obs.misfit(nstep, h)
        Jo += mis[nstep].dot(mis[nstep]) / sigma_R ** 2
    J = 0.5 * (Jo + Jb)

    adh = np.zeros_like(h)
    adF = np.zeros_like(h)
    adX = np.zeros_like(X)
    if nstep in obs_set:
        adh = adh + obs.adj(nstep, mis[nstep], states[nstep])
    for i in reversed(range(len(cps) - 1)):
        c, n = cps[i], cps[i + 1] - cps[i]
        adF = adF + n * dt / (3600 * 24) * np.nan_to_num(adh)
        adh = qgm.step_adj(adh, states[c], hb, n)
        if c % nstep_check == 0:
            adX = adX + basis.operg_transpose(time_basis[c // nstep_check], adF)
            adF = np.zeros_like(adF)
        if c in obs_set:
            adh = adh + obs.adj(c, mis[c], states[c])
    G = Q * adX + X0 if prec else adX + X0 / Q ** 2
    return J, G
