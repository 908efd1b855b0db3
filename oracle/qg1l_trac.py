"""Float64 NumPy restatement of the QG 1.5-layer model with passive tracers of
the reference (mapping/models/model_qg1l/jqgm.py, class ``Qgm_trac``,
1551-2151), forward only.

Test infrastructure only: a CUDA form of this model would be checked against
this module; the product never imports it.

Pinning: ``step`` reproduces golden vectors generated by the reference's own
``jqgm.py`` source (``tests/golden/gen_golden_trac.py``, checked in
``tests/test_oracle_qg1l_trac.py``).

The model (line numbers in jqgm.py):
- the SSH / PV part is ``Qgm``'s (h2uv 1699-1723, h2pv 1725-1754, pv2h
  1756-1769 are the same functions), with PV advection switchable
  (``advect_pv``) and the beta term inside that switch (1806-1815);
- every tracer is advected by the same 3rd-order upwind scheme with the
  geostrophic velocities (plus ageostrophic ones when ``ageo_velocities``),
  diffused with ``Kdiffus_trac``, and zeroed on land only (1827-1866);
- after each step the tracers get open boundary conditions on the domain
  edge (Mellor 1996, with the start-of-step velocities and state, 1957-1996)
  or, with any other ``bc_trac``, their boundary values on the ring classes,
  then a relaxation to the boundary field with weights ``Wbc`` on the
  interior (2002-2003; ``Wbc`` defaults to 1 on class-1 points, 1657-1661);
- Euler and rk2 time schemes (1897-1922). The reference's rk4 (1924-1955)
  cannot run: it calls ``qrhs_jit``, which the class does not define, and
  names undefined variables. ``time_scheme='rk4'`` here is the classical
  Runge-Kutta 4 that method sets out to be, on the stacked state [q,
  tracers...]: k_s = dt * rhs(velocities of pv2h(q_s), state_s) with states
  var0, var0 + k1/2, var0 + k2/2, var0 + k3 (the reference's text has var0 +
  k2 for the last one, which is not RK4), var1 = var0 + (k1 + 2 k2 + 2 k3 +
  k4) / 6. It is an extension, checked by its order of convergence.

``ageo_velocities`` is restated but not pinned: with it the reference's
boundary stack holds the ageostrophic fields too (``cb = Xb[1:]``, 2079),
one more than the state's tracers, and its boundary loop indexes past them.
"""
import numpy as np

from oracle.qg1l import QgmOracle


class QgmTracOracle(QgmOracle):
    """Qgm_trac(dx, dy, dt, SSH, c, upwind, g, f, time_scheme, Wbc, Kdiffus,
    Kdiffus_trac, bc_trac, mdt, ageo_velocities, advect_pv)."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, upwind=3, g=9.81, f=1e-4,
                 time_scheme="Euler", Wbc=None, Kdiffus=None, Kdiffus_trac=None, bc_trac="OBC", mdt=None,
                 ageo_velocities=False, advect_pv=True, **kwargs):
        if time_scheme not in ("Euler", "rk2", "rk4"):
            raise ValueError("Qgm_trac steps with 'Euler', 'rk2' or 'rk4' (classical, an extension)")
        super().__init__(dx=dx, dy=dy, dt=dt, SSH=SSH, c=c, Kdiffus=Kdiffus, upwind=upwind, g=g, f=f,
                         time_scheme=time_scheme, mdt=mdt)
        if Wbc is None or np.all(np.asarray(Wbc) == 0.0):
            self.Wbc = np.zeros((self.ny, self.nx))
            self.Wbc[self.ind1] = 1.0
        else:
            self.Wbc = np.asarray(Wbc, dtype=np.float64)
        self.Kdiffus_trac = Kdiffus_trac
        self.bc_trac = bc_trac
        self.advect_pv = advect_pv
        self.ageo = ageo_velocities

    @staticmethod
    def _upwind(u, v):
        uT = 0.5 * (u[1:-1, 1:-1] + u[1:-1, 2:])
        vT = 0.5 * (v[1:-1, 1:-1] + v[2:, 1:-1])
        return (np.where(uT < 0, 0, uT), np.where(vT < 0, 0, vT), np.where(uT > 0, 0, uT),
                np.where(vT > 0, 0, vT))

    def _diffuse(self, r, a, K):
        r[2:-2, 2:-2] = r[2:-2, 2:-2] + K / self.dx ** 2 * (a[2:-2, 3:-1] + a[2:-2, 1:-3] - 2 * a[2:-2, 2:-2]) + \
            K / self.dy ** 2 * (a[3:-1, 2:-2] + a[1:-3, 2:-2] - 2 * a[2:-2, 2:-2])
        return r

    def rhs_state(self, u, v, ua, va, var):
        """Tendency of the stacked state [q, tracers...] (jqgm.py:1771-1874)."""
        q0 = var[0]
        up, vp, um, vm = self._upwind(u, v)
        if self.advect_pv:
            rq = self.adv(up, vp, um, vm, q0)
            if self.beta is not None:
                rq[2:-2, 2:-2] = rq[2:-2, 2:-2] - self.beta[1:-1, 2:-2] * (v[2:-2, 2:-2] + v[3:-1, 2:-2]) / 2
        else:
            rq = np.zeros_like(q0)
        if self.Kdiffus is not None:
            rq = self._diffuse(rq, q0, self.Kdiffus)
        rq = np.where(np.isnan(rq), 0, rq)
        rq[self.ind12] = 0
        rq[self.ind0] = 0
        out = [rq]
        if var.shape[0] > 1:
            if self.ageo:
                uap, vap, uam, vam = self._upwind(ua, va)
                up, vp, um, vm = up + uap, vp + vap, um + uam, vm + vam
            for ci in var[1:]:
                rc = self.adv(up, vp, um, vm, ci)
                if self.Kdiffus_trac is not None:
                    rc = self._diffuse(rc, ci, self.Kdiffus_trac)
                rc = np.where(np.isnan(rc), 0, rc)
                rc[self.ind0] = 0
                out.append(rc)
        return np.stack(out)

    def bc(self, var1, var0, u, v, varb):
        """Tracer boundary conditions and relaxation (jqgm.py:1957-2006)."""
        if varb.shape[0] <= 1:
            return var1
        var1 = var1.copy()
        dt, dx, dy = self.dt, self.dx, self.dy
        r1S = 0.5 * dt / dy * (v[1, 1:-1] + np.abs(v[1, 1:-1]))
        r2S = 0.5 * dt / dy * (v[1, 1:-1] - np.abs(v[1, 1:-1]))
        r1N = 0.5 * dt / dy * (v[-1, 1:-1] + np.abs(v[-1, 1:-1]))
        r2N = 0.5 * dt / dy * (v[-1, 1:-1] - np.abs(v[-1, 1:-1]))
        r1W = 0.5 * dt / dx * (u[1:-1, 1] + np.abs(u[1:-1, 1]))
        r2W = 0.5 * dt / dx * (u[1:-1, 1] - np.abs(u[1:-1, 1]))
        r1E = 0.5 * dt / dx * (u[1:-1, -1] + np.abs(u[1:-1, -1]))
        r2E = 0.5 * dt / dx * (u[1:-1, -1] - np.abs(u[1:-1, -1]))
        W = self.Wbc[1:-1, 1:-1]
        for i in range(1, varb.shape[0]):
            a, b = var0[i], varb[i]
            if self.bc_trac == "OBC":
                var1[i, 0, 1:-1] = a[0, 1:-1] - (r1S * (a[0, 1:-1] - b[0, 1:-1]) + r2S * (a[1, 1:-1] - a[0, 1:-1]))
                var1[i, -1, 1:-1] = a[-1, 1:-1] - (r1N * (a[-1, 1:-1] - a[-2, 1:-1]) +
                                                  r2N * (b[-1, 1:-1] - a[-1, 1:-1]))
                var1[i, 1:-1, 0] = a[1:-1, 0] - (r1W * (a[1:-1, 0] - b[1:-1, 0]) + r2W * (a[1:-1, 1] - a[1:-1, 0]))
                var1[i, 1:-1, -1] = a[1:-1, -1] - (r1E * (a[1:-1, -1] - a[1:-1, -2]) +
                                                  r2E * (b[1:-1, -1] - a[1:-1, -1]))
            else:
                var1[i][self.ind12] = b[self.ind12]
            var1[i, 1:-1, 1:-1] = W * b[1:-1, 1:-1] + (1 - W) * var1[i, 1:-1, 1:-1]
        return var1

    def one_step_state(self, h0, ua, va, var0, hb, varb):
        """jqgm.py:2008-2046."""
        u, v = self.h2uv(h0)
        qb = varb[0]
        incr = self.rhs_state(u, v, ua, va, var0)
        if self.time_scheme == "Euler":
            var1 = var0 + self.dt * incr
        elif self.time_scheme == "rk2":
            var12 = var0 + 0.5 * incr * self.dt
            u12, v12 = self.h2uv(self.pv2h(var12[0], hb, qb))
            var1 = var0 + self.dt * self.rhs_state(u12, v12, ua, va, var12)
        else:
            k = [incr * self.dt]
            for a in (0.5, 0.5, 1.0):
                vs = var0 + a * k[-1]
                us, ws = self.h2uv(self.pv2h(vs[0], hb, qb))
                k.append(self.rhs_state(us, ws, ua, va, vs) * self.dt)
            var1 = var0 + (k[0] + 2 * k[1] + 2 * k[2] + k[3]) / 6.0
        h1 = self.pv2h(var1[0], hb, qb)
        ubc, vbc = (u + ua, v + va) if ua is not None else (u, v)
        return h1, self.bc(var1, var0, ubc, vbc, varb)

    def step(self, X0, Xb, nstep=1):
        """jqgm.py:2057-2139: X0 is the SSH, or [SSH, (ua, va,) tracers...]."""
        X0 = np.array(X0, dtype=np.float64)
        Xb = np.array(Xb, dtype=np.float64)
        stacked = X0.ndim == 3
        ua = va = None
        if stacked:
            h0 = X0[0].copy()
            if self.ageo:
                ua, va = X0[1].copy(), X0[2].copy()
                c0 = X0[3:].copy()
            else:
                c0 = X0[1:].copy()
            hb = Xb[0].copy()
            cb = Xb[1:].copy()
            c0[:, self.ind0] = 0
            cb[:, self.ind0] = 0
        else:
            h0, hb, c0, cb = X0.copy(), Xb.copy(), None, None
        if self.mdt is not None:
            h0 = h0 + self.mdt
            hb = hb + self.mdt
        q0 = self.h2pv(h0, hb)
        qb = self.h2pv(hb, hb)
        var = q0[None] if c0 is None else np.concatenate([q0[None], c0])
        varb = qb[None] if cb is None else np.concatenate([qb[None], cb])
        h1 = h0
        for _ in range(int(nstep)):
            h1, var = self.one_step_state(h1, ua, va, var, hb, varb)
        h1 = h1.copy()
        h1[self.ind0] = np.nan
        var = var.copy()
        var[1:, self.ind0] = np.nan
        if self.mdt is not None:
            h1 = h1 - self.mdt
        if not stacked:
            return h1
        parts = [h1[None]] + ([ua[None], va[None]] if self.ageo else []) + [var[1:]]
        return np.concatenate(parts)
