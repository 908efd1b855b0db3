"""Float64 NumPy restatement of the QG 1.5-layer model with passive tracers of
the reference (mapping/models/model_qg1l/jqgm.py, class ``Qgm_trac``,
1551-2151): forward, tangent linear and adjoint.

Test infrastructure only: a CUDA form of this model would be checked against
this module; the product never imports it.

Pinning: ``step`` reproduces golden vectors generated by the reference's own
``jqgm.py`` source (``tests/golden/gen_golden_trac.py``, checked in
``tests/test_oracle_qg1l_trac.py``). ``step_tgl`` / ``step_adj`` (jax.jvp /
jax.vjp of ``step``, jqgm.py:2141-2151) are hand-derived from the same
pieces and checked against central differences of ``step`` and by a
dot-product test (same file).

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


def _butcher(scheme, dt):
    if scheme == "Euler":
        return [[]], [dt]
    if scheme == "rk2":
        return [[], [0.5 * dt]], [0.0, dt]
    return [[], [0.5 * dt], [0.0, 0.5 * dt], [0.0, 0.0, dt]], [dt / 6, dt / 3, dt / 3, dt / 6]


class QgmTracTLAD(QgmTracOracle):
    """Tangent linear and adjoint of ``QgmTracOracle.step`` with respect to X0
    (jax.jvp / jax.vjp, jqgm.py:2141-2151), without ``ageo_velocities``.

    Derivative rules of the forward's jnp.where / abs (as jax applies them):
    where(u < 0, 0, u) passes the derivative for u >= 0, where(u > 0, 0, u)
    for u <= 0; a NaN-guarded value passes none; |w| has derivative sign(w)
    (0 at 0); values overwritten with constants (land, ring classes, NaN on
    land at the end) pass none. The boundary fields Xb are not differentiated.
    """

    # ---- raw (unguarded) tendencies, for the NaN guards
    def _raw_q(self, u, v, q):
        up, vp, um, vm = self._upwind(u, v)
        rq = self.adv(up, vp, um, vm, q) if self.advect_pv else np.zeros_like(q)
        if self.advect_pv and self.beta is not None:
            rq[2:-2, 2:-2] = rq[2:-2, 2:-2] - self.beta[1:-1, 2:-2] * (v[2:-2, 2:-2] + v[3:-1, 2:-2]) / 2
        if self.Kdiffus is not None:
            rq = self._diffuse(rq, q, self.Kdiffus)
        return rq

    def _raw_c(self, u, v, c):
        up, vp, um, vm = self._upwind(u, v)
        rc = self.adv(up, vp, um, vm, c)
        if self.Kdiffus_trac is not None:
            rc = self._diffuse(rc, c, self.Kdiffus_trac)
        return rc

    def _dsplit(self, u, v, du, dv):
        uT, vT = self._velocities_on_T(u, v)
        duT, dvT = self._velocities_on_T(du, dv)
        return (np.where(uT < 0, 0, duT), np.where(vT < 0, 0, dvT), np.where(uT > 0, 0, duT),
                np.where(vT > 0, 0, dvT))

    def rhs_state_tl(self, u, v, var, du, dv, dvar):
        up, vp, um, vm = self._upwind(u, v)
        dup, dvp, dum, dvm = self._dsplit(u, v, du, dv)
        q, dq = var[0], dvar[0]
        if self.advect_pv:
            rq = self.adv(dup, dvp, dum, dvm, q) + self.adv(up, vp, um, vm, dq)
            if self.beta is not None:
                rq[2:-2, 2:-2] = rq[2:-2, 2:-2] - self.beta[1:-1, 2:-2] * (dv[2:-2, 2:-2] + dv[3:-1, 2:-2]) / 2
        else:
            rq = np.zeros_like(q)
        if self.Kdiffus is not None:
            rq = self._diffuse(rq, dq, self.Kdiffus)
        rq[np.isnan(self._raw_q(u, v, q))] = 0
        rq[~self.ind3] = 0
        out = [rq]
        for c, dc in zip(var[1:], dvar[1:]):
            rc = self.adv(dup, dvp, dum, dvm, c) + self.adv(up, vp, um, vm, dc)
            if self.Kdiffus_trac is not None:
                rc = self._diffuse(rc, dc, self.Kdiffus_trac)
            rc[np.isnan(self._raw_c(u, v, c))] = 0
            rc[self.ind0] = 0
            out.append(rc)
        return np.stack(out)

    def _diffuse_adj(self, ad, a, K):
        kx, ky = K / self.dx ** 2, K / self.dy ** 2
        x = a[2:-2, 2:-2]
        ad[2:-2, 3:-1] += kx * x
        ad[2:-2, 1:-3] += kx * x
        ad[2:-2, 2:-2] -= 2 * kx * x + 2 * ky * x
        ad[3:-1, 2:-2] += ky * x
        ad[1:-3, 2:-2] += ky * x

    def rhs_state_adj(self, u, v, var, adr):
        """(adu, adv, advar) of the stacked tendency."""
        up, vp, um, vm = self._upwind(u, v)
        uT, vT = self._velocities_on_T(u, v)
        shp = up.shape
        adup, advp, adum, advm = (np.zeros(shp) for _ in range(4))
        adu = np.zeros((self.ny, self.nx))
        adv = np.zeros((self.ny, self.nx))
        advar = np.zeros_like(var)
        q = var[0]
        a = np.where(np.isnan(self._raw_q(u, v, q)) | ~self.ind3, 0, adr[0])
        if self.advect_pv:
            p1, p2, p3, p4, adq = self.adv_adj(up, vp, um, vm, q, a)
            adup += p1; advp += p2; adum += p3; advm += p4
            advar[0] += adq
            if self.beta is not None:
                t = - self.beta[1:-1, 2:-2] * a[2:-2, 2:-2] / 2
                adv[2:-2, 2:-2] += t
                adv[3:-1, 2:-2] += t
        if self.Kdiffus is not None:
            self._diffuse_adj(advar[0], a, self.Kdiffus)
        for i in range(1, var.shape[0]):
            c = var[i]
            a = np.where(np.isnan(self._raw_c(u, v, c)) | self.ind0, 0, adr[i])
            p1, p2, p3, p4, adc = self.adv_adj(up, vp, um, vm, c, a)
            adup += p1; advp += p2; adum += p3; advm += p4
            advar[i] += adc
            if self.Kdiffus_trac is not None:
                self._diffuse_adj(advar[i], a, self.Kdiffus_trac)
        aduT = np.where(uT < 0, 0, adup) + np.where(uT > 0, 0, adum)
        advT = np.where(vT < 0, 0, advp) + np.where(vT > 0, 0, advm)
        adu[1:-1, 1:-1] += 0.5 * aduT
        adu[1:-1, 2:] += 0.5 * aduT
        adv[1:-1, 1:-1] += 0.5 * advT
        adv[2:, 1:-1] += 0.5 * advT
        return adu, adv, advar

    # ---- boundary update (jqgm.py:1957-2006)
    def _ratios(self, w, r):
        return r * (w + np.abs(w)), r * (w - np.abs(w))

    def bc_tl(self, dvar1, var0, dvar0, u, v, du, dv, varb):
        if varb.shape[0] <= 1:
            return dvar1
        out = dvar1.copy()
        ry, rx = 0.5 * self.dt / self.dy, 0.5 * self.dt / self.dx
        W = self.Wbc[1:-1, 1:-1]
        edges = [(v[1, 1:-1], dv[1, 1:-1], ry), (v[-1, 1:-1], dv[-1, 1:-1], ry),
                 (u[1:-1, 1], du[1:-1, 1], rx), (u[1:-1, -1], du[1:-1, -1], rx)]
        R = []
        for w, dw, r in edges:
            r1, r2 = self._ratios(w, r)
            sg = np.sign(w)
            R.append((r1, r2, r * (dw + sg * dw), r * (dw - sg * dw)))
        for i in range(1, varb.shape[0]):
            a, da, b = var0[i], dvar0[i], varb[i]
            if self.bc_trac == "OBC":
                (r1, r2, d1, d2) = R[0]
                out[i, 0, 1:-1] = da[0, 1:-1] - (d1 * (a[0, 1:-1] - b[0, 1:-1]) + r1 * da[0, 1:-1] +
                                                 d2 * (a[1, 1:-1] - a[0, 1:-1]) + r2 * (da[1, 1:-1] - da[0, 1:-1]))
                (r1, r2, d1, d2) = R[1]
                out[i, -1, 1:-1] = da[-1, 1:-1] - (d1 * (a[-1, 1:-1] - a[-2, 1:-1]) +
                                                   r1 * (da[-1, 1:-1] - da[-2, 1:-1]) +
                                                   d2 * (b[-1, 1:-1] - a[-1, 1:-1]) - r2 * da[-1, 1:-1])
                (r1, r2, d1, d2) = R[2]
                out[i, 1:-1, 0] = da[1:-1, 0] - (d1 * (a[1:-1, 0] - b[1:-1, 0]) + r1 * da[1:-1, 0] +
                                                 d2 * (a[1:-1, 1] - a[1:-1, 0]) + r2 * (da[1:-1, 1] - da[1:-1, 0]))
                (r1, r2, d1, d2) = R[3]
                out[i, 1:-1, -1] = da[1:-1, -1] - (d1 * (a[1:-1, -1] - a[1:-1, -2]) +
                                                   r1 * (da[1:-1, -1] - da[1:-1, -2]) +
                                                   d2 * (b[1:-1, -1] - a[1:-1, -1]) - r2 * da[1:-1, -1])
            else:
                out[i][self.ind12] = 0
            out[i, 1:-1, 1:-1] = (1 - W) * out[i, 1:-1, 1:-1]
        return out

    def bc_adj(self, adx, var0, u, v, varb):
        """adjoint of bc: (ad var1 before the update, ad var0, adu, adv)."""
        adpre = adx.copy()
        ad0 = np.zeros_like(var0)
        adu = np.zeros((self.ny, self.nx))
        adv = np.zeros((self.ny, self.nx))
        if varb.shape[0] <= 1:
            return adpre, ad0, adu, adv
        ry, rx = 0.5 * self.dt / self.dy, 0.5 * self.dt / self.dx
        W = self.Wbc[1:-1, 1:-1]
        for i in range(1, varb.shape[0]):
            x = adx[i].copy()
            x[1:-1, 1:-1] = (1 - W) * x[1:-1, 1:-1]
            a, b = var0[i], varb[i]
            if self.bc_trac == "OBC":
                # row 0 (w = v[1, 1:-1])
                w = v[1, 1:-1]; r1, r2 = self._ratios(w, ry); s = np.sign(w)
                g = x[0, 1:-1]
                ad0[i, 0, 1:-1] += g * (1 - r1 + r2)
                ad0[i, 1, 1:-1] += -g * r2
                gr1, gr2 = -g * (a[0, 1:-1] - b[0, 1:-1]), -g * (a[1, 1:-1] - a[0, 1:-1])
                adv[1, 1:-1] += ry * (gr1 * (1 + s) + gr2 * (1 - s))
                # row ny-1 (w = v[-1, 1:-1])
                w = v[-1, 1:-1]; r1, r2 = self._ratios(w, ry); s = np.sign(w)
                g = x[-1, 1:-1]
                ad0[i, -1, 1:-1] += g * (1 - r1 + r2)
                ad0[i, -2, 1:-1] += g * r1
                gr1, gr2 = -g * (a[-1, 1:-1] - a[-2, 1:-1]), -g * (b[-1, 1:-1] - a[-1, 1:-1])
                adv[-1, 1:-1] += ry * (gr1 * (1 + s) + gr2 * (1 - s))
                # column 0 (w = u[1:-1, 1])
                w = u[1:-1, 1]; r1, r2 = self._ratios(w, rx); s = np.sign(w)
                g = x[1:-1, 0]
                ad0[i, 1:-1, 0] += g * (1 - r1 + r2)
                ad0[i, 1:-1, 1] += -g * r2
                gr1, gr2 = -g * (a[1:-1, 0] - b[1:-1, 0]), -g * (a[1:-1, 1] - a[1:-1, 0])
                adu[1:-1, 1] += rx * (gr1 * (1 + s) + gr2 * (1 - s))
                # column nx-1 (w = u[1:-1, -1])
                w = u[1:-1, -1]; r1, r2 = self._ratios(w, rx); s = np.sign(w)
                g = x[1:-1, -1]
                ad0[i, 1:-1, -1] += g * (1 - r1 + r2)
                ad0[i, 1:-1, -2] += g * r1
                gr1, gr2 = -g * (a[1:-1, -1] - a[1:-1, -2]), -g * (b[1:-1, -1] - a[1:-1, -1])
                adu[1:-1, -1] += rx * (gr1 * (1 + s) + gr2 * (1 - s))
                x[0, 1:-1] = 0
                x[-1, 1:-1] = 0
                x[1:-1, 0] = 0
                x[1:-1, -1] = 0
            else:
                x[self.ind12] = 0
            adpre[i] = x
        return adpre, ad0, adu, adv

    # ---- trajectory
    def _prepare(self, X0, Xb):
        if self.ageo:
            raise NotImplementedError("tangent/adjoint with ageo_velocities")
        X0 = np.array(X0, dtype=np.float64)
        Xb = np.array(Xb, dtype=np.float64)
        stacked = X0.ndim == 3
        if stacked:
            h0, c0, hb, cb = X0[0].copy(), X0[1:].copy(), Xb[0].copy(), Xb[1:].copy()
            c0[:, self.ind0] = 0
            cb[:, self.ind0] = 0
        else:
            h0, hb = X0.copy(), Xb.copy()
            c0 = cb = np.zeros((0, self.ny, self.nx))
        if self.mdt is not None:
            h0 = h0 + self.mdt
            hb = hb + self.mdt
        q0 = self.h2pv(h0, hb)
        qb = self.h2pv(hb, hb)
        return stacked, h0, hb, np.concatenate([q0[None], c0]), np.concatenate([qb[None], cb])

    def _traj(self, h0, hb, var0, varb, nstep):
        A, b = _butcher(self.time_scheme, self.dt)
        qb = varb[0]
        traj = []
        h, var = h0, var0
        for _ in range(int(nstep)):
            stages, ks = [], []
            for s in range(len(b)):
                if s == 0:
                    hs, vs = h, var
                else:
                    vs = var + sum(A[s][i] * ks[i] for i in range(s))
                    hs = self.pv2h(vs[0], hb, qb)
                us, ws = self.h2uv(hs)
                stages.append((hs, vs, us, ws))
                ks.append(self.rhs_state(us, ws, None, None, vs))
            traj.append(stages)
            var1 = var + sum(b[s] * ks[s] for s in range(len(b)))
            h = self.pv2h(var1[0], hb, qb)
            var = self.bc(var1, var, stages[0][2], stages[0][3], varb)
        return traj

    def step_tgl(self, dX0, X0, Xb, nstep=1):
        stacked, h0, hb, var0, varb = self._prepare(X0, Xb)
        dX0 = np.array(dX0, dtype=np.float64)
        if stacked:
            dh, dc = dX0[0].copy(), dX0[1:].copy()
            dc[:, self.ind0] = 0
        else:
            dh, dc = dX0.copy(), np.zeros((0, self.ny, self.nx))
        dvar = np.concatenate([self.h2pv_tl(dh, h0)[None], dc])
        traj = self._traj(h0, hb, var0, varb, nstep)
        A, b = _butcher(self.time_scheme, self.dt)
        for n in range(int(nstep)):
            dks = []
            st = traj[n]
            dus = None
            for s in range(len(b)):
                hs, vs, us, ws = st[s]
                if s == 0:
                    dhs, dvs = dh, dvar
                else:
                    dvs = dvar + sum(A[s][i] * dks[i] for i in range(s))
                    dhs = self.pv2h_tl(dvs[0])
                du, dv = self.h2uv_tl(dhs, hs)
                if s == 0:
                    dus = (du, dv)
                dks.append(self.rhs_state_tl(us, ws, vs, du, dv, dvs))
            dvar1 = dvar + sum(b[s] * dks[s] for s in range(len(b)))
            dh = self.pv2h_tl(dvar1[0])
            dvar = self.bc_tl(dvar1, st[0][1], dvar, st[0][2], st[0][3], dus[0], dus[1], varb)
        dh = dh.copy()
        dh[self.ind0] = 0
        if not stacked:
            return dh
        dc = dvar[1:].copy()
        dc[:, self.ind0] = 0
        return np.concatenate([dh[None], dc])

    def step_adj(self, adX1, X0, Xb, nstep=1):
        stacked, h0, hb, var0, varb = self._prepare(X0, Xb)
        ad = np.nan_to_num(np.array(adX1, dtype=np.float64))
        if stacked:
            adh, adc = ad[0].copy(), ad[1:].copy()
            adc[:, self.ind0] = 0
        else:
            adh, adc = ad.copy(), np.zeros((0, self.ny, self.nx))
        adh[self.ind0] = 0
        advar = np.concatenate([np.zeros((1, self.ny, self.nx)), adc])
        traj = self._traj(h0, hb, var0, varb, nstep)
        A, b = _butcher(self.time_scheme, self.dt)
        S = len(b)
        for n in reversed(range(int(nstep))):
            st = traj[n]
            adpre, ad0, adub, advb = self.bc_adj(advar, st[0][1], st[0][2], st[0][3], varb)
            adpre[0] = adpre[0] + self.pv2h_adj(adh)
            adk = [b[s] * adpre for s in range(S)]
            acc = adpre + ad0
            adh_out = None
            for s in reversed(range(S)):
                hs, vs, us, ws = st[s]
                adu, adv, advs = self.rhs_state_adj(us, ws, vs, adk[s])
                if s == 0:
                    adu = adu + adub
                    adv = adv + advb
                adhs = self.h2uv_adj(adu, adv, hs)
                if s == 0:
                    adh_out = adhs
                    acc = acc + advs
                else:
                    advs[0] = advs[0] + self.pv2h_adj(adhs)
                    acc = acc + advs
                    for i in range(s):
                        if A[s][i] != 0.0:
                            adk[i] = adk[i] + A[s][i] * advs
            adh, advar = adh_out, acc
        adh0 = adh + self.h2pv_adj(advar[0], h0)
        if not stacked:
            return adh0
        adc0 = advar[1:].copy()
        adc0[:, self.ind0] = 0
        return np.concatenate([adh0[None], adc0])
