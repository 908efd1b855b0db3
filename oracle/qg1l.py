"""Float64 NumPy restatement of the QG 1.5-layer model of the reference
(mapping/models/model_qg1l/jqgm.py, class ``Qgm``), with hand-derived
tangent-linear and adjoint models.

Test infrastructure only: the CUDA path is checked against this module; the
product never imports it.

Pinning: the forward functions reproduce golden vectors generated by the
reference's own ``jqgm.py`` source (``tests/golden/gen_golden.py``); the
tangent and adjoint are checked against finite differences of this forward and
by dot-product tests (``tests/test_oracle_qg1l.py``).

Differences from the reference that are deliberate and documented:
- ``time_scheme='rk4'`` (classical Runge-Kutta 4) is an extension: ``Qgm``
  (jqgm.py:493-498) offers only Euler, rk2 and rk3.
- Tangent/adjoint are written out by hand instead of ``jax.jvp``/``jax.vjp``
  (jqgm.py:559-569); they follow jax's derivative conventions for
  ``jnp.where`` (jqgm.py:344-347): d/du of ``where(u<0,0,u)`` is 1 for u>=0 and
  d/du of ``where(u>0,0,u)`` is 1 for u<=0; NaN guards pass no derivative where
  the primal value was NaN.
"""
import numpy as np
import scipy.fft

SECONDS_PER_DAY = 3600.0 * 24.0


# --------------------------------------------------------------------------
# DST-I (jqgm.py:75-91)
# --------------------------------------------------------------------------
def dst1(x, axis=-1):
    """Orthonormal DST-I along ``axis``.

    jqgm.py:75-77 computes it as ``irfft(-1j*pad(x))`` of length 2(n+1);
    the two agree to rounding (checked in the tests against
    :func:`dst1_via_irfft`)."""
    return scipy.fft.dst(x, type=1, norm="ortho", axis=axis)


def dst1_via_irfft(x):
    """Literal restatement of jqgm.py:75-77 for a 2-D array: ``jnp.pad`` pads
    BOTH axes by one, irfft runs along the last axis, the slice drops the
    padded rows and keeps columns 1..n."""
    n0, n1 = x.shape
    xp = np.pad(x, 1)
    return np.fft.irfft(-1j * xp, axis=-1, norm="ortho")[1:n0 + 1, 1:n1 + 1]


def dst2(x):
    """2-D DST-I, last axis first then the first axis (jqgm.py:79-81)."""
    return dst1(dst1(x, axis=-1), axis=-2)


def inverse_elliptic_dst(f, operator_dst):
    """DST2(DST2(f)/operator) (jqgm.py:83-91)."""
    return dst2(dst2(f) / operator_dst)


# --------------------------------------------------------------------------
# Constants and masks (jqgm.py:113-217)
# --------------------------------------------------------------------------
def helmholtz_eigenvalues(ny, nx, dx, dy, g, f, c):
    """Eigenvalues of the 5-point Helmholtz operator g/f*lap - g*f/c^2 on the
    (ny-2) x (nx-2) interior with Dirichlet walls (jqgm.py:166-172)."""
    x, y = np.meshgrid(np.arange(1, nx - 1, dtype="float64"),
                       np.arange(1, ny - 1, dtype="float64"))
    laplace_dst = 2 * (np.cos(np.pi / (nx - 1) * x) - 1) / dx ** 2 + \
        2 * (np.cos(np.pi / (ny - 1) * y) - 1) / dy ** 2
    return g / f * laplace_dst - g * f / c ** 2


def _dilate(b, r):
    """Chebyshev-distance dilation of a boolean map by r cells."""
    out = np.zeros_like(b)
    ny, nx = b.shape
    padded = np.pad(b, r)
    for p1 in range(-r, r + 1):
        for p2 in range(-r, r + 1):
            out |= padded[r + p1:r + p1 + ny, r + p2:r + p2 + nx]
    return out


def build_mask(ny, nx, ssh=None):
    """Integer mask of jqgm.py:178-217: 3 away from walls/coasts, 1 on the
    outer ring and on land-adjacent cells, 2 on the second ring (rows/cols 1,
    -2, -3 -- the reference marks -3 but not 2) and within two cells of land,
    0 on land (NaN in ``ssh``).

    The reference loops over land points; the result does not depend on the
    visiting order, so it is computed here with two dilations."""
    mask = 3 * np.ones((ny, nx), dtype="int64")
    mask[0, :] = 1
    mask[:, 0] = 1
    mask[-1, :] = 1
    mask[:, -1] = 1
    mask[1, 1:-1] = 2
    mask[1:-1, 1] = 2
    mask[-2, 1:-1] = 2
    mask[-3, 1:-1] = 2
    mask[1:-1, -2] = 2
    mask[1:-1, -3] = 2
    if ssh is not None:
        land = np.isnan(ssh)
        if land.any():
            near1 = _dilate(land, 1) & ~land
            near2 = _dilate(land, 2) & ~land
            new = mask.copy()
            new[near2 & (mask == 3)] = 2
            new[near1 & (mask >= 2)] = 1
            new[land] = 0
            mask = new
    return mask


# --------------------------------------------------------------------------
# Time-scheme tableaux (jqgm.py:398-477; rk4 is an extension)
# --------------------------------------------------------------------------
def butcher(time_scheme, dt):
    """(A, b) with q_s = q + sum_i A[s][i] k_i and q_new = q + sum_s b_s k_s."""
    if time_scheme == "Euler":
        return [[]], [dt]
    if time_scheme == "rk2":
        return [[], [0.5 * dt]], [0.0, dt]
    if time_scheme == "rk3":
        return [[], [0.5 * dt], [-dt, 2 * dt]], [dt / 6, 4 * dt / 6, dt / 6]
    if time_scheme == "rk4":
        return ([[], [0.5 * dt], [0.0, 0.5 * dt], [0.0, 0.0, dt]],
                [dt / 6, dt / 3, dt / 3, dt / 6])
    raise ValueError(f"unknown time_scheme {time_scheme!r}")


class QgmOracle:
    """Restatement of ``Qgm`` (jqgm.py:108-569) in float64 NumPy."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None,
                 upwind=3, g=9.81, f=1e-4, time_scheme="Euler", mdt=None,
                 bathymetry_PV_term=None, **kwargs):
        ny, nx = np.shape(dx)                                 # jqgm.py:122
        self.ny, self.nx = ny, nx
        self.dx = float(np.asarray(dx)[int(ny / 2), int(nx / 2)])   # 127-128
        self.dy = float(np.asarray(dy)[int(ny / 2), int(nx / 2)])
        self.dt = float(dt)
        self.g = float(g)
        if np.ndim(f) > 0:                                   # 140-146
            f = np.asarray(f, dtype="float64")
            self.f = float(np.nanmean(f))
            self.beta = (f[2:, :] - f[:-2, :]) / (2 * self.dy)
        else:
            self.f = float(f)
            self.beta = None
        self.c = float(np.nanmean(c)) if np.ndim(c) > 0 else float(c)   # 150-153
        self.mdt = None if mdt is None else np.asarray(mdt, dtype="float64")
        self.bathymetry_PV_term = (None if bathymetry_PV_term is None else
                                   np.asarray(bathymetry_PV_term, dtype="float64"))
        self.upwind = upwind
        self.time_scheme = time_scheme
        self.Kdiffus = Kdiffus
        self.helmoltz_dst = helmholtz_eigenvalues(ny, nx, self.dx, self.dy,
                                                  self.g, self.f, self.c)
        self.mask = build_mask(ny, nx, None if SSH is None else np.asarray(SSH))
        self.ind0 = self.mask == 0
        self.ind1 = self.mask == 1
        self.ind2 = self.mask == 2
        self.ind12 = self.ind1 | self.ind2
        self.ind3 = self.mask == 3

    # ---------------- forward pieces ----------------
    def h2uv(self, h):
        """Geostrophic velocities (jqgm.py:238-262)."""
        g, f, dx, dy = self.g, self.f, self.dx, self.dy
        u = np.zeros((self.ny, self.nx))
        v = np.zeros((self.ny, self.nx))
        u[1:-1, 1:] = - g / f * (h[2:, :-1] + h[2:, 1:] - h[:-2, 1:] - h[:-2, :-1]) / (4 * dy)
        v[1:, 1:-1] = g / f * (h[1:, 2:] + h[:-1, 2:] - h[:-1, :-2] - h[1:, :-2]) / (4 * dx)
        u = np.where(np.isnan(u), 0, u)
        v = np.where(np.isnan(v), 0, v)
        return u, v

    def _h2pv_interior(self, h):
        g, f, c, dx, dy = self.g, self.f, self.c, self.dx, self.dy
        return g / f * ((h[2:, 1:-1] + h[:-2, 1:-1] - 2 * h[1:-1, 1:-1]) / dy ** 2 +
                        (h[1:-1, 2:] + h[1:-1, :-2] - 2 * h[1:-1, 1:-1]) / dx ** 2) - \
            g * f / (c ** 2) * h[1:-1, 1:-1]

    def h2pv(self, h, hb):
        """SSH -> PV (jqgm.py:264-293)."""
        q = np.zeros((self.ny, self.nx))
        q[1:-1, 1:-1] = self._h2pv_interior(h)
        q = np.where(np.isnan(q), 0, q)
        q[self.ind12] = - self.g * self.f / (self.c ** 2) * hb[self.ind12]
        q[self.ind0] = 0
        return q

    def pv2h(self, q, hb, qb):
        """PV -> SSH by the DST Helmholtz inversion (jqgm.py:295-319)."""
        qin = q[1:-1, 1:-1] - qb[1:-1, 1:-1]
        h = np.zeros((self.ny, self.nx))
        h[1:-1, 1:-1] = inverse_elliptic_dst(qin, self.helmoltz_dst)
        return h + hb

    def _coef(self):
        return 1 / (6 * self.dx), 1 / (6 * self.dy)

    def adv(self, up, vp, um, vm, q0):
        """3rd-order upwind advection on [2:-2, 2:-2] (jqgm.py:377-396)."""
        dx, dy = self.dx, self.dy
        out = np.zeros_like(q0)
        out[2:-2, 2:-2] = (
            - up[1:-1, 1:-1] * 1 / (6 * dx) *
            (2 * q0[2:-2, 3:-1] + 3 * q0[2:-2, 2:-2] - 6 * q0[2:-2, 1:-3] + q0[2:-2, :-4])
            + um[1:-1, 1:-1] * 1 / (6 * dx) *
            (q0[2:-2, 4:] - 6 * q0[2:-2, 3:-1] + 3 * q0[2:-2, 2:-2] + 2 * q0[2:-2, 1:-3])
            - vp[1:-1, 1:-1] * 1 / (6 * dy) *
            (2 * q0[3:-1, 2:-2] + 3 * q0[2:-2, 2:-2] - 6 * q0[1:-3, 2:-2] + q0[:-4, 2:-2])
            + vm[1:-1, 1:-1] * 1 / (6 * dy) *
            (q0[4:, 2:-2] - 6 * q0[3:-1, 2:-2] + 3 * q0[2:-2, 2:-2] + 2 * q0[1:-3, 2:-2]))
        return out

    @staticmethod
    def _split(uT):
        up = np.where(uT < 0, 0, uT)
        um = np.where(uT > 0, 0, uT)
        return up, um

    def _velocities_on_T(self, u, v):
        uT = 0.5 * (u[1:-1, 1:-1] + u[1:-1, 2:])
        vT = 0.5 * (v[1:-1, 1:-1] + v[2:, 1:-1])
        return uT, vT

    def _rhs_raw(self, u, v, q):
        uT, vT = self._velocities_on_T(u, v)
        up, um = self._split(uT)
        vp, vm = self._split(vT)
        r = self.adv(up, vp, um, vm, q)
        if self.bathymetry_PV_term is not None:
            r = r + self.adv(up, vp, um, vm, self.f * self.bathymetry_PV_term)
        if self.beta is not None:
            r[2:-2, 2:-2] = r[2:-2, 2:-2] - \
                self.beta[1:-1, 2:-2] * (v[2:-2, 2:-2] + v[3:-1, 2:-2]) / 2
        if self.Kdiffus is not None:
            K = self.Kdiffus
            r[2:-2, 2:-2] = r[2:-2, 2:-2] + \
                K / (self.dx ** 2) * (q[2:-2, 3:-1] + q[2:-2, 1:-3] - 2 * q[2:-2, 2:-2]) + \
                K / (self.dy ** 2) * (q[3:-1, 2:-2] + q[1:-3, 2:-2] - 2 * q[2:-2, 2:-2])
        return r

    def rhs(self, u, v, q):
        """PV tendency (jqgm.py:321-375) with way=+1."""
        r = self._rhs_raw(u, v, q)
        r = np.where(np.isnan(r), 0, r)
        r[self.ind12] = 0
        r[self.ind0] = 0
        return r

    def _tend(self, h, q):
        u, v = self.h2uv(h)
        return self.rhs(u, v, q)

    def one_step(self, h0, q0, hb, qb):
        """One model step (jqgm.py:480-503 with euler 398-404, rk2 406-431,
        rk3 433-477; rk4 is the classical extension)."""
        dt = self.dt
        incr = self._tend(h0, q0)
        ts = self.time_scheme
        if ts == "Euler":
            q1 = q0 + dt * incr
        elif ts == "rk2":
            q12 = q0 + 0.5 * incr * dt
            incr12 = self._tend(self.pv2h(q12, hb, qb), q12)
            q1 = q0 + dt * incr12
        elif ts == "rk3":
            q12 = q0 + 0.5 * dt * incr
            incr12 = self._tend(self.pv2h(q12, hb, qb), q12)
            q13 = q0 - dt * incr + 2 * dt * incr12
            incr13 = self._tend(self.pv2h(q13, hb, qb), q13)
            q1 = q0 + (dt / 6) * (incr + 4 * incr12 + incr13)
        elif ts == "rk4":
            q2 = q0 + 0.5 * dt * incr
            k2 = self._tend(self.pv2h(q2, hb, qb), q2)
            q3 = q0 + 0.5 * dt * k2
            k3 = self._tend(self.pv2h(q3, hb, qb), q3)
            q4 = q0 + dt * k3
            k4 = self._tend(self.pv2h(q4, hb, qb), q4)
            q1 = q0 + (dt / 6) * (incr + 2 * k2 + 2 * k3 + k4)
        else:
            raise ValueError(ts)
        return self.pv2h(q1, hb, qb), q1

    def step(self, h0, hb, nstep=1):
        """nstep steps from SSH h0 with boundary/background SSH hb
        (jqgm.py:517-557)."""
        h0 = np.array(h0, dtype="float64")
        hb = np.array(hb, dtype="float64")
        if self.mdt is not None:
            h0 = h0 + self.mdt
            hb = hb + self.mdt
        q0 = self.h2pv(h0, hb)
        qb = self.h2pv(hb, hb)
        h1, q1 = +h0, +q0
        for _ in range(nstep):
            h1, q1 = self.one_step(h1, q1, hb, qb)
        h1 = h1.copy()
        h1[self.ind0] = np.nan
        if self.mdt is not None:
            h1 = h1 - self.mdt
        return h1

    # ---------------- stage form used by tangent/adjoint ----------------
    def _trajectory(self, h0, hb, nstep):
        """Forward run keeping every stage state (h_s, q_s) of every step."""
        h0 = np.array(h0, dtype="float64")
        hb = np.array(hb, dtype="float64")
        if self.mdt is not None:
            h0 = h0 + self.mdt
            hb = hb + self.mdt
        A, b = butcher(self.time_scheme, self.dt)
        q0 = self.h2pv(h0, hb)
        qb = self.h2pv(hb, hb)
        traj = []
        h, q = h0, q0
        for _ in range(nstep):
            stages = []
            ks = []
            for s in range(len(b)):
                if s == 0:
                    hs, qs = h, q
                else:
                    qs = q + sum(A[s][i] * ks[i] for i in range(s))
                    hs = self.pv2h(qs, hb, qb)
                stages.append((hs, qs))
                ks.append(self._tend(hs, qs))
            traj.append(stages)
            q = q + sum(b[s] * ks[s] for s in range(len(b)))
            h = self.pv2h(q, hb, qb)
        return h0, hb, qb, traj

    # ---------------- tangent linear ----------------
    def h2uv_tl(self, dh, h):
        g, f, dx, dy = self.g, self.f, self.dx, self.dy
        u, v = self._h2uv_raw(h)
        du = np.zeros((self.ny, self.nx))
        dv = np.zeros((self.ny, self.nx))
        du[1:-1, 1:] = - g / f * (dh[2:, :-1] + dh[2:, 1:] - dh[:-2, 1:] - dh[:-2, :-1]) / (4 * dy)
        dv[1:, 1:-1] = g / f * (dh[1:, 2:] + dh[:-1, 2:] - dh[:-1, :-2] - dh[1:, :-2]) / (4 * dx)
        du[np.isnan(u)] = 0
        dv[np.isnan(v)] = 0
        return du, dv

    def _h2uv_raw(self, h):
        g, f, dx, dy = self.g, self.f, self.dx, self.dy
        u = np.zeros((self.ny, self.nx))
        v = np.zeros((self.ny, self.nx))
        u[1:-1, 1:] = - g / f * (h[2:, :-1] + h[2:, 1:] - h[:-2, 1:] - h[:-2, :-1]) / (4 * dy)
        v[1:, 1:-1] = g / f * (h[1:, 2:] + h[:-1, 2:] - h[:-1, :-2] - h[1:, :-2]) / (4 * dx)
        return u, v

    def rhs_tl(self, u, v, q, du, dv, dq):
        uT, vT = self._velocities_on_T(u, v)
        duT, dvT = self._velocities_on_T(du, dv)
        up, um = self._split(uT)
        vp, vm = self._split(vT)
        dup = np.where(uT < 0, 0, duT)
        dum = np.where(uT > 0, 0, duT)
        dvp = np.where(vT < 0, 0, dvT)
        dvm = np.where(vT > 0, 0, dvT)
        qa = q if self.bathymetry_PV_term is None else q + self.f * self.bathymetry_PV_term
        r = self.adv(dup, dvp, dum, dvm, qa) + self.adv(up, vp, um, vm, dq)
        if self.beta is not None:
            r[2:-2, 2:-2] -= self.beta[1:-1, 2:-2] * (dv[2:-2, 2:-2] + dv[3:-1, 2:-2]) / 2
        if self.Kdiffus is not None:
            K = self.Kdiffus
            r[2:-2, 2:-2] += K / (self.dx ** 2) * (dq[2:-2, 3:-1] + dq[2:-2, 1:-3] - 2 * dq[2:-2, 2:-2]) + \
                K / (self.dy ** 2) * (dq[3:-1, 2:-2] + dq[1:-3, 2:-2] - 2 * dq[2:-2, 2:-2])
        r[np.isnan(self._rhs_raw(u, v, q))] = 0
        r[~self.ind3] = 0
        return r

    def pv2h_tl(self, dq):
        h = np.zeros((self.ny, self.nx))
        h[1:-1, 1:-1] = inverse_elliptic_dst(dq[1:-1, 1:-1], self.helmoltz_dst)
        return h

    def h2pv_tl(self, dh, h):
        dq = np.zeros((self.ny, self.nx))
        dq[1:-1, 1:-1] = self._h2pv_interior(dh)
        qraw = np.zeros((self.ny, self.nx))
        qraw[1:-1, 1:-1] = self._h2pv_interior(h)
        dq[np.isnan(qraw)] = 0
        dq[~self.ind3] = 0
        return dq

    def _tend_tl(self, h, q, dh, dq):
        u, v = self.h2uv(h)
        du, dv = self.h2uv_tl(dh, h)
        return self.rhs_tl(u, v, q, du, dv, dq)

    def step_tgl(self, dh0, h0, hb, nstep=1):
        """Tangent of :meth:`step` w.r.t. h0 (jqgm.py:559-563)."""
        h0s, hbs, qb, traj = self._trajectory(h0, hb, nstep)
        A, b = butcher(self.time_scheme, self.dt)
        dh = np.array(dh0, dtype="float64")
        dq = self.h2pv_tl(dh, h0s)
        for n in range(nstep):
            dks = []
            for s in range(len(b)):
                hs, qs = traj[n][s]
                if s == 0:
                    dhs, dqs = dh, dq
                else:
                    dqs = dq + sum(A[s][i] * dks[i] for i in range(s))
                    dhs = self.pv2h_tl(dqs)
                dks.append(self._tend_tl(hs, qs, dhs, dqs))
            dq = dq + sum(b[s] * dks[s] for s in range(len(b)))
            dh = self.pv2h_tl(dq)
        dh = dh.copy()
        # jqgm.py:551 overwrites land with a constant (NaN): its tangent is 0
        dh[self.ind0] = 0.0
        return dh

    # ---------------- adjoint ----------------
    def h2uv_adj(self, adu, adv, h):
        g, f, dx, dy = self.g, self.f, self.dx, self.dy
        u, v = self._h2uv_raw(h)
        adu = np.where(np.isnan(u), 0, adu)
        adv = np.where(np.isnan(v), 0, adv)
        adh = np.zeros((self.ny, self.nx))
        cu = - g / f / (4 * dy)
        cv = g / f / (4 * dx)
        a = cu * adu[1:-1, 1:]
        adh[2:, :-1] += a
        adh[2:, 1:] += a
        adh[:-2, 1:] -= a
        adh[:-2, :-1] -= a
        b = cv * adv[1:, 1:-1]
        adh[1:, 2:] += b
        adh[:-1, 2:] += b
        adh[:-1, :-2] -= b
        adh[1:, :-2] -= b
        return adh

    def adv_adj(self, up, vp, um, vm, q, ad):
        """Adjoint of :meth:`adv` w.r.t. (up, vp, um, vm) and q."""
        cx, cy = self._coef()
        a = ad[2:-2, 2:-2]
        upc, umc = up[1:-1, 1:-1], um[1:-1, 1:-1]
        vpc, vmc = vp[1:-1, 1:-1], vm[1:-1, 1:-1]
        adq = np.zeros_like(q)
        adq[2:-2, 3:-1] += a * (-2 * cx * upc - 6 * cx * umc)
        adq[2:-2, 2:-2] += a * (-3 * cx * upc + 3 * cx * umc - 3 * cy * vpc + 3 * cy * vmc)
        adq[2:-2, 1:-3] += a * (6 * cx * upc + 2 * cx * umc)
        adq[2:-2, :-4] += a * (-cx * upc)
        adq[2:-2, 4:] += a * (cx * umc)
        adq[3:-1, 2:-2] += a * (-2 * cy * vpc - 6 * cy * vmc)
        adq[1:-3, 2:-2] += a * (6 * cy * vpc + 2 * cy * vmc)
        adq[:-4, 2:-2] += a * (-cy * vpc)
        adq[4:, 2:-2] += a * (cy * vmc)
        Dpx = 2 * q[2:-2, 3:-1] + 3 * q[2:-2, 2:-2] - 6 * q[2:-2, 1:-3] + q[2:-2, :-4]
        Dmx = q[2:-2, 4:] - 6 * q[2:-2, 3:-1] + 3 * q[2:-2, 2:-2] + 2 * q[2:-2, 1:-3]
        Dpy = 2 * q[3:-1, 2:-2] + 3 * q[2:-2, 2:-2] - 6 * q[1:-3, 2:-2] + q[:-4, 2:-2]
        Dmy = q[4:, 2:-2] - 6 * q[3:-1, 2:-2] + 3 * q[2:-2, 2:-2] + 2 * q[1:-3, 2:-2]
        shp = up.shape
        adup = np.zeros(shp); adum = np.zeros(shp)
        advp = np.zeros(shp); advm = np.zeros(shp)
        adup[1:-1, 1:-1] = -cx * Dpx * a
        adum[1:-1, 1:-1] = cx * Dmx * a
        advp[1:-1, 1:-1] = -cy * Dpy * a
        advm[1:-1, 1:-1] = cy * Dmy * a
        return adup, advp, adum, advm, adq

    def rhs_adj(self, u, v, q, adr):
        """Adjoint of :meth:`rhs` w.r.t. (u, v, q)."""
        adr = np.where(np.isnan(self._rhs_raw(u, v, q)), 0, adr)
        adr = np.where(self.ind3, adr, 0)
        uT, vT = self._velocities_on_T(u, v)
        up, um = self._split(uT)
        vp, vm = self._split(vT)
        qa = q if self.bathymetry_PV_term is None else q + self.f * self.bathymetry_PV_term
        adup, advp, adum, advm, _ = self.adv_adj(up, vp, um, vm, qa, adr)
        _, _, _, _, adq = self.adv_adj(up, vp, um, vm, q, adr)
        aduT = np.where(uT < 0, 0, adup) + np.where(uT > 0, 0, adum)
        advT = np.where(vT < 0, 0, advp) + np.where(vT > 0, 0, advm)
        adu = np.zeros((self.ny, self.nx))
        adv = np.zeros((self.ny, self.nx))
        if self.beta is not None:
            t = - self.beta[1:-1, 2:-2] * adr[2:-2, 2:-2] / 2
            adv[2:-2, 2:-2] += t
            adv[3:-1, 2:-2] += t
        if self.Kdiffus is not None:
            K = self.Kdiffus
            a = adr[2:-2, 2:-2]
            kx, ky = K / (self.dx ** 2), K / (self.dy ** 2)
            adq[2:-2, 3:-1] += kx * a
            adq[2:-2, 1:-3] += kx * a
            adq[2:-2, 2:-2] -= 2 * kx * a + 2 * ky * a
            adq[3:-1, 2:-2] += ky * a
            adq[1:-3, 2:-2] += ky * a
        adu[1:-1, 1:-1] += 0.5 * aduT
        adu[1:-1, 2:] += 0.5 * aduT
        adv[1:-1, 1:-1] += 0.5 * advT
        adv[2:, 1:-1] += 0.5 * advT
        return adu, adv, adq

    def pv2h_adj(self, adh):
        """Adjoint of the interior DST solve w.r.t. q (the solve is symmetric)."""
        adq = np.zeros((self.ny, self.nx))
        adq[1:-1, 1:-1] = inverse_elliptic_dst(adh[1:-1, 1:-1], self.helmoltz_dst)
        return adq

    def h2pv_adj(self, adq, h):
        g, f, c, dx, dy = self.g, self.f, self.c, self.dx, self.dy
        qraw = np.zeros((self.ny, self.nx))
        qraw[1:-1, 1:-1] = self._h2pv_interior(h)
        a = np.where(self.ind3 & ~np.isnan(qraw), adq, 0)[1:-1, 1:-1]
        adh = np.zeros((self.ny, self.nx))
        gf = g / f
        adh[2:, 1:-1] += gf / dy ** 2 * a
        adh[:-2, 1:-1] += gf / dy ** 2 * a
        adh[1:-1, 2:] += gf / dx ** 2 * a
        adh[1:-1, :-2] += gf / dx ** 2 * a
        adh[1:-1, 1:-1] += (-2 * gf / dy ** 2 - 2 * gf / dx ** 2 - g * f / c ** 2) * a
        return adh

    def _tend_adj(self, h, q, adk):
        u, v = self.h2uv(h)
        adu, adv, adq = self.rhs_adj(u, v, q, adk)
        return self.h2uv_adj(adu, adv, h), adq

    def step_adj(self, adh1, h0, hb, nstep=1):
        """Adjoint of :meth:`step` w.r.t. h0 (jqgm.py:565-569)."""
        h0s, hbs, qb, traj = self._trajectory(h0, hb, nstep)
        A, b = butcher(self.time_scheme, self.dt)
        S = len(b)
        adh = np.array(adh1, dtype="float64")
        adh = np.where(self.ind0, 0, adh)
        adh = np.nan_to_num(adh)
        adq = np.zeros((self.ny, self.nx))
        for n in reversed(range(nstep)):
            adq = adq + self.pv2h_adj(adh)
            adk = [b[s] * adq for s in range(S)]
            adq_acc = adq.copy()
            adh_out = None
            for s in reversed(range(S)):
                hs, qs = traj[n][s]
                adhs, adqs = self._tend_adj(hs, qs, adk[s])
                if s == 0:
                    adh_out = adhs
                    adq_acc = adq_acc + adqs
                else:
                    adqs = adqs + self.pv2h_adj(adhs)
                    adq_acc = adq_acc + adqs
                    for i in range(s):
                        if A[s][i] != 0.0:
                            adk[i] = adk[i] + A[s][i] * adqs
            adh, adq = adh_out, adq_acc
        return adh + self.h2pv_adj(adq, h0s)


# --------------------------------------------------------------------------
# Model wrapper semantics (mapping/src/mod.py:867-1076, Model_qg1l_jax)
# --------------------------------------------------------------------------
def model_step(qgm, ssh, Fssh, hb, nstep):
    """State update of ``Model_qg1l_jax.step`` (mod.py:867-913): model step
    then the SSH forcing ``nstep*dt/86400*Fssh`` (mod.py:911-913)."""
    out = qgm.step(ssh, hb, nstep)
    if Fssh is not None:
        out = out + nstep * qgm.dt / SECONDS_PER_DAY * Fssh
    return out


def model_step_tgl(qgm, dssh, dFssh, ssh, hb, nstep):
    """``Model_qg1l_jax.step_tgl`` (mod.py:957-1016)."""
    out = qgm.step_tgl(dssh, ssh, hb, nstep)
    if dFssh is not None:
        out = out + nstep * qgm.dt / SECONDS_PER_DAY * dFssh
    return out


def model_step_adj(qgm, adssh, adFssh, ssh, hb, nstep):
    """``Model_qg1l_jax.step_adj`` (mod.py:1018-1076): returns the new
    (adssh, adFssh); the parameter adjoint ACCUMULATES nstep*dt/86400 times
    the incoming SSH adjoint (mod.py:1058-1068)."""
    new_ad = qgm.step_adj(adssh, ssh, hb, nstep)
    if adFssh is not None:
        adFssh = adFssh + nstep * qgm.dt / SECONDS_PER_DAY * adssh
    return new_ad, adFssh


class QgmSfOracle:
    """Restatement of ``Qgm_sf`` (jqgm.py:571-1031), the streamfunction form.

    The state is phi = g/f h with f the (possibly varying) Coriolis field
    (jqgm.py:1004-1005); PV q = lap(phi) - (f0/c)^2 phi (724-741), inversion
    with lap_dst - (f0/c)^2 (627-631), velocities from phi without the g/f
    factor (698-719), f0 = mean(f) (606), the bathymetry term f*bathymetry
    with the f field (819-820), the same beta and mask as Qgm. In phi these
    are exactly Qgm's equations with g = f = f0 and the bathymetry term
    scaled by f/f0, so the model part is a ``QgmOracle`` built that way."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None,
                 upwind=3, g=9.81, f=1e-4, time_scheme="Euler", mdt=None,
                 bathymetry_PV_term=None, **kwargs):
        ny, nx = np.shape(dx)
        f_arr = np.broadcast_to(np.asarray(f, dtype="float64"), (ny, nx))
        self.f0 = float(np.mean(f_arr))
        self.g = float(g)
        bathy = None
        if bathymetry_PV_term is not None:
            bathy = np.asarray(bathymetry_PV_term, dtype="float64") * (f_arr / self.f0)
        self.core = QgmOracle(dx=dx, dy=dy, dt=dt, SSH=SSH, c=c, Kdiffus=Kdiffus, upwind=upwind,
                              g=self.f0, f=(np.asarray(f, dtype="float64") if np.ndim(f) > 0 else self.f0),
                              time_scheme=time_scheme, bathymetry_PV_term=bathy)
        self.s = self.g / f_arr                 # h -> phi
        self.mdt = None if mdt is None else np.asarray(mdt, dtype="float64")
        self.mask = self.core.mask
        self.ind0 = self.core.ind0

    def phi2uv(self, phi):
        return self.core.h2uv(phi)

    def phi2pv(self, phi, phib):
        return self.core.h2pv(phi, phib)

    def pv2phi(self, q, phib, qb):
        return self.core.pv2h(q, phib, qb)

    def _in(self, h0, hb):
        h0 = np.array(h0, dtype="float64")
        hb = np.array(hb, dtype="float64")
        if self.mdt is not None:
            h0 = h0 + self.mdt
            hb = hb + self.mdt
        return self.s * h0, self.s * hb

    def step(self, h0, hb, nstep=1):
        phi0, phib = self._in(h0, hb)
        h1 = self.core.step(phi0, phib, nstep) / self.s
        if self.mdt is not None:
            h1 = h1 - self.mdt
        return h1

    def step_tgl(self, dh0, h0, hb, nstep=1):
        phi0, phib = self._in(h0, hb)
        return self.core.step_tgl(self.s * np.asarray(dh0, dtype="float64"), phi0, phib, nstep) / self.s

    def step_adj(self, adh1, h0, hb, nstep=1):
        phi0, phib = self._in(h0, hb)
        return self.s * self.core.step_adj(np.asarray(adh1, dtype="float64") / self.s, phi0, phib, nstep)
