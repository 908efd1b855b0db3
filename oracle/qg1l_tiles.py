"""Float64 NumPy restatement of the overlapping-tile QG 1.5-layer model of the
reference (mapping/models/model_qg1l/jqgm.py, class ``QgmWithTiles``,
1033-1376).

Test infrastructure only: a CUDA form of this model would be checked against
this module; the product never imports it.

Pinning: ``step`` reproduces golden vectors generated by the reference's own
``jqgm.py`` source (``tests/golden/gen_golden_tiles.py``, checked in
``tests/test_oracle_qg1l_tiles.py``). ``step_tgl`` / ``step_adj`` (jax.jvp /
vjp of the blended step, jqgm.py:1358-1376) are hand-derived: every tile is
the full-domain oracle's model with the tile's f, c and masks, so the tile
Jacobians are that oracle's tangent and adjoint; they are checked against
central differences of ``step`` and by a dot-product test.

The model (all line numbers in jqgm.py):
- the domain's masks are the full-domain model's (178-217): classes 1/2 on
  the rings and around land, 0 on land;
- the domain is covered by square tiles of ``tile_size`` overlapping by
  ``tile_overlap``, the last tile of a row or column moved back inside the
  domain (1087-1101);
- every tile runs an independent QG1.5L model for ``nstep`` steps
  (1300-1330) with the tile means of f and c (1313-1314), no beta and no
  bathymetry term (1184-1231), the domain masks sliced to the tile, a PV
  computed on the tile interior (1124-1147), and the Helmholtz inversion on
  the tile with Dirichlet values hb on its edge (1149-1170);
- the tile results, NaN on land, are blended with separable Gaspari-Cohn
  weights in the overlaps (1069-1079, 1333-1349), MDT added before and
  removed after (1343-1356).
"""
import numpy as np

from oracle.qg1l import QgmOracle, build_mask, inverse_elliptic_dst


def gaspari_cohn(r, c):
    """Gaspari-Cohn taper of jqgm.py:22-53 (zero beyond 2c/2 = c)."""
    ra = np.atleast_1d(np.asarray(r, dtype=np.float64))
    if c <= 0:
        return np.zeros_like(ra)
    ra = 2 * np.abs(ra) / c
    gp = np.zeros_like(ra)
    i = ra <= 1.0
    gp[i] = -0.25 * ra[i] ** 5 + 0.5 * ra[i] ** 4 + 0.625 * ra[i] ** 3 - 5.0 / 3.0 * ra[i] ** 2 + 1.0
    i = (ra > 1.0) & (ra <= 2.0)
    gp[i] = (1.0 / 12.0 * ra[i] ** 5 - 0.5 * ra[i] ** 4 + 0.625 * ra[i] ** 3 + 5.0 / 3.0 * ra[i] ** 2
             - 5.0 * ra[i] + 4.0 - 2.0 / 3.0 / ra[i])
    return gp


def tile_origins(ny, nx, size, overlap):
    """(y, x) origins of the tiles (jqgm.py:1087-1101)."""
    out = []
    step = size - overlap
    for y in range(0, ny, step):
        for x in range(0, nx, step):
            ys = ny - size if y + size > ny else max(y, 0)
            xs = nx - size if x + size > nx else max(x, 0)
            out.append((ys, xs))
    return out


def tile_weights(size, overlap):
    """Separable taper of one tile (jqgm.py:1069-1073)."""
    w = np.ones(size)
    gc = gaspari_cohn(np.arange(0, size), overlap)[:overlap]
    w[:overlap] = gc[::-1]
    w[-overlap:] = gc
    return w[:, None] * w[None, :]


class _TileModel(QgmOracle):
    """One tile as the full-domain oracle's model: the tile's f and c, no beta
    or bathymetry, the domain's mask classes sliced to the tile. Two point
    sets replace the full domain's single interior set: PV is a function of h
    on the tile interior [1:-1] (``ind_pv``), the tendency acts on [2:-2]
    (``ind3``); both exclude the domain's ring classes and land."""

    def __init__(self, T, dx, dy, dt, g, f, c, Kdiffus, scheme, ind12, ind0):
        super().__init__(dx=np.full((T, T), dx), dy=np.full((T, T), dy), dt=dt, SSH=None, c=c, Kdiffus=Kdiffus,
                         g=g, f=f, time_scheme=scheme)
        self.ind0 = ind0
        self.ind12 = ind12
        self.ind1 = ind12
        self.ind2 = np.zeros_like(ind12)
        free = ~(ind12 | ind0)
        core = np.zeros((T, T), bool)
        core[2:-2, 2:-2] = True
        inner = np.zeros((T, T), bool)
        inner[1:-1, 1:-1] = True
        self.ind3 = free & core
        self.ind_pv = free & inner

    def h2pv_tl(self, dh, h):
        dq = np.zeros((self.ny, self.nx))
        dq[1:-1, 1:-1] = self._h2pv_interior(dh)
        qraw = np.zeros((self.ny, self.nx))
        qraw[1:-1, 1:-1] = self._h2pv_interior(h)
        dq[np.isnan(qraw)] = 0
        dq[~self.ind_pv] = 0
        return dq

    def h2pv_adj(self, adq, h):
        ind3 = self.ind3
        self.ind3 = self.ind_pv
        try:
            return super().h2pv_adj(adq, h)
        finally:
            self.ind3 = ind3


class QgmTilesOracle:
    """QgmWithTiles(dx, dy, dt, SSH, c, Kdiffus, g, f, time_scheme, mdt,
    tile_size, tile_overlap); time_scheme 'Euler' or 'rk2' (the tile model's
    one_step knows only these, jqgm.py:1269-1276)."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None, g=9.81, f=1e-4,
                 time_scheme="Euler", mdt=None, tile_size=64, tile_overlap=8, **kwargs):
        if time_scheme not in ("Euler", "rk2"):
            raise ValueError("the tile model steps with 'Euler' or 'rk2'")
        dx = np.asarray(dx, dtype=np.float64)
        dy = np.asarray(dy, dtype=np.float64)
        self.ny, self.nx = dx.shape
        # centre spacings (jqgm.py:126-128)
        self.dx = float(dx[self.ny // 2, self.nx // 2])
        self.dy = float(dy[self.ny // 2, self.nx // 2])
        self.dt, self.g, self.K = float(dt), float(g), Kdiffus
        self.scheme = time_scheme
        self.f = np.broadcast_to(np.asarray(f, dtype=np.float64), (self.ny, self.nx))
        self.c = np.broadcast_to(np.asarray(c, dtype=np.float64), (self.ny, self.nx))
        self.mdt = None if mdt is None else np.asarray(mdt, dtype=np.float64)
        mask = build_mask(self.ny, self.nx, None if SSH is None else np.asarray(SSH, dtype=np.float64))
        self.ind0 = mask == 0
        self.ind12 = (mask == 1) | (mask == 2)
        self.T, self.ov = int(tile_size), int(tile_overlap)
        self.tiles = tile_origins(self.ny, self.nx, self.T, self.ov)
        x, y = np.meshgrid(np.arange(1, self.T - 1, dtype=np.float64), np.arange(1, self.T - 1, dtype=np.float64))
        self.lap_tile = 2 * (np.cos(np.pi / (self.T - 1) * x) - 1) / self.dx ** 2 + \
            2 * (np.cos(np.pi / (self.T - 1) * y) - 1) / self.dy ** 2
        self.w = tile_weights(self.T, self.ov)
        self.wsum = np.zeros((self.ny, self.nx))
        for ys, xs in self.tiles:
            self.wsum[ys:ys + self.T, xs:xs + self.T] += self.w

    # ---------------- one tile (jqgm.py:1105-1330) ----------------
    def _h2uv(self, h, f):
        g, dx, dy = self.g, self.dx, self.dy
        u = np.zeros_like(h)
        v = np.zeros_like(h)
        u[1:-1, 1:] = - g / f * (h[2:, :-1] + h[2:, 1:] - h[:-2, 1:] - h[:-2, :-1]) / (4 * dy)
        v[1:, 1:-1] = g / f * (h[1:, 2:] + h[:-1, 2:] - h[:-1, :-2] - h[1:, :-2]) / (4 * dx)
        return np.where(np.isnan(u), 0, u), np.where(np.isnan(v), 0, v)

    def _h2pv(self, h, hb, f, c, i12, i0):
        g, dx, dy = self.g, self.dx, self.dy
        q = np.zeros((self.T, self.T))
        q[1:-1, 1:-1] = g / f * ((h[2:, 1:-1] + h[:-2, 1:-1] - 2 * h[1:-1, 1:-1]) / dy ** 2 +
                                 (h[1:-1, 2:] + h[1:-1, :-2] - 2 * h[1:-1, 1:-1]) / dx ** 2) - \
            g * f / c ** 2 * h[1:-1, 1:-1]
        q = np.where(np.isnan(q), 0, q)
        q = np.where(i12, - g * f / c ** 2 * hb, q)
        return np.where(i0, 0, q)

    def _pv2h(self, q, hb, qb, f, c):
        helm = self.g / f * self.lap_tile - self.g * f / c ** 2
        h = np.zeros((self.T, self.T))
        h[1:-1, 1:-1] = inverse_elliptic_dst(q[1:-1, 1:-1] - qb[1:-1, 1:-1], helm)
        return h + hb

    def _rhs(self, u, v, q, i12, i0):
        dx, dy = self.dx, self.dy
        uT = 0.5 * (u[1:-1, 1:-1] + u[1:-1, 2:])
        vT = 0.5 * (v[1:-1, 1:-1] + v[2:, 1:-1])
        up, um = np.where(uT < 0, 0, uT), np.where(uT > 0, 0, uT)
        vp, vm = np.where(vT < 0, 0, vT), np.where(vT > 0, 0, vT)
        r = np.zeros_like(q)
        r[2:-2, 2:-2] = (
            - up[1:-1, 1:-1] / (6 * dx) * (2 * q[2:-2, 3:-1] + 3 * q[2:-2, 2:-2] - 6 * q[2:-2, 1:-3] + q[2:-2, :-4])
            + um[1:-1, 1:-1] / (6 * dx) * (q[2:-2, 4:] - 6 * q[2:-2, 3:-1] + 3 * q[2:-2, 2:-2] + 2 * q[2:-2, 1:-3])
            - vp[1:-1, 1:-1] / (6 * dy) * (2 * q[3:-1, 2:-2] + 3 * q[2:-2, 2:-2] - 6 * q[1:-3, 2:-2] + q[:-4, 2:-2])
            + vm[1:-1, 1:-1] / (6 * dy) * (q[4:, 2:-2] - 6 * q[3:-1, 2:-2] + 3 * q[2:-2, 2:-2] + 2 * q[1:-3, 2:-2]))
        if self.K is not None:
            K = self.K
            r[2:-2, 2:-2] = r[2:-2, 2:-2] + \
                K / dx ** 2 * (q[2:-2, 3:-1] + q[2:-2, 1:-3] - 2 * q[2:-2, 2:-2]) + \
                K / dy ** 2 * (q[3:-1, 2:-2] + q[1:-3, 2:-2] - 2 * q[2:-2, 2:-2])
        r = np.where(np.isnan(r), 0, r)
        r = np.where(i12, 0, r)
        return np.where(i0, 0, r)

    def _one_step(self, h, q, hb, qb, f, c, i12, i0):
        u, v = self._h2uv(h, f)
        k = self._rhs(u, v, q, i12, i0)
        if self.scheme == "Euler":
            q1 = q + self.dt * k
        else:
            q12 = q + 0.5 * k * self.dt
            u12, v12 = self._h2uv(self._pv2h(q12, hb, qb, f, c), f)
            q1 = q + self.dt * self._rhs(u12, v12, q12, i12, i0)
        return self._pv2h(q1, hb, qb, f, c), q1

    def step_tile(self, ys, xs, h, hb, nstep=1):
        s = (slice(ys, ys + self.T), slice(xs, xs + self.T))
        h0, hbt = h[s], hb[s]
        f = np.nanmean(self.f[s])
        c = np.nanmean(self.c[s])
        i12, i0 = self.ind12[s], self.ind0[s]
        q = self._h2pv(h0, hbt, f, c, i12, i0)
        qb = self._h2pv(hbt, hbt, f, c, i12, i0)
        h1 = h0
        for _ in range(int(nstep)):
            h1, q = self._one_step(h1, q, hbt, qb, f, c, i12, i0)
        return np.where(i0, np.nan, h1)

    def _tile_model(self, k):
        ys, xs = self.tiles[k]
        s = (slice(ys, ys + self.T), slice(xs, xs + self.T))
        return _TileModel(self.T, self.dx, self.dy, self.dt, self.g, float(np.nanmean(self.f[s])),
                          float(np.nanmean(self.c[s])), self.K, self.scheme, self.ind12[s], self.ind0[s]), s

    def _with_mdt(self, h, hb):
        h = np.asarray(h, dtype=np.float64)
        hb = np.asarray(hb, dtype=np.float64)
        if self.mdt is not None:
            return h + self.mdt, hb + self.mdt
        return h, hb

    def step_tgl(self, dh0, h0, hb, nstep=1):
        """jax.jvp of the blended step with respect to h0 (jqgm.py:1358-1362);
        zero on land, as the derivative of where(ind0, nan, h)."""
        h, hbm = self._with_mdt(h0, hb)
        dh0 = np.asarray(dh0, dtype=np.float64)
        acc = np.zeros((self.ny, self.nx))
        for k in range(len(self.tiles)):
            m, s = self._tile_model(k)
            acc[s] += self.w * m.step_tgl(dh0[s], h[s], hbm[s], nstep)
        return acc / self.wsum

    def step_adj(self, adh1, h0, hb, nstep=1):
        """jax.vjp of the blended step with respect to h0 (jqgm.py:1364-1376)."""
        h, hbm = self._with_mdt(h0, hb)
        a = np.asarray(adh1, dtype=np.float64) / self.wsum
        out = np.zeros((self.ny, self.nx))
        for k in range(len(self.tiles)):
            m, s = self._tile_model(k)
            out[s] += m.step_adj(self.w * a[s], h[s], hbm[s], nstep)
        return out

    # ---------------- the blended step (jqgm.py:1333-1376) ----------------
    def step(self, h, hb, nstep=1):
        h = np.asarray(h, dtype=np.float64)
        hb = np.asarray(hb, dtype=np.float64)
        if self.mdt is not None:
            h = h + self.mdt
            hb = hb + self.mdt
        acc = np.zeros((self.ny, self.nx))
        for ys, xs in self.tiles:
            acc[ys:ys + self.T, xs:xs + self.T] += self.w * self.step_tile(ys, xs, h, hb, nstep)
        h1 = acc / self.wsum
        if self.mdt is not None:
            h1 = h1 - self.mdt
        return h1
