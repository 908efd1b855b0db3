"""Oracle (test infrastructure only): restatement of the reduced bases of the
reference (Gaussian space-time and wave-packet) in float64 NumPy/SciPy, in
the reference's own sparse form (CSC space matrices and time weights per
basis time).

  - Basis_gauss3d            mapping/src/basis.py:1170-1555
    (lattice 1291-1324, Q 1359, space 1393-1421, time 1423-1446,
     operg 1489-1524, operg_transpose 1526-1555, norm_fact 1278-1283)
  - Basis_multi              mapping/src/basis.py:4039-4135
  - Basis_bm / Basis_bm_jax  mapping/src/basis.py:472-1168 (wave packets)
  - mywindow / mywindow_flux mapping/src/basis.py:4138-4144

Two coordinate forms:
  geo=True   lon/lat in degrees, exactly the reference's formulas
             (km2deg = 1/110, longitude spacing stretched by cos(lat),
             longitude differences wrapped to [-180, 180)).
  geo=False  planar x/y in km for the Cartesian synthetic grids: the same
             formulas with km2deg = 1, cos(lat) = 1 and no wrap.

Parity status: pinned to golden vectors produced by the reference's own
Basis_gauss3d, Basis_bm and Basis_wavelet3d on a lon/lat grid with land
(tests/golden/gen_golden_basis.py, gen_golden_bm.py, gen_golden_wavelet.py;
G and G^T <= 1e-13), and checked by the transpose (dot-product) identity and
the analytic footprint values.
"""
import numpy as np
from scipy.sparse import csc_matrix

KM2DEG = 1. / 110


def mywindow(x):
    """cos^2 window (basis.py:4138-4140)."""
    return np.cos(x * 0.5 * np.pi) ** 2


def mywindow_flux(x):
    """Flux window (basis.py:4142-4144)."""
    return -np.pi * np.sin(x * 0.5 * np.pi) * np.cos(x * 0.5 * np.pi)


class Gauss3dOracle:
    """One Gaussian (cos^2) space-time basis component.

    lon, lat: 2-D coordinate arrays of the grid (degrees if geo, km if not);
    mask: 2-D bool, True = excluded (land), or None."""

    def __init__(self, lon, lat, sigma_D, sigma_T, facns=2.0, facnlt=1.0, sigma_Q=0.01,
                 normalize_fact=True, time_spinup=None, mask=None, flux=False, geo=False):
        lon = np.asarray(lon, float)
        lat = np.asarray(lat, float)
        self.shape_phys = lon.shape
        self.lon1d, self.lat1d = lon.ravel(), lat.ravel()
        self.lon_min, self.lon_max = np.nanmin(lon), np.nanmax(lon)
        self.lat_min, self.lat_max = np.nanmin(lat), np.nanmax(lat)
        self.sigma_D, self.sigma_T = float(sigma_D), float(sigma_T)
        self.facns, self.facnlt, self.sigma_Q = float(facns), float(facnlt), float(sigma_Q)
        self.time_spinup = time_spinup
        self.geo = geo
        self.km2deg = KM2DEG if geo else 1.0
        self.mask1d = None
        if mask is not None and np.any(mask):
            self.mask1d = np.asarray(mask, bool).ravel()
        self.window = mywindow_flux if flux else mywindow
        self.normalize_fact = normalize_fact
        if normalize_fact:                                       # basis.py:1278-1283
            tt = np.linspace(-self.sigma_T, self.sigma_T)
            tmp = np.zeros_like(tt)
            for i in range(tt.size - 1):
                tmp[i + 1] = tmp[i] + self.window(tt[i] / self.sigma_T) * (tt[i + 1] - tt[i])
            self.norm_fact = tmp.max()

    def _cos(self, lat_deg):
        return np.cos(lat_deg * np.pi / 180.) if self.geo else 1.0

    def _dlon(self, d):
        return np.mod(d + 180, 360) - 180 if self.geo else d

    def set_basis(self, time):
        """Lattice, prior std Q, space and time components (basis.py:1291-1390).
        Returns (Xb, Q); Xb is zero (basis.py:1388-1389)."""
        time = np.asarray(time, float)
        TIME_MIN, TIME_MAX = time.min(), time.max()
        LON_MIN, LON_MAX = self.lon_min, self.lon_max
        LAT_MIN, LAT_MAX = self.lat_min, self.lat_max
        if LON_MAX < LON_MIN:
            LON_MAX = LON_MAX + 360.
        k = self.km2deg
        dlat = self.sigma_D / self.facns * k
        lat0 = LAT_MIN - LAT_MIN % dlat - self.sigma_D * (1 - 1. / self.facns) * k
        lat1 = LAT_MAX + 1.5 * dlat
        ENSLAT1 = np.arange(lat0, lat1, dlat)
        ENSLAT, ENSLON = [], []
        for la in ENSLAT1:
            cl = self._cos(la)
            dlon = self.sigma_D / self.facns / cl * k
            lon0 = LON_MIN - LON_MIN % dlon - self.sigma_D * (1 - 1. / self.facns) / cl * k
            lon1 = LON_MAX + dlon * 1.5
            ENSLON1 = np.arange(lon0, lon1, dlon)
            ENSLAT.append(np.repeat(la, ENSLON1.size))
            ENSLON.append(ENSLON1)
        self.ENSLAT1 = ENSLAT1
        self.ENSLAT = np.concatenate(ENSLAT)
        self.ENSLON = np.concatenate(ENSLON)
        self.ENST = np.arange(-self.sigma_T * (1 - 1. / self.facnlt),
                              (TIME_MAX - TIME_MIN) + 1.5 * self.sigma_T / self.facnlt,
                              self.sigma_T / self.facnlt)
        self.Nx = self.ENSLAT.size
        self.nbasis = self.ENST.size * self.Nx
        self.Q = self.sigma_Q / ((self.facns * self.facnlt)) ** .5 * np.ones(self.nbasis)
        self.Gauss_xy = self._space()
        self.Gauss_t, self.Nt = self._time(time)
        return np.zeros_like(self.Q), self.Q

    def _space(self):
        """cos^2 x cos^2 footprints of half-width sigma_D (basis.py:1393-1421)."""
        k = self.km2deg
        data, indices, sizes = [], [], []
        for lat0, lon0 in zip(self.ENSLAT, self.ENSLON):
            cl = self._cos(lat0)
            xall = self._dlon(self.lon1d - lon0) / k * cl
            yall = (self.lat1d - lat0) / k
            ind = np.where((np.abs(xall) <= self.sigma_D) & (np.abs(yall) <= self.sigma_D))[0]
            xx, yy = xall[ind], yall[ind]
            if self.mask1d is not None:
                keep = ~self.mask1d[ind]
                ind, xx, yy = ind[keep], xx[keep], yy[keep]
            data.append(mywindow(xx / self.sigma_D) * mywindow(yy / self.sigma_D))
            indices.append(ind)
            sizes.append(ind.size)
        indptr = np.zeros(len(sizes) + 1, dtype=np.int64)
        indptr[1:] = np.cumsum(sizes)
        return csc_matrix((np.concatenate(data), np.concatenate(indices), indptr),
                          shape=(self.lon1d.size, self.Nx))

    def time_weights(self, t):
        """[(it, fact)] of the time centres active at t (basis.py:1423-1446)."""
        out = []
        for it, tc in enumerate(self.ENST):
            dt = t - tc
            if abs(dt) < self.sigma_T:
                fact = self.window(dt / self.sigma_T)
                if self.normalize_fact:
                    fact /= self.norm_fact
                if self.time_spinup is not None and t < self.time_spinup:
                    fact *= (1 - self.window(t / self.time_spinup))
                if fact != 0:
                    out.append((it, fact))
        return out

    def _time(self, time):
        Gt, Nt = {}, {}
        for t in time:
            g = np.zeros(self.Nx * self.ENST.size)
            act = self.time_weights(t)
            for it, fact in act:
                g[it * self.Nx:(it + 1) * self.Nx] = fact
            Gt[float(t)], Nt[float(t)] = g, len(act)
        return Gt, Nt

    def operg(self, t, X):
        """phi = G(t) X on the grid (basis.py:1489-1524)."""
        g = self.Gauss_t[float(t)]
        ind0 = np.nonzero(g)[0]
        phi = np.zeros(self.lon1d.size)
        if ind0.size:
            GtX = (g * X)[ind0].reshape(self.Nt[float(t)], self.Nx)
            phi += self.Gauss_xy.dot(GtX.sum(axis=0))
        return phi.reshape(self.shape_phys)

    def operg_transpose(self, t, adphi):
        """adX = G(t)^T adphi (basis.py:1526-1555; the reference's JAX form
        1686-1737 takes the vjp of operg, which is this product)."""
        adX = np.zeros(self.nbasis)
        g = self.Gauss_t[float(t)]
        ind0 = np.nonzero(g)[0]
        if ind0.size:
            Gt = g[ind0].reshape(self.Nt[float(t)], self.Nx)
            ad = self.Gauss_xy.T.dot(np.asarray(adphi).ravel())
            adX[ind0] += (Gt * ad[None, :]).ravel()
        return adX


class MultiOracle:
    """Concatenation of components (basis.py:4039-4135): the projections add
    up into one field, the transpose concatenates."""

    def __init__(self, comps):
        self.comps = comps

    def set_basis(self, time):
        Xb, Q, self.slices, n = [], [], [], 0
        for c in self.comps:
            xb, q = c.set_basis(time)
            self.slices.append(slice(n, n + c.nbasis))
            n += c.nbasis
            Xb.append(xb)
            Q.append(q)
        self.nbasis = n
        return np.concatenate(Xb), np.concatenate(Q)

    def operg(self, t, X):
        return sum(c.operg(t, X[s]) for c, s in zip(self.comps, self.slices))

    def operg_transpose(self, t, adphi):
        return np.concatenate([c.operg_transpose(t, adphi) for c in self.comps])


class BMOracle:
    """Wave-packet basis of the reference (Basis_bm / Basis_bm_jax,
    mapping/src/basis.py:472-1168), in the reference's sparse form.

    Frequencies ff (pseudo-wavelengths between lmin and lmax, 577-583),
    directions theta (587), per frequency a lattice of centres spaced
    DX/facns (611-649, centres whose footprint of radius 1/ff is fully
    masked are dropped), atoms sqrt(2) cos^2(pi xx/2DX) cos^2(pi yy/2DX)
    {cos, sin}(kx xx + ky yy) (736-772), per-frequency time centres spaced
    tdec/facnlt from -time_ref mod tdec (652-667), time weights of the JAX
    form (|dt| <= tdec, 1026-1035), prior std Q (671-690). Coefficients of
    one frequency are ordered [time centre][space centre][theta][cos, sin].
    geo=False: planar x/y in km (km2deg = 1, cos(lat) = 1)."""

    def __init__(self, lon, lat, npsp=3.5, facpsp=1.5, lmin=80., lmax=900., facns=1., facnlt=2.,
                 tdecmin=2., tdecmax=20., factdec=1., sloptdec=-1.28, Qmax=1e-3, slopQ=-2., lmeso=300.,
                 tmeso=20., norm_time=True, flux=False, time_ref=0.0, mask=None, geo=False):
        lon = np.asarray(lon, float)
        lat = np.asarray(lat, float)
        self.shape_phys = lon.shape
        self.lon1d, self.lat1d = lon.ravel(), lat.ravel()
        self.lon_min, self.lon_max = lon.min(), lon.max()
        self.lat_min, self.lat_max = lat.min(), lat.max()
        self.npsp, self.facpsp, self.lmin, self.lmax = float(npsp), float(facpsp), float(lmin), float(lmax)
        self.facns, self.facnlt = float(facns), float(facnlt)
        self.tdecmin, self.tdecmax, self.factdec, self.sloptdec = float(tdecmin), float(tdecmax), float(factdec), \
            float(sloptdec)
        self.Qmax, self.slopQ, self.lmeso, self.tmeso = float(Qmax), float(slopQ), float(lmeso), float(tmeso)
        self.norm_time = norm_time
        self.window = mywindow_flux if flux else mywindow
        self.time_ref = float(time_ref)
        self.geo = geo
        self.km2deg = KM2DEG if geo else 1.0
        self.mask1d = None
        if mask is not None and np.any(mask):
            self.mask1d = np.asarray(mask, bool).ravel()

    def _cos(self, lat_deg):
        return np.cos(lat_deg * np.pi / 180.) if self.geo else 1.0

    def set_basis(self, time):
        time = np.asarray(time, float)
        TIME_MIN, TIME_MAX = time.min(), time.max()
        LON_MIN, LON_MAX, LAT_MIN, LAT_MAX = self.lon_min, self.lon_max, self.lat_min, self.lat_max
        k2 = self.km2deg
        logff = np.arange(np.log(1. / self.lmin), np.log(1. / self.lmax) - np.log(1 + self.facpsp / self.npsp),
                          -np.log(1 + self.facpsp / self.npsp))[::-1]
        ff = np.exp(logff)
        dff = ff[1:] - ff[:-1]
        theta = np.linspace(0, np.pi, int(np.pi * ff[0] / dff[0] * self.facpsp))[:-1]
        ntheta, nf = len(theta), len(ff)
        deltat = TIME_MAX - TIME_MIN
        DX = 1. / ff * self.npsp * 0.5
        DXG = DX / self.facns
        ENSLON, ENSLAT, enst, tdec, norm_fact = [], [], [], [], []
        NP = np.zeros(nf, dtype=int)
        for iff in range(nf):
            el, ea = [], []
            dlat = DXG[iff] * k2
            lat0 = LAT_MIN - LAT_MIN % dlat - DX[iff] * k2
            lat1 = LAT_MAX + DX[iff] * k2 * 1.5
            for la in np.arange(lat0, lat1, dlat):
                cl = self._cos(la)
                dlon = DXG[iff] / cl * k2
                lon0 = LON_MIN - LON_MIN % dlon - DX[iff] / cl * k2
                lon1 = LON_MAX + DX[iff] / cl * k2 * 1.5
                for lo in np.arange(lon0, lon1, dlon):
                    if self.mask1d is not None:
                        ind = np.where((np.abs((self.lon1d - lo) / k2 * self._cos(la)) <= 1. / ff[iff]) &
                                       (np.abs((self.lat1d - la) / k2) <= 1. / ff[iff]))[0]
                        if np.all(self.mask1d[ind]):
                            continue
                    el.append(lo)
                    ea.append(la)
            ENSLON.append(np.array(el))
            ENSLAT.append(np.array(ea))
            NP[iff] = len(el)
            td = self.tmeso * self.lmeso ** self.sloptdec * ff[iff] ** self.sloptdec
            td *= self.factdec
            td = min(max(td, self.tdecmin), self.tdecmax)
            tdec.append(td)
            t0 = -self.time_ref % td
            enst.append(np.arange(t0 - td / self.facnlt, deltat + td / self.facnlt, td / self.facnlt))
            tt = np.linspace(-td, td)
            tmp = np.zeros_like(tt)
            for i in range(tt.size - 1):
                tmp[i + 1] = tmp[i] + self.window(tt[i] / td) * (tt[i + 1] - tt[i])
            norm_fact.append(tmp.max())
        Q, bounds, iw = [], [], 0
        for iff in range(nf):
            bounds.append(iw)
            n = 2 * len(enst[iff]) * ntheta * NP[iff]
            if NP[iff] > 0:
                if 1 / ff[iff] > self.lmeso:
                    Q.append(self.Qmax / self.facns * np.ones(n))
                else:
                    Q.append(self.Qmax / self.facns * self.lmeso ** self.slopQ * ff[iff] ** self.slopQ * np.ones(n))
                iw += n
        bounds.append(iw)
        self.ff, self.theta, self.ntheta, self.nf, self.DX = ff, theta, ntheta, nf, DX
        self.ENSLON, self.ENSLAT, self.NP, self.enst, self.tdec, self.norm_fact = ENSLON, ENSLAT, NP, enst, tdec, \
            norm_fact
        self.k = 2 * np.pi * ff
        self.bounds = bounds
        self.nbasis = iw
        self.Q = np.concatenate(Q) if Q else np.zeros(0)
        self.Gx = [self._space(iff) for iff in range(nf)]
        self.times = time
        return np.zeros_like(self.Q), self.Q

    def _space(self, iff):
        k2 = self.km2deg
        cols_data, cols_ind = [], []
        for P in range(self.NP[iff]):
            lo, la = self.ENSLON[iff][P], self.ENSLAT[iff][P]
            cl = self._cos(la)
            xall = (self.lon1d - lo) / k2 * cl
            yall = (self.lat1d - la) / k2
            ind = np.where((np.abs(xall) <= self.DX[iff]) & (np.abs(yall) <= self.DX[iff]))[0]
            xx, yy = xall[ind], yall[ind]
            if self.mask1d is not None:
                keep = ~self.mask1d[ind]
                ind, xx, yy = ind[keep], xx[keep], yy[keep]
            facs = mywindow(xx / self.DX[iff]) * mywindow(yy / self.DX[iff])
            for th in self.theta:
                kx, ky = self.k[iff] * np.cos(th), self.k[iff] * np.sin(th)
                cols_data.append(np.sqrt(2) * facs * np.cos(kx * xx + ky * yy))
                cols_ind.append(ind)
                cols_data.append(np.sqrt(2) * facs * np.sin(kx * xx + ky * yy))
                cols_ind.append(ind)
        sizes = [len(c) for c in cols_ind]
        indptr = np.zeros(len(sizes) + 1, dtype=np.int64)
        indptr[1:] = np.cumsum(sizes)
        data = np.concatenate(cols_data) if cols_data else np.zeros(0)
        indices = np.concatenate(cols_ind) if cols_ind else np.zeros(0, dtype=np.int64)
        return csc_matrix((data, indices, indptr), shape=(self.lon1d.size, len(sizes)))

    def time_weights(self, iff, t):
        """[(it, fact)] of frequency iff at time t (JAX form, basis.py:1026-1035)."""
        out = []
        td = self.tdec[iff]
        for it, tc in enumerate(self.enst[iff]):
            dt = t - tc
            if not (abs(dt) > td or np.isnan(tc)):
                fact = self.window(dt / td)
                if self.norm_time:
                    fact /= self.norm_fact[iff]
                out.append((it, fact))
        return out

    def operg(self, t, X):
        phi = np.zeros(self.lon1d.size)
        for iff in range(self.nf):
            nx_ = 2 * self.ntheta * self.NP[iff]
            Xf = X[self.bounds[iff]:self.bounds[iff + 1]].reshape(len(self.enst[iff]), nx_) if nx_ else None
            if nx_ == 0:
                continue
            z = np.zeros(nx_)
            for it, fct in self.time_weights(iff, t):
                z += fct * Xf[it]
            phi += self.Gx[iff].dot(z)
        return phi.reshape(self.shape_phys)

    def operg_transpose(self, t, adphi):
        adX = np.zeros(self.nbasis)
        for iff in range(self.nf):
            nx_ = 2 * self.ntheta * self.NP[iff]
            if nx_ == 0:
                continue
            ad = self.Gx[iff].T.dot(np.asarray(adphi).ravel())
            blk = adX[self.bounds[iff]:self.bounds[iff + 1]].reshape(len(self.enst[iff]), nx_)
            for it, fct in self.time_weights(iff, t):
                blk[it] += fct * ad
        return adX


def gaspari_cohn(r, c=1):
    """Gaspari-Cohn taper of mapping/src/tools.py:16-46 (scalar r)."""
    if c <= 0:
        return 0.0
    ra = 2 * abs(r) / c
    if ra <= 1.:
        return -0.25 * ra ** 5 + 0.5 * ra ** 4 + 0.625 * ra ** 3 - 5. / 3. * ra ** 2 + 1.
    if 1. < ra <= 2.:
        return 1. / 12. * ra ** 5 - 0.5 * ra ** 4 + 0.625 * ra ** 3 + 5. / 3. * ra ** 2 - 5. * ra + 4. - 2. / 3. / ra
    return 0.0


class WaveletOracle(BMOracle):
    """Wavelet basis of the reference (Basis_wavelet3d, mapping/src/basis.py:
    2640-2985; the numpy form: the jax subclass's time routine reads
    attributes the class never sets).

    Space and time pseudo-frequencies between lmin..lmax and tmin..tmax
    (2689-2707, periods above the maximum dropped), directions (2710), per
    space frequency a lattice laid out from the domain centre with spacing
    DXs/facnst (2717-2771; a centre whose box of half-width 0.5/fs is fully
    masked is dropped), per time frequency centres from the time centre with
    spacing DXt/facnst (2773-2796), Gaspari-Cohn time weights divided by the
    running integral's maximum (|dt| < DXt, kept when non-zero, 2902-2922),
    Q = sigma_Q. Coefficients of one space frequency: [time centre over all
    time frequencies][space centre][theta][cos, sin]."""

    def __init__(self, lon, lat, npsp=3.5, facpsp=1.5, facnst=1., lmin=80., lmax=900., tmin=2., tmax=20.,
                 sigma_Q=1.0, mask=None, geo=False):
        super().__init__(lon, lat, npsp=npsp, facpsp=facpsp, lmin=lmin, lmax=lmax, mask=mask, geo=geo)
        self.facnst, self.tmin, self.tmax, self.sigma_Q = float(facnst), float(tmin), float(tmax), float(sigma_Q)

    @staticmethod
    def _centred(c, lo, hi, step):
        return np.concatenate((np.arange(c, lo, -step)[::-1], np.arange(c, hi, step)[1:]))

    def set_basis(self, time):
        time = np.asarray(time, float)
        TIME_MIN, TIME_MAX = time.min(), time.max()
        LON_MIN, LON_MAX, LAT_MIN, LAT_MAX = self.lon_min, self.lon_max, self.lat_min, self.lat_max
        if LON_MAX < LON_MIN:
            LON_MAX = LON_MAX + 360.
        k2 = self.km2deg
        step = np.log(1 + self.facpsp / self.npsp)
        logfs = np.arange(np.log(1. / self.lmin), np.log(1. / self.lmax) - step, -step)[::-1]
        fs = np.exp(logfs)
        fs = fs[1 / fs <= self.lmax]
        dfs = fs[1:] - fs[:-1]
        logft = np.arange(np.log(1. / self.tmin), np.log(1. / self.tmax) - step, -step)[::-1]
        ft = np.exp(logft)
        ft = ft[1 / ft <= self.tmax]
        theta = np.linspace(0, np.pi, int(np.pi * fs[0] / dfs[0] * self.facpsp))[:-1]
        ntheta, nf = len(theta), len(fs)
        DXs = 1. / fs * self.npsp * 0.5
        ENSLON, ENSLAT = [], []
        NS = np.zeros(nf, dtype=int)
        for iff in range(nf):
            el, ea = [], []
            lats = self._centred((LAT_MIN + LAT_MAX) / 2, LAT_MIN - DXs[iff] * k2, LAT_MAX + DXs[iff] * k2,
                                 DXs[iff] / self.facnst * k2)
            for la in lats:
                cl = self._cos(la)
                lons = self._centred((LON_MIN + LON_MAX) / 2, LON_MIN - DXs[iff] / cl * k2,
                                     LON_MAX + DXs[iff] / cl * k2, DXs[iff] / self.facnst / cl * k2)
                for lo in lons:
                    if self.mask1d is not None:
                        ind = np.where((np.abs((self.lon1d - lo) / k2 * cl) <= .5 / fs[iff]) &
                                       (np.abs((self.lat1d - la) / k2) <= .5 / fs[iff]))[0]
                        if np.all(self.mask1d[ind]):
                            continue
                    el.append(lo)
                    ea.append(la)
            ENSLON.append(np.array(el))
            ENSLAT.append(np.array(ea))
            NS[iff] = len(el)
        DXt = 1. / ft * self.npsp * 0.5
        enst, tsc, tnorm = [], [], []
        for ift in range(len(ft)):
            e = self._centred((TIME_MIN + TIME_MAX) / 2, TIME_MIN - DXt[ift], TIME_MAX + DXt[ift],
                              DXt[ift] / self.facnst)
            tt = np.linspace(-DXt[ift], DXt[ift])
            tmp = np.zeros_like(tt)
            for i in range(tt.size - 1):
                tmp[i + 1] = tmp[i] + gaspari_cohn(tt[i], DXt[ift]) * (tt[i + 1] - tt[i])
            enst.extend(e.tolist())
            tsc.extend([DXt[ift]] * e.size)
            tnorm.extend([tmp.max()] * e.size)
        Q, bounds, iw = [], [], 0
        for iff in range(nf):
            bounds.append(iw)
            if NS[iff] > 0:
                n = 2 * len(enst) * ntheta * NS[iff]
                Q.append(self.sigma_Q * np.ones(n))
                iw += n
        bounds.append(iw)
        self.ff, self.theta, self.ntheta, self.nf, self.DX = fs, theta, ntheta, nf, DXs
        self.ENSLON, self.ENSLAT, self.NP = ENSLON, ENSLAT, NS
        self.enst = [np.array(enst)] * nf
        self.tscale, self.tnorm = np.array(tsc), np.array(tnorm)
        self.k = 2 * np.pi * fs
        self.bounds = bounds
        self.nbasis = iw
        self.Q = np.concatenate(Q) if Q else np.zeros(0)
        self.Gx = [self._space(iff) for iff in range(nf)]
        self.times = time
        return np.zeros_like(self.Q), self.Q

    def time_weights(self, iff, t):
        out = []
        for it, tc in enumerate(self.enst[iff]):
            dt = t - tc
            if abs(dt) < self.tscale[it]:
                fact = gaspari_cohn(dt, self.tscale[it]) / self.tnorm[it]
                if fact != 0:
                    out.append((it, fact))
        return out


def aux_interp_mean(fc, latc, lonc, data, f, elon, elat):
    """np.nanmean of ``data.interp(f=f, lon=elon, lat=elat)`` for 1-D lon /
    lat indexers (basis.py:2071, 2134): xarray interpolates orthogonally
    (the outer product of the lon and lat values), multilinearly, NaN outside
    the coordinates. data is [f][lat][lon] on ascending coordinates. Returns
    NaN when every value is NaN."""
    from scipy.interpolate import RegularGridInterpolator
    rgi = RegularGridInterpolator((np.asarray(fc, float), np.asarray(latc, float), np.asarray(lonc, float)),
                                  np.asarray(data, float), method="linear", bounds_error=False, fill_value=np.nan)
    la, lo = np.meshgrid(np.asarray(elat, float), np.asarray(elon, float), indexing="ij")
    pts = np.stack([np.full(la.size, float(f)), la.ravel(), lo.ravel()], axis=1)
    v = rgi(pts)
    return np.nan if np.all(np.isnan(v)) else float(np.nanmean(v))


class BMauxOracle:
    """Wave-packet basis with per-location decorrelation times and variances
    of the reference (Basis_bmaux / Basis_bmaux_jax, mapping/src/basis.py
    1741-2638), without depth tapering, facQ_aux file or C-grid variables.

    The atoms are the wave packets of Basis_bm. What differs (basis.py):
    - the lattice ends at LAT_MAX + DX and LON_MAX + DX/cos (1947-1954), not
      1.5 DX;
    - every space centre P of frequency f has its own decorrelation time
      tdec = factdec * nanmean of Tdec(f, lon, lat) over a 10 x 10 grid of its
      box of half-width DX, clipped to [tdecmin, tdecmax] (2004-2015), its own
      window integral norm_fact (2017-2024) and its own time centres from
      -time_ref mod tdec, spaced tdec / facnlt (2026-2027); the time axis of
      a frequency is padded with NaN centres to its longest list (2029-2035);
    - Q of (time centre, P) is facQ * nanmean of Std over the same box (1e-10
      where every value is NaN), or 1e-10 * facQ on a padded centre
      (2041-2100);
    - G(t) phi = sum_f Gx_f sum_it Gt(t)[it, P] X[it, P, :] with Gt = window(
      dt / tdec_P) / norm_fact_P for |dt| <= tdec_P, 0 otherwise or on a
      padded centre (jax form, 2473-2530; the numpy operg of 2303-2340
      accumulates into a variable it never returns).
    aux = dict(f, lat, lon, Tdec, Std) with Tdec, Std [f][lat][lon] on
    ascending coordinates (in the grid's longitude convention)."""

    def __init__(self, lon, lat, aux, npsp=3.5, facpsp=1.5, lmin=80., lmax=900., facns=1., facnlt=2.,
                 tdecmin=2., tdecmax=20., factdec=1., facQ=1., norm_time=True, flux=False, time_ref=0.0,
                 mask=None, geo=True):
        lon = np.asarray(lon, float)
        lat = np.asarray(lat, float)
        self.shape_phys = lon.shape
        self.lon1d, self.lat1d = lon.ravel(), lat.ravel()
        self.lon_min, self.lon_max = lon.min(), lon.max()
        self.lat_min, self.lat_max = lat.min(), lat.max()
        self.aux = aux
        self.npsp, self.facpsp, self.lmin, self.lmax = float(npsp), float(facpsp), float(lmin), float(lmax)
        self.facns, self.facnlt = float(facns), float(facnlt)
        self.tdecmin, self.tdecmax, self.factdec, self.facQ = float(tdecmin), float(tdecmax), float(factdec), \
            float(facQ)
        self.norm_time = norm_time
        self.window = mywindow_flux if flux else mywindow
        self.time_ref = float(time_ref)
        self.geo = geo
        self.km2deg = KM2DEG if geo else 1.0
        self.mask1d = None
        if mask is not None and np.any(mask):
            self.mask1d = np.asarray(mask, bool).ravel()

    def _cos(self, lat_deg):
        return np.cos(lat_deg * np.pi / 180.) if self.geo else 1.0

    def _box_mean(self, name, iff, P):
        k2 = self.km2deg
        lo, la = self.ENSLON[iff][P], self.ENSLAT[iff][P]
        dlon = self.DX[iff] * k2 / self._cos(la)
        dlat = self.DX[iff] * k2
        elon = np.linspace(lo - dlon, lo + dlon, 10)
        elat = np.linspace(la - dlat, la + dlat, 10)
        a = self.aux
        return aux_interp_mean(a["f"], a["lat"], a["lon"], a[name], self.ff[iff], elon, elat)

    def set_basis(self, time):
        time = np.asarray(time, float)
        TIME_MIN, TIME_MAX = time.min(), time.max()
        LON_MIN, LON_MAX, LAT_MIN, LAT_MAX = self.lon_min, self.lon_max, self.lat_min, self.lat_max
        if LON_MAX < LON_MIN:
            LON_MAX = LON_MAX + 360.
        k2 = self.km2deg
        logff = np.arange(np.log(1. / self.lmin), np.log(1. / self.lmax) - np.log(1 + self.facpsp / self.npsp),
                          -np.log(1 + self.facpsp / self.npsp))[::-1]
        ff = np.exp(logff)
        dff = ff[1:] - ff[:-1]
        theta = np.linspace(0, np.pi, int(np.pi * ff[0] / dff[0] * self.facpsp))[:-1]
        ntheta, nf = len(theta), len(ff)
        deltat = TIME_MAX - TIME_MIN
        DX = 1. / ff * self.npsp * 0.5
        DXG = DX / self.facns
        self.ff, self.DX = ff, DX
        ENSLON, ENSLAT = [], []
        NP = np.zeros(nf, dtype=int)
        for iff in range(nf):
            el, ea = [], []
            dlat = DXG[iff] * k2
            lat0 = LAT_MIN - LAT_MIN % dlat - DX[iff] * k2
            lat1 = LAT_MAX + DX[iff] * k2
            for la in np.arange(lat0, lat1, dlat):
                cl = self._cos(la)
                dlon = DXG[iff] / cl * k2
                lon0 = LON_MIN - LON_MIN % dlon - DX[iff] / cl * k2
                lon1 = LON_MAX + DX[iff] / cl * k2
                for lo in np.arange(lon0, lon1, dlon):
                    if self.mask1d is not None:
                        ind = np.where((np.abs((self.lon1d - lo) / k2 * self._cos(la)) <= 1. / ff[iff]) &
                                       (np.abs((self.lat1d - la) / k2) <= 1. / ff[iff]))[0]
                        if np.all(self.mask1d[ind]):
                            continue
                    el.append(lo)
                    ea.append(la)
            ENSLON.append(np.array(el))
            ENSLAT.append(np.array(ea))
            NP[iff] = len(el)
        self.ENSLON, self.ENSLAT, self.NP = ENSLON, ENSLAT, NP
        tdec, norm_fact, enst, std = [], [], [], []
        for iff in range(nf):
            td_f, nf_f, en_f, sd_f = [], [], [], []
            for P in range(NP[iff]):
                m = self._box_mean("Tdec", iff, P)
                td = 0.0 if np.isnan(m) else m
                td *= self.factdec
                td = min(max(td, self.tdecmin), self.tdecmax)
                if self.norm_time:
                    tt = np.linspace(-td, td)
                    tmp = np.zeros_like(tt)
                    for i in range(tt.size - 1):
                        tmp[i + 1] = tmp[i] + self.window(tt[i] / td) * (tt[i + 1] - tt[i])
                    nrm = tmp.max()
                else:
                    nrm = 1.0
                t0 = -self.time_ref % td
                td_f.append(td)
                nf_f.append(nrm)
                en_f.append(np.arange(t0 - td / self.facnlt, deltat + td / self.facnlt, td / self.facnlt))
                s = self._box_mean("Std", iff, P)
                sd_f.append(1e-10 if np.isnan(s) else s)
            nit = max((e.size for e in en_f), default=0)
            pad = np.full((NP[iff], nit), np.nan)
            for P in range(NP[iff]):
                pad[P, :en_f[P].size] = en_f[P]
            tdec.append(np.array(td_f))
            norm_fact.append(np.array(nf_f))
            enst.append(pad)
            std.append(np.array(sd_f))
        Q, bounds, iw = [], [], 0
        for iff in range(nf):
            bounds.append(iw)
            nit = enst[iff].shape[1]
            for it in range(nit):
                for P in range(NP[iff]):
                    q = 1e-10 if np.isnan(enst[iff][P, it]) else std[iff][P]
                    Q.append(np.full(2 * ntheta, q * self.facQ))
            iw += 2 * ntheta * NP[iff] * nit
        bounds.append(iw)
        self.theta, self.ntheta, self.nf = theta, ntheta, nf
        self.tdec, self.norm_fact, self.enst, self.std = tdec, norm_fact, enst, std
        self.k = 2 * np.pi * ff
        self.bounds = bounds
        self.nbasis = iw
        self.Q = np.concatenate(Q) if Q else np.zeros(0)
        self.Gx = [BMOracle._space(self, iff) for iff in range(nf)]
        self.times = time
        return np.zeros_like(self.Q), self.Q

    def time_weights(self, iff, t):
        """Gt(t) of frequency iff as [time centre][space centre]."""
        en = self.enst[iff]
        g = np.zeros(en.shape)
        for P in range(en.shape[0]):
            td = self.tdec[iff][P]
            for it in range(en.shape[1]):
                dt = t - en[P, it]
                if not (abs(dt) > td or np.isnan(en[P, it])):
                    g[P, it] = self.window(dt / td) / self.norm_fact[iff][P]
        return g.T

    def operg(self, t, X):
        phi = np.zeros(self.lon1d.size)
        for iff in range(self.nf):
            nx_ = 2 * self.ntheta * self.NP[iff]
            if nx_ == 0:
                continue
            nit = self.enst[iff].shape[1]
            Xf = X[self.bounds[iff]:self.bounds[iff + 1]].reshape(nit, self.NP[iff], 2 * self.ntheta)
            z = (self.time_weights(iff, t)[:, :, None] * Xf).sum(axis=0).ravel()
            phi += self.Gx[iff].dot(z)
        return phi.reshape(self.shape_phys)

    def operg_transpose(self, t, adphi):
        adX = np.zeros(self.nbasis)
        for iff in range(self.nf):
            nx_ = 2 * self.ntheta * self.NP[iff]
            if nx_ == 0:
                continue
            nit = self.enst[iff].shape[1]
            ad = self.Gx[iff].T.dot(np.asarray(adphi).ravel()).reshape(self.NP[iff], 2 * self.ntheta)
            blk = adX[self.bounds[iff]:self.bounds[iff + 1]].reshape(nit, self.NP[iff], 2 * self.ntheta)
            blk += self.time_weights(iff, t)[:, :, None] * ad[None]
        return adX
