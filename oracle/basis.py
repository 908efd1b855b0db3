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
