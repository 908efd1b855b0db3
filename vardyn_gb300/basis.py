"""Gaussian space-time reduced basis on the GPU (Basis_gauss3d / Basis_multi).

:class:`BasisPlan` owns one ``vd_basis_plan`` (lattice and banded footprint
tables built by the library on the host, uploaded once) and projects batched
control vectors with ``vd_basis_project`` / ``vd_basis_project_T`` on torch's
current stream.

:class:`Basis_gauss3d` and :class:`Basis_multi` mirror the reference classes
(mapping/src/basis.py:1170-1555 and 4039-4135): the constructor takes
``(config, State)``, ``set_basis(time, return_q=True)`` returns ``(Xb, Q)``,
``operg(t, X, State=State.params)`` writes the projected field into the
parameter dict, and ``operg_transpose(t, adState=adState.params)`` returns
the coefficient adjoint and zeroes the parameter adjoint. ``t`` is looked up
among the basis times by exact equality, as the reference does
(basis.py:1636-1640).
"""
import contextlib
import ctypes

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Gauss3dParams:
    """Parameters of one Basis_gauss3d component (config.BASIS fields,
    basis.py:1176-1187)."""

    def __init__(self, sigma_D, sigma_T, facns=1.0, facnlt=2.0, sigma_Q=1.0, normalize_fact=True,
                 flux=False, time_spinup=None):
        self.sigma_D = float(sigma_D)
        self.sigma_T = float(sigma_T)
        self.facns = float(facns)
        self.facnlt = float(facnlt)
        self.sigma_Q = float(sigma_Q)
        self.normalize_fact = bool(normalize_fact)
        self.flux = bool(flux)
        self.time_spinup = time_spinup

    def to_c(self):
        return _lib.VdGauss3dParams(self.sigma_D, self.sigma_T, self.facns, self.facnlt, self.sigma_Q,
                                    int(self.normalize_fact), int(self.flux),
                                    int(self.time_spinup is not None),
                                    float(self.time_spinup) if self.time_spinup is not None else 0.0)


class _SeparablePlan:
    """Shared plumbing of the basis plans: grid description, workspace, batched
    G / G^T calls on torch's current stream."""

    _prefix = None

    def _grid(self, xc, yc, time, land, geographic, dtype, device, host_only):
        self.xc = np.ascontiguousarray(xc, dtype=np.float64)
        self.yc = np.ascontiguousarray(yc, dtype=np.float64)
        self.ny, self.nx = self.yc.size, self.xc.size
        self.times = np.ascontiguousarray(np.atleast_1d(time), dtype=np.float64)
        self.dtype = dtype
        self.host_only = host_only
        self.device = None
        if not host_only:
            if not torch.cuda.is_available():
                raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
            dev = torch.device(device or "cuda")
            self.device = torch.device("cuda", dev.index if dev.index is not None else torch.cuda.current_device())
        self._land = None
        if land is not None:
            land = np.asarray(land, dtype=bool)
            if land.shape != (self.ny, self.nx):
                raise ValueError("land must be [ny, nx]")
            self._land = np.ascontiguousarray(land.astype(np.int8))
        dptr = ctypes.POINTER(ctypes.c_double)
        self._gridc = _lib.VdBasisGrid(
            self.ny, self.nx, _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32, int(geographic),
            self.xc.ctypes.data_as(dptr), self.yc.ctypes.data_as(dptr),
            self._land.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)) if self._land is not None else None,
            self.times.size, self.times.ctypes.data_as(dptr), int(host_only))
        self.lib = _lib.load()
        self._ws = None

    def _on_device(self):
        """Context that makes the plan's device current for a C call (the
        caller's current device is restored afterwards)."""
        return contextlib.nullcontext() if self.host_only else torch.cuda.device(self.device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                getattr(self.lib, self._prefix + "_plan_destroy")(h)
            except Exception:
                pass
            self._h = None

    def time_index(self, t):
        """Index of basis time t (exact match, as basis.py:1636-1640)."""
        k = np.nonzero(self.times == float(t))[0]
        if k.size == 0:
            raise KeyError(f"time {t} is not a basis time")
        return int(k[0])

    def workspace(self, batch):
        n = int(getattr(self.lib, self._prefix + "_workspace_bytes")(self._h, batch))
        if self._ws is None or self._ws.numel() < n:
            self._ws = torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)
        return self._ws

    def _batch_X(self, X):
        if X.dim() == 1:
            X = X.unsqueeze(0)
        if X.dim() != 2 or X.shape[1] != self.nbasis:
            raise ValueError(f"control must be [batch, {self.nbasis}]")
        if X.dtype != self.dtype or X.device != self.device or X.stride(1) != 1 or X.stride(0) < self.nbasis:
            raise ValueError("control must be a contiguous tensor of the plan's dtype on its device")
        return X

    def project(self, k, X, out=None, accumulate=False):
        """phi [B, ny, nx] = G(t_k) X (+ out if accumulate)."""
        X = self._batch_X(X)
        B = X.shape[0]
        if out is None:
            out = torch.empty(B, self.ny, self.nx, dtype=self.dtype, device=self.device)
            accumulate = False
        ws = self.workspace(B)
        with self._on_device():
            _lib.check(getattr(self.lib, self._prefix + "_project")(
                self._h, B, int(k), _ptr(X), X.stride(0), _ptr(out), int(bool(accumulate)), _ptr(ws), ws.numel(),
                _stream()), self._prefix + "_project")
        return out

    def project_T(self, k, adphi, adX):
        """adX [B, nbasis] += G(t_k)^T adphi [B, ny, nx]."""
        adX = self._batch_X(adX)
        B = adX.shape[0]
        adphi = adphi.reshape(B, self.ny, self.nx)
        if not adphi.is_contiguous():
            raise ValueError("adphi must be contiguous")
        ws = self.workspace(B)
        with self._on_device():
            _lib.check(getattr(self.lib, self._prefix + "_project_T")(
                self._h, B, int(k), _ptr(adphi), _ptr(adX), adX.stride(0), _ptr(ws), ws.numel(), _stream()),
                self._prefix + "_project_T")
        return adX

    def q(self):
        """Prior standard deviation of every coefficient (float64 [nbasis])."""
        q = np.zeros(self.nbasis)
        _lib.check(getattr(self.lib, self._prefix + "_q")(self._h, q.ctypes.data), self._prefix + "_q")
        return q


class BasisPlan(_SeparablePlan):
    """One or more Gaussian components on a rectilinear grid.

    xc [nx], yc [ny]: column / row coordinates (km, or lon/lat in degrees when
    ``geographic``); time: the basis times in days (set_basis's argument);
    land: bool [ny, nx] (True = excluded) or None. ``host_only`` builds the
    tables without a GPU (queries only)."""

    _prefix = "vd_basis"

    def __init__(self, xc, yc, time, comps, land=None, geographic=False, dtype=torch.float32,
                 device=None, host_only=False):
        self._grid(xc, yc, time, land, geographic, dtype, device, host_only)
        self.comps = list(comps)
        params = (_lib.VdGauss3dParams * len(self.comps))(*[c.to_c() for c in self.comps])
        h = ctypes.c_void_p()
        with self._on_device():
            _lib.check(self.lib.vd_basis_plan_create(ctypes.byref(h), ctypes.byref(self._gridc), len(self.comps),
                                                     params), "vd_basis_plan_create")
        self._h = h
        self.nbasis = int(self.lib.vd_basis_nbasis(h))

    def component(self, c):
        off, nt, ns = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.vd_basis_component(self._h, c, ctypes.byref(off), ctypes.byref(nt),
                                               ctypes.byref(ns)), "vd_basis_component")
        return off.value, nt.value, ns.value

    def lattice(self, c):
        """(ENST, ENSLAT, ENSLON) of component c."""
        _, nt, ns = self.component(c)
        enst, lat, lon = np.zeros(nt), np.zeros(ns), np.zeros(ns)
        _lib.check(self.lib.vd_basis_lattice(self._h, c, enst.ctypes.data, lat.ctypes.data, lon.ctypes.data),
                   "vd_basis_lattice")
        return enst, lat, lon

    def time_weights(self, k, c):
        n = ctypes.c_int()
        _lib.check(self.lib.vd_basis_time_weights(self._h, k, c, ctypes.byref(n), None, None),
                   "vd_basis_time_weights")
        it = np.zeros(max(n.value, 1), dtype=np.int32)
        w = np.zeros(max(n.value, 1))
        _lib.check(self.lib.vd_basis_time_weights(self._h, k, c, ctypes.byref(n), it.ctypes.data,
                                                  w.ctypes.data), "vd_basis_time_weights")
        return list(zip(it[:n.value].tolist(), w[:n.value].tolist()))


class BMParams:
    """Parameters of the wave-packet basis (config.BASIS fields of Basis_bm,
    basis.py:478-496); ``time_ref`` is the window start in days since
    1950-01-01 (basis.py:527)."""

    def __init__(self, npsp=3.5, facpsp=1.5, lmin=80., lmax=900., facns=1., facnlt=2., tdecmin=2.,
                 tdecmax=20., factdec=1., sloptdec=-1.28, Qmax=1e-3, slopQ=-2., lmeso=300., tmeso=20.,
                 norm_time=True, flux=False, time_ref=0.0):
        self.__dict__.update(dict(npsp=npsp, facpsp=facpsp, lmin=lmin, lmax=lmax, facns=facns, facnlt=facnlt,
                                  tdecmin=tdecmin, tdecmax=tdecmax, factdec=factdec, sloptdec=sloptdec,
                                  Qmax=Qmax, slopQ=slopQ, lmeso=lmeso, tmeso=tmeso, norm_time=norm_time,
                                  flux=flux, time_ref=time_ref))

    def to_c(self):
        return _lib.VdBmParams(*[float(getattr(self, k)) for k in (
            "npsp", "facpsp", "lmin", "lmax", "facns", "facnlt", "tdecmin", "tdecmax", "factdec", "sloptdec",
            "Qmax", "slopQ", "lmeso", "tmeso")], int(bool(self.norm_time)), int(bool(self.flux)),
            float(self.time_ref))


class BMPlan(_SeparablePlan):
    """Wave-packet basis (Basis_bm, basis.py:472-1168) on a rectilinear grid."""

    _prefix = "vd_bm"

    def __init__(self, xc, yc, time, params, land=None, geographic=False, dtype=torch.float32, device=None,
                 host_only=False):
        self._grid(xc, yc, time, land, geographic, dtype, device, host_only)
        self.params = params
        h = ctypes.c_void_p()
        pc = params.to_c()
        with self._on_device():
            _lib.check(self.lib.vd_bm_plan_create(ctypes.byref(h), ctypes.byref(self._gridc), ctypes.byref(pc)),
                       "vd_bm_plan_create")
        self._h = h
        self.nbasis = int(self.lib.vd_bm_nbasis(h))
        nf, nth = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.vd_bm_shape(h, ctypes.byref(nf), ctypes.byref(nth), None), "vd_bm_shape")
        self.nf, self.ntheta = nf.value, nth.value
        self.theta = np.zeros(self.ntheta)
        _lib.check(self.lib.vd_bm_shape(h, None, None, self.theta.ctypes.data), "vd_bm_shape")

    def frequency(self, iff):
        """(ff, tdec, offset, n time centres, n space centres) of frequency iff."""
        ff, td, off, nt, ns = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong(), ctypes.c_int(), \
            ctypes.c_int()
        _lib.check(self.lib.vd_bm_frequency(self._h, iff, ctypes.byref(ff), ctypes.byref(td), ctypes.byref(off),
                                            ctypes.byref(nt), ctypes.byref(ns)), "vd_bm_frequency")
        return ff.value, td.value, off.value, nt.value, ns.value

    def lattice(self, iff):
        _, _, _, nt, ns = self.frequency(iff)
        enst, lat, lon = np.zeros(nt), np.zeros(ns), np.zeros(ns)
        _lib.check(self.lib.vd_bm_lattice(self._h, iff, enst.ctypes.data, lat.ctypes.data, lon.ctypes.data),
                   "vd_bm_lattice")
        return enst, lat, lon

    def time_weights(self, k, iff):
        n = ctypes.c_int()
        _lib.check(self.lib.vd_bm_time_weights(self._h, k, iff, ctypes.byref(n), None, None),
                   "vd_bm_time_weights")
        it = np.zeros(max(n.value, 1), dtype=np.int32)
        w = np.zeros(max(n.value, 1))
        _lib.check(self.lib.vd_bm_time_weights(self._h, k, iff, ctypes.byref(n), it.ctypes.data, w.ctypes.data),
                   "vd_bm_time_weights")
        return list(zip(it[:n.value].tolist(), w[:n.value].tolist()))


class WaveletParams:
    """Parameters of the wavelet basis (config.BASIS fields of
    Basis_wavelet3d, basis.py:2647-2656)."""

    def __init__(self, npsp=3.5, facpsp=1.5, facnst=1., lmin=80., lmax=900., tmin=2., tmax=20., sigma_Q=1.0):
        self.__dict__.update(dict(npsp=npsp, facpsp=facpsp, facnst=facnst, lmin=lmin, lmax=lmax, tmin=tmin,
                                  tmax=tmax, sigma_Q=sigma_Q))

    def to_c(self):
        return _lib.VdWaveletParams(*[float(getattr(self, k)) for k in (
            "npsp", "facpsp", "facnst", "lmin", "lmax", "tmin", "tmax", "sigma_Q")])


class WaveletPlan(BMPlan):
    """Wavelet basis (Basis_wavelet3d, basis.py:2640-2985) on a rectilinear
    grid: the wave-packet plan's atoms and kernels with the wavelet lattice
    and Gaspari-Cohn time weights."""

    def __init__(self, xc, yc, time, params, land=None, geographic=False, dtype=torch.float32, device=None,
                 host_only=False):
        self._grid(xc, yc, time, land, geographic, dtype, device, host_only)
        self.params = params
        h = ctypes.c_void_p()
        pc = params.to_c()
        with self._on_device():
            _lib.check(self.lib.vd_wavelet_plan_create(ctypes.byref(h), ctypes.byref(self._gridc), ctypes.byref(pc)),
                       "vd_wavelet_plan_create")
        self._h = h
        self.nbasis = int(self.lib.vd_bm_nbasis(h))
        nf, nth = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.vd_bm_shape(h, ctypes.byref(nf), ctypes.byref(nth), None), "vd_bm_shape")
        self.nf, self.ntheta = nf.value, nth.value
        self.theta = np.zeros(self.ntheta)
        _lib.check(self.lib.vd_bm_shape(h, None, None, self.theta.ctypes.data), "vd_bm_shape")


class BMauxParams:
    """Parameters of the wave-packet basis with auxiliary fields (config.BASIS
    fields of Basis_bmaux, basis.py:1748-1765) and the auxiliary fields
    themselves: ``aux`` = dict(f, lat, lon, Tdec, Std), Tdec / Std
    [f][lat][lon] on ascending coordinates in the grid's longitude
    convention (Basis_bmaux.prepare_aux puts a dataset in that form)."""

    def __init__(self, aux, npsp=3.5, facpsp=1.5, lmin=80., lmax=900., facns=1., facnlt=2., tdecmin=2.,
                 tdecmax=20., factdec=1., facQ=1., norm_time=True, flux=False, time_ref=0.0):
        self.__dict__.update(dict(npsp=npsp, facpsp=facpsp, lmin=lmin, lmax=lmax, facns=facns, facnlt=facnlt,
                                  tdecmin=tdecmin, tdecmax=tdecmax, factdec=factdec, facQ=facQ,
                                  norm_time=norm_time, flux=flux, time_ref=time_ref))
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.aux = {k: c(aux[k]) for k in ("f", "lat", "lon", "Tdec", "Std")}
        shape = (self.aux["f"].size, self.aux["lat"].size, self.aux["lon"].size)
        for k in ("Tdec", "Std"):
            if self.aux[k].shape != shape:
                raise ValueError(f"aux['{k}'] must be [f, lat, lon] = {shape}")

    def to_c(self):
        dp = ctypes.POINTER(ctypes.c_double)
        a = self.aux
        return _lib.VdBmauxParams(*[float(getattr(self, k)) for k in (
            "npsp", "facpsp", "lmin", "lmax", "facns", "facnlt", "tdecmin", "tdecmax", "factdec", "facQ")],
            int(bool(self.norm_time)), int(bool(self.flux)), float(self.time_ref),
            a["f"].size, a["lat"].size, a["lon"].size, *[a[k].ctypes.data_as(dp) for k in (
                "f", "lat", "lon", "Tdec", "Std")])


class BMauxPlan(BMPlan):
    """Wave-packet basis with per-location decorrelation times and variances
    (Basis_bmaux, basis.py:1741-2638) on a rectilinear grid: the wave-packet
    plan's atoms and passes, after a per-centre time reduction."""

    def __init__(self, xc, yc, time, params, land=None, geographic=False, dtype=torch.float32, device=None,
                 host_only=False):
        self._grid(xc, yc, time, land, geographic, dtype, device, host_only)
        self.params = params
        h = ctypes.c_void_p()
        pc = params.to_c()
        with self._on_device():
            _lib.check(self.lib.vd_bmaux_plan_create(ctypes.byref(h), ctypes.byref(self._gridc), ctypes.byref(pc)),
                       "vd_bmaux_plan_create")
        self._h = h
        self.nbasis = int(self.lib.vd_bm_nbasis(h))
        nf, nth = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.vd_bm_shape(h, ctypes.byref(nf), ctypes.byref(nth), None), "vd_bm_shape")
        self.nf, self.ntheta = nf.value, nth.value
        self.theta = np.zeros(self.ntheta)
        _lib.check(self.lib.vd_bm_shape(h, None, None, self.theta.ctypes.data), "vd_bm_shape")

    def lattice(self, iff):
        """(enst [NP][padded time centres], lat, lon) of frequency iff."""
        _, _, _, nt, ns = self.frequency(iff)
        enst, lat, lon = np.zeros((ns, nt)), np.zeros(ns), np.zeros(ns)
        _lib.check(self.lib.vd_bm_lattice(self._h, iff, enst.ctypes.data, lat.ctypes.data, lon.ctypes.data),
                   "vd_bm_lattice")
        return enst, lat, lon

    def centres(self, iff):
        """(tdec, norm_fact, time-centre count) per space centre of frequency iff."""
        ns = self.frequency(iff)[4]
        td, nrm, nt = np.zeros(ns), np.zeros(ns), np.zeros(ns, dtype=np.int32)
        _lib.check(self.lib.vd_bmaux_centres(self._h, iff, td.ctypes.data, nrm.ctypes.data, nt.ctypes.data),
                   "vd_bmaux_centres")
        return td, nrm, nt

    def time_weights(self, k, iff):
        raise NotImplementedError("the auxiliary-field basis weights time per space centre")


# ---------------------------------------------------------------------------
# Reference-facing classes
# ---------------------------------------------------------------------------
def _grid_axes(State):
    """1-D axes of a rectilinear State grid (lon varies along columns only,
    lat along rows only)."""
    lon = np.asarray(State.lon, dtype=np.float64)
    lat = np.asarray(State.lat, dtype=np.float64)
    if lon.ndim == 1 and lat.ndim == 1:
        return lon, lat
    if not (np.all(lon == lon[:1, :]) and np.all(lat == lat[:, :1])):
        raise NotImplementedError("the GPU basis needs a rectilinear grid (lon per column, lat per row)")
    return lon[0, :].copy(), lat[:, 0].copy()


def _params_from_config(cb):
    for name, bad in (("flag_variable_Q", True), ("compute_velocities", True)):
        if getattr(cb, name, False) == bad:
            raise NotImplementedError(f"config.BASIS.{name} is not supported by the GPU basis")
    if getattr(cb, "c_grid_var", None) is not None:
        raise NotImplementedError("config.BASIS.c_grid_var is not supported by the GPU basis")
    return Gauss3dParams(cb.sigma_D, cb.sigma_T, facns=cb.facns, facnlt=cb.facnlt, sigma_Q=cb.sigma_Q,
                         normalize_fact=cb.normalize_fact, flux=getattr(cb, "flux", False),
                         time_spinup=getattr(cb, "time_spinup", None))


def _to_tensor(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous(), True
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=device).to(dtype).contiguous(), False


class Basis_gauss3d:
    """Drop-in for Basis_gauss3d / Basis_gauss3d_jax (basis.py:1170-1739)
    with the GPU projection. Arrays may be NumPy (returned as NumPy) or torch
    tensors (returned as tensors on the plan's device)."""

    def __init__(self, config, State, multi_mode=False, dtype=torch.float32, device=None):
        self.params = _params_from_config(config.BASIS)
        self.name_mod_var = config.BASIS.name_mod_var
        self.multi_mode = multi_mode
        self.lon, self.lat = _grid_axes(State)
        self.geographic = True
        self.ny, self.nx = State.ny, State.nx
        self.mask = None
        if getattr(State, "mask", None) is not None and np.any(State.mask):
            self.mask = np.asarray(State.mask, dtype=bool)
        self.dtype = dtype
        self.device = torch.device(device or "cuda")
        self.plan = None

    def _components(self):
        return [self.params]

    def _make_plan(self, time):
        return BasisPlan(self.lon, self.lat, time, self._components(), land=self.mask,
                         geographic=self.geographic, dtype=self.dtype, device=self.device)

    def set_basis(self, time, return_q=False, **kwargs):
        self.plan = self._make_plan(time)
        self.nbasis = self.plan.nbasis
        self.time = np.asarray(time, dtype=np.float64)
        if return_q:
            Q = self.plan.q()
            return np.zeros_like(Q), Q

    def _phi(self, t, X):
        Xt, is_t = _to_tensor(X, self.dtype, self.device)
        phi = self.plan.project(self.plan.time_index(t), Xt.reshape(1, -1))[0]
        return phi, is_t

    def operg(self, t, X, State=None):
        """Projection to the grid (basis.py:1489-1524, 1690-1717)."""
        phi, is_t = self._phi(t, X)
        if State is None:
            return phi if is_t else phi.double().cpu().numpy()
        cur = State.get(self.name_mod_var)
        if not self.multi_mode or cur is None:
            State[self.name_mod_var] = phi if is_t else phi.double().cpu().numpy()
        else:
            State[self.name_mod_var] = cur + (phi if isinstance(cur, torch.Tensor) else phi.double().cpu().numpy())

    def operg_transpose(self, t, adState):
        """Coefficient adjoint; zeroes adState[name_mod_var] unless in
        multi mode (basis.py:1526-1555, 1719-1737)."""
        ad = adState.get(self.name_mod_var)
        if ad is None:
            ad = np.zeros((self.ny, self.nx))
        adt, is_t = _to_tensor(ad, self.dtype, self.device)
        adX = torch.zeros(1, self.nbasis, dtype=self.dtype, device=self.device)
        self.plan.project_T(self.plan.time_index(t), adt.reshape(1, self.ny, self.nx), adX)
        if not self.multi_mode:
            adState[self.name_mod_var] = ad * 0.
        return adX[0] if is_t else adX[0].double().cpu().numpy()


class Basis_bm(Basis_gauss3d):
    """Drop-in for Basis_bm / Basis_bm_jax (basis.py:472-1168) with the GPU
    projection; ``config.EXP.init_date`` gives the time reference of the
    wavelet time lattice (basis.py:527). Depth tapering (file_depth) and
    background files are not supported."""

    def __init__(self, config, State, multi_mode=False, dtype=torch.float32, device=None):
        cb = config.BASIS
        if getattr(cb, "file_depth", None) is not None:
            raise NotImplementedError("config.BASIS.file_depth is not supported by the GPU basis")
        if getattr(cb, "compute_velocities", False):
            raise NotImplementedError("config.BASIS.compute_velocities is not supported by the GPU basis")
        import datetime
        tref = (config.EXP.init_date - datetime.datetime(1950, 1, 1, 0)).total_seconds() / 24 / 3600
        self.params = BMParams(npsp=cb.npsp, facpsp=cb.facpsp, lmin=cb.lmin, lmax=cb.lmax, facns=cb.facns,
                               facnlt=cb.facnlt, tdecmin=cb.tdecmin, tdecmax=cb.tdecmax, factdec=cb.factdec,
                               sloptdec=cb.sloptdec, Qmax=cb.Qmax, slopQ=cb.slopQ, lmeso=cb.lmeso, tmeso=cb.tmeso,
                               norm_time=cb.norm_time, flux=getattr(cb, "flux", False), time_ref=tref)
        self.name_mod_var = cb.name_mod_var
        self.multi_mode = multi_mode
        self.lon, self.lat = _grid_axes(State)
        self.geographic = True
        self.ny, self.nx = State.ny, State.nx
        self.mask = None
        if getattr(State, "mask", None) is not None and np.any(State.mask):
            self.mask = np.asarray(State.mask, dtype=bool)
        self.dtype = dtype
        self.device = torch.device(device or "cuda")
        self.plan = None

    def _make_plan(self, time):
        return BMPlan(self.lon, self.lat, time, self.params, land=self.mask, geographic=self.geographic,
                      dtype=self.dtype, device=self.device)


class Basis_multi:
    """Drop-in for Basis_multi (basis.py:4039-4135) over Gaussian components.
    ``config.BASIS`` maps names to component configs, as in the reference.
    One plan holds every component, so one projection call sums them into
    the parameter field (the reference zeroes it, then adds each component,
    basis.py:4097-4106); without a State the components' fields come back
    concatenated, as the reference's operg returns them (4108-4114)."""

    def __init__(self, config, State, verbose=True, dtype=torch.float32, device=None):
        subs = [config.BASIS[k] for k in config.BASIS]
        self.params = [_params_from_config(b) for b in subs]
        self.name_mod_var = subs[0].name_mod_var
        if any(b.name_mod_var != self.name_mod_var for b in subs):
            raise NotImplementedError("all components must project onto the same parameter")
        self.lon, self.lat = _grid_axes(State)
        self.ny, self.nx = State.ny, State.nx
        self.mask = None
        if getattr(State, "mask", None) is not None and np.any(State.mask):
            self.mask = np.asarray(State.mask, dtype=bool)
        self.dtype = dtype
        self.device = torch.device(device or "cuda")
        self.geographic = True
        self.multi_mode = False
        self.plan = None

    def _components(self):
        return list(self.params)

    _make_plan = Basis_gauss3d._make_plan
    set_basis = Basis_gauss3d.set_basis
    _phi = Basis_gauss3d._phi
    operg_transpose = Basis_gauss3d.operg_transpose

    def operg(self, t, X, State=None):
        if State is not None:
            return Basis_gauss3d.operg(self, t, X, State=State)
        Xt, is_t = _to_tensor(X, self.dtype, self.device)
        k = self.plan.time_index(t)
        parts = []
        for c in range(len(self.params)):
            off, nt, ns = self.plan.component(c)
            Xc = torch.zeros_like(Xt)
            Xc[off:off + nt * ns] = Xt[off:off + nt * ns]
            parts.append(self.plan.project(k, Xc.reshape(1, -1))[0].reshape(-1))
        phi = torch.cat(parts)
        return phi if is_t else phi.double().cpu().numpy()


class Basis_wavelet3d(Basis_gauss3d):
    """Drop-in for Basis_wavelet3d (basis.py:2640-2985) with the GPU
    projection; background files (path_background) are not supported."""

    def __init__(self, config, State, multi_mode=False, dtype=torch.float32, device=None):
        cb = config.BASIS
        pb = getattr(cb, "path_background", None)
        if pb is not None:
            import os
            if os.path.exists(pb):
                raise NotImplementedError("config.BASIS.path_background is not supported by the GPU basis")
        self.params = WaveletParams(npsp=cb.npsp, facpsp=cb.facpsp, facnst=cb.facnst, lmin=cb.lmin, lmax=cb.lmax,
                                    tmin=cb.tmin, tmax=cb.tmax, sigma_Q=cb.sigma_Q)
        self.name_mod_var = cb.name_mod_var
        self.multi_mode = multi_mode
        self.lon, self.lat = _grid_axes(State)
        self.geographic = True
        self.ny, self.nx = State.ny, State.nx
        self.mask = None
        if getattr(State, "mask", None) is not None and np.any(State.mask):
            self.mask = np.asarray(State.mask, dtype=bool)
        self.dtype = dtype
        self.device = torch.device(device or "cuda")
        self.plan = None

    def _make_plan(self, time):
        return WaveletPlan(self.lon, self.lat, time, self.params, land=self.mask, geographic=self.geographic,
                           dtype=self.dtype, device=self.device)


class Basis_bmaux(Basis_gauss3d):
    """Drop-in for Basis_bmaux / Basis_bmaux_jax (basis.py:1741-2638) with
    the GPU projection: the jax class's operg / operg_transpose (the numpy
    class's operg returns a field it never fills, 2303-2320).

    ``config.BASIS.file_aux`` is the auxiliary dataset the reference opens
    with xarray (1943-1950): here a mapping with 1-D ``lon``, ``lat``, ``f``
    and 3-D ``Tdec``, ``Std`` [f][lat][lon] (no NetCDF reader ships with this
    build); its longitudes are converted to the grid's convention and sorted
    as the reference does. Not supported (they raise): depth tapering
    (file_depth), a facQ_aux file, C-grid variables, geostrophic velocities
    and background files."""

    def __init__(self, config, State, multi_mode=False, dtype=torch.float32, device=None):
        cb = config.BASIS
        for name in ("file_depth", "file_facQaux", "c_grid_var"):
            if getattr(cb, name, None) is not None:
                raise NotImplementedError(f"config.BASIS.{name} is not supported by the GPU basis")
        if getattr(cb, "compute_velocities", False):
            raise NotImplementedError("config.BASIS.compute_velocities is not supported by the GPU basis")
        pb = getattr(cb, "path_background", None)
        if pb is not None:
            import os
            if os.path.exists(pb):
                raise NotImplementedError("config.BASIS.path_background is not supported by the GPU basis")
        import datetime
        tref = (config.EXP.init_date - datetime.datetime(1950, 1, 1, 0)).total_seconds() / 24 / 3600
        aux = self.prepare_aux(cb.file_aux, getattr(State, "lon_unit", "-180_180"))
        self.params = BMauxParams(aux, npsp=cb.npsp, facpsp=cb.facpsp, lmin=cb.lmin, lmax=cb.lmax, facns=cb.facns,
                                  facnlt=cb.facnlt, tdecmin=cb.tdecmin, tdecmax=cb.tdecmax, factdec=cb.factdec,
                                  facQ=cb.facQ, norm_time=cb.norm_time, flux=getattr(cb, "flux", False),
                                  time_ref=tref)
        self.name_mod_var = cb.name_mod_var
        self.multi_mode = multi_mode
        self.lon, self.lat = _grid_axes(State)
        self.geographic = True
        self.ny, self.nx = State.ny, State.nx
        self.mask = None
        if getattr(State, "mask", None) is not None and np.any(State.mask):
            self.mask = np.asarray(State.mask, dtype=bool)
        self.dtype = dtype
        self.device = torch.device(device or "cuda")
        self.plan = None

    @staticmethod
    def prepare_aux(ds, lon_unit):
        """The reference's longitude handling of the auxiliary dataset
        (basis.py:1944-1948): to [0, 360) for a '0_360' grid when the
        dataset has negative longitudes, to [-180, 180) for a '-180_180'
        grid when it has none or some above 180; then sorted by longitude."""
        lon = np.asarray(ds["lon"], dtype=np.float64)
        if np.sign(lon.min()) == -1 and lon_unit == "0_360":
            lon = lon % 360
        elif (np.sign(lon.min()) >= 0 or lon.max() > 180) and lon_unit == "-180_180":
            lon = (lon + 180) % 360 - 180
        order = np.argsort(lon, kind="stable")
        return dict(f=np.asarray(ds["f"], dtype=np.float64), lat=np.asarray(ds["lat"], dtype=np.float64),
                    lon=lon[order], Tdec=np.asarray(ds["Tdec"], dtype=np.float64)[..., order],
                    Std=np.asarray(ds["Std"], dtype=np.float64)[..., order])

    def _make_plan(self, time):
        return BMauxPlan(self.lon, self.lat, time, self.params, land=self.mask, geographic=self.geographic,
                         dtype=self.dtype, device=self.device)
