"""Drop-in QG 1.5-layer model class backed by the GB300 kernels.

Point the reference's ``config.MOD.dir_model`` at this directory: the model
wrapper loads ``{dir_model}/jqgm.py`` by path and instantiates
``getattr(module, config.MOD.name_class)`` with the keyword arguments of
mapping/src/mod.py:697-718, then calls ``step_jit(X, Xb, nstep=)``,
``step_tgl_jit(dX, X, Xb, nstep=)`` and ``step_adj_jit(adX, X, Xb, nstep=)``
(mod.py:721-723, 892, 991, 1055). ``Qgm`` here keeps those names, arguments
and return values (mapping/models/model_qg1l/jqgm.py:108-569); arrays may be
NumPy (returned as NumPy) or CUDA torch tensors (returned as tensors).

Precision follows the reference's global flag: float32 unless
``VARDYN_GB300_FLOAT64=1`` is set or ``dtype='float64'`` is passed.
"""
import ctypes
import os

import numpy as np
import torch

from vardyn_gb300.qg1l import QG1LPlan, build_mask


def _default_dtype():
    return torch.float64 if os.environ.get("VARDYN_GB300_FLOAT64", "0") == "1" else torch.float32


class Qgm:
    """QG 1.5-layer model with the constructor of jqgm.py:113."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None, upwind=3,
                 g=9.81, f=1e-4, time_scheme="Euler", compile=True, mdt=None,
                 bathymetry_PV_term=None, dtype=None, device=None, **kwargs):
        if dtype is None:
            dtype = _default_dtype()
        elif isinstance(dtype, str):
            dtype = torch.float64 if dtype == "float64" else torch.float32
        self.dtype = dtype
        ny, nx = np.shape(dx)
        self.ny, self.nx = ny, nx
        self.dx = float(np.asarray(dx)[int(ny / 2), int(nx / 2)])       # jqgm.py:126-131
        self.dy = float(np.asarray(dy)[int(ny / 2), int(nx / 2)])
        self.dt = float(dt)
        self.g = float(g)
        beta = None
        if np.ndim(f) > 0:                                               # jqgm.py:137-146
            fa = np.asarray(f, dtype=np.float64)
            self.f = float(np.nanmean(fa))
            beta = np.zeros((ny, nx))
            beta[1:-1, :] = (fa[2:, :] - fa[:-2, :]) / (2 * self.dy)
        else:
            self.f = float(f)
        self.c = float(np.nanmean(c)) if np.ndim(c) > 0 else float(c)  # jqgm.py:149-153
        self.upwind = upwind
        self.time_scheme = time_scheme
        self.Kdiffus = Kdiffus
        self.mask = build_mask(ny, nx, None if SSH is None else np.asarray(SSH))
        self.ind0 = self.mask == 0
        fb = None
        if bathymetry_PV_term is not None:
            fb = self.f * np.asarray(bathymetry_PV_term, dtype=np.float64)
        self.plan = QG1LPlan(ny, nx, self.dx, self.dy, self.dt, self.f, self.c, g=self.g,
                             time_scheme=time_scheme, dtype=dtype, Kdiffus=Kdiffus,
                             mask=self.mask, beta=beta, fbathy=fb, device=device)
        self.device = self.plan.device
        self._mdt = None if mdt is None else self._to_dev(mdt)
        # the reference binds jitted aliases (jqgm.py:221-236)
        self.h2uv_jit = self.h2uv
        self.h2pv_jit = self.h2pv
        self.pv2h_jit = self.pv2h
        self.rhs_jit = self.rhs
        self.step_jit = self.step
        self.step_tgl_jit = self.step_tgl
        self.step_adj_jit = self.step_adj

    # ---------------- conversions ----------------
    def _to_dev(self, x):
        if isinstance(x, torch.Tensor):
            return x.to(device=self.device, dtype=self.dtype).contiguous()
        return torch.as_tensor(np.asarray(x, dtype=np.float64), device=self.device).to(self.dtype).contiguous()

    def _wrap(self, like, *outs):
        res = [o.squeeze(0) if like.dim() == 2 else o for o in outs] if isinstance(like, torch.Tensor) else \
            [o.squeeze(0).cpu().numpy() if np.ndim(like) == 2 else o.cpu().numpy() for o in outs]
        return res[0] if len(res) == 1 else tuple(res)

    # ---------------- pieces ----------------
    def h2uv(self, h):
        u, v = self.plan.h2uv(self._to_dev(h))
        return self._wrap(h, u, v)

    def h2pv(self, h, hb, c=None):
        return self._wrap(h, self.plan.h2pv(self._to_dev(h), self._to_dev(hb)))

    def pv2h(self, q, hb, qb):
        return self._wrap(q, self.plan.pv2h(self._to_dev(q), self._to_dev(hb), self._to_dev(qb)))

    def rhs(self, u, v, q, way=1):
        if way != 1:
            raise NotImplementedError("way=-1 is not used by any caller of the reference")
        return self._wrap(q, self.plan.rhs(self._to_dev(u), self._to_dev(v), self._to_dev(q)))

    # ---------------- model ----------------
    def _mdt_in(self, h0, hb):
        if self._mdt is None:
            return h0, hb
        return h0 + self._mdt, hb + self._mdt

    def step(self, h0, hb, nstep=1):
        """nstep steps of the model from SSH h0 (jqgm.py:517-557)."""
        H0, HB = self._mdt_in(self._to_dev(h0), self._to_dev(hb))
        out = self.plan.step(H0, HB, int(nstep))
        if self._mdt is not None:
            out = out - self._mdt
        return self._wrap(h0, out)

    def step_tgl(self, dh0, h0, hb, nstep=1):
        """Tangent linear of :meth:`step` w.r.t. h0 (jqgm.py:559-563)."""
        H0, HB = self._mdt_in(self._to_dev(h0), self._to_dev(hb))
        return self._wrap(h0, self.plan.step_tgl(self._to_dev(dh0), H0, HB, int(nstep)))

    def step_adj(self, adh0, h0, hb, nstep=1):
        """Adjoint of :meth:`step` w.r.t. h0 (jqgm.py:565-569)."""
        H0, HB = self._mdt_in(self._to_dev(h0), self._to_dev(hb))
        return self._wrap(h0, self.plan.step_adj(self._to_dev(adh0), H0, HB, int(nstep)))


class Qgm_sf(Qgm):
    """Streamfunction form of the model with the constructor of jqgm.py:576.

    The state is phi = g/f h with f the (possibly varying) Coriolis field
    (jqgm.py:1004-1005); PV q = lap(phi) - (f0/c)^2 phi with f0 = mean(f)
    (606, 724-741), the inversion lap_dst - (f0/c)^2 (627-631), velocities
    from phi without the g/f factor (698-719), the bathymetry term f*bathymetry
    with the f field (819-820), the same beta and mask as Qgm. In phi these
    are Qgm's equations with g = f = f0 and the bathymetry term scaled by
    f/f0, so the GPU plan is built that way; the conversions h <-> phi are
    pointwise scalings (their own adjoints). ``phi2uv``, ``phi2pv``,
    ``pv2phi`` and ``rhs`` act on phi as in the reference."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None, upwind=3,
                 g=9.81, f=1e-4, time_scheme="Euler", compile=True, mdt=None,
                 bathymetry_PV_term=None, dtype=None, device=None, **kwargs):
        ny, nx = np.shape(dx)
        f_arr = np.broadcast_to(np.asarray(f, dtype=np.float64), (ny, nx))
        f0 = float(np.mean(f_arr))
        bathy = None
        if bathymetry_PV_term is not None:
            bathy = np.asarray(bathymetry_PV_term, dtype=np.float64) * (f_arr / f0)
        super().__init__(dx=dx, dy=dy, dt=dt, SSH=SSH, c=c, Kdiffus=Kdiffus, upwind=upwind, g=f0,
                         f=(np.asarray(f, dtype=np.float64) if np.ndim(f) > 0 else f0),
                         time_scheme=time_scheme, compile=compile, mdt=None, bathymetry_PV_term=bathy,
                         dtype=dtype, device=device)
        self.g = float(g)
        self.f0 = f0
        self._s = self._to_dev(self.g / f_arr)          # h -> phi
        self._sinv = self._to_dev(f_arr / self.g)       # phi -> h
        self._mdt = None if mdt is None else self._to_dev(mdt)
        self.phi2uv_jit = self.phi2uv
        self.phi2pv_jit = self.phi2pv
        self.pv2phi_jit = self.pv2phi

    def phi2uv(self, phi):
        return Qgm.h2uv(self, phi)

    def phi2pv(self, phi, phib, c=None):
        return Qgm.h2pv(self, phi, phib)

    def pv2phi(self, q, phib, qb):
        return Qgm.pv2h(self, q, phib, qb)

    def _phi_in(self, h0, hb):
        H0, HB = self._mdt_in(self._to_dev(h0), self._to_dev(hb))
        return self.plan.scale(H0, self._s), self.plan.scale(HB, self._s)

    def step(self, h0, hb, nstep=1):
        """nstep steps from SSH h0 (jqgm.py:981-1021)."""
        P0, PB = self._phi_in(h0, hb)
        out = self.plan.scale(self.plan.step(P0, PB, int(nstep)), self._sinv)
        if self._mdt is not None:
            out = out - self._mdt
        return self._wrap(h0, out)

    def step_tgl(self, dh0, h0, hb, nstep=1):
        """Tangent linear of :meth:`step` w.r.t. h0 (jqgm.py:1023-1027)."""
        P0, PB = self._phi_in(h0, hb)
        dP = self.plan.scale(self._to_dev(dh0), self._s)
        return self._wrap(h0, self.plan.scale(self.plan.step_tgl(dP, P0, PB, int(nstep)), self._sinv))

    def step_adj(self, adh0, h0, hb, nstep=1):
        """Adjoint of :meth:`step` w.r.t. h0 (jqgm.py:1029-1033)."""
        P0, PB = self._phi_in(h0, hb)
        adP = self.plan.scale(self._to_dev(adh0), self._sinv)
        return self._wrap(h0, self.plan.scale(self.plan.step_adj(adP, P0, PB, int(nstep)), self._s))


def _gaspari_cohn(r, c):
    """Gaspari-Cohn taper (jqgm.py:22-53): 1 at 0, zero beyond distance c."""
    ra = 2 * np.abs(np.asarray(r, dtype=np.float64)) / c
    gp = np.zeros_like(ra)
    i = ra <= 1.0
    gp[i] = -0.25 * ra[i] ** 5 + 0.5 * ra[i] ** 4 + 0.625 * ra[i] ** 3 - 5.0 / 3.0 * ra[i] ** 2 + 1.0
    i = (ra > 1.0) & (ra <= 2.0)
    gp[i] = (ra[i] ** 5 / 12.0 - 0.5 * ra[i] ** 4 + 0.625 * ra[i] ** 3 + 5.0 / 3.0 * ra[i] ** 2 - 5.0 * ra[i]
             + 4.0 - 2.0 / 3.0 / ra[i])
    return gp


class QgmWithTiles:
    """Overlapping-tile QG 1.5-layer model with the constructor of
    jqgm.py:1035-1085. ``step`` runs on the GPU (vd_qgt_step): every tile of
    ``tile_size`` (overlap ``tile_overlap``) is an independent QG1.5L model
    with the tile means of f and c and Dirichlet hb on its edge, the tiles are
    blended with Gaspari-Cohn tapers. ``time_scheme`` is 'Euler' or 'rk2' (the
    reference's tile model knows only these). The tangent linear and adjoint
    (jax.jvp / vjp of the blended step) run on the GPU too (vd_qgt_step_tgl /
    vd_qgt_step_adj)."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, Kdiffus=None, upwind=3, g=9.81, f=1e-4,
                 time_scheme="Euler", mdt=None, tile_size=64, tile_overlap=8, dtype=None, device=None, **kwargs):
        from vardyn_gb300 import _lib
        if time_scheme not in ("Euler", "rk2"):
            raise ValueError("QgmWithTiles steps with 'Euler' or 'rk2' (jqgm.py:1269-1276)")
        if dtype is None:
            dtype = _default_dtype()
        elif isinstance(dtype, str):
            dtype = torch.float64 if dtype == "float64" else torch.float32
        self.dtype = dtype
        self.device = torch.device(device if device is not None else "cuda")
        self._lib = _lib
        ny, nx = np.shape(dx)
        self.ny, self.nx = ny, nx
        self.dx = float(np.asarray(dx)[int(ny / 2), int(nx / 2)])       # jqgm.py:126-131
        self.dy = float(np.asarray(dy)[int(ny / 2), int(nx / 2)])
        self.dt, self.g = float(dt), float(g)
        self.time_scheme, self.Kdiffus = time_scheme, Kdiffus
        T, ov = int(tile_size), int(tile_overlap)
        if not (8 <= T <= min(ny, nx)) or not (0 < ov < T):
            raise ValueError("tile_size must lie in [8, min(ny, nx)] and 0 < tile_overlap < tile_size")
        esz = 8 if dtype == torch.float64 else 4
        need = _lib.load().vd_qgt_shared_bytes(T, _lib.VD_F64 if esz == 8 else _lib.VD_F32)
        if need > 227 * 1024:
            raise ValueError(f"tile_size {T} needs {need} B of shared memory per tile (more than 227 KiB)")
        self.tile_size, self.tile_overlap = T, ov
        self.mask = build_mask(ny, nx, None if SSH is None else np.asarray(SSH))
        fa = np.broadcast_to(np.asarray(f, dtype=np.float64), (ny, nx))
        ca = np.broadcast_to(np.asarray(c, dtype=np.float64), (ny, nx))
        # tiles (jqgm.py:1087-1101): the last tile of a row / column moved back inside
        tiles = []
        for y in range(0, ny, T - ov):
            for x in range(0, nx, T - ov):
                tiles.append((ny - T if y + T > ny else y, nx - T if x + T > nx else x))
        self.tiles = tiles
        org = np.asarray(tiles, dtype=np.int32)
        assert org.min() >= 0 and (org[:, 0] <= ny - T).all() and (org[:, 1] <= nx - T).all()
        ftile = np.array([np.nanmean(fa[a:a + T, b:b + T]) for a, b in tiles])       # jqgm.py:1313-1314
        ctile = np.array([np.nanmean(ca[a:a + T, b:b + T]) for a, b in tiles])
        # tile taper (jqgm.py:1069-1079)
        w = np.ones(T)
        gc = _gaspari_cohn(np.arange(0, T), ov)[:ov]
        w[:ov] = gc[::-1]
        w[-ov:] = gc
        wt = w[:, None] * w[None, :]
        wsum = np.zeros((ny, nx))
        for a, b in tiles:
            wsum[a:a + T, b:b + T] += wt
        # orthonormal DST-I of the tile interior and its Laplacian eigenvalues (jqgm.py:1063-1067)
        n = T - 2
        k = np.arange(1, n + 1)
        S = np.sqrt(2.0 / (n + 1)) * np.sin(np.pi * np.outer(k, k) / (n + 1))
        xg, yg = np.meshgrid(np.arange(1, T - 1, dtype=np.float64), np.arange(1, T - 1, dtype=np.float64))
        lap = 2 * (np.cos(np.pi / (T - 1) * xg) - 1) / self.dx ** 2 + 2 * (np.cos(np.pi / (T - 1) * yg) - 1) / \
            self.dy ** 2
        dev, R = self.device, dtype
        self._t = {
            "origins": torch.as_tensor(org.reshape(-1), device=dev),
            "f_tile": torch.as_tensor(ftile, dtype=torch.float64, device=dev),
            "c_tile": torch.as_tensor(ctile, dtype=torch.float64, device=dev),
            "mask": torch.as_tensor(self.mask.astype(np.int8), device=dev),
            "S": torch.as_tensor(S, device=dev).to(R).contiguous(),
            "lap": torch.as_tensor(lap, device=dev).to(R).contiguous(),
            "weights": torch.as_tensor(wt, device=dev).to(R).contiguous(),
            "wsum": torch.as_tensor(wsum, device=dev).to(R).contiguous(),
        }
        self._mdt = None if mdt is None else torch.as_tensor(np.asarray(mdt, dtype=np.float64),
                                                               device=dev).to(R).contiguous()
        d = _lib.VdQgtDesc()
        d.ny, d.nx, d.tile, d.ntiles = ny, nx, T, len(tiles)
        d.dtype = _lib.VD_F64 if esz == 8 else _lib.VD_F32
        d.time_scheme = 0 if time_scheme == "Euler" else 1
        d.has_Kdiffus = 0 if Kdiffus is None else 1
        d.dx, d.dy, d.dt, d.g = self.dx, self.dy, self.dt, self.g
        d.Kdiffus = 0.0 if Kdiffus is None else float(Kdiffus)
        for key, val in self._t.items():
            setattr(d, key, val.data_ptr())
        d.mdt = None if self._mdt is None else self._mdt.data_ptr()
        self._desc = d
        self._work = torch.empty(_lib.load().vd_qgt_workspace_bytes(ctypes.byref(d)) // esz, dtype=R, device=dev)
        self._ad_work = {}
        self.step_jit = self.step
        self.step_tgl_jit = self.step_tgl
        self.step_adj_jit = self.step_adj

    def step(self, h0, hb, nstep=1):
        """QgmWithTiles.step (jqgm.py:1333-1356)."""
        as_np = not isinstance(h0, torch.Tensor)
        H0 = (h0 if not as_np else torch.as_tensor(np.asarray(h0, dtype=np.float64))).to(
            device=self.device, dtype=self.dtype).contiguous()
        HB = (hb if isinstance(hb, torch.Tensor) else torch.as_tensor(np.asarray(hb, dtype=np.float64))).to(
            device=self.device, dtype=self.dtype).contiguous()
        if tuple(H0.shape) != (self.ny, self.nx) or tuple(HB.shape) != (self.ny, self.nx):
            raise ValueError(f"h0 and hb must be ({self.ny}, {self.nx})")
        out = torch.empty_like(H0)
        self._lib.call("vd_qgt_step", ctypes.byref(self._desc), ctypes.c_void_p(H0.data_ptr()),
                       ctypes.c_void_p(HB.data_ptr()), int(nstep), ctypes.c_void_p(out.data_ptr()),
                       ctypes.c_void_p(self._work.data_ptr()), self._work.numel() * self._work.element_size(),
                       ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return out.cpu().numpy() if as_np else out

    def _field(self, x):
        t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.float64))
        t = t.to(device=self.device, dtype=self.dtype).contiguous()
        if tuple(t.shape) != (self.ny, self.nx):
            raise ValueError(f"fields must be ({self.ny}, {self.nx})")
        return t

    def _ad(self, name, adjoint, x, h0, hb, nstep):
        as_np = not isinstance(h0, torch.Tensor)
        X, H0, HB = self._field(x), self._field(h0), self._field(hb)
        nbytes = self._lib.load().vd_qgt_ad_workspace_bytes(ctypes.byref(self._desc), int(nstep), int(adjoint))
        esz = X.element_size()
        key = (adjoint, int(nstep))
        if self._ad_work.get(key) is None:
            self._ad_work = {key: torch.empty(nbytes // esz, dtype=self.dtype, device=self.device)}
        work = self._ad_work[key]
        out = torch.empty_like(H0)
        self._lib.call(name, ctypes.byref(self._desc), ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(H0.data_ptr()),
                       ctypes.c_void_p(HB.data_ptr()), int(nstep), ctypes.c_void_p(out.data_ptr()),
                       ctypes.c_void_p(work.data_ptr()), work.numel() * esz,
                       ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return out.cpu().numpy() if as_np else out

    def step_tgl(self, dh0, h0, hb, nstep=1):
        """jax.jvp of the blended step with respect to h0 (jqgm.py:1358-1362),
        on the GPU (vd_qgt_step_tgl); zero on land."""
        return self._ad("vd_qgt_step_tgl", 0, dh0, h0, hb, nstep)

    def step_adj(self, adh0, h0, hb, nstep=1):
        """jax.vjp of the blended step with respect to h0 (jqgm.py:1364-1376),
        on the GPU (vd_qgt_step_adj): the adjoint keeps every tile's stage
        inputs of every step in its workspace."""
        return self._ad("vd_qgt_step_adj", 1, adh0, h0, hb, nstep)


class Qgm_trac(Qgm):
    """QG 1.5-layer model with passive tracers, with the constructor of
    jqgm.py:1553-1697. ``step(X0, Xb, nstep)`` runs on the GPU
    (vd_qgtrac_step): X0 is the SSH [ny, nx], or [SSH, tracers...] stacked
    [1 + ntrac, ny, nx], Xb the boundary fields of the same shape; the result
    has the shape of X0, NaN on land (jqgm.py:2057-2139).

    - ``Wbc``: relaxation weights on rows/columns 1..n-2 (None or all zero: 1
      on the outer ring class, jqgm.py:1657-1661);
    - ``bc_trac``: 'OBC' for the open boundaries of Mellor (1996) on the
      edge, anything else for the boundary values on the ring classes;
    - ``advect_pv``: False leaves the PV only diffused;
    - ``time_scheme``: 'Euler', 'rk2', or 'rk4', the classical Runge-Kutta 4
      that the reference's rk4 for this class sets out to be (that one
      cannot run, jqgm.py:1924-1955).

    ``step_tgl`` / ``step_adj`` (jax.jvp / vjp of step, jqgm.py:2141-2151) run
    on the GPU too (vd_qgtrac_step_tgl / vd_qgtrac_step_adj).

    Not built: ``ageo_velocities`` (the reference's boundary stack then holds
    the ageostrophic fields, jqgm.py:2079, and its boundary loop indexes past
    the tracers)."""

    def __init__(self, dx=None, dy=None, dt=None, SSH=None, c=None, upwind=3, g=9.81, f=1e-4,
                 time_scheme="Euler", Wbc=None, Kdiffus=None, Kdiffus_trac=None, bc_trac="OBC", mdt=None,
                 ageo_velocities=False, advect_pv=True, dtype=None, device=None, **kwargs):
        from vardyn_gb300 import _lib
        if time_scheme not in ("Euler", "rk2", "rk4"):
            raise ValueError("Qgm_trac steps with 'Euler', 'rk2' or 'rk4'")
        if ageo_velocities:
            raise NotImplementedError("Qgm_trac with ageo_velocities is not built")
        super().__init__(dx=dx, dy=dy, dt=dt, SSH=SSH, c=c, Kdiffus=Kdiffus, upwind=upwind, g=g, f=f,
                         time_scheme=time_scheme, mdt=mdt, dtype=dtype, device=device)
        self._lib = _lib
        ny, nx = self.ny, self.nx
        if Wbc is None or np.all(np.asarray(Wbc) == 0.0):
            w = np.zeros((ny, nx))
            w[self.mask == 1] = 1.0
        else:
            w = np.asarray(Wbc, dtype=np.float64)
        if w.shape != (ny, nx):
            raise ValueError(f"Wbc must be [ny, nx] = {(ny, nx)}, got {w.shape}")
        if self._mdt is not None and tuple(self._mdt.shape) != (ny, nx):
            raise ValueError(f"mdt must be [ny, nx] = {(ny, nx)}, got {tuple(self._mdt.shape)}")
        self.Wbc = self._to_dev(w)
        self.Kdiffus_trac = Kdiffus_trac
        self.bc_trac = bc_trac
        self.advect_pv = bool(advect_pv)
        self.ageo_velocities = False
        self._ws = {}

    def _desc(self, ntrac):
        d = self._lib.VdQgtracDesc()
        d.ntrac = int(ntrac)
        d.time_scheme = self._lib.SCHEMES[self.time_scheme]
        d.advect_pv = 1 if self.advect_pv else 0
        d.bc_obc = 1 if self.bc_trac == "OBC" else 0
        d.has_Kdiffus_trac = 0 if self.Kdiffus_trac is None else 1
        d.Kdiffus_trac = 0.0 if self.Kdiffus_trac is None else float(self.Kdiffus_trac)
        d.wbc = self.Wbc.data_ptr()
        d.mdt = None if self._mdt is None else self._mdt.data_ptr()
        return d

    def step_windows(self, h0, c0, hb, cb, nstep=1):
        """Batched step on device tensors: h0, hb [B, ny, nx]; c0, cb
        [B, ntrac, ny, nx] (ntrac may be 0). Returns (h1, c1)."""
        h0, hb = self._to_dev(h0), self._to_dev(hb)
        c0, cb = self._to_dev(c0), self._to_dev(cb)
        B = h0.shape[0]
        if h0.dim() != 3 or hb.shape != h0.shape or h0.shape[1:] != (self.ny, self.nx):
            raise ValueError("h0 and hb must be [B, ny, nx] on the model grid")
        if c0.dim() != 4 or cb.shape != c0.shape or c0.shape[0] != B or c0.shape[2:] != (self.ny, self.nx):
            raise ValueError("c0 and cb must be [B, ntrac, ny, nx] with the batch of h0")
        nt = c0.shape[1]
        d = self._desc(nt)
        key = (B, nt)
        ws = self._ws.get(key)
        if ws is None:
            nbytes = self._lib.load().vd_qgtrac_workspace_bytes(self.plan.handle, ctypes.byref(d), B)
            if nbytes == 0:
                raise ValueError("vd_qgtrac_workspace_bytes rejected the configuration")
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        h1 = torch.empty_like(h0)
        c1 = torch.empty_like(c0)
        p = (lambda t: ctypes.c_void_p(t.data_ptr() if t.numel() else None))
        self._lib.call("vd_qgtrac_step", self.plan.handle, ctypes.byref(d), B, p(h0), p(c0), p(hb), p(cb),
                       int(nstep), p(h1), p(c1), p(ws), ws.numel(),
                       ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return h1, c1

    def step(self, X0, Xb, nstep=1):
        """nstep steps from X0 with boundary fields Xb (jqgm.py:2057-2139)."""
        X, XB = self._to_dev(X0), self._to_dev(Xb)
        if X.shape != XB.shape:
            raise ValueError("X0 and Xb must have the same shape")
        if X.dim() == 2:
            h1, _ = self.step_windows(X[None], X.new_empty((1, 0) + X.shape), XB[None],
                                      XB.new_empty((1, 0) + XB.shape), nstep)
            out = h1[0]
        elif X.dim() == 3:
            h1, c1 = self.step_windows(X[:1], X[None, 1:], XB[:1], XB[None, 1:], nstep)
            out = torch.cat([h1, c1[0]], dim=0)
        else:
            raise ValueError("X0 is [ny, nx] or [1 + ntrac, ny, nx]")
        return out if isinstance(X0, torch.Tensor) else out.cpu().numpy()

    def rhs(self, *args, **kwargs):
        raise NotImplementedError("Qgm_trac.rhs takes the stacked state; the GPU step fuses it")

    def _ad_windows(self, name, adjoint, h0, c0, hb, cb, xh, xc, nstep):
        h0, hb, xh = self._to_dev(h0), self._to_dev(hb), self._to_dev(xh)
        c0, cb, xc = self._to_dev(c0), self._to_dev(cb), self._to_dev(xc)
        B = h0.shape[0]
        if h0.dim() != 3 or hb.shape != h0.shape or xh.shape != h0.shape or h0.shape[1:] != (self.ny, self.nx):
            raise ValueError("h0, hb and the direction must be [B, ny, nx] on the model grid")
        if c0.dim() != 4 or cb.shape != c0.shape or xc.shape != c0.shape or c0.shape[0] != B or \
                c0.shape[2:] != (self.ny, self.nx):
            raise ValueError("c0, cb and the tracer direction must be [B, ntrac, ny, nx] with the batch of h0")
        nt = c0.shape[1]
        d = self._desc(nt)
        nbytes = self._lib.load().vd_qgtrac_ad_workspace_bytes(self.plan.handle, ctypes.byref(d), B, int(nstep),
                                                                int(adjoint))
        if nbytes == 0:
            raise ValueError("vd_qgtrac_ad_workspace_bytes rejected the configuration")
        key = ("ad", B, nt)
        ws = self._ws.get(key)
        if ws is None or ws.numel() < nbytes:
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        oh = torch.empty_like(h0)
        oc = torch.empty_like(c0)
        p = (lambda t: ctypes.c_void_p(t.data_ptr() if t.numel() else None))
        self._lib.call(name, self.plan.handle, ctypes.byref(d), B, p(h0), p(c0), p(hb), p(cb), p(xh), p(xc),
                       int(nstep), p(oh), p(oc), p(ws), ws.numel(),
                       ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return oh, oc

    def step_tgl_windows(self, dh0, dc0, h0, c0, hb, cb, nstep=1):
        """Batched tangent linear on device tensors (shapes of step_windows)."""
        return self._ad_windows("vd_qgtrac_step_tgl", 0, h0, c0, hb, cb, dh0, dc0, nstep)

    def step_adj_windows(self, adh1, adc1, h0, c0, hb, cb, nstep=1):
        """Batched adjoint on device tensors (shapes of step_windows)."""
        return self._ad_windows("vd_qgtrac_step_adj", 1, h0, c0, hb, cb, adh1, adc1, nstep)

    def _ad(self, adjoint, dX, X0, Xb, nstep):
        X, XB, D = self._to_dev(X0), self._to_dev(Xb), self._to_dev(dX)
        if X.shape != XB.shape or D.shape != X.shape:
            raise ValueError("the direction, X0 and Xb must have the same shape")
        f = self.step_adj_windows if adjoint else self.step_tgl_windows
        if X.dim() == 2:
            e = X.new_empty((1, 0) + tuple(X.shape))
            oh, _ = f(D[None], e, X[None], e, XB[None], e, nstep)
            out = oh[0]
        elif X.dim() == 3:
            oh, oc = f(D[:1], D[None, 1:], X[:1], X[None, 1:], XB[:1], XB[None, 1:], nstep)
            out = torch.cat([oh, oc[0]], dim=0)
        else:
            raise ValueError("X0 is [ny, nx] or [1 + ntrac, ny, nx]")
        return out if isinstance(X0, torch.Tensor) else out.cpu().numpy()

    def step_tgl(self, dX0, X0, Xb, way=1, nstep=1):
        """jax.jvp of step with respect to X0 (jqgm.py:2141-2145), on the GPU
        (vd_qgtrac_step_tgl); zero on land."""
        return self._ad(0, dX0, X0, Xb, nstep)

    def step_adj(self, adX0, X0, Xb, way=1, nstep=1):
        """jax.vjp of step with respect to X0 (jqgm.py:2147-2151), on the GPU
        (vd_qgtrac_step_adj); NaN in adX0 reads as 0."""
        return self._ad(1, adX0, X0, Xb, nstep)
