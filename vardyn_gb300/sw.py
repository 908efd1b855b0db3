"""Torch-facing wrapper of the multilayer rotating shallow-water model of
libvardyn_gb300 (mapping/models/model_qgsw/sw.py ``SW``).

Fields keep the reference's layout ``[n_ens, nl, x, y]``: u ``[.., nx+1, ny]``,
v ``[.., nx, ny+1]``, h ``[.., nx, ny]``; step inputs and outputs are physical
fields as in ``SW.step`` (sw.py:752-904). A :class:`SWPlan` owns one
``vd_sw_plan`` (metrics, Coriolis, masks, reference thickness, wind factors
and sponge rates on the GPU); the C calls run on torch's current stream.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .qg1l import _ptr, _stream

_FORCING = {"direct": 0, "mass_consistent": 1}


def _f64(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class SWMasks:
    """Masks of masks.py:57-158 from the library's host mask builder: float
    arrays ``h``, ``u``, ``v``, ``w``, ``psi`` (shapes of the reference without
    its two leading unit axes), the vorticity boundary classes, the WENO
    stencil selectors and the irregular psi-boundary indices. ``obc``: the
    open-boundary face masks of sw.py:365-369 (outer u / v faces 1)."""

    def __init__(self, nx, ny, mask=None, obc=False):
        m = None if mask is None else _f64(mask)
        if m is not None and m.shape != (nx, ny):
            raise ValueError(f"mask must be ({nx}, {ny}), got {m.shape}")
        fh = np.zeros((nx, ny), np.uint8)
        fu = np.zeros((nx + 1, ny), np.uint8)
        fv = np.zeros((nx, ny + 1), np.uint8)
        fw = np.zeros((nx + 1, ny + 1), np.uint8)
        _lib.call("vd_sw_masks", nx, ny, None if m is None else m.ctypes.data_as(ctypes.c_void_p),
                  fh.ctypes.data_as(ctypes.c_void_p), fu.ctypes.data_as(ctypes.c_void_p),
                  fv.ctypes.data_as(ctypes.c_void_p), fw.ctypes.data_as(ctypes.c_void_p))
        b = lambda f, k: ((f >> k) & 1).astype(np.float64)
        self.h, self.u, self.v = b(fh, 0), b(fu, 0), b(fv, 0)
        if obc:
            self.u[0, :] = self.u[-1, :] = 1.0
            self.v[:, 0] = self.v[:, -1] = 1.0
        self.w_valid, self.w_cornerout_bound = b(fw, 0), b(fw, 1)
        self.w_vertical_bound, self.w_horizontal_bound = b(fw, 2), b(fw, 3)
        self.w, self.psi = b(fw, 4), b(fw, 5)
        self.u_sten_hx_eq2, self.u_sten_hx_eq4, self.u_sten_hx_gt6 = b(fu, 1), b(fu, 2), b(fu, 3)
        self.u_sten_wy_eq2, self.u_sten_wy_eq4, self.u_sten_wy_gt4 = b(fu, 4), b(fu, 5), b(fu, 6)
        self.v_sten_hy_eq2, self.v_sten_hy_eq4, self.v_sten_hy_gt6 = b(fv, 1), b(fv, 2), b(fv, 3)
        self.v_sten_wx_eq2, self.v_sten_wx_eq4, self.v_sten_wx_gt6 = b(fv, 4), b(fv, 5), b(fv, 6)
        self.not_psi = 1.0 - self.psi
        # irregular psi boundary (masks.py:98-101): not psi, with a psi point
        # in its 3 x 3 neighbourhood
        p = self.psi
        nb = sum(p[a:a + nx - 1, c:c + ny - 1] for a in range(3) for c in range(3))
        self.psi_irrbound_xids, self.psi_irrbound_yids = np.where((p[1:-1, 1:-1] == 0) & (nb > 0))


class SWPlan:
    """Constants of one shallow-water configuration on one GPU; the keyword
    arguments are the reference's ``param`` keys (sw.py:103-383)."""

    def __init__(self, nx, ny, nl, dx, dy, f, H, g_prime, dt, mask=None, slip_coef=1.0, bottom_drag_coef=0.0,
                 rho_water=1025.0, h_min=0.1, h_min_sharpness=10.0, visc_coef=0.0, diff_coef=0.0, sponge_coef=0.0,
                 flag_linear=False, forcing_momentum="direct", h_wind=None, taux=0.0, tauy=0.0, sponge_u=None,
                 sponge_v=None, sponge_h=None, dtype=torch.float64, device=None, H_wind=None,
                 barotropic_filter=False, bf_lambd=None, flag_obc=False):
        """``H_wind`` (without ``h_wind``): the layer thicknesses the wind
        depth is taken from, when they differ from ``H`` (a model stepped
        with a perturbed H keeps its own H there, sw.py:622-630).

        ``barotropic_filter``: the spectral barotropic filter in every
        right-hand side (sw.py:305-320, 720-750), all-ocean masks only;
        ``bf_lambd`` its ``lambd`` (a scalar or an [nx, ny] field; None: from
        ``H``), which a model stepped with a perturbed H keeps from its own.
        ``flag_obc``: open boundaries (sw.py:353-371)."""
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        self.device = torch.device(device if device is not None else "cuda")
        self.nx, self.ny, self.nl = int(nx), int(ny), int(nl)
        self.dtype = dtype
        self.dt = float(dt)
        nx, ny, nl = self.nx, self.ny, self.nl
        if forcing_momentum not in _FORCING:
            raise ValueError(f"forcing_momentum must be one of {sorted(_FORCING)}")
        keep = []
        k = lambda a: (keep.append(a), a)[1]
        d = _lib.VdSwDesc()
        d.nx, d.ny, d.nl = nx, ny, nl
        d.dtype = _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32
        dxa = np.broadcast_to(_f64(dx), (nx, ny))
        dya = np.broadcast_to(_f64(dy), (nx, ny))
        d.dx_host = _dp(k(np.ascontiguousarray(dxa)))
        d.dy_host = _dp(k(np.ascontiguousarray(dya)))
        fa = _f64(f)
        if fa.shape != (nx + 1, ny + 1):
            raise ValueError(f"f must be ({nx + 1}, {ny + 1})")
        d.f_host = _dp(k(fa))
        Ha = _f64(H)
        if Ha.size == nl:
            d.H_spatial = 0
            d.H_host = _dp(k(Ha.reshape(nl)))
        else:
            d.H_spatial = 1
            d.H_host = _dp(k(np.ascontiguousarray(np.broadcast_to(Ha.reshape((nl,) + Ha.shape[-2:]), (nl, nx, ny)))))
        gp = _f64(g_prime).reshape(-1)
        if gp.size != nl:
            raise ValueError("g_prime needs one value per layer")
        d.g_prime_host = _dp(k(gp))
        self.mask = None if mask is None else _f64(mask)
        d.mask_host = _dp(k(self.mask)) if mask is not None else None
        d.slip_coef, d.bottom_drag_coef, d.rho_water = float(slip_coef), float(bottom_drag_coef), float(rho_water)
        d.h_min, d.h_min_sharpness = float(h_min), float(h_min_sharpness)
        d.visc_coef, d.diff_coef = float(visc_coef or 0.0), float(diff_coef or 0.0)
        d.dt, d.sponge_coef = float(dt), float(sponge_coef or 0.0)
        d.flag_linear = 1 if flag_linear else 0
        d.forcing_momentum = _FORCING[forcing_momentum]
        if h_wind is None:
            d.h_wind_mode = 0
            if H_wind is not None:
                Hw = _f64(H_wind)
                Hw0 = Hw.reshape(-1)[0] if Hw.size == nl else Hw.reshape((nl,) + Hw.shape[-2:])[0]
                d.Hwind_host = _dp(k(np.ascontiguousarray(np.broadcast_to(Hw0, (nx, ny)))))
        elif np.ndim(h_wind) == 0:
            d.h_wind_mode, d.h_wind_scalar = 1, float(h_wind)
        else:
            d.h_wind_mode = 2
            d.h_wind_host = _dp(k(np.ascontiguousarray(np.broadcast_to(_f64(h_wind), (nx, ny)))))
        for name, val, shape in (("taux", taux, (nx - 1, ny)), ("tauy", tauy, (nx, ny - 1))):
            if np.ndim(val) == 0:
                setattr(d, name + "_scalar", float(val))
            else:
                setattr(d, name + "_host", _dp(k(np.ascontiguousarray(np.broadcast_to(_f64(val), shape)))))
        for name, val, shape in (("sponge_u", sponge_u, (nx + 1, ny)), ("sponge_v", sponge_v, (nx, ny + 1)),
                                 ("sponge_h", sponge_h, (nx, ny))):
            if val is not None:
                setattr(d, name + "_host", _dp(k(np.ascontiguousarray(np.broadcast_to(_f64(val).reshape(
                    np.shape(val)[-2:]), shape)))))
        if barotropic_filter:
            d.barotropic_filter = 1
            if bf_lambd is not None:
                lam = _f64(bf_lambd)
                if lam.size == 1:
                    d.bf_lambd_host, d.bf_lambd_spatial = _dp(k(lam.reshape(1))), 0
                else:
                    d.bf_lambd_host = _dp(k(np.ascontiguousarray(np.broadcast_to(lam.reshape(lam.shape[-2:]),
                                                                                   (nx, ny)))))
                    d.bf_lambd_spatial = 1
        self.barotropic_filter = bool(barotropic_filter)
        d.flag_obc = 1 if flag_obc else 0
        self.masks = SWMasks(nx, ny, mask, obc=bool(flag_obc))
        self.forcing_momentum = forcing_momentum
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("vd_sw_plan_create", ctypes.byref(handle), ctypes.byref(d))
        self._h = handle
        self._lib = _lib.load()
        self._ws = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.vd_sw_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    # ---------------- buffers and shapes ----------------
    def shapes(self, batch):
        nx, ny, nl = self.nx, self.ny, self.nl
        return (batch, nl, nx + 1, ny), (batch, nl, nx, ny + 1), (batch, nl, nx, ny)

    def workspace(self, batch, nstep):
        nbytes = self._lib.vd_sw_workspace_bytes(self._h, batch, nstep)
        ws = self._ws.get("buf")
        if ws is None or ws.numel() < nbytes:
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._ws["buf"] = ws
        return ws

    def _field(self, x, shape, name):
        if x is None:
            return None
        x = torch.as_tensor(x, device=self.device)
        if x.dtype != self.dtype:
            x = x.to(self.dtype)
        if tuple(x.shape[-2:]) != shape[-2:] or x.numel() != int(np.prod(shape)):
            raise ValueError(f"{name} has shape {tuple(x.shape)}, expected {shape}")
        return x.reshape(shape).contiguous()

    def _uvh(self, u, v, h, B, prefix=""):
        su, sv, sh = self.shapes(B)
        return (self._field(u, su, prefix + "u"), self._field(v, sv, prefix + "v"), self._field(h, sh, prefix + "h"))

    def _batch(self, u):
        u = torch.as_tensor(u)
        return u.shape[0] if u.dim() == 4 else 1

    def _tau(self, taux, tauy):
        tx = None if taux is None else self._field(torch.as_tensor(taux, device=self.device).broadcast_to(
            (self.nx - 1, self.ny)), (self.nx - 1, self.ny), "taux")
        ty = None if tauy is None else self._field(torch.as_tensor(tauy, device=self.device).broadcast_to(
            (self.nx, self.ny - 1)), (self.nx, self.ny - 1), "tauy")
        return tx, ty

    # ---------------- API ----------------
    def step(self, u0, v0, h0, nstep=1, ub=None, vb=None, hb=None, Fu=None, Fv=None, Fh=None, taux=None, tauy=None):
        B = self._batch(u0)
        u0, v0, h0 = self._uvh(u0, v0, h0, B)
        ub, vb, hb = self._uvh(ub, vb, hb, B, "b_") if ub is not None else (None, None, None)
        Fu, Fv, Fh = self._fill_forcing(Fu, Fv, Fh, B)
        tx, ty = self._tau(taux, tauy)
        u1, v1, h1 = torch.empty_like(u0), torch.empty_like(v0), torch.empty_like(h0)
        ws = self.workspace(B, int(nstep))
        _lib.call("vd_sw_step", self._h, B, _ptr(u0), _ptr(v0), _ptr(h0), int(nstep), _ptr(ub), _ptr(vb), _ptr(hb),
                  _ptr(Fu), _ptr(Fv), _ptr(Fh), _ptr(tx), _ptr(ty), _ptr(u1), _ptr(v1), _ptr(h1), _ptr(ws),
                  ws.numel(), _stream())
        return u1, v1, h1

    def _fill_forcing(self, Fu, Fv, Fh, B):
        if Fu is None and Fv is None and Fh is None:
            return None, None, None
        su, sv, sh = self.shapes(B)
        z = lambda s: torch.zeros(s, dtype=self.dtype, device=self.device)
        return (self._field(Fu, su, "Fu") if Fu is not None else z(su),
                self._field(Fv, sv, "Fv") if Fv is not None else z(sv),
                self._field(Fh, sh, "Fh") if Fh is not None else z(sh))

    def step_tgl(self, u0, v0, h0, du0, dv0, dh0, nstep=1, ub=None, vb=None, hb=None, dub=None, dvb=None, dhb=None,
                 Fu=None, Fv=None, Fh=None, dFu=None, dFv=None, dFh=None, taux=None, tauy=None, dH=None,
                 dh_wind=None):
        """Tangent of :meth:`step`; ``dH`` (broadcast to [nl, nx, ny]) and
        ``dh_wind`` ([nx, ny], or a scalar for a scalar h_wind) perturb the
        layer thicknesses and the wind depth (vd_sw_set_ref_tangent)."""
        if dH is not None or dh_wind is not None:
            esz = 8 if self.dtype == torch.float64 else 4
            buf = torch.zeros(self._lib.vd_sw_ref_adj_bytes(self._h) // esz, dtype=self.dtype, device=self.device)
            dHh = None
            if dH is not None:
                a = np.asarray(dH.detach().cpu() if torch.is_tensor(dH) else dH, dtype=np.float64)
                while a.ndim < 3:
                    a = a[None]
                dHh = np.ascontiguousarray(np.broadcast_to(a, (self.nl, self.nx, self.ny)))
            dhw = None
            if dh_wind is not None:
                a = np.asarray(dh_wind.detach().cpu() if torch.is_tensor(dh_wind) else dh_wind, dtype=np.float64)
                dhw = np.ascontiguousarray(a.reshape(1) if a.size == 1 else np.broadcast_to(a, (self.nx, self.ny)))
            hp = lambda a: None if a is None else ctypes.c_void_p(a.ctypes.data)   # noqa: E731
            _lib.call("vd_sw_set_ref_tangent", self._h, hp(dHh), hp(dhw), _ptr(buf))
            try:
                return self.step_tgl(u0, v0, h0, du0, dv0, dh0, nstep=nstep, ub=ub, vb=vb, hb=hb, dub=dub, dvb=dvb,
                                     dhb=dhb, Fu=Fu, Fv=Fv, Fh=Fh, dFu=dFu, dFv=dFv, dFh=dFh, taux=taux, tauy=tauy)
            finally:
                _lib.call("vd_sw_set_ref_tangent", self._h, None, None, None)
        B = self._batch(u0)
        u0, v0, h0 = self._uvh(u0, v0, h0, B)
        du0, dv0, dh0 = self._uvh(du0, dv0, dh0, B, "d")
        ub, vb, hb = self._uvh(ub, vb, hb, B, "b_") if ub is not None else (None, None, None)
        if ub is not None and dub is not None:
            dub, dvb, dhb = self._uvh(dub, dvb, dhb, B, "db_")
        else:
            dub = dvb = dhb = None
        Fu, Fv, Fh = self._fill_forcing(Fu, Fv, Fh, B)
        dFu, dFv, dFh = self._fill_forcing(dFu, dFv, dFh, B)
        tx, ty = self._tau(taux, tauy)
        du1, dv1, dh1 = torch.empty_like(u0), torch.empty_like(v0), torch.empty_like(h0)
        ws = self.workspace(B, int(nstep))
        _lib.call("vd_sw_step_tgl", self._h, B, _ptr(u0), _ptr(v0), _ptr(h0), _ptr(du0), _ptr(dv0), _ptr(dh0),
                  int(nstep), _ptr(ub), _ptr(vb), _ptr(hb), _ptr(dub), _ptr(dvb), _ptr(dhb), _ptr(Fu), _ptr(Fv),
                  _ptr(Fh), _ptr(dFu), _ptr(dFv), _ptr(dFh), _ptr(tx), _ptr(ty), _ptr(du1), _ptr(dv1), _ptr(dh1),
                  _ptr(ws), ws.numel(), _stream())
        return du1, dv1, dh1

    def step_adj(self, u0, v0, h0, adu1, adv1, adh1, nstep=1, ub=None, vb=None, hb=None, Fu=None, Fv=None, Fh=None,
                 taux=None, tauy=None, want_bc=False, want_forcing=False, want_ref=False):
        """Adjoint of :meth:`step`; returns a dict with ``u0``, ``v0``, ``h0``
        and, when asked, ``ub``, ``vb``, ``hb`` / ``Fu``, ``Fv``, ``Fh`` /
        ``H`` (the cotangent of every layer's thickness, [nl, nx, ny]) and
        ``h_wind`` ([nx, ny]; zero unless the plan's h_wind is a field)."""
        if want_ref:
            esz = 8 if self.dtype == torch.float64 else 4
            buf = torch.zeros(self._lib.vd_sw_ref_adj_bytes(self._h) // esz, dtype=self.dtype,
                              device=self.device)
            _lib.call("vd_sw_set_ref_adj", self._h, _ptr(buf))
            try:
                out = self.step_adj(u0, v0, h0, adu1, adv1, adh1, nstep=nstep, ub=ub, vb=vb, hb=hb, Fu=Fu, Fv=Fv,
                                    Fh=Fh, taux=taux, tauy=tauy, want_bc=want_bc, want_forcing=want_forcing)
            finally:
                _lib.call("vd_sw_set_ref_adj", self._h, None)
            out["H"] = torch.empty((self.nl, self.nx, self.ny), dtype=self.dtype, device=self.device)
            out["h_wind"] = torch.empty((self.nx, self.ny), dtype=self.dtype, device=self.device)
            _lib.call("vd_sw_ref_pullback", self._h, _ptr(buf), _ptr(out["H"]), _ptr(out["h_wind"]), _stream())
            return out
        B = self._batch(u0)
        u0, v0, h0 = self._uvh(u0, v0, h0, B)
        a1 = self._uvh(adu1, adv1, adh1, B, "ad")
        ub, vb, hb = self._uvh(ub, vb, hb, B, "b_") if ub is not None else (None, None, None)
        Fu, Fv, Fh = self._fill_forcing(Fu, Fv, Fh, B)
        tx, ty = self._tau(taux, tauy)
        out = {"u0": torch.empty_like(u0), "v0": torch.empty_like(v0), "h0": torch.empty_like(h0)}
        bc = (torch.empty_like(u0), torch.empty_like(v0), torch.empty_like(h0)) if (want_bc and ub is not None) \
            else (None, None, None)
        fo = (torch.empty_like(u0), torch.empty_like(v0), torch.empty_like(h0)) if want_forcing else (None, None, None)
        ws = self.workspace(B, int(nstep))
        _lib.call("vd_sw_step_adj", self._h, B, _ptr(u0), _ptr(v0), _ptr(h0), _ptr(a1[0]), _ptr(a1[1]), _ptr(a1[2]),
                  int(nstep), _ptr(ub), _ptr(vb), _ptr(hb), _ptr(Fu), _ptr(Fv), _ptr(Fh), _ptr(tx), _ptr(ty),
                  _ptr(out["u0"]), _ptr(out["v0"]), _ptr(out["h0"]), _ptr(bc[0]), _ptr(bc[1]), _ptr(bc[2]),
                  _ptr(fo[0]), _ptr(fo[1]), _ptr(fo[2]), _ptr(ws), ws.numel(), _stream())
        if want_bc:
            out["ub"], out["vb"], out["hb"] = bc
        if want_forcing:
            out["Fu"], out["Fv"], out["Fh"] = fo
        return out

    def rhs(self, u, v, h, taux=None, tauy=None):
        """compute_time_derivatives of model-space fields (u dx, v dy,
        h area)."""
        B = self._batch(u)
        u, v, h = self._uvh(u, v, h, B)
        tx, ty = self._tau(taux, tauy)
        du, dv, dh = torch.empty_like(u), torch.empty_like(v), torch.empty_like(h)
        ws = self.workspace(B, 0)
        _lib.call("vd_sw_rhs", self._h, B, _ptr(u), _ptr(v), _ptr(h), _ptr(tx), _ptr(ty), _ptr(du), _ptr(dv),
                  _ptr(dh), _ptr(ws), ws.numel(), _stream())
        return du, dv, dh

    # ---------------- building blocks (model space) ----------------
    def rhs_tgl(self, u, v, h, du, dv, dh, taux=None, tauy=None):
        B = self._batch(u)
        u, v, h = self._uvh(u, v, h, B)
        du, dv, dh = self._uvh(du, dv, dh, B, "d")
        tx, ty = self._tau(taux, tauy)
        k = [torch.empty_like(a) for a in (u, v, h)]
        dk = [torch.empty_like(a) for a in (u, v, h)]
        ws = self.workspace(B, 0)
        _lib.call("vd_sw_rhs_tgl", self._h, B, _ptr(u), _ptr(v), _ptr(h), _ptr(du), _ptr(dv), _ptr(dh), _ptr(tx),
                  _ptr(ty), *[_ptr(a) for a in k + dk], _ptr(ws), ws.numel(), _stream())
        return tuple(k), tuple(dk)

    def rhs_adj(self, u, v, h, aku, akv, akh, out):
        """out (adu, adv, adh) += J_rhs(u, v, h)^T (aku, akv, akh)."""
        B = self._batch(u)
        ws = self.workspace(B, 0)
        _lib.call("vd_sw_rhs_adj", self._h, B, _ptr(u), _ptr(v), _ptr(h), _ptr(aku), _ptr(akv), _ptr(akh),
                  _ptr(out[0]), _ptr(out[1]), _ptr(out[2]), _ptr(ws), ws.numel(), _stream())

    @staticmethod
    def _ptrs(fields):
        arr = (ctypes.c_void_p * len(fields))(*[None if f is None else f.data_ptr() for f in fields])
        return arr

    def stage(self, B, stage, x, r, k0, k1, xb, F, ks, nxt):
        f = list(x) + list(r) + list(k0 or (None,) * 3) + list(k1 or (None,) * 3) + list(xb) + \
            list(F or (None,) * 3) + list(ks or (None,) * 3) + list(nxt)
        _lib.call("vd_sw_stage", self._h, B, stage, self._ptrs(f), _stream())

    def stage_adj(self, B, stage, adn, adk, a0, a1, adb):
        _lib.call("vd_sw_stage_adj", self._h, B, stage, self._ptrs(list(adn) + list(adk) + list(a0) + list(a1) +
                                                                   list(adb)), _stream())

    def scale(self, B, to_physical, x, out):
        _lib.call("vd_sw_scale", self._h, B, 1 if to_physical else 0, *[_ptr(a) for a in x],
                  *[_ptr(a) for a in out], _stream())

    def force_mc(self, B, x, F, out):
        _lib.call("vd_sw_force_mc", self._h, B, self._ptrs(list(x) + list(F) + list(out)), _stream())

    def force_mc_adj(self, B, x, Fh, ad, adFh):
        _lib.call("vd_sw_force_mc_adj", self._h, B, self._ptrs(list(x) + [Fh] + list(ad) + [adFh]), _stream())
